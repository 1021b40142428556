// Batched IC-GN (6-DOF first pass and 2-DOF Subpb1) as one persistent kernel.
//
// This header holds the kernel template and its device code.  Each team
// width is instantiated in its own translation units (icgn_batched_tw{1,2,4,8}.cu
// without the staged g footprint, icgn_batched_tw{1,2,4,8}s.cu with it) so
// that they compile in parallel; icgn_batched.cu holds the host side and the
// FP64 factor kernel.
//
// Teams of warps pull subsets from a global work queue and run each with the
// control flow, mask logic and result codes of the plain FP64 kernels
// (funICGNQuadtree.m / funICGN_Subpb1.m).  The queue is a counting sort by
// subset size; in the split form the large subsets go first to teams of
// several warps and the rest to single warps, smallest first, so that neither
// a large subset nor a small one that runs to the iteration limit starts late.
//
// Per-subset scratch (interpolated g tile, tempf for the 2-DOF form, four
// flood-fill bitmaps) lives in shared memory when the tile fits the team's
// shared slot and otherwise in a per-warp slice of a global scratch buffer, so
// occupancy is set by registers, not by the largest subset of the batch.
//
// Precision: warped positions are an integer base plus an FP32 offset;
// bicubic weights, interpolation and residuals are FP32.  The per-iteration
// sums (sum J g for the b-vector; the g statistics as one-pass sums shifted by
// meanf, so that the variance does not cancel) are per-lane FP32 FMA chains
// reduced across lanes in FP32, and so are the set-up's f statistics (two
// passes: the mean, then the sums around it) and the Hessian (it only scales
// the step, never the converged point).  The 6x6 Hessian is reduced,
// factorised (Cholesky, else LU with partial pivoting) and inverted in FP64
// once per subset; every iteration applies that FP64 inverse to the FP32
// right-hand side in double-float arithmetic (FP32 pairs with exact products
// and error-free sums, about 2^-48 relative), because GB300's FP64 pipe issues
// at a small fraction of the FP32 rate.  The warp-parameter update is FP32.
#pragma once

#include "device_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

template <int TW>
struct Team {
  int id;  // team index in the CTA
  int tl;  // thread index in the team
  static constexpr int TT = TW * 32;
  STDIC_DEV void sync() const {
    if constexpr (TW == 1) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(id + 1), "r"(TT) : "memory");
  }
  STDIC_DEV int any(int v, int* scr) const {
    const int r = __any_sync(0xffffffffu, v);
    if constexpr (TW == 1) return r;
    sync();
    if ((tl & 31) == 0) scr[tl >> 5] = r;
    sync();
    int o = 0;
#pragma unroll
    for (int k = 0; k < TW; ++k) o |= scr[k];
    sync();
    return o;
  }
  STDIC_DEV int sum_int(int v, int* scr) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if constexpr (TW == 1) return v;
    sync();
    if ((tl & 31) == 0) scr[tl >> 5] = v;
    sync();
    int s = 0;
#pragma unroll
    for (int k = 0; k < TW; ++k) s += scr[k];
    sync();
    return s;
  }
  // Team reduce-scatter of K <= 32 FP32 values: team thread k < K returns
  // the team total of v[k] (the others return partial sums).  Within a warp
  // each level exchanges half of the remaining values with the partner lane,
  // 31 shuffles in all instead of 5 K.
  template <int K>
  STDIC_DEV float scatter_sum32(const float (&v)[K], float* scr) const {
    static_assert(K <= 32, "at most 32 values");
    const int lane = tl & 31;
    float a[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = k < K ? v[k] : 0.f;
#pragma unroll
    for (int lev = 0; lev < 5; ++lev) {
      const int o = 16 >> lev, h = 16 >> lev;
      const bool up = (lane & o) != 0;
#pragma unroll
      for (int k = 0; k < h; ++k) {
        const float send = up ? a[k] : a[k + h];
        const float keep = up ? a[k + h] : a[k];
        a[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    }
    float t = a[0];  // warp total of v[lane]
    if constexpr (TW > 1) {
      sync();
      scr[(tl >> 5) * 32 + lane] = t;
      sync();
      t = 0.f;
#pragma unroll
      for (int w = 0; w < TW; ++w) t += scr[w * 32 + lane];
      sync();
    }
    return t;
  }
  // In-place team sum of K <= 16 FP32 values, every thread receiving the
  // totals: a warp reduce-scatter (value k ends in lanes 2k, 2k+1 after 16
  // shuffles), then K shuffles (or shared-memory reads across the team) to
  // give every lane all K totals; 16 + K shuffles instead of 5 K.
  template <int K>
  STDIC_DEV void sumf16(float (&v)[K], float* scr) const {
    static_assert(K <= 16, "at most 16 values");
    const int lane = tl & 31;
    float a[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = k < K ? v[k] : 0.f;
#pragma unroll
    for (int lev = 0; lev < 4; ++lev) {
      const int o = 16 >> lev, h = 8 >> lev;
      const bool up = (lane & o) != 0;
#pragma unroll
      for (int k = 0; k < h; ++k) {
        const float send = up ? a[k] : a[k + h];
        const float keep = up ? a[k + h] : a[k];
        a[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    }
    const float t = a[0] + __shfl_xor_sync(0xffffffffu, a[0], 1);  // total of value lane >> 1
    if constexpr (TW == 1) {
#pragma unroll
      for (int k = 0; k < K; ++k) v[k] = __shfl_sync(0xffffffffu, t, 2 * k);
    } else {
      sync();
      if ((lane & 1) == 0) scr[(tl >> 5) * 16 + (lane >> 1)] = t;
      sync();
#pragma unroll
      for (int k = 0; k < K; ++k) {
        float s2 = 0.f;
#pragma unroll
        for (int w = 0; w < TW; ++w) s2 += scr[w * 16 + k];
        v[k] = s2;
      }
      sync();
    }
  }
  // in-place team sum of K FP32 values (every thread receives the totals)
  template <int K>
  STDIC_DEV void sumf(float (&v)[K], float* scr) const {
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
    if constexpr (TW > 1) {
      sync();
      if ((tl & 31) == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) scr[k * TW + (tl >> 5)] = v[k];
      sync();
#pragma unroll
      for (int k = 0; k < K; ++k) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < TW; ++w) s += scr[k * TW + w];
        v[k] = s;
      }
      sync();
    }
  }
};

// P <- P o DeltaP^-1 (funICGNQuadtree.m:393-411) in FP32.  Every lane holds
// the same D and P and computes all six parameters, so the lanes stay
// identical without shuffles or lane-specialised branches.  Returns false (P
// unchanged) when det(DeltaP) == 0.
STDIC_DEV bool compose_warp(float P[6], const float D[6], int lane) {
  (void)lane;
  const float det = (1.f + D[0]) * (1.f + D[3]) - D[1] * D[2];
  if (!(det != 0.f)) return false;
  const float inv = 1.f / det;
  const float T0 = (-D[0] - D[0] * D[3] + D[1] * D[2]) * inv;
  const float T1 = -D[1] * inv;
  const float T2 = -D[2] * inv;
  const float T3 = (-D[3] - D[0] * D[3] + D[1] * D[2]) * inv;
  const float T4 = (-D[4] - D[3] * D[4] + D[2] * D[5]) * inv;
  const float T5 = (-D[5] - D[0] * D[5] + D[1] * D[4]) * inv;
  const float a = 1.f + P[0], d = 1.f + P[3];
  const float n0 = P[0] + (a * T0 + P[2] * T1);
  const float n1 = P[1] * (1.f + T0) + d * T1;
  const float n2 = a * T2 + P[2] * (1.f + T3);
  const float n3 = P[3] + (P[1] * T2 + d * T3);
  const float n4 = P[4] + (a * T4 + P[2] * T5);
  const float n5 = P[5] + (P[1] * T4 + d * T5);
  P[0] = n0; P[1] = n1; P[2] = n2; P[3] = n3; P[4] = n4; P[5] = n5;
  return true;
}

// Bounds test of the warp P over the tile [x1, x1+mx-1] x [y1, y1+my-1]: lanes
// 0..7 evaluate one coordinate of one corner each (the warp is affine); the
// integer node position is kept apart from the FP32 offset.
STDIC_DEV bool corners_oob_warp(const float P[6], int x0, int y0, int x1, int y1, int mx, int my,
                                int W, int H, int lane) {
  bool bad = false;
  if (lane < 8) {
    const int cn = lane >> 1;
    const float dx = (float)((cn & 1 ? x1 + mx - 1 : x1) - x0);
    const float dy = (float)((cn & 2 ? y1 + my - 1 : y1) - y0);
    if ((lane & 1) == 0) {
      const float o = (1.f + P[0]) * dx + P[2] * dy + P[4];
      bad = o < (float)(3 - x0) || o > (float)(W - 2 - x0);
    } else {
      const float o = P[1] * dx + (1.f + P[3]) * dy + P[5];
      bad = o < (float)(3 - y0) || o > (float)(H - 2 - y0);
    }
  }
  return __any_sync(0xffffffffu, bad);
}

// Runs of the set bits of A that contain a bit of S (S subset of A): adding S
// to A carries through each seeded run and clears it, so ((A + S) ^ A) & A
// marks every bit from the seed to the top of its run; the bit-reversed form
// gives the part below the seed.
STDIC_DEV uint64_t run_fill(uint64_t A, uint64_t S) {
  const uint64_t up = ((A + S) ^ A) & A;
  const uint64_t Ar = __brevll(A), Sr = __brevll(S);
  const uint64_t dn = __brevll(((Ar + Sr) ^ Ar) & Ar);
  return up | dn | S;
}

// bwselect on an m x n tile (m <= 64, n <= 96) by one warp with bitmaps: lane
// l owns the tile columns l, l+32, l+64 (fixed dim-2 index), each a 64-bit
// mask over dim 1.  Every round fills the seeded runs of each column and then
// lets each column take the pixels of its neighbour columns' selection
// (shifted by one for 8-connectivity); rounds repeat until no column changes,
// at most m*n rounds since each productive round adds a pixel.
STDIC_DEV void bwselect_warp_bits(const uint8_t* allow, uint8_t* sel, int m, int n, int r1, int c1,
                                  int conn) {
  const int lane = threadIdx.x & 31;
  uint64_t A[3], S[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int j = lane + 32 * c;
    uint64_t a = 0;
    if (j < n)
      for (int i = 0; i < m; ++i) a |= (uint64_t)(allow[i + j * m] != 0) << i;
    A[c] = a;
    S[c] = 0;
    if (r1 >= 1 && r1 <= m && c1 >= 1 && c1 <= n && j == c1 - 1) S[c] = a & (1ull << (r1 - 1));
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) S[c] = run_fill(A[c], S[c]);
  for (;;) {
    uint64_t L[3], R[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const uint64_t up = __shfl_up_sync(0xffffffffu, S[c], 1);
      const uint64_t dn = __shfl_down_sync(0xffffffffu, S[c], 1);
      const uint64_t wrapL = c > 0 ? __shfl_sync(0xffffffffu, S[c > 0 ? c - 1 : 0], 31) : 0ull;
      const uint64_t wrapR = c < 2 ? __shfl_sync(0xffffffffu, S[c < 2 ? c + 1 : 2], 0) : 0ull;
      L[c] = lane == 0 ? wrapL : up;
      R[c] = lane == 31 ? wrapR : dn;
    }
    bool changed = false;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      uint64_t nb = L[c] | R[c];
      if (conn == 8) nb |= (L[c] << 1) | (L[c] >> 1) | (R[c] << 1) | (R[c] >> 1);
      const uint64_t t = S[c] | (nb & A[c]);
      const uint64_t f = t != S[c] ? run_fill(A[c], t) : t;
      changed |= f != S[c];
      S[c] = f;
    }
    if (!__any_sync(0xffffffffu, changed)) break;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int j = lane + 32 * c;
    if (j < n)
      for (int i = 0; i < m; ++i) sel[i + j * m] = (uint8_t)((S[c] >> i) & 1);
  }
  __syncwarp();
}

// The same fill for m <= 32, n <= 32 with one 32-bit column word per lane.
STDIC_DEV uint32_t run_fill32(uint32_t A, uint32_t S) {
  const uint32_t up = ((A + S) ^ A) & A;
  const uint32_t Ar = __brev(A), Sr = __brev(S);
  const uint32_t dn = __brev(((Ar + Sr) ^ Ar) & Ar);
  return up | dn | S;
}

STDIC_DEV void bwselect_warp_bits32(const uint8_t* allow, uint8_t* sel, int m, int n, int r1, int c1,
                                    int conn) {
  const int lane = threadIdx.x & 31;
  uint32_t A = 0, S = 0;
  if (lane < n) {
    const uint8_t* col = allow + lane * m;
    for (int i = 0; i < m; ++i) A |= (uint32_t)(col[i] != 0) << i;
  }
  if (r1 >= 1 && r1 <= m && c1 >= 1 && c1 <= n && lane == c1 - 1) S = A & (1u << (r1 - 1));
  S = run_fill32(A, S);
  for (;;) {
    const uint32_t L = __shfl_up_sync(0xffffffffu, S, 1), R = __shfl_down_sync(0xffffffffu, S, 1);
    uint32_t nb = (lane > 0 ? L : 0u) | (lane < 31 ? R : 0u);
    if (conn == 8) nb |= (nb << 1) | (nb >> 1);
    const uint32_t t = S | (nb & A);
    const uint32_t f = t != S ? run_fill32(A, t) : t;
    const bool changed = f != S;
    S = f;
    if (!__any_sync(0xffffffffu, changed)) break;
  }
  if (lane < n) {
    uint8_t* col = sel + lane * m;
    for (int i = 0; i < m; ++i) col[i] = (uint8_t)((S >> i) & 1u);
  }
  __syncwarp();
}

// flood fill of bwselect restricted to a team (see bwselect_block): tiles up
// to 64 x 96 by the first warp of the team with bitmaps, larger ones by
// alternating sweeps of the whole team
template <int TW>
STDIC_DEV void bwselect_team(const Team<TW>& tm, const uint8_t* allow, uint8_t* sel_, int m, int n,
                             int r1, int c1, int conn, int* iscr) {
  if (m <= 64 && n <= 96) {
    tm.sync();
    if (tm.tl < 32) {
      if (m <= 32 && n <= 32) bwselect_warp_bits32(allow, sel_, m, n, r1, c1, conn);
      else bwselect_warp_bits(allow, sel_, m, n, r1, c1, conn);
    }
    tm.sync();
    return;
  }
  volatile uint8_t* sel = sel_;
  const int npx = m * n;
  for (int p = tm.tl; p < npx; p += tm.TT) sel[p] = 0;
  tm.sync();
  if (tm.tl == 0 && r1 >= 1 && r1 <= m && c1 >= 1 && c1 <= n) {
    const int s = (r1 - 1) + (c1 - 1) * m;
    if (allow[s]) sel[s] = 1;
  }
  tm.sync();
  for (;;) {
    int changed = 0;
    for (int j = tm.tl; j < n; j += tm.TT) {
      for (int i = 0; i < m; ++i) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
      for (int i = m - 1; i >= 0; --i) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
    }
    tm.sync();
    for (int i = tm.tl; i < m; i += tm.TT) {
      for (int j = 0; j < n; ++j) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
      for (int j = n - 1; j >= 0; --j) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
    }
    if (!tm.any(changed, iscr)) break;
  }
  tm.sync();
}

struct Frame32 {
  const float* __restrict__ f;
  const float* __restrict__ g;
  const uint8_t* __restrict__ mask;
  const float* __restrict__ gx;
  const float* __restrict__ gy;
  int W, H;
  STDIC_DEV float F(long long x1, long long y1) const { return __ldg(f + (y1 - 1) * W + (x1 - 1)); }
  STDIC_DEV float M(long long x1, long long y1) const {
    return (float)__ldg(mask + (y1 - 1) * W + (x1 - 1));
  }
  STDIC_DEV float GX(long long x1, long long y1) const {
    return __ldg(gx + (y1 - 4) * (long long)(W - 6) + (x1 - 4));
  }
  STDIC_DEV float GY(long long x1, long long y1) const {
    return __ldg(gy + (y1 - 4) * (long long)(W - 6) + (x1 - 4));
  }
};

STDIC_DEV bool crop_ok32(const Frame32& fr, long long x1, long long x3, long long y1, long long y3) {
  return x1 >= 4 && x3 <= fr.W - 3 && y1 >= 4 && y3 <= fr.H - 3;
}
STDIC_DEV bool mask_crop_ok32(const Frame32& fr, long long x1, long long x3, long long y1,
                              long long y3) {
  return x1 >= 1 && x3 <= fr.W && y1 >= 1 && y3 <= fr.H;
}

// Keys (a = -1/2) weights of the four taps at fractional offset d in [0, 1),
// in factored form: w0 = -d (1-d)^2 / 2, w1 = (1-d)(2 + 2d - 3d^2) / 2,
// w2 = d (1 + 4d - 3d^2) / 2, w3 = -d^2 (1-d) / 2.  They equal the expanded
// polynomials of ba_interp2.cpp, but in FP32 the expanded w0, w1 and w3 cancel
// catastrophically as d -> 1 (terms of order 1 summing to order (1-d)^2):
// there a weight of 1e-8 can come out as exactly 0, and an interpolated value
// that is tiny but nonzero in FP64 becomes 0, which changes the subset's
// selection of nonzero g pixels.  The factored forms keep every weight to a
// few FP32 ulps of its value, and a weight is exactly 0 only where it is 0 in
// exact arithmetic (d = 0).  1 - d is exact for d >= 1/2.
STDIC_DEV void keys_weights(float d, float& w0, float& w1, float& w2, float& w3) {
  const float e = 1.f - d, hd = 0.5f * d;
  w0 = -hd * e * e;
  w1 = 0.5f * e * fmaf(d, fmaf(-3.f, d, 2.f), 2.f);
  w2 = hd * fmaf(d, fmaf(-3.f, d, 4.f), 1.f);
  w3 = -hd * d * e;
}

// Bicubic sample of g at (iu + su, iv + sv): integer base + FP32 offset.
STDIC_DEV float cubic32(const float* __restrict__ g, int W, int H, int iu, float su, int iv,
                        float sv) {
  const float fu = floorf(su), fv = floorf(sv);
  const float dx = su - fu, dy = sv - fv;
  // 0-based first tap (x = dim 1); the FP64 corner test keeps positions in
  // [3, W-2] x [3, H-2], the clamp only guards FP32 rounding at that edge
  const int xb = min(max(iu + (int)fu - 2, 0), W - 4);
  const int yb = min(max(iv + (int)fv - 2, 0), H - 4);
  float wx0, wx1, wx2, wx3, wy0, wy1, wy2, wy3;
  keys_weights(dx, wx0, wx1, wx2, wx3);
  keys_weights(dy, wy0, wy1, wy2, wy3);
  const float* r = g + (long long)yb * W + xb;
  const float s0 = wx0 * __ldg(r) + wx1 * __ldg(r + 1) + wx2 * __ldg(r + 2) + wx3 * __ldg(r + 3);
  r += W;
  const float s1 = wx0 * __ldg(r) + wx1 * __ldg(r + 1) + wx2 * __ldg(r + 2) + wx3 * __ldg(r + 3);
  r += W;
  const float s2 = wx0 * __ldg(r) + wx1 * __ldg(r + 1) + wx2 * __ldg(r + 2) + wx3 * __ldg(r + 3);
  r += W;
  const float s3 = wx0 * __ldg(r) + wx1 * __ldg(r + 1) + wx2 * __ldg(r + 2) + wx3 * __ldg(r + 3);
  return wy0 * s0 + wy1 * s1 + wy2 * s2 + wy3 * s3;
}

// (i, j) of tile pixel p = i + j*mx, advanced by a fixed stride without division
struct PixIter {
  int i, j, di, dj, mx;
  STDIC_DEV PixIter(int p0, int stride, int mx_) : mx(mx_) {
    i = p0 % mx_; j = p0 / mx_; di = stride % mx_; dj = stride / mx_;
  }
  STDIC_DEV PixIter(const int4& start, int mx_) : i(start.x), j(start.y), di(start.z), dj(start.w), mx(mx_) {}
  STDIC_DEV void next() {
    i += di; j += dj;
    if (i >= mx) { i -= mx; ++j; }
  }
};

struct TeamCtl {
  // inverse Hessian of the team's current subset (6-DOF, row-major), split
  // into FP32 pairs hh + hl that carry its FP64 value to about 2^-48
  float hh[36], hl[36];
  float jf[6], j1[6];
  int item;
  int pad[3];
  unsigned long long mbar;  // completion barrier of the team's footprint copies (TMA)
};

// Double-float helpers: a pair (hi, lo) of FP32 values represents hi + lo.
// fp64 -> pair (exact to about 2^-48 relative)
STDIC_DEV void split_f64(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// sum_q (hh_q + hl_q) * x_q in double-float arithmetic, rounded once to FP32:
// each product is split exactly by an FMA into p_q + e_q, and the p_q are
// added pairwise (a tree of depth log2 K) by error-free TwoSums whose errors
// join the e_q, so the result matches an FP64 dot product of the same operands
// rounded to FP32, without using the FP64 pipe.  The tree keeps the chain of
// dependent operations short: this sits on the serial path of every iteration.
STDIC_DEV void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}
template <int K>
STDIC_DEV float dot_df(const float* hh, const float* hl, const float* x) {
  float p[K], e[K];
#pragma unroll
  for (int q = 0; q < K; ++q) {
    p[q] = __fmul_rn(hh[q], x[q]);
    e[q] = fmaf(hl[q], x[q], fmaf(hh[q], x[q], -p[q]));
  }
#pragma unroll
  for (int w = 1; w < K; w *= 2) {
#pragma unroll
    for (int q = 0; q + w < K; q += 2 * w) {
      float t, err;
      two_sum(p[q], p[q + w], t, err);
      p[q] = t;
      e[q] = __fadd_rn(__fadd_rn(e[q], e[q + w]), err);
    }
  }
  return __fadd_rn(p[0], e[0]);
}

// kg += J t for the 6-DOF steepest-descent images J = [dx gx, dx gy, dy gx,
// dy gy, gx, gy] of a pixel with masked gradients g2 = (gx, gy) at offset
// (dx, dy) from the node: (gx t, gy t) once, then scaled by dx and dy.
STDIC_DEV void add_jt6(float (&kg)[6], float2 g2, float dx, float dy, float t) {
  const float a = g2.x * t, b = g2.y * t;
  kg[0] = fmaf(dx, a, kg[0]);
  kg[1] = fmaf(dx, b, kg[1]);
  kg[2] = fmaf(dy, a, kg[2]);
  kg[3] = fmaf(dy, b, kg[3]);
  kg[4] += a;
  kg[5] += b;
}

// Team slot layout: per-pixel arrays, the staged g footprint, the control
// block and the reduction scratch.
// Bytes per tile pixel: 6-DOF: the masked gradients (float2) cached for the
// iterations, tempg and five bitmaps; 2-DOF: tempg, tempf and five bitmaps.
__host__ __device__ __forceinline__ int tile_px_bytes(bool two) { return two ? 13 : 17; }
__host__ __device__ __forceinline__ size_t tiles_bytes(int px, bool two) {
  return ((size_t)px * tile_px_bytes(two) + 127) / 128 * 128;
}
// Bytes of one warp's global scratch slice (the per-pixel arrays for npx_max
// pixels), a multiple of 16 so that every slice keeps the alignment of the
// buffer for its float arrays.
__host__ __device__ __forceinline__ size_t slice_bytes(int npx_max, bool two) {
  return ((size_t)npx_max * tile_px_bytes(two) + 15) / 16 * 16;
}
__host__ __device__ __forceinline__ size_t gtile_bytes(int gt) {
  return ((size_t)(gt > 0 ? gt : 0) * 4 + 127) / 128 * 128;
}
// a team's slot, a multiple of 128 bytes so that every team's staging area
// (right after its 128-byte-rounded tiles) starts on a 128-byte boundary
__host__ __device__ __forceinline__ size_t team_bytes(int px, bool two, int tw, int gt) {
  const size_t b = tiles_bytes(px, two) + gtile_bytes(gt) + sizeof(TeamCtl) + sizeof(float) * 32 * tw + 16 * tw + 64;
  return (b + 127) / 128 * 128;
}

// Asynchronous 4-byte global -> shared copy (no register staging) and the
// wait for all of this thread's copies.
STDIC_DEV void cp_async4(float* smem, const float* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
STDIC_DEV void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// cubic32 reading its 16 taps from a staged tile of g whose first element is
// image element (gx0, gy0) (0-based) and whose rows are gtw floats: the same
// taps and arithmetic as cubic32, so the same result.  Local indices are
// clamped to the tile, so a read never leaves it.
STDIC_DEV float cubic_tile(const float* __restrict__ gt, int gtw, int gth, int gx0, int gy0, int W,
                           int H, int iu, float su, int iv, float sv) {
  const float fu = floorf(su), fv = floorf(sv);
  const float dx = su - fu, dy = sv - fv;
  const int xb = min(max(iu + (int)fu - 2, 0), W - 4);
  const int yb = min(max(iv + (int)fv - 2, 0), H - 4);
  const int lx = min(max(xb - gx0, 0), gtw - 4), ly = min(max(yb - gy0, 0), gth - 4);
  float wx0, wx1, wx2, wx3, wy0, wy1, wy2, wy3;
  keys_weights(dx, wx0, wx1, wx2, wx3);
  keys_weights(dy, wy0, wy1, wy2, wy3);
  const float* r = gt + ly * gtw + lx;
  const float s0 = wx0 * r[0] + wx1 * r[1] + wx2 * r[2] + wx3 * r[3];
  r += gtw;
  const float s1 = wx0 * r[0] + wx1 * r[1] + wx2 * r[2] + wx3 * r[3];
  r += gtw;
  const float s2 = wx0 * r[0] + wx1 * r[1] + wx2 * r[2] + wx3 * r[3];
  r += gtw;
  const float s3 = wx0 * r[0] + wx1 * r[1] + wx2 * r[2] + wx3 * r[3];
  return wy0 * s0 + wy1 * s1 + wy2 * s2 + wy3 * s3;
}

}  // namespace

// TMA copy of a box x box float tile of the deformed frame at image position
// (x, y) (x a multiple of 4: TMA's 16-byte rule) into the team's staging
// area, completing on the team's mbarrier.  The fence orders the generic
// accesses that the team's synchronisation before this call has completed
// with the copy's writes (the area may have held other data).
STDIC_DEV void tma_box_issue(const CUtensorMap* map, float* dst, int x, int y, unsigned long long* mbar,
                             unsigned bytes) {
  const unsigned sbar = (unsigned)__cvta_generic_to_shared(mbar);
  const unsigned sdst = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sbar), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          sdst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(sbar)
      : "memory");
}

// Bounded wait for the completion of the mbarrier phase of the given parity.
STDIC_DEV bool tma_box_wait(unsigned long long* mbar, unsigned parity, int polls) {
  const unsigned sbar = (unsigned)__cvta_generic_to_shared(mbar);
  for (int it = 0; it < polls; ++it) {
    unsigned done;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done)
                 : "r"(sbar), "r"(parity)
                 : "memory");
    if (done) return true;
  }
  return false;
}

// One subset on one team: set-up, iterations and outputs.  base/ctl/fscr/iscr
// are the team's shared slot of smpx tile pixels, gt its staging area of gcap
// floats for the warped g footprint, gbase its global slice.
template <int TW, bool TWO, int STAGE, bool STG>
STDIC_DEV void run_subset(const BatchedArgs& B, const Team<TW>& tm, int item, unsigned char* base,
                          TeamCtl* ctl, float* fscr, int* iscr, unsigned char* gbase, int smpx,
                          float* gt, int gcap, unsigned& gphase, bool& tma_ok) {
  const IcgnArgs& a = B.a;
  const int lane = threadIdx.x & 31;
  constexpr int stage = STAGE;
  SubsetState6* st6 = (SubsetState6*)B.st6;
  const int Ntot = a.N * (B.frames > 0 ? B.frames : 1);
  const float tolf = (float)a.tol;
  const int node = item % a.N;
  const int frame = item / a.N;
  Frame32 fr{B.f32, B.g32 + (long long)frame * B.g_stride, a.mask, B.dfdx32, B.dfdy32, a.W, a.H};
  const long long x0 = llround(a.coords[node]), y0 = llround(a.coords[a.N + node]);

  // ---------------- per-subset set-up ----------------
  int wx, wy;
  float P[6];  // warp parameters [F11 F21 F12 F22 u v] in FP32
  if constexpr (TWO) {
    wx = a.wsl2[node]; wy = a.wsl2[a.N + node];
#pragma unroll
    for (int k = 0; k < 4; ++k) P[k] = (float)a.FOld[4 * item + k];
    P[4] = (float)a.UOld[2 * item]; P[5] = (float)a.UOld[2 * item + 1];
  } else {
    wx = wy = a.ws_list ? a.ws_list[node] : a.ws_all;
    P[0] = P[1] = P[2] = P[3] = 0.f;
    P[4] = (float)a.U0[2 * item]; P[5] = (float)a.U0[2 * item + 1];
  }
  const int ws0 = wx;
  float uold0 = 0.f, uold1 = 0.f, vd0 = 0.f, vd1 = 0.f;
  if constexpr (TWO) {
    uold0 = P[4]; uold1 = P[5];
    vd0 = (float)a.vdual[2 * item]; vd1 = (float)a.vdual[2 * item + 1];
  }
  long long x1 = x0 - wx / 2, x3 = x0 + wx / 2, y1 = y0 - wy / 2, y3 = y0 + wy / 2;
  int code = 0;
  bool nan_out = false;
  const int err_code = TWO ? 0 : -1;  // value the reference leaves on a run-time error
  int cntf = 0;
  float meanf = 0.f, bottomf = 0.f, sabs = 0.f;
  int mx = 0, my = 0, npx = 0, sc = 0, sr = 0;
  int4 pstart = make_int4(0, 0, 0, 0);  // PixIter start of this thread for the tile
  float* tg = nullptr;
  float* tf = nullptr;
  float2* gq = nullptr;  // 6-DOF iterations: (gx, gy) of each tile pixel times the f selection
  uint8_t *mtile = nullptr, *bwf = nullptr, *bwg = nullptr, *tmp = nullptr, *bwm8 = nullptr;
  bool have_m8 = false;  // bwm8 holds the 8-connected selection of the mask tile
  bool have_mtile = false;  // mtile holds the mask tile
  bool has_masked = false;
  bool decided = false;  // outputs of this subset already written by the set-up stage
  const double npx0 = (double)(wx + 1) * (double)(wy + 1);
  // 6-DOF set-up: the first pass keeps f .* mask of each pixel in the tile
  // slot's f plane when the window fits the slot; if the window then neither
  // grows nor holds a masked pixel, the tile is exactly that window and the
  // mask tile and f pass read it back instead of f and the mask
  bool fm_cached = false;

  // 6-DOF iterations: the subset's inverse Hessian pairs and f-side sums are
  // loaded here, with its state, and written to the control block after the
  // tile set-up, so that their latency overlaps the state's
  float2 hpre = make_float2(0.f, 0.f), hpre2 = make_float2(0.f, 0.f);
  float jpre = 0.f;
  if (stage == 2) {
    const float2* hp = reinterpret_cast<const float2*>(B.Hinv6) + (size_t)item * 36;
    if (tm.tl < 36) hpre = hp[tm.tl];
    if (tm.tl + tm.TT < 36) hpre2 = hp[tm.tl + tm.TT];
    if (tm.tl < 12) jpre = tm.tl < 6 ? st6[item].Jf[tm.tl] : st6[item].J1[tm.tl - 6];
    const SubsetState6 s6 = st6[item];
    if (s6.code != 0) {
      decided = true;
    } else {
      wx = wy = s6.ws;
      x1 = x0 - wx / 2; x3 = x0 + wx / 2; y1 = y0 - wy / 2; y3 = y0 + wy / 2;
      cntf = s6.cntf;
      has_masked = s6.masked != 0;
      meanf = s6.meanf; bottomf = s6.bottomf; sabs = s6.sabs;
    }
  } else {
    const bool crop_valid = !((wx & 1) || (wy & 1)) && wx >= 0 && wy >= 0 && wx <= a.ws_max &&
                            wy <= a.ws_max && mask_crop_ok32(fr, x1, x3, y1, y3);
    int nanf = 0;
    if (crop_valid) {
      const int mx0 = wx + 1, np0 = (wx + 1) * (wy + 1);
      const bool keep = STAGE == 1 && !TWO && np0 <= smpx;
      // the f plane of the tile slot as the tile set-up below lays it out
      float* fm = (float*)(base + 8 * (size_t)smpx);
      PixIter it(tm.tl, tm.TT, mx0);
      #pragma unroll 4
      for (int p = tm.tl; p < np0; p += tm.TT, it.next()) {
        const float t = fr.F(x1 + it.i, y1 + it.j) * fr.M(x1 + it.i, y1 + it.j);
        if (keep) fm[p] = t;
        if (t != t) nanf = 1;
        if (t == 0.f) ++cntf;
      }
      fm_cached = keep;
    }
    cntf = tm.sum_int(cntf, iscr);
    nanf = tm.any(nanf, iscr);
    if constexpr (!TWO) {
      if (a.mark && tm.tl == 0) a.mark[item] = (!crop_valid || cntf > 0) ? 1 : 0;
    }
    if (!crop_valid || !crop_ok32(fr, x1, x3, y1, y3) || nanf) {
      code = err_code; nan_out = true;
    } else if (!((double)cntf < 0.4 * npx0)) {
      code = kMaxIter + 2;
    } else if ((double)cntf > 0.0 * npx0) {
      fm_cached = false;  // masked pixels, and the window grows
      if constexpr (TWO) {
        {
          const double aa = (double)(wx + 1) * (double)(wy + 1);
          wx = (int)grow_window(aa, aa - (double)cntf, wx);
        }
        {
          const double aa = (double)(wx + 1) * (double)(wy + 1);
          wy = (int)grow_window(aa, aa - (double)cntf, wy);
        }
      } else {
        wx = wy = (int)grow_window(npx0, npx0 - (double)cntf, wx);
      }
      x1 = x0 - wx / 2; x3 = x0 + wx / 2; y1 = y0 - wy / 2; y3 = y0 + wy / 2;
      if (!mask_crop_ok32(fr, x1, x3, y1, y3) || !crop_ok32(fr, x1, x3, y1, y3) ||
          (wx + 1) * (wy + 1) > a.npx_max) {
        code = err_code; nan_out = true;
      }
    }
  }
  // tile storage, mask tile and the 4-connected f selection
  if (!decided && code == 0 && !nan_out) {
    mx = wx + 1; my = wy + 1; npx = mx * my;
    sc = (wx + 1) / 2; sr = (wy + 1) / 2;
    pstart = make_int4(tm.tl % mx, tm.tl / mx, tm.TT % mx, tm.TT / mx);
    const bool in_smem = npx <= smpx;
    const int cap = in_smem ? smpx : a.npx_max;
    unsigned char* stp = in_smem ? base : gbase;
    if constexpr (!TWO) {
      gq = (float2*)stp;
      stp += 8 * (size_t)cap;
    }
    tg = (float*)stp;
    tf = tg + cap;
    mtile = (uint8_t*)(tg + (TWO ? 2 : 1) * cap);
    bwf = mtile + cap;
    bwg = bwf + cap;
    tmp = bwg + cap;
    bwm8 = tmp + cap;
    // the mask tile: the set-up stage needs it to find masked subsets; the
    // iteration stage only for a masked subset (its f selection) and, lazily,
    // for the rare unmasked subset whose interpolated g has an exact zero
    if (fm_cached) {
      // no pixel of the window is masked (cntf == 0): every mask value is
      // nonzero, so the mask tile is all ones and the f selection is whole
      has_masked = false;
    } else if (stage != 2 || has_masked) {
      int z = 0;
      PixIter it(pstart, mx);
      #pragma unroll 4
      for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
        const uint8_t mk = __ldg(fr.mask + (y1 + it.j - 1) * fr.W + (x1 + it.i - 1)) != 0;
        mtile[p] = mk;
        if (!mk) z = 1;
      }
      have_mtile = true;
      if (stage != 2) has_masked = tm.any(z, iscr) != 0;
      if (has_masked) bwselect_team(tm, mtile, bwf, mx, my, sr, sc, 4, iscr);
    }
    tm.sync();
  }

  const uint8_t* bw = has_masked ? bwf : nullptr;  // nullptr: every pixel selected
  if constexpr (!TWO) {
    // the iterations' steepest-descent images depend on the fixed f selection
    // only: each thread caches the masked gradients of its own pixels
    if (stage == 2 && !decided && code == 0 && !nan_out) {
      PixIter it(pstart, mx);
      #pragma unroll 4
      for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
        const float s = bw ? (float)bw[p] : 1.f;
        gq[p] = make_float2(fr.GX(x1 + it.i, y1 + it.j) * s, fr.GY(x1 + it.i, y1 + it.j) * s);
      }
    }
  }
  constexpr int NQ = TWO ? 2 : 6;  // parameters of the b-vector
  // inverse of the 2x2 system (2-DOF) as double-float pairs: row k of lane k < 2
  float ih[2] = {0.f, 0.f}, il[2] = {0.f, 0.f};
  // f-side parts of b: jf = sum J (tempf - meanf), j1 = sum J
  float jf[NQ], j1[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) { jf[q] = 0.f; j1[q] = 0.f; }
  // steepest-descent images J of pixel (i, j): [dx gx, dx gy, dy gx, dy gy, gx, gy]
  // (6-DOF) or [gx, gy] (2-DOF), gx/gy masked by the current selection
  // the same from the cached gradients of pixel p (6-DOF iterations)
  auto jacq = [&](int p, int i, int j, float (&J)[NQ]) {
    if constexpr (!TWO) {
      const float2 g2 = gq[p];
      const float dx = (float)(int)(x1 + i - x0), dy = (float)(int)(y1 + j - y0);
      J[0] = dx * g2.x; J[1] = dx * g2.y; J[2] = dy * g2.x; J[3] = dy * g2.y; J[4] = g2.x; J[5] = g2.y;
    }
  };
  auto jac = [&](int i, int j, float s, float (&J)[NQ]) {
    const float gx = fr.GX(x1 + i, y1 + j) * s, gy = fr.GY(x1 + i, y1 + j) * s;
    if constexpr (TWO) {
      J[0] = gx; J[1] = gy;
    } else {
      const float dx = (float)(int)(x1 + i - x0), dy = (float)(int)(y1 + j - y0);
      J[0] = dx * gx; J[1] = dx * gy; J[2] = dy * gx; J[3] = dy * gy; J[4] = gx; J[5] = gy;
    }
  };
  // f-side statistics: Hessian (6x6 or 2x2), meanf, bottomf, sum |tempf|, jf, j1.
  // The 6-DOF set-up stage stores them; the 2-DOF form recomputes them when
  // the g selection changes (funICGN_Subpb1.m:171-190).
  auto f_side = [&]() {
    float hs[21];
#pragma unroll
    for (int k = 0; k < 21; ++k) hs[k] = 0.f;
    float sf = 0.f, nf = 0.f, sa = 0.f;
    PixIter it(pstart, mx);
    #pragma unroll 2
    for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
      const int i = it.i, j = it.j;
      const float s = bw ? (float)bw[p] : 1.f;
      const float fv = (fm_cached ? tg[p] : fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j)) * s;
      sa += fabsf(fv);
      if (fabsf(fv) > 1e-10f) { sf += fv; nf += 1.f; }
      float J[NQ];
      jac(i, j, s, J);
      // the second pass reads f and the masked gradients back from the tile
      if constexpr (TWO) tf[p] = fv;
      else { tg[p] = fv; gq[p] = make_float2(J[4], J[5]); }
      int q = 0;
#pragma unroll
      for (int aa = 0; aa < NQ; ++aa)
#pragma unroll
        for (int bb = aa; bb < NQ; ++bb) hs[q++] += J[aa] * J[bb];
    }
    float st3[3] = {sf, nf, sa};
    tm.template sumf<3>(st3, fscr);
    const float cnt = st3[1];
    const float mean = st3[0] / cnt;
    float q = 0.f, kjf[NQ], kj1[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) { kjf[k] = 0.f; kj1[k] = 0.f; }
    PixIter it2(pstart, mx);
    for (int p = tm.tl; p < npx; p += tm.TT, it2.next()) {
      const float s = bw ? (float)bw[p] : 1.f;
      const float fv = TWO ? tf[p] : tg[p];
      const float d = fv - mean;
      if (fabsf(fv) > 1e-10f) q = fmaf(d, d, q);
      float J[NQ];
      if constexpr (TWO) jac(it2.i, it2.j, s, J);
      else jacq(p, it2.i, it2.j, J);
#pragma unroll
      for (int k = 0; k < NQ; ++k) { kjf[k] = fmaf(J[k], d, kjf[k]); kj1[k] += J[k]; }
    }
    float qq[1 + 2 * NQ];
    qq[0] = q;
#pragma unroll
    for (int k = 0; k < NQ; ++k) { qq[1 + k] = kjf[k]; qq[1 + NQ + k] = kj1[k]; }
    tm.template sumf<1 + 2 * NQ>(qq, fscr);
#pragma unroll
    for (int k = 0; k < NQ; ++k) { jf[k] = qq[1 + k]; j1[k] = qq[1 + NQ + k]; }
    const float var = cnt == 0.f ? __int_as_float(0x7fc00000) : (cnt == 1.f ? 0.f : qq[0] / (cnt - 1.f));
    meanf = mean;
    bottomf = sqrtf((cnt - 1.f) * var);
    sabs = st3[2];
    if constexpr (TWO) {
      tm.template sumf<3>(*reinterpret_cast<float(*)[3]>(hs), fscr);
      // H2 + 1e-3 max(diag H2) I of funICGN_Subpb1.m:391-394, inverted in FP64
      // by the two lanes that apply it (lane k holds row k)
      if (lane < 2) {
        const double s2 = 2.0 / ((double)bottomf * (double)bottomf);
        const double A11 = (double)hs[0] * s2 + a.mu, A12 = (double)hs[1] * s2, A22 = (double)hs[2] * s2 + a.mu;
        const double dmax = isnan(A11) ? A22 : (isnan(A22) ? A11 : fmax(A11, A22));
        const double h11 = A11 + 1e-3 * dmax, h22 = A22 + 1e-3 * dmax;
        const double det = h11 * h22 - A12 * A12;
        double r0, r1;
        if (h11 > 0 && h22 > 0 && det > 1e-8 * (h11 * h22)) {
          // well-conditioned symmetric positive definite: the adjugate
          const double rd = 1.0 / det;
          r0 = (lane == 0 ? h22 : -A12) * rd;
          r1 = (lane == 0 ? -A12 : h11) * rd;
        } else {
          // Cholesky or pivoted elimination of mldivide on e_lane
          solve2(h11, A12, h22, lane == 0 ? 1.0 : 0.0, lane == 0 ? 0.0 : 1.0, &r0, &r1);
        }
        split_f64(r0, ih[0], il[0]);
        split_f64(r1, ih[1], il[1]);
      }
    } else {
      // each of the 21 sums is needed by one thread only (the one that
      // writes it): a reduce-scatter leaves sum k with team thread k
      const float v = tm.scatter_sum32(hs, fscr);
      // packed lower (row-major) Hessian for the factor kernel and the output
      if (tm.tl < 21) {
        // hs index of (row aa, col bb >= aa) -> packed lower (bb, aa)
        int aa = 0, rem = tm.tl;
        while (rem >= 6 - aa) { rem -= 6 - aa; ++aa; }
        const int bb = aa + rem;
        B.H6[(size_t)item * 21 + bb * (bb + 1) / 2 + aa] = (double)v;
        // HGlobal = [H(1:6) H(8:12) ...]: column aa, rows aa..5 in the order of hs
        if (a.Hpk) a.Hpk[(size_t)tm.tl * Ntot + item] = (double)v;
      }
    }
    tm.sync();
  };

  if (stage != 2 && !decided && code == 0 && !nan_out) f_side();

  if (stage == 1) {
    // hand the subset to the factor kernel and the iteration stage
    if (tm.tl == 0) {
      SubsetState6 s6;
      s6.code = nan_out ? -1 : code;
      s6.ws = wx; s6.cntf = cntf; s6.masked = has_masked ? 1 : 0;
      s6.meanf = meanf; s6.bottomf = bottomf; s6.sabs = sabs; s6.pad = 0.f;
#pragma unroll
      for (int k = 0; k < 6; ++k) { s6.Jf[k] = jf[k < NQ ? k : 0]; s6.J1[k] = j1[k < NQ ? k : 0]; }
      st6[item] = s6;
      if (B.order2 && code == 0 && !nan_out) {
        // masked subsets refill their selections every iteration: with the
        // large ones they go to the wide teams of the split form
        const bool wide = B.split && (cntf > 0 || has_masked || wx >= B.split_ws);
        const int slot = atomicAdd(&B.n2[wide ? 0 : 1], 1);
        // the single-warp list is filled from its end, so that the iteration
        // stage takes it in the reverse of the set-up order (smallest first)
        B.order2[wide ? (size_t)slot : 2 * (size_t)Ntot - 1 - slot] = item;
      }
      if (code != 0 || nan_out) {
        a.conv[item] = code;
        // decided in the set-up: P is still the initial guess, passed through in FP64
        a.U[2 * item] = nan_out ? nan("") : a.U0[2 * item];
        a.U[2 * item + 1] = nan_out ? nan("") : a.U0[2 * item + 1];
#pragma unroll
        for (int k = 0; k < 4; ++k) a.F[4 * item + k] = nan_out ? nan("") : 0.0;
        if (a.Hpk)
          for (int q = 0; q < 21; ++q) a.Hpk[(size_t)q * Ntot + item] = 0.0;
      }
    }
    tm.sync();
    return;
  }
  if (decided) {
    tm.sync();
    return;
  }
  if constexpr (!TWO) {
    // the subset's inverse Hessian and f-side sums (loaded with its state),
    // once, into the team's control block
    if (tm.tl < 36) { ctl->hh[tm.tl] = hpre.x; ctl->hl[tm.tl] = hpre.y; }
    if (tm.tl + tm.TT < 36) { ctl->hh[tm.tl + tm.TT] = hpre2.x; ctl->hl[tm.tl + tm.TT] = hpre2.y; }
    if (tm.tl < 6) ctl->jf[tm.tl] = jpre;
    else if (tm.tl < 12) ctl->j1[tm.tl - 6] = jpre;
    tm.sync();
  }
  const bool run = (code == 0 && !nan_out);
  float normNew = 1.f, normAbs = 1.f, normInit = 0.f;
  int step = 0, cg = 0, nupd = 0, last_cg = -1, last_nws = wx;
  bool err = false;
  bool oob = run ? corners_oob_warp(P, (int)x0, (int)y0, (int)x1, (int)y1, mx, my, a.W, a.H, lane) : false;
  float ibf = 1.f / bottomf;
  // the g box staged by TMA for this subset (tbox 0: none): image position of
  // its first element and its side; reused while the footprint stays inside
  int tbox = 0, bgx0 = 0, bgy0 = 0;
  while (run && step <= kMaxIter && normNew > tolf && normAbs > tolf) {
    ++step;
    if constexpr (!TWO) {
      if (step > 1 && cntf > 0) {
        // window growth test of funICGNQuadtree.m:140 (FP64, recomputed only
        // when the count of selected g pixels changes)
        int nws = last_nws;
        if (cg != last_cg) {
          // nws = 2 ceil(r), r = sqrt((ws0+1)^2 / cg) wx / 2, decided in
          // integers: ceil(r) is the least k with 4 k^2 cg >= (ws0+1)^2 wx^2.
          // When r is not an integer it lies at least 1/(8 cg k) from one,
          // far beyond the FP64 rounding of the reference's expression, so
          // both give the same k; an integer r takes the FP64 value itself.
          if (cg <= 0) { err = true; break; }
          const long long A = (long long)(ws0 + 1) * (ws0 + 1);
          const long long rhs = A * (long long)wx * (long long)wx;
          long long k = (long long)ceilf(sqrtf((float)A / (float)cg) * (float)wx * 0.5f);
          if (k < 0) k = 0;
          while (k > 0 && 4 * (k - 1) * (k - 1) * cg >= rhs) --k;
          while (4 * k * k * cg < rhs) ++k;
          if (4 * k * k * cg == rhs) k = (long long)ceil(sqrt((double)A / (double)cg) * wx / 2);
          nws = 2 * (int)k;
          last_cg = cg;
          last_nws = nws;
        }
        if (nws != wx) {
          const long long nx1 = x0 - nws / 2, nx3 = x0 + nws / 2, ny1 = y0 - nws / 2, ny3 = y0 + nws / 2;
          if (!mask_crop_ok32(fr, nx1, nx3, ny1, ny3)) { err = true; break; }
          if (corners_oob_warp(P, (int)x0, (int)y0, (int)nx1, (int)ny1, nws + 1, nws + 1, a.W, a.H, lane)) { normNew = 1e6f; break; }
          err = true;
          break;
        }
      }
    }
    if (oob) { normNew = 1e6f; break; }
    // integer base + FP32 offsets of the warp
    const float flu = floorf(P[4]), flv = floorf(P[5]);
    const int iu = (int)x0 + (int)flu, iv = (int)y0 + (int)flv;
    const float fu = P[4] - flu, fv0 = P[5] - flv;
    const float p0 = 1.f + P[0], p1 = P[1], p2 = P[2], p3 = 1.f + P[3];
    const float dx0 = (float)(int)(x1 - x0), dy0 = (float)(int)(y1 - y0);
    const float shift = meanf;  // one-pass variance around meanf
    // one pass: interpolation, zero count, g statistics and sum J g.
    // Slots: zero count, sum g and sum g^2 (shifted), count, sum J g.  A NaN
    // in the interpolated tile shows in sum gx g (the kR + NQ - 2 slot): every
    // J holds gx or gy of a finite gradient times the selection (0 or 1), and
    // 0 * NaN is NaN, so that sum is NaN exactly when a tile value is.
    constexpr int kR = 4;  // first sum J g slot
    constexpr int NR = kR + NQ;
    float red[NR];
    {
      int zg = 0;
      float sg = 0.f, qg = 0.f;
      float kg[NQ];
#pragma unroll
      for (int k = 0; k < NQ; ++k) kg[k] = 0.f;
      float ng = 0.f;
      PixIter it(pstart, mx);
      auto one = [&](int p, float dx, float dy, int i, int j, float t) {
        tg[p] = t;
        if (t == 0.f) ++zg;
        if (fabsf(t) > 1e-10f) {
          const float d = t - shift;
          sg += d;
          qg = fmaf(d, d, qg);
          ng += 1.f;
        }
        if constexpr (TWO) {
          float J[NQ];
          jac(i, j, bw ? (float)bw[p] : 1.f, J);
#pragma unroll
          for (int k = 0; k < NQ; ++k) kg[k] = fmaf(J[k], t, kg[k]);
        } else {
          add_jt6(*reinterpret_cast<float(*)[6]>(kg), gq[p], dx, dy, t);
        }
      };
      // Stage the warped footprint of g in shared memory when it fits: the
      // tap range follows from the four corners (the warp is affine), with a
      // one-pixel margin, clipped to the image.
      int gx0 = 0, gy0 = 0, gtw = 0, gth = 0;
      bool staged = false;
      if (STG && gcap > 0) {
        const float xa = dx0, xb2 = dx0 + (float)(mx - 1), ya = dy0, yb2 = dy0 + (float)(my - 1);
        const float u00 = fu + p0 * xa + p2 * ya, u10 = fu + p0 * xb2 + p2 * ya;
        const float u01 = fu + p0 * xa + p2 * yb2, u11 = fu + p0 * xb2 + p2 * yb2;
        const float v00 = fv0 + p1 * xa + p3 * ya, v10 = fv0 + p1 * xb2 + p3 * ya;
        const float v01 = fv0 + p1 * xa + p3 * yb2, v11 = fv0 + p1 * xb2 + p3 * yb2;
        const float umin = fminf(fminf(u00, u10), fminf(u01, u11)), umax = fmaxf(fmaxf(u00, u10), fmaxf(u01, u11));
        const float vmin = fminf(fminf(v00, v10), fminf(v01, v11)), vmax = fmaxf(fmaxf(v00, v10), fmaxf(v01, v11));
        if (umin >= -1e6f && umax <= 1e6f && vmin >= -1e6f && vmax <= 1e6f) {
          const long long ax0 = (long long)iu + (long long)floorf(umin) - 3;
          const long long ax1 = (long long)iu + (long long)floorf(umax) + 2;
          const long long ay0 = (long long)iv + (long long)floorf(vmin) - 3;
          const long long ay1 = (long long)iv + (long long)floorf(vmax) + 2;
          const long long cx0 = ax0 < 0 ? 0 : ax0, cx1 = ax1 > fr.W - 1 ? fr.W - 1 : ax1;
          const long long cy0 = ay0 < 0 ? 0 : ay0, cy1 = ay1 > fr.H - 1 ? fr.H - 1 : ay1;
          const long long w_ = cx1 - cx0 + 1, h_ = cy1 - cy0 + 1;
          if (B.gbox_n > 0 && tma_ok) {
            // one TMA box per subset, with a 2-pixel margin, copied again
            // only when the footprint leaves it
            if (!(tbox > 0 && cx0 >= bgx0 && cx1 < bgx0 + tbox && cy0 >= bgy0 && cy1 < bgy0 + tbox)) {
              constexpr long long M = 2;
              const long long bx = ((cx0 - M) >> 2) << 2;  // floor to a multiple of 4
              const long long by = cy0 - M;
              const long long need = max(cx1 + M - bx + 1, cy1 + M - by + 1);
              int k = 0;
              while (k < B.gbox_n && gbox_side(k) < need) ++k;
              tbox = 0;
              if (k < B.gbox_n && (long long)gbox_side(k) * gbox_side(k) <= gcap) {
                const int box = gbox_side(k);
                tm.sync();  // every thread is done with the previous box
                if (tm.tl == 0)
                  tma_box_issue(&B.gmap[k], gt, (int)bx, frame * fr.H + (int)by, &ctl->mbar,
                                (unsigned)(box * box * 4));
                const bool done = tma_box_wait(&ctl->mbar, gphase, 1 << 22);
                if (!tm.any(!done, iscr)) {
                  gphase ^= 1u;
                  tbox = box; bgx0 = (int)bx; bgy0 = (int)by;
                } else {
                  // last resort: the copy has not landed after 2^22 polls.  The
                  // error is recorded, the team polls once more for a bounded
                  // interval so that no copy is left writing its shared memory,
                  // and it gathers from global memory from here on
                  if (tm.tl == 0 && B.tma_err) atomicExch(B.tma_err, 1);
                  tma_box_wait(&ctl->mbar, gphase, 1 << 22);
                  tma_ok = false;
                }
              }
            }
            if (tbox > 0) {
              gx0 = bgx0; gy0 = bgy0; gtw = gth = tbox;
              staged = true;
            }
          } else if (w_ >= 4 && h_ >= 4 && w_ <= gcap && h_ <= gcap && w_ * h_ <= gcap) {
            gx0 = (int)cx0; gy0 = (int)cy0; gtw = (int)w_; gth = (int)h_;
            staged = true;
          }
        }
      }
      if (staged && tbox == 0) {
        PixIter ti(tm.tl, tm.TT, gtw);
        const int ng_ = gtw * gth;
        for (int k = tm.tl; k < ng_; k += tm.TT, ti.next())
          cp_async4(gt + k, fr.g + (long long)(gy0 + ti.j) * fr.W + gx0 + ti.i);
        cp_async_wait_all();
        tm.sync();
      }
      auto sample = [&](float su, float sv) {
        return staged ? cubic_tile(gt, gtw, gth, gx0, gy0, fr.W, fr.H, iu, su, iv, sv)
                      : cubic32(fr.g, fr.W, fr.H, iu, su, iv, sv);
      };
      int p = tm.tl;
      // two pixels per trip so that both pixels' taps are in flight together.
      // The trip count is the same on every lane (trips whose both pixels
      // exist on the team's last thread); the rest, fewer than 2 TT pixels,
      // is taken below as two single-pixel steps, so that a tile of
      // 2 k TT + TT + 1 pixels (17^2 = 289 on one warp) does not run its
      // last pair on one lane while the others wait to run their single one.
      for (; p - tm.tl + 2 * tm.TT <= npx; p += 2 * tm.TT) {
        const int ia = it.i, ja = it.j;
        it.next();
        const int ib = it.i, jb = it.j;
        it.next();
        const float dxa = dx0 + (float)ia, dya = dy0 + (float)ja;
        const float dxb = dx0 + (float)ib, dyb = dy0 + (float)jb;
        const float ta = sample(fu + p0 * dxa + p2 * dya, fv0 + p1 * dxa + p3 * dya);
        const float tb2 = sample(fu + p0 * dxb + p2 * dyb, fv0 + p1 * dxb + p3 * dyb);
        one(p, dxa, dya, ia, ja, ta);
        one(p + tm.TT, dxb, dyb, ib, jb, tb2);
      }
      if (p < npx) {
        const float dx = dx0 + (float)it.i, dy = dy0 + (float)it.j;
        const float t = sample(fu + p0 * dx + p2 * dy, fv0 + p1 * dx + p3 * dy);
        one(p, dx, dy, it.i, it.j, t);
        p += tm.TT;
        it.next();
        if (p < npx) {
          const float dxb = dx0 + (float)it.i, dyb = dy0 + (float)it.j;
          const float tb = sample(fu + p0 * dxb + p2 * dyb, fv0 + p1 * dxb + p3 * dyb);
          one(p, dxb, dyb, it.i, it.j, tb);
        }
      }
      red[0] = (float)zg;
      red[1] = sg; red[2] = qg; red[3] = ng;
#pragma unroll
      for (int k = 0; k < NQ; ++k) red[kR + k] = kg[k];
    }
    tm.template sumf16<NR>(red, fscr);
    if (isnan(red[kR + NQ - 2])) { err = true; break; }
    if (cntf > 0 || red[0] > 0.f) {
      for (int p = tm.tl; p < npx; p += tm.TT) tmp[p] = tg[p] != 0.f;
      tm.sync();
      bwselect_team(tm, tmp, bwg, mx, my, sr, sc, TWO ? 4 : 8, iscr);
      int anyzero = 0;
      for (int p = tm.tl; p < npx; p += tm.TT) anyzero |= !bwg[p];
      if (!tm.any(anyzero, iscr)) {
        // the 8-connected selection of the mask tile does not change between
        // iterations: filled once per subset, then copied
        if (!have_m8) {
          if (!have_mtile) {
            PixIter it(pstart, mx);
            for (int p = tm.tl; p < npx; p += tm.TT, it.next())
              mtile[p] = __ldg(fr.mask + (y1 + it.j - 1) * fr.W + (x1 + it.i - 1)) != 0;
            have_mtile = true;
            tm.sync();
          }
          bwselect_team(tm, mtile, bwm8, mx, my, sr, sc, 8, iscr);
          have_m8 = true;
        }
        for (int p = tm.tl; p < npx; p += tm.TT) bwg[p] = bwm8[p];
        tm.sync();
      }
      if constexpr (TWO) {
        // the f side depends on the tile and the selection only: it is kept
        // while the selection equals the one it was last evaluated for, which
        // bwf holds (bw nullptr: every pixel)
        int diff = 0;
        for (int p = tm.tl; p < npx; p += tm.TT) diff |= bwg[p] != (bw ? bw[p] : 1);
        if (tm.any(diff, iscr)) {
          for (int p = tm.tl; p < npx; p += tm.TT) bwf[p] = bwg[p];
          tm.sync();
          bw = bwf;
          f_side();
          ibf = 1.f / bottomf;
        }
      }
      if constexpr (!TWO) {
        // The g tile restricted to its selection.  J depends only on the fixed
        // f selection here, so the sums of the first pass stay valid for the
        // kept pixels: only the removed pixels' parts are summed and taken off.
        int cnt = 0, rem = 0;
        float rsg = 0.f, rqg = 0.f;
        float rkg[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float rng = 0.f;
        PixIter it(pstart, mx);
        for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
          const int keep = bwg[p];
          cnt += keep;
          if (!keep) {
            const float t = tg[p];
            if (t != 0.f) {
              rem = 1;
              tg[p] = 0.f;
              if (fabsf(t) > 1e-10f) {
                const float d = t - shift;
                rsg += d;
                rqg = fmaf(d, d, rqg);
                rng += 1.f;
              }
              add_jt6(rkg, gq[p], dx0 + (float)it.i, dy0 + (float)it.j, t);
            }
          }
        }
        cg = tm.sum_int(cnt, iscr);
        if (tm.any(rem, iscr)) {
          float rr[NR];
          rr[0] = 0.f;
          rr[1] = rsg; rr[2] = rqg; rr[3] = rng;
#pragma unroll
          for (int k = 0; k < NQ; ++k) rr[kR + k] = rkg[k < 6 ? k : 0];
          tm.template sumf16<NR>(rr, fscr);
#pragma unroll
          for (int k = 1; k < NR; ++k) red[k] -= rr[k];
        }
        red[0] = (float)cg;
      } else {
        // the g tile restricted to its selection, and its sums again (the f
        // selection, and with it J, follows the g selection in this form)
        int cnt = 0;
        float sg = 0.f, qg = 0.f;
        float kg[NQ];
#pragma unroll
        for (int k = 0; k < NQ; ++k) kg[k] = 0.f;
        float ng = 0.f;
        PixIter it(pstart, mx);
        for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
          const float t = tg[p] * (float)bwg[p];
          tg[p] = t;
          cnt += bwg[p];
          if (fabsf(t) > 1e-10f) {
            const float d = t - shift;
            sg += d;
            qg = fmaf(d, d, qg);
            ng += 1.f;
          }
          float J[NQ];
          jac(it.i, it.j, bw ? (float)bw[p] : 1.f, J);
#pragma unroll
          for (int k = 0; k < NQ; ++k) kg[k] = fmaf(J[k], t, kg[k]);
        }
        red[0] = (float)cnt;
        red[1] = sg; red[2] = qg; red[3] = ng;
#pragma unroll
        for (int k = 0; k < NQ; ++k) red[kR + k] = kg[k];
        tm.template sumf16<NR>(red, fscr);
        cg = (int)red[0];
      }
    }
    // g statistics from the shifted one-pass sums: mean and
    // sqrt((n-1) var) = sqrt(max(s2 - s1^2/n, 0)) (NaN for n = 0, 0 for n = 1)
    const float cntg = red[3];
    const float s1 = red[1], s2 = red[2];
    const float icnt = 1.f / cntg;
    const float meang = shift + s1 * icnt;
    float bg2 = fmaxf(s2 - s1 * s1 * icnt, 0.f);
    if (cntg == 1.f) bg2 = 0.f;
    if (cntg == 0.f) bg2 = __int_as_float(0x7fc00000);
    const float ibg = 1.f / sqrtf(bg2);
    // b2 = sum J [(tempf - meanf)/bottomf - (tempg - meang)/bottomg]; the
    // 6-DOF f-side sums come from the set-up stage (read here, not held
    // in registers across the pixel pass)
    if constexpr (!TWO) {
#pragma unroll
      for (int k = 0; k < NQ; ++k) { jf[k] = ctl->jf[k]; j1[k] = ctl->j1[k]; }
    }
    float b2[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      const float jg = red[kR + k];
      b2[k] = jf[k] * ibf - (jg - meang * j1[k]) * ibg;
    }
    // convergence test (FP32) and the update, identical on every lane
    int done = 0;
    float nb = 0.f;
    float D[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if constexpr (TWO) {
      const float b0 = bottomf * b2[0], b1 = bottomf * b2[1];
      const float sc2 = 2.f / (bottomf * bottomf);
      const float tb0 = b0 * sc2 + (float)a.mu * (P[4] - uold0 - vd0);
      const float tb1 = b1 * sc2 + (float)a.mu * (P[5] - uold1 - vd1);
      nb = tb0 * tb0 + tb1 * tb1;
      // 2x2 solve with the FP64 inverse: lane 0 forms DeltaP_5, lane 1 DeltaP_6
      const float tb[2] = {tb0, tb1};
      const float dkf = -dot_df<2>(ih, il, tb);
      D[4] = __shfl_sync(0xffffffffu, dkf, 0);
      D[5] = __shfl_sync(0xffffffffu, dkf, 1);
    } else {
      float b[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) { b[q] = bottomf * b2[q < NQ ? q : 0]; nb += b[q] * b[q]; }
      // DeltaP = -H^-1 b with the FP64 inverse: every lane holds b, lane k
      // forms row k in double-float arithmetic
      const int r = (lane < 6 ? lane : 0) * 6;
      const float dkf = -dot_df<6>(ctl->hh + r, ctl->hl + r, b);
#pragma unroll
      for (int q = 0; q < 6; ++q) D[q] = __shfl_sync(0xffffffffu, dkf, q);
    }
    float nN = sqrtf(nb);
    const float nA = nN;
    if (step == 1) normInit = nN;
    nN = normInit > tolf ? nN / normInit : 0.f;
    normNew = nN;
    normAbs = nA;
    if (nN < tolf || nA < tolf) done = 1;
    else if (!compose_warp(P, D, lane)) done = 2;
    else ++nupd;
    if (done) break;
    oob = corners_oob_warp(P, (int)x0, (int)y0, (int)x1, (int)y1, mx, my, a.W, a.H, lane);
  }
  if (run) {
    if (err) { code = err_code; nan_out = true; }
    else {
      code = step;
      if (!(normNew < tolf || normAbs < tolf)) code = kMaxIter + 1;
      if (isnan(normNew)) code = kMaxIter + 1;
      if constexpr (TWO) {
        float v[1] = {0.f};
        for (int p = tm.tl; p < npx; p += tm.TT) v[0] += fabsf(tf[p]);
        tm.template sumf<1>(v, fscr);
        sabs = v[0];
      }
      if (sabs < 1e-6f) code = kMaxIter + 3;
    }
  }
  if (tm.tl == 0) {
    a.conv[item] = code;
    // a subset that never updated P returns its initial guess bit-exactly
    const bool moved = nupd > 0;
    if constexpr (TWO) {
      a.U[2 * item] = nan_out ? nan("") : (moved ? (double)P[4] : a.UOld[2 * item]);
      a.U[2 * item + 1] = nan_out ? nan("") : (moved ? (double)P[5] : a.UOld[2 * item + 1]);
    } else {
      a.U[2 * item] = nan_out ? nan("") : (moved ? (double)P[4] : a.U0[2 * item]);
      a.U[2 * item + 1] = nan_out ? nan("") : (moved ? (double)P[5] : a.U0[2 * item + 1]);
    }
    if constexpr (!TWO) {
#pragma unroll
      for (int k = 0; k < 4; ++k) a.F[4 * item + k] = nan_out ? nan("") : (double)P[k];
      if (a.Hpk && nan_out)
        for (int q = 0; q < 21; ++q) a.Hpk[(size_t)q * Ntot + item] = 0.0;
    }
  }
  tm.sync();
}

// Pulls queue positions [lo, hi) from counter *head, one subset per team.
// Frames are interleaved so that every frame's largest subsets start first.
template <int TW, bool TWO, int STAGE, bool STG>
STDIC_DEV void team_loop(const BatchedArgs& B, const Team<TW>& tm, int* head, int lo, int hi,
                         unsigned char* base, int smpx, int gcap, unsigned char* gbase,
                         const int32_t* list = nullptr) {
  const size_t tiles_b = tiles_bytes(smpx, TWO);
  float* gt = (float*)(base + tiles_b);
  TeamCtl* ctl = (TeamCtl*)(base + tiles_b + gtile_bytes(gcap));
  float* fscr = (float*)(ctl + 1);
  int* iscr = (int*)(fscr + 32 * TW);
  const int nf = B.frames > 0 ? B.frames : 1;
  // the team's footprint-copy barrier (its slot moves between the team and
  // the single-warp phases of the split form, so it lives per call)
  unsigned gphase = 0;
  bool tma_ok = STG && B.gbox_n > 0;
  const unsigned sbar = (unsigned)__cvta_generic_to_shared(&ctl->mbar);
  if (tma_ok) {
    if (tm.tl == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tm.sync();
  }
  for (;;) {
    if (tm.tl == 0) {
      const int q = lo + atomicAdd(head, 1);
      // list: subset ids as they are; otherwise node order with frames interleaved
      ctl->item = q >= hi ? -1 : (list ? list[q] : B.order[q / nf] + (q % nf) * B.a.N);
    }
    tm.sync();
    const int item = ctl->item;
    tm.sync();
    if (item < 0) break;
    run_subset<TW, TWO, STAGE, STG>(B, tm, item, base, ctl, fscr, iscr, gbase, smpx, gt, gcap, gphase, tma_ok);
  }
  if (STG && B.gbox_n > 0) {
    tm.sync();
    if (tm.tl == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(sbar) : "memory");
    tm.sync();
  }
}

// The persistent kernel.  Without B.split every subset runs on a team of TW
// warps.  With B.split (TW > 1) the queue is ordered by decreasing size and
// the first *B.n_big positions (subsets of at least B.big_ws pixels a side)
// run on teams of TW warps; once they are all taken, each warp of a team
// pulls the remaining small subsets on its own, in a 1/TW share of the team's
// shared slot (B.smem_px_small tile pixels).  The largest subsets thus start
// first and get the widest teams, and no warp idles while small work is left.
//
// Shared memory per team: smem_px floats (tempg) [+ smem_px floats (tempf,
// 2-DOF)] + 5 smem_px bytes of bitmaps, the staged g footprint, then the
// control block and reduction scratch.  Global scratch: one slice of the same layout for npx_max pixels
// per warp (a team uses the slice of its first warp).
//
// Stages (B.stage): 0 runs the 2-DOF form fused; for the 6-DOF form stage 1
// does the per-subset set-up (window, masks, f statistics, FP32 Hessian) and
// stage 2 the iterations with the inverse Hessian the factor kernel produced
// in FP64 between them.  Every lane of a team holds the team totals after each
// reduction and runs the same update on them, so all warps carry bit-identical
// P without a shared-memory broadcast.
template <int TW, bool TWO, int STAGE, bool STG>
__global__ void __launch_bounds__(256, STAGE == 1 ? 3 : 2) icgn_batched_kernel(const __grid_constant__ BatchedArgs B) {
  extern __shared__ __align__(128) unsigned char dsm_raw[];
  // team slots from a 128-byte boundary (TMA copies land there); the launch
  // adds 128 bytes of dynamic shared memory for this
  unsigned char* const dsm = dsm_raw + ((128u - ((unsigned)__cvta_generic_to_shared(dsm_raw) & 127u)) & 127u);
  const int nf = B.frames > 0 ? B.frames : 1;
  const int Ntot = B.a.N * nf;
  const int warp = threadIdx.x >> 5;
  const size_t gstride = slice_bytes(B.a.npx_max, TWO);
  const long long gwarp0 = (long long)blockIdx.x * (blockDim.x >> 5);
  const size_t tb = team_bytes(B.smem_px, TWO, TW, B.gtile);
  Team<TW> tm;
  tm.id = threadIdx.x / Team<TW>::TT;
  tm.tl = threadIdx.x % Team<TW>::TT;
  unsigned char* tbase = dsm + tb * tm.id;
  const bool split = TW > 1 && B.split;
  unsigned char* const gteam = B.scratch + gstride * (gwarp0 + (long long)tm.id * TW);
  if (STAGE == 2 && B.order2) {
    // the lists the set-up stage left: wide teams first, then single warps
    // (without the split every subset is in the second list)
    const int nwide = B.n2[0], nrest = B.n2[1];
    if (split)
      team_loop<TW, TWO, STAGE, STG>(B, tm, B.queue_head, 0, nwide, tbase, B.smem_px, B.gtile, gteam, B.order2);
    else
      team_loop<TW, TWO, STAGE, STG>(B, tm, B.queue_head, 0, nrest, tbase, B.smem_px, B.gtile, gteam,
                                B.order2 + 2 * (size_t)Ntot - nrest);
    if constexpr (TW > 1) {
      if (split) {
        Team<1> t1;
        t1.id = warp;
        t1.tl = threadIdx.x & 31;
        const size_t sub = (tb / TW) & ~(size_t)127;
        team_loop<1, TWO, STAGE, STG>(B, t1, B.queue_head + 1, 0, nrest, tbase + sub * (warp % TW),
                                 B.smem_px_small, B.gtile_small, B.scratch + gstride * (gwarp0 + warp),
                                 B.order2 + 2 * (size_t)Ntot - nrest);
      }
    }
    return;
  }
  if (STAGE == 1 && B.band_list) {
    // one band of a frame uploaded in row bands: its nodes, big ones first
    const int lo = B.band_off[B.band], n = B.band_off[B.band + 1] - lo;
    const int32_t* lst = B.band_list + lo;
    const int nbg = split ? min(B.band_nbig[B.band], n) : n;
    team_loop<TW, TWO, STAGE, STG>(B, tm, B.queue_head, 0, nbg, tbase, B.smem_px, B.gtile, gteam, lst);
    if constexpr (TW > 1) {
      if (split) {
        Team<1> t1;
        t1.id = warp;
        t1.tl = threadIdx.x & 31;
        const size_t sub = (tb / TW) & ~(size_t)127;
        team_loop<1, TWO, STAGE, STG>(B, t1, B.queue_head + 1, nbg, n, tbase + sub * (warp % TW),
                                      B.smem_px_small, B.gtile_small, B.scratch + gstride * (gwarp0 + warp), lst);
      }
    }
    return;
  }
  const int split_q = split ? min(*B.n_big * nf, Ntot) : Ntot;
  team_loop<TW, TWO, STAGE, STG>(B, tm, B.queue_head, 0, split_q, tbase, B.smem_px, B.gtile, gteam);
  if constexpr (TW > 1) {
    if (split) {
      Team<1> t1;
      t1.id = warp;
      t1.tl = threadIdx.x & 31;
      const size_t sub = (tb / TW) & ~(size_t)127;
      team_loop<1, TWO, STAGE, STG>(B, t1, B.queue_head + 1, split_q, Ntot,
                               tbase + sub * (warp % TW), B.smem_px_small, B.gtile_small,
                               B.scratch + gstride * (gwarp0 + warp));
    }
  }
}

// Launch and occupancy of the instantiations of one team width.
template <int TW, bool TWO, int STAGE, bool STG>
inline cudaError_t launch_tw(const BatchedArgs& b, int blocks, int threads, cudaStream_t s) {
  const int teams = threads / (TW * 32);
  const size_t smem = batched_team_bytes(b.smem_px, TWO, TW, b.gtile) * teams + 128;
  if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(icgn_batched_kernel<TW, TWO, STAGE, STG>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  icgn_batched_kernel<TW, TWO, STAGE, STG><<<blocks, threads, smem, s>>>(b);
  return cudaGetLastError();
}

// Shapes without a staged g footprint run instantiations compiled without the
// staging code (STG = false), which leaves its registers and issue slots to
// the rest (the iteration stage ran 11 % faster at 2048²); the set-up stage
// never reads g.  Each (team width, STG) pair is its own translation unit.
template <int TW, bool STG>
inline cudaError_t launch_stage(const BatchedArgs& b, int blocks, int threads, cudaStream_t s) {
  if (b.two_dof) return launch_tw<TW, true, 0, STG>(b, blocks, threads, s);
  if (b.stage == 1) {
    if constexpr (STG) return cudaErrorInvalidValue;  // compiled in the STG = false units only
    else return launch_tw<TW, false, 1, false>(b, blocks, threads, s);
  }
  return launch_tw<TW, false, 2, STG>(b, blocks, threads, s);
}

template <int TW, bool TWO, int STAGE, bool STG>
inline int occupancy_of(int threads, size_t smem) {
  int nb = 0;
  cudaError_t e = cudaFuncSetAttribute(icgn_batched_kernel<TW, TWO, STAGE, STG>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, icgn_batched_kernel<TW, TWO, STAGE, STG>, threads, smem);
  return e == cudaSuccess ? nb : 0;
}

// stage 1: the 6-DOF set-up; any other stage: the iterations or the fused 2-DOF form
template <int TW, bool STG>
inline int blocks_per_sm_of(bool two, int threads, size_t smem, int stage) {
  if (two) return occupancy_of<TW, true, 0, STG>(threads, smem);
  if (stage == 1) {
    if constexpr (STG) return 0;
    else return occupancy_of<TW, false, 1, false>(threads, smem);
  }
  return occupancy_of<TW, false, 2, STG>(threads, smem);
}

// The entry points of one (team width, staging) translation unit: the
// instantiations without staging carry the suffix u, those with it s.
#define STDIC_BATCHED_UNIT(TW, STG, SFX)                                                                    \
  cudaError_t launch_icgn_batched_tw##TW##SFX(const BatchedArgs& b, int blocks, int threads, cudaStream_t s) { \
    return launch_stage<TW, STG>(b, blocks, threads, s);                                                     \
  }                                                                                                          \
  int batched_blocks_per_sm_tw##TW##SFX(bool two, int threads, size_t smem, int stage) {                    \
    return blocks_per_sm_of<TW, STG>(two, threads, smem, stage);                                             \
  }

#define STDIC_BATCHED_DECL(TW, SFX)                                                                      \
  cudaError_t launch_icgn_batched_tw##TW##SFX(const BatchedArgs& b, int blocks, int threads, cudaStream_t s); \
  int batched_blocks_per_sm_tw##TW##SFX(bool two, int threads, size_t smem, int stage);
STDIC_BATCHED_DECL(1, u)
STDIC_BATCHED_DECL(2, u)
STDIC_BATCHED_DECL(4, u)
STDIC_BATCHED_DECL(8, u)
STDIC_BATCHED_DECL(1, s)
STDIC_BATCHED_DECL(2, s)
STDIC_BATCHED_DECL(4, s)
STDIC_BATCHED_DECL(8, s)
#undef STDIC_BATCHED_DECL

}  // namespace stdic
