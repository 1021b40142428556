// Batched IC-GN (6-DOF first pass and 2-DOF Subpb1) as one persistent kernel.
//
// A team of TW warps (one warp by default) pulls the next subset from a global
// work queue ordered by decreasing subset size, so the longest solves start
// first, and runs it with the control flow, mask logic and result codes of the
// plain FP64 kernels (funICGNQuadtree.m / funICGN_Subpb1.m).
//
// Per-subset scratch (interpolated g tile, tempf for the 2-DOF form, four
// flood-fill bitmaps) lives in shared memory when the tile fits the team's
// shared slot and otherwise in a per-team slice of a global scratch buffer, so
// occupancy is set by registers, not by the largest subset of the batch.
//
// Precision: warped positions are an integer base plus an FP32 offset;
// bicubic weights, interpolation and residuals are FP32.  Per-lane sums are
// Kahan-compensated FP32 (b-vector and g statistics; the g variance is a
// one-pass shifted sum around meanf), reduced across lanes in FP32 together
// with their compensations; the Hessian is accumulated in plain FP32 (it only
// scales the step, never the converged point).  Team totals, the Cholesky
// factor of the 6x6 Hessian (once per subset), the triangular solves of every
// iteration and the warp-parameter update are FP64.
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

// Warp-parallel FP64 Gauss-Newton update.  Lane k < 6 holds row k of H^-1
// (6x6 form) and produces DeltaP_k; the inverse-compositional update of P and
// the image-bounds test of the next warp are also split over lanes, so the
// narrow FP64 pipe sees a few dozen instructions per iteration.
STDIC_DEV double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// P <- P o DeltaP^-1 (funICGNQuadtree.m:393-411) with D known on every lane.
// Returns false (P unchanged) when det(DeltaP) == 0.
STDIC_DEV bool compose_warp(double P[6], const double D[6], int lane) {
  const double det = (1 + D[0]) * (1 + D[3]) - D[1] * D[2];
  if (!(det != 0)) return false;
  const double inv = 1.0 / det;
  // lane k < 6 forms tempP_(k+1)
  double t = 0;
  switch (lane) {
    case 0: t = (-D[0] - D[0] * D[3] + D[1] * D[2]) * inv; break;
    case 1: t = -D[1] * inv; break;
    case 2: t = -D[2] * inv; break;
    case 3: t = (-D[3] - D[0] * D[3] + D[1] * D[2]) * inv; break;
    case 4: t = (-D[4] - D[3] * D[4] + D[2] * D[5]) * inv; break;
    case 5: t = (-D[5] - D[0] * D[5] + D[1] * D[4]) * inv; break;
  }
  double T[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) T[k] = shfl_d(t, k);
  // lane k < 6 forms the new P_(k+1)
  double pn = 0;
  switch (lane) {
    case 0: pn = (1 + P[0]) * (1 + T[0]) + P[2] * T[1] - 1; break;
    case 1: pn = P[1] * (1 + T[0]) + (1 + P[3]) * T[1]; break;
    case 2: pn = (1 + P[0]) * T[2] + P[2] * (1 + T[3]); break;
    case 3: pn = P[1] * T[2] + (1 + P[3]) * (1 + T[3]) - 1; break;
    case 4: pn = (1 + P[0]) * T[4] + P[2] * T[5] + P[4]; break;
    case 5: pn = P[1] * T[4] + (1 + P[3]) * T[5] + P[5]; break;
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) P[k] = shfl_d(pn, k);
  return true;
}

// Bounds test of the warp P over the tile [x1, x1+mx-1] x [y1, y1+my-1]: lanes
// 0..7 evaluate one coordinate of one corner each (the warp is affine).
STDIC_DEV bool corners_oob_warp(const double P[6], long long x0, long long y0, long long x1,
                                long long y1, int mx, int my, int W, int H, int lane) {
  bool bad = false;
  if (lane < 8) {
    const int cn = lane >> 1;
    const double dx = (double)((cn & 1 ? x1 + mx - 1 : x1) - x0);
    const double dy = (double)((cn & 2 ? y1 + my - 1 : y1) - y0);
    if ((lane & 1) == 0) {
      const double u22 = (1 + P[0]) * dx + P[2] * dy + ((double)x0 + P[4]);
      bad = u22 < 3 || u22 > (double)W - 2;
    } else {
      const double v22 = P[1] * dx + (1 + P[3]) * dy + ((double)y0 + P[5]);
      bad = v22 < 3 || v22 > (double)H - 2;
    }
  }
  return __any_sync(0xffffffffu, bad);
}

struct Kahan {
  float s = 0.f, c = 0.f;
  STDIC_DEV void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// flood fill of bwselect restricted to a team (see bwselect_block)
template <int TW>
STDIC_DEV void bwselect_team(const Team<TW>& tm, const uint8_t* allow, uint8_t* sel_, int m, int n,
                             int r1, int c1, int conn, int* iscr) {
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

// Affine warp is linear in (dx, dy): the tile's extreme positions are at its corners.
STDIC_DEV bool corners_oob(const Frame32& fr, const double P[6], long long x0, long long y0,
                           long long x1, long long y1, int mx, int my) {
  const double dxs[2] = {(double)(x1 - x0), (double)(x1 + mx - 1 - x0)};
  const double dys[2] = {(double)(y1 - y0), (double)(y1 + my - 1 - y0)};
  bool bad = false;
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const double u22 = (1 + P[0]) * dxs[a] + P[2] * dys[b] + ((double)x0 + P[4]);
      const double v22 = P[1] * dxs[a] + (1 + P[3]) * dys[b] + ((double)y0 + P[5]);
      bad |= (u22 < 3 || u22 > (double)fr.W - 2 || v22 < 3 || v22 > (double)fr.H - 2);
    }
  return bad;
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
  const float dx2 = dx * dx, dx3 = dx2 * dx, dy2 = dy * dy, dy3 = dy2 * dy;
  const float wx0 = 0.5f * (-dx + 2.f * dx2 - dx3), wx1 = 0.5f * (2.f - 5.f * dx2 + 3.f * dx3);
  const float wx2 = 0.5f * (dx + 4.f * dx2 - 3.f * dx3), wx3 = 0.5f * (-dx2 + dx3);
  const float wy0 = 0.5f * (-dy + 2.f * dy2 - dy3), wy1 = 0.5f * (2.f - 5.f * dy2 + 3.f * dy3);
  const float wy2 = 0.5f * (dy + 4.f * dy2 - 3.f * dy3), wy3 = 0.5f * (-dy2 + dy3);
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
  STDIC_DEV void next() {
    i += di; j += dj;
    if (i >= mx) { i -= mx; ++j; }
  }
};

// Packed lower-triangular Cholesky of a 6x6 SPD matrix in registers.
struct Chol6 {
  double l[21];  // row-major packed: l[r*(r+1)/2 + c], c <= r
  bool ok;
};

STDIC_DEV void chol6_factor(const double H[21], Chol6& C) {
  C.ok = true;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double d = H[j * (j + 1) / 2 + j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= C.l[j * (j + 1) / 2 + k] * C.l[j * (j + 1) / 2 + k];
    C.ok = C.ok && (d > 0);
    const double ljj = sqrt(d > 0 ? d : 1.0);
    C.l[j * (j + 1) / 2 + j] = ljj;
    const double inv = 1.0 / ljj;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double s = H[i * (i + 1) / 2 + j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= C.l[i * (i + 1) / 2 + k] * C.l[j * (j + 1) / 2 + k];
      C.l[i * (i + 1) / 2 + j] = s * inv;
    }
  }
}

STDIC_DEV void chol6_solve(const Chol6& C, const double b[6], double x[6]) {
  double y[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double s = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s -= C.l[i * (i + 1) / 2 + k] * y[k];
    y[i] = s / C.l[i * (i + 1) / 2 + i];
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    double s = y[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) s -= C.l[k * (k + 1) / 2 + i] * x[k];
    x[i] = s / C.l[i * (i + 1) / 2 + i];
  }
}

struct TeamCtl {
  double P[6];
  double Hm[36];
  double nN, nA, nI;
  int flag;
  int item;
};

}  // namespace

size_t batched_team_bytes(int sm_px, bool two, int tw) {
  return ((size_t)sm_px * (two ? 8 : 4) + 4 * (size_t)sm_px + 15) / 16 * 16 + sizeof(TeamCtl) +
         sizeof(float) * 32 * tw + 16 * tw + 64;
}

size_t batched_scratch_bytes(int npx_max, bool two, long long teams) {
  return ((size_t)npx_max * (two ? 8 : 4) + 4 * (size_t)npx_max) * (size_t)teams + 256;
}

// Shared memory per team: smem_px floats (tempg) [+ smem_px floats (tempf,
// 2-DOF)] + 4 smem_px bytes of bitmaps, then the control block and reduction
// scratch.  Global scratch per team: the same layout for npx_max pixels.
//
// Every warp of a team holds the team totals after each reduction and runs the
// same FP64 update on them, so all warps carry bit-identical P without a
// shared-memory broadcast.
template <int TW, bool TWO>
__global__ void __launch_bounds__(256, 2) icgn_batched_kernel(BatchedArgs B) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const IcgnArgs& a = B.a;
  Team<TW> tm;
  tm.id = threadIdx.x / Team<TW>::TT;
  tm.tl = threadIdx.x % Team<TW>::TT;
  const int lane = threadIdx.x & 31;
  const int teams_per_block = blockDim.x / Team<TW>::TT;
  const long long gteam = (long long)blockIdx.x * teams_per_block + tm.id;
  const int smpx = B.smem_px;
  const size_t tiles_b = ((size_t)smpx * (TWO ? 8 : 4) + 4 * (size_t)smpx + 15) / 16 * 16;
  const size_t tb = tiles_b + sizeof(TeamCtl) + sizeof(float) * 32 * TW + 16 * TW + 64;
  unsigned char* base = dsm + tb * tm.id;
  TeamCtl* ctl = (TeamCtl*)(base + tiles_b);
  float* fscr = (float*)(ctl + 1);
  int* iscr = (int*)(fscr + 32 * TW);
  const size_t gstride = (size_t)a.npx_max * (TWO ? 8 : 4) + 4 * (size_t)a.npx_max;
  unsigned char* gbase = B.scratch + gstride * gteam;

  const int Ntot = a.N * (B.frames > 0 ? B.frames : 1);
  const float tolf = (float)a.tol;
  for (;;) {
    if (tm.tl == 0) {
      // frames interleaved so that every frame's largest subsets start first
      const int q = atomicAdd(B.queue_head, 1);
      const int nf = B.frames > 0 ? B.frames : 1;
      ctl->item = q < Ntot ? B.order[q / nf] + (q % nf) * a.N : -1;
    }
    tm.sync();
    const int item = ctl->item;
    tm.sync();
    if (item < 0) break;
    const int node = item % a.N;
    const int frame = item / a.N;
    Frame32 fr{B.f32, B.g32 + (long long)frame * B.g_stride, a.mask, B.dfdx32, B.dfdy32, a.W, a.H};
    const long long x0 = llround(a.coords[node]), y0 = llround(a.coords[a.N + node]);

    // ---------------- per-subset set-up ----------------
    int wx, wy;
    double P[6];
    if constexpr (TWO) {
      wx = a.wsl2[node]; wy = a.wsl2[a.N + node];
#pragma unroll
      for (int k = 0; k < 4; ++k) P[k] = a.FOld[4 * item + k];
      P[4] = a.UOld[2 * item]; P[5] = a.UOld[2 * item + 1];
    } else {
      wx = wy = a.ws_list ? a.ws_list[node] : a.ws_all;
      P[0] = P[1] = P[2] = P[3] = 0;
      P[4] = a.U0[2 * item]; P[5] = a.U0[2 * item + 1];
    }
    const int ws0 = wx;
    long long x1 = x0 - wx / 2, x3 = x0 + wx / 2, y1 = y0 - wy / 2, y3 = y0 + wy / 2;
    int code = 0;
    bool nan_out = false;
    bool hdone = false;
    const int err_code = TWO ? 0 : -1;  // value the reference leaves on a run-time error
    const bool crop_valid = !((wx & 1) || (wy & 1)) && wx >= 0 && wy >= 0 && wx <= a.ws_max &&
                            wy <= a.ws_max && mask_crop_ok32(fr, x1, x3, y1, y3);
    int cntf = 0, nanf = 0;
    if (crop_valid) {
      const int mx0 = wx + 1, np0 = (wx + 1) * (wy + 1);
      PixIter it(tm.tl, tm.TT, mx0);
      for (int p = tm.tl; p < np0; p += tm.TT, it.next()) {
        const float t = fr.F(x1 + it.i, y1 + it.j) * fr.M(x1 + it.i, y1 + it.j);
        if (t != t) nanf = 1;
        if (t == 0.f) ++cntf;
      }
    }
    cntf = tm.sum_int(cntf, iscr);
    nanf = tm.any(nanf, iscr);
    if constexpr (!TWO) {
      if (a.mark && tm.tl == 0) a.mark[item] = (!crop_valid || cntf > 0) ? 1 : 0;
    }
    const double npx0 = (double)(wx + 1) * (double)(wy + 1);
    float meanf = 0.f, bottomf = 0.f, sabs = 0.f;
    double A11 = 0, A12 = 0, A22 = 0;
    int mx = 0, my = 0, npx = 0, sc = 0, sr = 0;
    float* tg = nullptr;
    float* tf = nullptr;
    uint8_t *mtile = nullptr, *bwf = nullptr, *bwg = nullptr, *tmp = nullptr;
    bool has_masked = false;
    if (!crop_valid || !crop_ok32(fr, x1, x3, y1, y3) || nanf) {
      code = err_code; nan_out = true;
    } else if (!((double)cntf < 0.4 * npx0)) {
      code = kMaxIter + 2;
    } else {
      if ((double)cntf > 0.0 * npx0) {
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
      if (!nan_out) {
        mx = wx + 1; my = wy + 1; npx = mx * my;
        sc = (wx + 1) / 2; sr = (wy + 1) / 2;
        // tile storage: the team's shared slot when it fits, else its global slice
        const bool in_smem = npx <= smpx;
        const int cap = in_smem ? smpx : a.npx_max;
        unsigned char* st = in_smem ? base : gbase;
        tg = (float*)st;
        tf = tg + cap;
        mtile = (uint8_t*)(tg + (TWO ? 2 : 1) * cap);
        bwf = mtile + cap;
        bwg = bwf + cap;
        tmp = bwg + cap;
        int z = 0;
        PixIter it(tm.tl, tm.TT, mx);
        for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
          const uint8_t mk = __ldg(fr.mask + (y1 + it.j - 1) * fr.W + (x1 + it.i - 1)) != 0;
          mtile[p] = mk;
          if (!mk) z = 1;
        }
        has_masked = tm.any(z, iscr) != 0;
        if (has_masked) bwselect_team(tm, mtile, bwf, mx, my, sr, sc, 4, iscr);
        tm.sync();
      }
    }

    const uint8_t* bw = has_masked ? bwf : nullptr;  // nullptr: every pixel selected
    double hinv[6];  // lane k < 6: row k of the inverse Hessian (6-DOF)
    bool hok = false;
    double i00 = 0, i01 = 0, i10 = 0, i11 = 0;  // inverse of the 2x2 system (2-DOF)
    // f-side statistics: Hessian (6x6 or 2x2), meanf, bottomf, sum |tempf|
    auto f_side = [&]() {
      float hs[21];
#pragma unroll
      for (int k = 0; k < 21; ++k) hs[k] = 0.f;
      Kahan sf;
      float nf = 0.f, sa = 0.f;
      PixIter it(tm.tl, tm.TT, mx);
      for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
        const int i = it.i, j = it.j;
        const float s = bw ? (float)bw[p] : 1.f;
        const float gx = fr.GX(x1 + i, y1 + j) * s, gy = fr.GY(x1 + i, y1 + j) * s;
        const float fv = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j) * s;
        if constexpr (TWO) tf[p] = fv;
        sa += fabsf(fv);
        if (fabsf(fv) > 1e-10f) { sf.add(fv); nf += 1.f; }
        if constexpr (TWO) {
          hs[0] += gx * gx; hs[1] += gx * gy; hs[2] += gy * gy;
        } else {
          const float dx = (float)(int)(x1 + i - x0), dy = (float)(int)(y1 + j - y0);
          const float J[6] = {dx * gx, dx * gy, dy * gx, dy * gy, gx, gy};
          int q = 0;
#pragma unroll
          for (int aa = 0; aa < 6; ++aa)
#pragma unroll
            for (int bb = aa; bb < 6; ++bb) hs[q++] += J[aa] * J[bb];
        }
      }
      float st4[4] = {sf.s, -sf.c, nf, sa};
      tm.template sumf<4>(st4, fscr);
      const float cnt = st4[2];
      const float mean = (st4[0] + st4[1]) / cnt;
      Kahan q;
      PixIter it2(tm.tl, tm.TT, mx);
      for (int p = tm.tl; p < npx; p += tm.TT, it2.next()) {
        float fv;
        if constexpr (TWO) fv = tf[p];
        else fv = fr.F(x1 + it2.i, y1 + it2.j) * fr.M(x1 + it2.i, y1 + it2.j) * (bw ? (float)bw[p] : 1.f);
        if (fabsf(fv) > 1e-10f) { const float d = fv - mean; q.add(d * d); }
      }
      float qq[2] = {q.s, -q.c};
      tm.template sumf<2>(qq, fscr);
      const float var = cnt == 0.f ? __int_as_float(0x7fc00000) : (cnt == 1.f ? 0.f : (qq[0] + qq[1]) / (cnt - 1.f));
      meanf = mean;
      bottomf = sqrtf((cnt - 1.f) * var);
      sabs = st4[3];
      if constexpr (TWO) {
        tm.template sumf<3>(*reinterpret_cast<float(*)[3]>(hs), fscr);
        const double b2 = (double)bottomf * (double)bottomf;
        A11 = (double)hs[0] * 2 / b2 + a.mu;
        A12 = (double)hs[1] * 2 / b2;
        A22 = (double)hs[2] * 2 / b2 + a.mu;
        // H2 + 1e-3 max(diag H2) I of funICGN_Subpb1.m:391-394, inverted once per change
        const double dmax = isnan(A11) ? A22 : (isnan(A22) ? A11 : fmax(A11, A22));
        solve2(A11 + 1e-3 * dmax, A12, A22 + 1e-3 * dmax, 1.0, 0.0, &i00, &i10);
        solve2(A11 + 1e-3 * dmax, A12, A22 + 1e-3 * dmax, 0.0, 1.0, &i01, &i11);
      } else {
        tm.template sumf<21>(hs, fscr);
        // Cholesky of H (every lane, FP64), then lane k < 6 solves for column k
        // of H^-1 (= row k by symmetry)
        double Hp[21];
#pragma unroll
        for (int k = 0; k < 21; ++k) Hp[k] = 0;
        {
          int q2 = 0;
#pragma unroll
          for (int aa = 0; aa < 6; ++aa)
#pragma unroll
            for (int bb = aa; bb < 6; ++bb) {
              // hs is (row aa, col bb >= aa); packed lower storage wants (bb, aa)
              Hp[bb * (bb + 1) / 2 + aa] = (double)hs[q2];
              ++q2;
            }
        }
        if (tm.tl == 0) {
          int q3 = 0;
          for (int aa = 0; aa < 6; ++aa)
            for (int bb = aa; bb < 6; ++bb) {
              ctl->Hm[aa * 6 + bb] = (double)hs[q3]; ctl->Hm[bb * 6 + aa] = (double)hs[q3]; ++q3;
            }
        }
        Chol6 ch;
        chol6_factor(Hp, ch);
        hok = ch.ok;
        double e[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) e[k] = (lane == k) ? 1.0 : 0.0;
        chol6_solve(ch, e, hinv);
      }
      tm.sync();
    };

    const bool run = (code == 0 && !nan_out);
    if (run) {
      f_side();
      hdone = true;
    }
    float normNew = 1.f, normAbs = 1.f, normInit = 0.f;
    int step = 0, cg = 0;
    bool err = false;
    bool oob = run ? corners_oob_warp(P, x0, y0, x1, y1, mx, my, a.W, a.H, lane) : false;
    while (run && step <= kMaxIter && normNew > tolf && normAbs > tolf) {
      ++step;
      if constexpr (!TWO) {
        if (step > 1 && (double)cntf > 0.0 * npx0) {
          const double r = sqrt((double)((ws0 + 1) * (ws0 + 1)) / (double)cg) * wx / 2;
          if (!isfinite(r)) { err = true; break; }
          const int nws = 2 * (int)ceil(r);
          if (nws != wx) {
            const long long nx1 = x0 - nws / 2, nx3 = x0 + nws / 2, ny1 = y0 - nws / 2, ny3 = y0 + nws / 2;
            if (!mask_crop_ok32(fr, nx1, nx3, ny1, ny3)) { err = true; break; }
            if (corners_oob_warp(P, x0, y0, nx1, ny1, nws + 1, nws + 1, a.W, a.H, lane)) { normNew = 1e6f; break; }
            err = true;
            break;
          }
        }
      }
      if (oob) { normNew = 1e6f; break; }
      // integer base + FP32 offsets of the warp
      const double bu = (double)x0 + P[4], bv = (double)y0 + P[5];
      const int iu = (int)floor(bu), iv = (int)floor(bv);
      const float fu = (float)(bu - iu), fv0 = (float)(bv - iv);
      const float p0 = (float)(1 + P[0]), p1 = (float)P[1], p2 = (float)P[2], p3 = (float)(1 + P[3]);
      const float dx0 = (float)(int)(x1 - x0), dy0 = (float)(int)(y1 - y0);
      const float shift = meanf;  // one-pass variance around meanf
      int zg = 0, nang = 0;
      Kahan sg, qg;
      float ng = 0.f;
      {
        PixIter it(tm.tl, tm.TT, mx);
        for (int p = tm.tl; p < npx; p += tm.TT, it.next()) {
          const float dx = dx0 + (float)it.i, dy = dy0 + (float)it.j;
          const float su = fu + p0 * dx + p2 * dy;
          const float sv = fv0 + p1 * dx + p3 * dy;
          const float t = cubic32(fr.g, fr.W, fr.H, iu, su, iv, sv);
          tg[p] = t;
          if (t != t) nang = 1;
          if (t == 0.f) ++zg;
          if (fabsf(t) > 1e-10f) {
            const float d = t - shift;
            sg.add(d);
            qg.add(d * d);
            ng += 1.f;
          }
        }
      }
      zg = tm.sum_int(zg, iscr);
      if (tm.any(nang, iscr)) { err = true; break; }
      if (cntf > 0 || zg > 0) {
        for (int p = tm.tl; p < npx; p += tm.TT) tmp[p] = tg[p] != 0.f;
        tm.sync();
        bwselect_team(tm, tmp, bwg, mx, my, sr, sc, TWO ? 4 : 8, iscr);
        int anyzero = 0;
        for (int p = tm.tl; p < npx; p += tm.TT) anyzero |= !bwg[p];
        if (!tm.any(anyzero, iscr)) bwselect_team(tm, mtile, bwg, mx, my, sr, sc, 8, iscr);
        int cnt = 0;
        sg = Kahan(); qg = Kahan(); ng = 0.f;
        for (int p = tm.tl; p < npx; p += tm.TT) {
          const float t = tg[p] * (float)bwg[p];
          tg[p] = t;
          cnt += bwg[p];
          if (fabsf(t) > 1e-10f) {
            const float d = t - shift;
            sg.add(d);
            qg.add(d * d);
            ng += 1.f;
          }
        }
        cg = tm.sum_int(cnt, iscr);
        if constexpr (TWO) {
          bw = bwg;
          f_side();
        }
      }
      // g statistics: mean and sqrt((n-1) var) from the shifted one-pass sums
      float gs[5] = {sg.s, -sg.c, qg.s, -qg.c, ng};
      tm.template sumf<5>(gs, fscr);
      const float cntg = gs[4];
      const float s1 = gs[0] + gs[1], s2 = gs[2] + gs[3];
      const float meang = shift + s1 / cntg;
      const float varg = cntg == 0.f ? __int_as_float(0x7fc00000)
                                     : (cntg == 1.f ? 0.f : fmaxf(s2 - s1 * s1 / cntg, 0.f) / (cntg - 1.f));
      const float bottomg = sqrtf((cntg - 1.f) * varg);
      const float mf = meanf, ibf = 1.f / bottomf;
      const float mg = meang, ibg = 1.f / bottomg;
      float bsum[TWO ? 4 : 12];
      if constexpr (TWO) {
        Kahan k0, k1;
        PixIter it3(tm.tl, tm.TT, mx);
        for (int p = tm.tl; p < npx; p += tm.TT, it3.next()) {
          const float s = bw ? (float)bw[p] : 1.f;
          const float gx = fr.GX(x1 + it3.i, y1 + it3.j) * s, gy = fr.GY(x1 + it3.i, y1 + it3.j) * s;
          const float r = (tf[p] - mf) * ibf - (tg[p] - mg) * ibg;
          k0.add(gx * r);
          k1.add(gy * r);
        }
        bsum[0] = k0.s; bsum[1] = -k0.c; bsum[2] = k1.s; bsum[3] = -k1.c;
        tm.template sumf<4>(bsum, fscr);
      } else {
        Kahan k[6];
        PixIter it3(tm.tl, tm.TT, mx);
        for (int p = tm.tl; p < npx; p += tm.TT, it3.next()) {
          const int i = it3.i, j = it3.j;
          const float s = bw ? (float)bw[p] : 1.f;
          const float gx = fr.GX(x1 + i, y1 + j) * s, gy = fr.GY(x1 + i, y1 + j) * s;
          const float fv = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j) * s;
          const float dx = dx0 + (float)i, dy = dy0 + (float)j;
          const float r = (fv - mf) * ibf - (tg[p] - mg) * ibg;
          const float gxr = gx * r, gyr = gy * r;
          k[0].add(dx * gxr); k[1].add(dx * gyr); k[2].add(dy * gxr); k[3].add(dy * gyr);
          k[4].add(gxr); k[5].add(gyr);
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) { bsum[2 * q] = k[q].s; bsum[2 * q + 1] = -k[q].c; }
        tm.template sumf<12>(bsum, fscr);
      }
      // convergence test (FP32) and the FP64 update, identical on every warp
      int done = 0;
      float nb = 0.f;
      double D[6] = {0, 0, 0, 0, 0, 0};
      if constexpr (TWO) {
        const float b0 = bottomf * (bsum[0] + bsum[1]), b1 = bottomf * (bsum[2] + bsum[3]);
        const float sc2 = 2.f / (bottomf * bottomf);
        const float tb0 = b0 * sc2 + (float)(a.mu * (P[4] - a.UOld[2 * item] - a.vdual[2 * item]));
        const float tb1 = b1 * sc2 + (float)(a.mu * (P[5] - a.UOld[2 * item + 1] - a.vdual[2 * item + 1]));
        nb = tb0 * tb0 + tb1 * tb1;
        D[4] = -(i00 * (double)tb0 + i01 * (double)tb1);
        D[5] = -(i10 * (double)tb0 + i11 * (double)tb1);
      } else {
        float b[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) { b[q] = bottomf * (bsum[2 * q] + bsum[2 * q + 1]); nb += b[q] * b[q]; }
        if (hok) {
          double dk = 0;
#pragma unroll
          for (int q = 0; q < 6; ++q) dk += hinv[q] * (double)b[q];
#pragma unroll
          for (int q = 0; q < 6; ++q) D[q] = -shfl_d(dk, q);
        } else {
          double bd[6];
#pragma unroll
          for (int q = 0; q < 6; ++q) bd[q] = (double)b[q];
          small_solve(ctl->Hm, bd, 6, D);
#pragma unroll
          for (int q = 0; q < 6; ++q) D[q] = -D[q];
        }
      }
      float nN = sqrtf(nb);
      const float nA = nN;
      if (step == 1) normInit = nN;
      nN = normInit > tolf ? nN / normInit : 0.f;
      normNew = nN;
      normAbs = nA;
      if (nN < tolf || nA < tolf) done = 1;
      else if (!compose_warp(P, D, lane)) done = 2;
      if (done) break;
      oob = corners_oob_warp(P, x0, y0, x1, y1, mx, my, a.W, a.H, lane);
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
      a.U[2 * item] = nan_out ? nan("") : P[4];
      a.U[2 * item + 1] = nan_out ? nan("") : P[5];
      if constexpr (!TWO) {
#pragma unroll
        for (int k = 0; k < 4; ++k) a.F[4 * item + k] = nan_out ? nan("") : P[k];
        if (a.Hpk) {
          int q = 0;
          const bool hv = hdone && !nan_out && code != kMaxIter + 2;
          for (int col = 0; col < 6; ++col)
            for (int row = col; row < 6; ++row)
              a.Hpk[(size_t)q++ * Ntot + item] = hv ? ctl->Hm[row * 6 + col] : 0.0;
        }
      }
    }
    tm.sync();
  }
}

template <int TW, bool TWO>
static cudaError_t launch_tw(const BatchedArgs& b, int blocks, int threads, cudaStream_t s) {
  const int teams = threads / (TW * 32);
  const size_t smem = batched_team_bytes(b.smem_px, TWO, TW) * teams;
  if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(icgn_batched_kernel<TW, TWO>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  icgn_batched_kernel<TW, TWO><<<blocks, threads, smem, s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_icgn_batched(const BatchedArgs& b, int blocks, int threads, cudaStream_t s) {
  const bool two = b.two_dof != 0;
  switch (b.warps_per_subset) {
    case 1: return two ? launch_tw<1, true>(b, blocks, threads, s) : launch_tw<1, false>(b, blocks, threads, s);
    case 2: return two ? launch_tw<2, true>(b, blocks, threads, s) : launch_tw<2, false>(b, blocks, threads, s);
    case 4: return two ? launch_tw<4, true>(b, blocks, threads, s) : launch_tw<4, false>(b, blocks, threads, s);
  }
  return cudaErrorInvalidValue;
}

// Resident blocks per SM of one configuration (for grid sizing and the autotuner).
int batched_blocks_per_sm(int tw, bool two, int threads, int smem_px) {
  const int teams = threads / (tw * 32);
  const size_t smem = batched_team_bytes(smem_px, two, tw) * teams;
  if (smem > 227 * 1024) return 0;
  int nb = 0;
  cudaError_t e = cudaSuccess;
#define STDIC_OCC(TWv, TWOv)                                                                 \
  e = cudaFuncSetAttribute(icgn_batched_kernel<TWv, TWOv>,                                   \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);          \
  if (e == cudaSuccess)                                                                      \
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, icgn_batched_kernel<TWv, TWOv>,   \
                                                      threads, smem);
  switch (tw) {
    case 1: if (two) { STDIC_OCC(1, true) } else { STDIC_OCC(1, false) } break;
    case 2: if (two) { STDIC_OCC(2, true) } else { STDIC_OCC(2, false) } break;
    case 4: if (two) { STDIC_OCC(4, true) } else { STDIC_OCC(4, false) } break;
    default: return 0;
  }
#undef STDIC_OCC
  return e == cudaSuccess ? nb : 0;
}

}  // namespace stdic
