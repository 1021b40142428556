// Device helpers shared by the STAQ-DIC kernels (sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define STDIC_DEV __device__ __forceinline__

namespace stdic {

constexpr int kMaxIter = 100;  // maxIterNum of funICGNQuadtree.m:59

// Exclusive prefix sum of n ints by one CTA of blockDim.x threads (a multiple
// of 32, at most 1024): each thread sums a contiguous segment, the segment
// sums are scanned with warp shuffles, then each thread writes its segment.
// out has n + 1 entries (out[n] = total).
STDIC_DEV void cta_exclusive_scan(const int* in, int* out, int n) {
  __shared__ int warp_tot[32];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b0 = min(n, (int)threadIdx.x * per), b1 = min(n, b0 + per);
  int s = 0;
  for (int k = b0; k < b1; ++k) s += in[k];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = s;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    int v = lane < nw ? warp_tot[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane < nw) warp_tot[lane] = v;  // inclusive warp totals
  }
  __syncthreads();
  int acc = inc - s + (wid ? warp_tot[wid - 1] : 0);
  for (int k = b0; k < b1; ++k) { const int t = in[k]; out[k] = acc; acc += t; }
  if (threadIdx.x == blockDim.x - 1) out[n] = acc;
}

// Correlation values within this of a map's maximum count as equal in the
// integer searches' peak choice: the first such lag (column-major) is the
// peak, which is findpeak's first maximum whenever the maximum is unique.  A
// degenerate map -- a template with a single nonzero pixel in a masked region
// -- holds several lags equal to 1 in exact arithmetic, and without the rule
// rounding alone would choose among them.
constexpr double kPeakTie = 1e-10;

// Index of the first of n values C[] (visible to the whole CTA) that lies
// within kPeakTie of their maximum; every thread receives it.  All threads of
// the CTA must call it (blockDim.x <= 1024).
STDIC_DEV int cta_first_near_max(const double* C, int n) {
  __shared__ double s_v[32];
  __shared__ int s_i[32];
  const int nw = (blockDim.x + 31) >> 5;
  double m = -INFINITY;
  for (int k = threadIdx.x; k < n; k += blockDim.x) m = fmax(m, C[k]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s_v[threadIdx.x >> 5] = m;
  __syncthreads();
  m = -INFINITY;
  for (int w = 0; w < nw; ++w) m = fmax(m, s_v[w]);
  int first = 0x7fffffff;
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    if (C[k] >= m - kPeakTie) { first = k; break; }
  for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
  if ((threadIdx.x & 31) == 0) s_i[threadIdx.x >> 5] = first;
  __syncthreads();
  first = 0x7fffffff;
  for (int w = 0; w < nw; ++w) first = min(first, s_i[w]);
  __syncthreads();
  return first;
}

// findpeak.m:40-68 on the 3 x 3 neighbourhood of a correlation maximum,
// v9[(dr+1) + 3 (dc+1)] at row offset dr and column offset dc: the least-
// squares quadratic [1 x y xy x^2 y^2] (x = column, y = row offset) in the
// closed form of that fixed 9-point design, its stationary point (xo, yo)
// and value there.  Returns false (the peak stays on the sample) when the fit
// moves it by more than one sample; otherwise the offsets are rounded to
// 1/1000 first, as the reference does, and the value is taken there.
STDIC_DEV bool findpeak_fit3(const double* v9, double* xo_out, double* yo_out, double* maxf) {
  double s0 = 0, sx = 0, sy = 0, sxy = 0, sxx = 0, syy = 0;
  for (int dc = -1; dc <= 1; ++dc)
    for (int dr = -1; dr <= 1; ++dr) {
      const double uu = v9[(dr + 1) + 3 * (dc + 1)];
      s0 += uu; sx += dc * uu; sy += dr * uu; sxy += dc * dr * uu;
      sxx += dc * dc * uu; syy += dr * dr * uu;
    }
  const double A2 = sx / 6, A3 = sy / 6, A4 = sxy / 4;
  const double Sv = (sxx + syy) / 2 - (2.0 / 3.0) * s0;
  const double Dd = (sxx - syy) / 2;
  const double A5 = (Sv + Dd) / 2, A6 = (Sv - Dd) / 2;
  const double A1 = (s0 - 6 * Sv) / 9;
  double xo = (-A3 * A4 + 2 * A6 * A2) / (A4 * A4 - 4 * A5 * A6);
  double yo = -1 / (A4 * A4 - 4 * A5 * A6) * (A4 * A2 - 2 * A5 * A3);
  if (fabs(xo) > 1 || fabs(yo) > 1) return false;
  xo = round(1000 * xo) / 1000;
  yo = round(1000 * yo) / 1000;
  *xo_out = xo;
  *yo_out = yo;
  *maxf = A1 + xo * A2 + yo * A3 + xo * yo * A4 + xo * xo * A5 + yo * yo * A6;
  return true;
}

// ---------------------------------------------------------------------------
// Keys cubic (a = -1/2) interpolation with clamp-to-edge borders, evaluated in
// the exact operation order of ba_interp2.cpp:188-233 with every product and
// sum rounded separately (no fused multiply-add), so results match the
// reference's compiled C++ bit for bit.  F is M x N column-major; X indexes
// dim 2 (column), Y dim 1 (row), both 1-based.
// ---------------------------------------------------------------------------
STDIC_DEV long long clamp_access(long long M, long long N, long long x, long long y) {
  x = x < 0 ? 0 : (x >= N ? N - 1 : x);
  y = y < 0 ? 0 : (y >= M ? M - 1 : y);
  return M * x + y;
}

STDIC_DEV double dm(double a, double b) { return __dmul_rn(a, b); }
STDIC_DEV double da(double a, double b) { return __dadd_rn(a, b); }
STDIC_DEV double ds(double a, double b) { return __dsub_rn(a, b); }

STDIC_DEV void cubic_weights_exact(double d, double w[4]) {
  const double dd = dm(d, d), ddd = dm(dd, d);
  // 0.5 * (-d + 2 dd - ddd), 0.5 * (2 - 5 dd + 3 ddd), 0.5 * (d + 4 dd - 3 ddd), 0.5 * (-dd + ddd)
  w[0] = dm(0.5, ds(da(-d, dm(2.0, dd)), ddd));
  w[1] = dm(0.5, da(ds(2.0, dm(5.0, dd)), dm(3.0, ddd)));
  w[2] = dm(0.5, ds(da(d, dm(4.0, dd)), dm(3.0, ddd)));
  w[3] = dm(0.5, da(-dd, ddd));
}

// The reference's single-precision template computes the weights in double
// (its literals are double) and rounds them once to float.
STDIC_DEV void cubic_weights_exact_f32(float d, float w[4]) {
  const float dd = __fmul_rn(d, d), ddd = __fmul_rn(dd, d);
  const double D = d, DD = dd, DDD = ddd;
  w[0] = (float)dm(0.5, ds(da(-D, dm(2.0, DD)), DDD));
  w[1] = (float)dm(0.5, da(ds(2.0, dm(5.0, DD)), dm(3.0, DDD)));
  w[2] = (float)dm(0.5, ds(da(D, dm(4.0, DD)), dm(3.0, DDD)));
  w[3] = (float)dm(0.5, da(-DD, DDD));
}

STDIC_DEV double ba_cubic_exact(const double* __restrict__ F, long long M, long long N, double X,
                                double Y) {
  const double xf = floor(X), yf = floor(Y);
  double wx[4], wy[4];
  cubic_weights_exact(ds(X, xf), wx);
  cubic_weights_exact(ds(Y, yf), wy);
  const long long x = (long long)(xf - 1), y = (long long)(yf - 1);
  const bool fast = !(x <= 2 || y <= 2 || x >= N - 3 || y >= M - 3);
  double acc = 0.0;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    double row;
    if (fast) {
      const long long base = M * (x - 1) + (y - 1 + b);
      row = dm(wx[0], __ldg(F + base));
      row = da(row, dm(wx[1], __ldg(F + base + M)));
      row = da(row, dm(wx[2], __ldg(F + base + 2 * M)));
      row = da(row, dm(wx[3], __ldg(F + base + 3 * M)));
    } else {
      row = dm(wx[0], __ldg(F + clamp_access(M, N, x - 1, y - 1 + b)));
      row = da(row, dm(wx[1], __ldg(F + clamp_access(M, N, x, y - 1 + b))));
      row = da(row, dm(wx[2], __ldg(F + clamp_access(M, N, x + 1, y - 1 + b))));
      row = da(row, dm(wx[3], __ldg(F + clamp_access(M, N, x + 2, y - 1 + b))));
    }
    acc = b == 0 ? dm(wy[0], row) : da(acc, dm(wy[b], row));
  }
  return acc;
}

STDIC_DEV float ba_cubic_exact_f32(const float* __restrict__ F, long long M, long long N, float X,
                                   float Y) {
  const float xf = floorf(X), yf = floorf(Y);
  float wx[4], wy[4];
  cubic_weights_exact_f32(__fsub_rn(X, xf), wx);
  cubic_weights_exact_f32(__fsub_rn(Y, yf), wy);
  const long long x = (long long)(xf - 1), y = (long long)(yf - 1);
  float acc = 0.f;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    float row = __fmul_rn(wx[0], __ldg(F + clamp_access(M, N, x - 1, y - 1 + b)));
    row = __fadd_rn(row, __fmul_rn(wx[1], __ldg(F + clamp_access(M, N, x, y - 1 + b))));
    row = __fadd_rn(row, __fmul_rn(wx[2], __ldg(F + clamp_access(M, N, x + 1, y - 1 + b))));
    row = __fadd_rn(row, __fmul_rn(wx[3], __ldg(F + clamp_access(M, N, x + 2, y - 1 + b))));
    acc = b == 0 ? __fmul_rn(wy[0], row) : __fadd_rn(acc, __fmul_rn(wy[b], row));
  }
  return acc;
}

// ---------------------------------------------------------------------------
// Block-wide sums of K doubles: warp shuffles, then one warp over the partials.
// scratch must hold K * 32 doubles.  Every thread returns the totals.
// ---------------------------------------------------------------------------
template <int K>
STDIC_DEV void block_sum(double (&v)[K], double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) scratch[k * 32 + warp] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double t = lane < nw ? scratch[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) scratch[k * 32] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = scratch[k * 32];
  __syncthreads();
}

STDIC_DEV int block_sum_int(int v, int* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int t = lane < nw ? scratch[lane] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) scratch[0] = t;
  }
  __syncthreads();
  const int r = scratch[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------------------
// bwselect(BW, c, r, conn) on an m x n tile in shared memory (BW[i + j*m]):
// the conn-connected component of the nonzero pixels that holds the 1-based
// seed (r = row along dim 1, c = column along dim 2).  An out-of-range or
// background seed selects nothing.  Line sweeps along both dimensions repeat
// until a full pass adds no pixel; every productive pass adds at least one
// pixel, so the loop ends after at most m*n passes.  Concurrent sweeps only
// ever set 0 -> 1, so reading a neighbour that another thread is setting can
// only delay propagation to the next pass, never change the fixed point.
// ---------------------------------------------------------------------------
STDIC_DEV bool sel_nb(const volatile uint8_t* s, int m, int n, int i, int j, int conn) {
  bool r = false;
  if (i > 0) r |= s[(i - 1) + j * m];
  if (i + 1 < m) r |= s[(i + 1) + j * m];
  if (j > 0) r |= s[i + (j - 1) * m];
  if (j + 1 < n) r |= s[i + (j + 1) * m];
  if (conn == 8) {
    if (i > 0 && j > 0) r |= s[(i - 1) + (j - 1) * m];
    if (i + 1 < m && j > 0) r |= s[(i + 1) + (j - 1) * m];
    if (i > 0 && j + 1 < n) r |= s[(i - 1) + (j + 1) * m];
    if (i + 1 < m && j + 1 < n) r |= s[(i + 1) + (j + 1) * m];
  }
  return r;
}

STDIC_DEV void bwselect_block(const uint8_t* allow, uint8_t* sel_, int m, int n, int r1, int c1,
                              int conn) {
  volatile uint8_t* sel = sel_;
  const int npx = m * n;
  for (int p = threadIdx.x; p < npx; p += blockDim.x) sel[p] = 0;
  __syncthreads();
  if (threadIdx.x == 0 && r1 >= 1 && r1 <= m && c1 >= 1 && c1 <= n) {
    const int s = (r1 - 1) + (c1 - 1) * m;
    if (allow[s]) sel[s] = 1;
  }
  __syncthreads();
  for (;;) {
    int changed = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      for (int i = 0; i < m; ++i) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
      for (int i = m - 1; i >= 0; --i) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      for (int j = 0; j < n; ++j) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
      for (int j = n - 1; j >= 0; --j) {
        const int p = i + j * m;
        if (!sel[p] && allow[p] && sel_nb(sel, m, n, i, j, conn)) { sel[p] = 1; changed = 1; }
      }
    }
    if (!__syncthreads_or(changed)) break;
  }
}

// ---------------------------------------------------------------------------
// x = A \ b for n <= 6: Cholesky when the diagonal is positive and the
// factorisation succeeds (MATLAB mldivide's path for a symmetric matrix with
// positive diagonal), otherwise LU with partial pivoting.  A is row-major.
// ---------------------------------------------------------------------------
STDIC_DEV void small_solve(const double* Ain, const double* b, int n, double* x) {
  double A[36], L[36];
  for (int k = 0; k < n * n; ++k) A[k] = Ain[k];
  bool spd = true;
  for (int i = 0; i < n; ++i)
    if (!(A[i * n + i] > 0)) spd = false;
  if (spd) {
    for (int k = 0; k < n * n; ++k) L[k] = 0;
    for (int j = 0; j < n && spd; ++j) {
      double d = A[j * n + j];
      for (int k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
      if (!(d > 0)) { spd = false; break; }
      const double ljj = sqrt(d);
      L[j * n + j] = ljj;
      for (int i = j + 1; i < n; ++i) {
        double s = A[i * n + j];
        for (int k = 0; k < j; ++k) s -= L[i * n + k] * L[j * n + k];
        L[i * n + j] = s / ljj;
      }
    }
    if (spd) {
      double y[6];
      for (int i = 0; i < n; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[i * n + k] * y[k];
        y[i] = s / L[i * n + i];
      }
      for (int i = n - 1; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < n; ++k) s -= L[k * n + i] * x[k];
        x[i] = s / L[i * n + i];
      }
      return;
    }
  }
  double bb[6];
  for (int i = 0; i < n; ++i) bb[i] = b[i];
  for (int k = 0; k < n; ++k) {
    int p = k;
    double amax = fabs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[i * n + k]) > amax) { amax = fabs(A[i * n + k]); p = i; }
    if (p != k) {
      for (int j = 0; j < n; ++j) { const double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
      const double t = bb[k]; bb[k] = bb[p]; bb[p] = t;
    }
    for (int i = k + 1; i < n; ++i) {
      const double f = A[i * n + k] / A[k * n + k];
      for (int j = k; j < n; ++j) A[i * n + j] -= f * A[k * n + j];
      bb[i] -= f * bb[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = bb[i];
    for (int j = i + 1; j < n; ++j) s -= A[i * n + j] * x[j];
    x[i] = s / A[i * n + i];
  }
}

// small_solve's Cholesky branch for n = 6 split in two, for a matrix that
// stays fixed while right-hand sides change: chol6_factor forms L (row-major,
// the same operations in the same order as small_solve) and returns false
// where small_solve would take its LU branch; chol6_solve then gives, for
// each b, the x small_solve gives.  With n fixed the arrays live in registers.
STDIC_DEV bool chol6_factor(const double* A, double* L) {
#pragma unroll
  for (int i = 0; i < 6; ++i)
    if (!(A[i * 6 + i] > 0)) return false;
  double l[36];
#pragma unroll
  for (int k = 0; k < 36; ++k) l[k] = 0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double d = A[j * 6 + j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= l[j * 6 + k] * l[j * 6 + k];
    if (!(d > 0)) return false;
    const double ljj = sqrt(d);
    l[j * 6 + j] = ljj;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double s = A[i * 6 + j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= l[i * 6 + k] * l[j * 6 + k];
      l[i * 6 + j] = s / ljj;
    }
  }
#pragma unroll
  for (int k = 0; k < 36; ++k) L[k] = l[k];
  return true;
}

STDIC_DEV void chol6_solve(const double* L, const double* b, double* x) {
  double y[6], z[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double s = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s -= L[i * 6 + k] * y[k];
    y[i] = s / L[i * 6 + i];
  }
#pragma unroll
  for (int i = 5; i >= 0; --i) {
    double s = y[i];
#pragma unroll
    for (int k = i + 1; k < 6; ++k) s -= L[k * 6 + i] * z[k];
    z[i] = s / L[i * 6 + i];
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) x[i] = z[i];
}

// x = A \ b for a symmetric 2x2 A = [a11 a12; a12 a22] in registers, with the
// branch structure of small_solve (Cholesky when it succeeds, else LU with
// partial pivoting).
STDIC_DEV void solve2(double a11, double a12, double a22, double b0, double b1, double* x0,
                      double* x1) {
  if (a11 > 0 && a22 > 0) {
    const double l11 = sqrt(a11);
    const double l21 = a12 / l11;
    const double d = a22 - l21 * l21;
    if (d > 0) {
      const double l22 = sqrt(d);
      const double y0 = b0 / l11, y1 = (b1 - l21 * y0) / l22;
      *x1 = y1 / l22;
      *x0 = (y0 - l21 * *x1) / l11;
      return;
    }
  }
  double r00 = a11, r01 = a12, r10 = a12, r11 = a22, c0 = b0, c1 = b1;
  if (fabs(r10) > fabs(r00)) {
    double t = r00; r00 = r10; r10 = t;
    t = r01; r01 = r11; r11 = t;
    t = c0; c0 = c1; c1 = t;
  }
  const double f = r10 / r00;
  r11 -= f * r01;
  c1 -= f * c0;
  *x1 = c1 / r11;
  *x0 = (c0 - r01 * *x1) / r00;
}

// Inverse-compositional update of P by DeltaP (funICGNQuadtree.m:393-411).
// Returns false when det(DeltaP) == 0 (the reference then leaves the loop).
STDIC_DEV bool compose_update(double P[6], const double D[6]) {
  const double det = (1 + D[0]) * (1 + D[3]) - D[1] * D[2];
  if (!(det != 0)) return false;
  const double t1 = (-D[0] - D[0] * D[3] + D[1] * D[2]) / det;
  const double t2 = -D[1] / det;
  const double t3 = -D[2] / det;
  const double t4 = (-D[3] - D[0] * D[3] + D[1] * D[2]) / det;
  const double t5 = (-D[4] - D[3] * D[4] + D[2] * D[5]) / det;
  const double t6 = (-D[5] - D[0] * D[5] + D[1] * D[4]) / det;
  const double a11 = 1 + P[0], a12 = P[2], a13 = P[4];
  const double a21 = P[1], a22 = 1 + P[3], a23 = P[5];
  const double b11 = 1 + t1, b12 = t3, b13 = t5;
  const double b21 = t2, b22 = 1 + t4, b23 = t6;
  const double m11 = a11 * b11 + a12 * b21;
  const double m21 = a21 * b11 + a22 * b21;
  const double m12 = a11 * b12 + a12 * b22;
  const double m22 = a21 * b12 + a22 * b22;
  const double m13 = a11 * b13 + a12 * b23 + a13;
  const double m23 = a21 * b13 + a22 * b23 + a23;
  P[0] = m11 - 1; P[1] = m21; P[2] = m12; P[3] = m22 - 1; P[4] = m13; P[5] = m23;
  return true;
}

// Warped position of tile pixel (dx, dy) = (X - x0, Y - y0), evaluated as
// (1+P1)*dx + P3*dy + (x0+P5) with separate roundings (funICGNQuadtree.m:151-152).
STDIC_DEV void warp_exact(const double P[6], double dx, double dy, double x0, double y0,
                          double* u22, double* v22) {
  *u22 = da(da(dm(1 + P[0], dx), dm(P[2], dy)), x0 + P[4]);
  *v22 = da(da(dm(P[1], dx), dm(1 + P[3], dy)), y0 + P[5]);
}

// Window growth used when part of a subset is masked (funICGNQuadtree.m:70):
// 2*ceil(sqrt(num/den) * ws / 2) in IEEE double.
STDIC_DEV double grow_window(double num, double den, int ws) {
  return 2.0 * ceil(sqrt(num / den) * ws / 2);
}

}  // namespace stdic
