// ORACLE — test infrastructure only.  CPU FP64 restatement of STAQ-DIC's
// augmented-Lagrangian hot path.  Only tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py may load this library, and only as the checker
// or the timed CPU baseline; the product path never calls it.
//
// Every routine follows one reference routine line by line (paths relative to
// the STAQ-DIC repository):
//   orc_interp_bicubic_*  ba_interp2.cpp:60-130 (access, indices_cubic),
//                         :184-234 (interpolate_bicubic_unrolled)
//   orc_img_gradient      func/funImgGradient.m:53-78
//   orc_integer_search    func/funIntegerSearch.m:3-27 (grid shrink),
//                         :82-203 (whole-field loop), func/findpeak.m:27-68,
//                         normxcorr2 restated from its published definition
//   orc_icgn6             func_quadtree/funICGNQuadtree.m:29-448 driven as in
//                         func_quadtree/LocalICGNQuadtree.m:67-147
//   orc_icgn2             func/funICGN_Subpb1.m:34-471 driven as in
//                         func_quadtree/Subpb1Quadtree.m:75-169
//   orc_nodal_strain      funGlobalNodalStrainQuadtree.m:80-257 (Gauss-point
//                         strains); nodal recovery is a local replacement
//   orc_fill_nans         local replacement of Subpb1Quadtree.m:193-259's fill
//   orc_adjoint           no counterpart: gradient of the ZNSSD subset cost of
//                         funICGNQuadtree.m:151-165 (pinned by finite differences)
//   orc_subpb2_assemble   func_quadtree/Subpb2Quadtree.m:30-336 (element loop,
//                         sparse triplets, Dirichlet lift); the linear solve of
//                         :339 is done by the Python side with a direct solver.
//
// Data layout is MATLAB's: column-major arrays, the first index contiguous.
// Images are W x H with x = dim 1.  Node coordinates are 1-based pixels.
// Arithmetic is plain IEEE double; build with -ffp-contract=off so that a
// compiler never fuses a multiply-add the reference evaluates as two roundings.
//
// MATLAB semantics kept on purpose:
//   * NaN comparisons are false, mean([]) and var([]) are NaN, var(scalar)=0;
//   * a MATLAB run-time error inside funICGNQuadtree (index out of range, size
//     mismatch, logical(NaN)) is caught by LocalICGNQuadtree and gives code -1
//     with NaN outputs; in Subpb1Quadtree the same catch leaves code 0 and NaN.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cfloat>
#include <vector>
#include <algorithm>

#ifdef _OPENMP
#include <omp.h>
#endif

// ---------------------------------------------------------------------------
// ba_interp2 (cubic).  F is M x N column-major, X indexes dim 2 (columns) and
// Y indexes dim 1 (rows), both 1-based.  Borders repeat the closest sample.
// ---------------------------------------------------------------------------
static inline long ba_access(long M, long N, long x, long y) {
  if (x < 0) x = 0; else if (x >= N) x = N - 1;
  if (y < 0) y = 0; else if (y >= M) y = M - 1;
  return M * x + y;
}

template <class REAL>
static inline REAL ba_cubic_one(const REAL* F, long M, long N, REAL X, REAL Y) {
  const REAL xf = std::floor(X), yf = std::floor(Y);
  const REAL dx = X - xf, dy = Y - yf;
  const REAL dxx = dx * dx, dxxx = dxx * dx;
  const REAL dyy = dy * dy, dyyy = dyy * dy;
  // Weights evaluated exactly as the reference writes them; the literal 0.5 and
  // 2.0 are doubles, so for REAL=float the weights round once from double.
  const REAL wx0 = 0.5 * (-dx + 2.0 * dxx - dxxx);
  const REAL wx1 = 0.5 * (2.0 - 5.0 * dxx + 3.0 * dxxx);
  const REAL wx2 = 0.5 * (dx + 4.0 * dxx - 3.0 * dxxx);
  const REAL wx3 = 0.5 * (-dxx + dxxx);
  const REAL wy0 = 0.5 * (-dy + 2.0 * dyy - dyyy);
  const REAL wy1 = 0.5 * (2.0 - 5.0 * dyy + 3.0 * dyyy);
  const REAL wy2 = 0.5 * (dy + 4.0 * dyy - 3.0 * dyyy);
  const REAL wy3 = 0.5 * (-dyy + dyyy);
  const long x = (long)(xf - 1), y = (long)(yf - 1);
  long i[4][4];  // i[col offset][row offset]
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) i[a][b] = ba_access(M, N, x - 1 + a, y - 1 + b);
  return wy0 * (wx0 * F[i[0][0]] + wx1 * F[i[1][0]] + wx2 * F[i[2][0]] + wx3 * F[i[3][0]]) +
         wy1 * (wx0 * F[i[0][1]] + wx1 * F[i[1][1]] + wx2 * F[i[2][1]] + wx3 * F[i[3][1]]) +
         wy2 * (wx0 * F[i[0][2]] + wx1 * F[i[1][2]] + wx2 * F[i[2][2]] + wx3 * F[i[3][2]]) +
         wy3 * (wx0 * F[i[0][3]] + wx1 * F[i[1][3]] + wx2 * F[i[2][3]] + wx3 * F[i[3][3]]);
}

extern "C" void orc_interp_bicubic_f64(const double* F, long M, long N, const double* X, const double* Y,
                            long n, double* out) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < n; ++k) out[k] = ba_cubic_one<double>(F, M, N, X[k], Y[k]);
}

extern "C" void orc_interp_bicubic_f32(const float* F, long M, long N, const float* X, const float* Y,
                            long n, float* out) {
#pragma omp parallel for schedule(static)
  for (long k = 0; k < n; ++k) out[k] = ba_cubic_one<float>(F, M, N, X[k], Y[k]);
}

// ---------------------------------------------------------------------------
// funImgGradient: 7-tap 6th-order central difference (correlation) along each
// dimension, crop 3, multiply by the mask.  Output (W-6) x (H-6).
// ---------------------------------------------------------------------------
extern "C" void orc_img_gradient(const double* img, const uint8_t* mask, long W, long H, double* dfdx,
                      double* dfdy) {
  static const double h[7] = {-1.0 / 60, 3.0 / 20, -3.0 / 4, 0.0, 3.0 / 4, -3.0 / 20, 1.0 / 60};
  const long Wo = W - 6, Ho = H - 6;
#pragma omp parallel for schedule(static)
  for (long j = 0; j < Ho; ++j) {
    for (long i = 0; i < Wo; ++i) {
      const long x = i + 3, y = j + 3;  // 0-based pixel of output (i, j)
      double sx = 0.0, sy = 0.0;
      for (int k = 0; k < 7; ++k) {
        sx += h[k] * img[y * W + (x + k - 3)];
        sy += h[k] * img[(y + k - 3) * W + x];
      }
      const double m = (double)mask[y * W + x];
      dfdx[j * Wo + i] = sx * m;
      dfdy[j * Wo + i] = sy * m;
    }
  }
}

// ---------------------------------------------------------------------------
// Small MATLAB helpers.
// ---------------------------------------------------------------------------
static inline double matlab_eps(double x) {
  x = std::fabs(x);
  if (!(x > 0)) return std::ldexp(1.0, -1074);
  if (!std::isfinite(x)) return NAN;
  int e;
  std::frexp(x, &e);  // x = f * 2^e, f in [0.5, 1)
  const int p = e - 53;
  return p < -1074 ? std::ldexp(1.0, -1074) : std::ldexp(1.0, p);
}

// Correlation values within this of the map's maximum count as equal in the
// integer searches' peak choice (the first such lag, column-major, wins).  A
// degenerate map -- a template with a single nonzero pixel inside a masked
// region -- has several lags equal to 1 in exact arithmetic, and rounding
// alone would pick among them.
static const double kPeakTie = 1e-10;

// bwselect(BW, c, r, n) on an m x n tile (column-major, BW[i + j*m]), seed at
// 1-based row r (dim 1) and column c (dim 2).  Returns the connected component
// of BW holding the seed; an out-of-range or background seed selects nothing.
static void bwselect_tile(const uint8_t* BW, int m, int nc, int r, int c, int conn, uint8_t* out) {
  std::memset(out, 0, (size_t)m * nc);
  if (r < 1 || r > m || c < 1 || c > nc) return;
  const int s = (r - 1) + (c - 1) * m;
  if (!BW[s]) return;
  std::vector<int> stack;
  stack.push_back(s);
  out[s] = 1;
  while (!stack.empty()) {
    const int p = stack.back();
    stack.pop_back();
    const int i = p % m, j = p / m;
    for (int dj = -1; dj <= 1; ++dj)
      for (int di = -1; di <= 1; ++di) {
        if (!di && !dj) continue;
        if (conn == 4 && di && dj) continue;
        const int ii = i + di, jj = j + dj;
        if (ii < 0 || ii >= m || jj < 0 || jj >= nc) continue;
        const int q = ii + jj * m;
        if (BW[q] && !out[q]) {
          out[q] = 1;
          stack.push_back(q);
        }
      }
  }
}

// mean / sqrt((n-1)*var) over the entries with |t| > 1e-10, as the reference
// computes meanf/bottomf (funICGNQuadtree.m:119-120).
static void masked_mean_bottom(const double* t, int n, double* mean_out, double* bottom_out) {
  double s = 0.0;
  long cnt = 0;
  for (int k = 0; k < n; ++k)
    if (std::fabs(t[k]) > 1e-10) { s += t[k]; ++cnt; }
  const double mean = s / (double)cnt;  // 0/0 = NaN for an empty selection
  double var;
  if (cnt == 0) var = NAN;
  else if (cnt == 1) var = 0.0;
  else {
    double q = 0.0;
    for (int k = 0; k < n; ++k)
      if (std::fabs(t[k]) > 1e-10) { const double d = t[k] - mean; q += d * d; }
    var = q / (double)(cnt - 1);
  }
  *mean_out = mean;
  *bottom_out = std::sqrt((double)(cnt - 1) * var);
}

// x = A \ b for a small dense SPD-looking matrix: Cholesky when it succeeds
// (MATLAB's mldivide path for a symmetric matrix with a positive diagonal),
// otherwise LU with partial pivoting.
static void small_solve(const double* Ain, const double* b, int n, double* x) {
  double A[36], L[36];
  std::memcpy(A, Ain, sizeof(double) * n * n);
  bool spd = true;
  for (int i = 0; i < n && spd; ++i)
    if (!(A[i * n + i] > 0)) spd = false;
  if (spd) {
    std::memset(L, 0, sizeof(L));
    for (int j = 0; j < n && spd; ++j) {
      double d = A[j * n + j];
      for (int k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
      if (!(d > 0)) { spd = false; break; }
      const double ljj = std::sqrt(d);
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
  // LU with partial pivoting
  double bb[6];
  for (int i = 0; i < n; ++i) bb[i] = b[i];
  for (int k = 0; k < n; ++k) {
    int p = k;
    double amax = std::fabs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > amax) { amax = std::fabs(A[i * n + k]); p = i; }
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
      std::swap(bb[k], bb[p]);
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

// Inverse-compositional update of P by DeltaP (funICGNQuadtree.m:393-411).
// Returns false when det(DeltaP) == 0 (the reference breaks out of the loop).
static bool compose_update(double P[6], const double D[6]) {
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

struct Frame {
  const double* f;      // reference image W x H
  const double* g;      // deformed image W x H
  const uint8_t* mask;  // reference mask W x H (0/1)
  const double* dfdx;   // (W-6) x (H-6)
  const double* dfdy;
  long W, H;
  inline double F(long x1, long y1) const { return f[(y1 - 1) * W + (x1 - 1)]; }
  inline double M(long x1, long y1) const { return (double)mask[(y1 - 1) * W + (x1 - 1)]; }
  inline double GX(long x1, long y1) const { return dfdx[(y1 - 4) * (W - 6) + (x1 - 4)]; }
  inline double GY(long x1, long y1) const { return dfdy[(y1 - 4) * (W - 6) + (x1 - 4)]; }
};

// The crops ImgRef(x1:x3, y1:y3) and Df.DfDx(x1-3:x3-3, y1-3:y3-3) are valid
// only for 4 <= x1, x3 <= W-3 (and the same in y); outside MATLAB throws.
static inline bool crop_ok(const Frame& fr, long x1, long x3, long y1, long y3) {
  return x1 >= 4 && x3 <= fr.W - 3 && y1 >= 4 && y3 <= fr.H - 3;
}
static inline bool mask_crop_ok(const Frame& fr, long x1, long x3, long y1, long y3) {
  return x1 >= 1 && x3 <= fr.W && y1 >= 1 && y3 <= fr.H;
}

struct Tile {
  int mx, my;  // tile extent in dim 1 / dim 2 = winsize_x+1, winsize_y+1
  long x1, y1;
  std::vector<double> f, gx, gy;
  std::vector<uint8_t> m;
  void load(const Frame& fr, long x1_, long y1_, int mx_, int my_) {
    mx = mx_; my = my_; x1 = x1_; y1 = y1_;
    const int n = mx * my;
    f.resize(n); gx.resize(n); gy.resize(n); m.resize(n);
    for (int j = 0; j < my; ++j)
      for (int i = 0; i < mx; ++i) {
        const int k = i + j * mx;
        const double mk = fr.M(x1 + i, y1 + j);
        m[k] = mk != 0;
        f[k] = fr.F(x1 + i, y1 + j) * mk;
        gx[k] = fr.GX(x1 + i, y1 + j);
        gy[k] = fr.GY(x1 + i, y1 + j);
      }
  }
};

static inline bool any_out_of_bounds(const Frame& fr, const double P[6], long x0, long y0, long x1,
                                     long y1, int mx, int my) {
  for (int j = 0; j < my; ++j)
    for (int i = 0; i < mx; ++i) {
      const double dx = (double)(x1 + i - x0), dy = (double)(y1 + j - y0);
      const double u22 = (1 + P[0]) * dx + P[2] * dy + ((double)x0 + P[4]);
      const double v22 = P[1] * dx + (1 + P[3]) * dy + ((double)y0 + P[5]);
      if (u22 < 3 || u22 > (double)fr.W - 2 || v22 < 3 || v22 > (double)fr.H - 2)
        return true;
    }
  return false;
}

// Warp the tile by P and sample g (ba_interp2(ImgDef, v22, u22)).
static void warp_sample(const Frame& fr, const double P[6], long x0, long y0, long x1, long y1,
                        int mx, int my, double* tg) {
  for (int j = 0; j < my; ++j)
    for (int i = 0; i < mx; ++i) {
      const double dx = (double)(x1 + i - x0), dy = (double)(y1 + j - y0);
      const double u22 = (1 + P[0]) * dx + P[2] * dy + ((double)x0 + P[4]);
      const double v22 = P[1] * dx + (1 + P[3]) * dy + ((double)y0 + P[5]);
      tg[i + j * mx] = ba_cubic_one<double>(fr.g, fr.W, fr.H, v22, u22);
    }
}

// ---------------------------------------------------------------------------
// funICGNQuadtree (6-DOF, Gauss-Newton) for one node.  Returns the code written
// to ConvItPerEle; P, Hpk (21 packed lower-triangle entries) are outputs.
// ---------------------------------------------------------------------------
// variant 0 follows the current source.  variant 1 restores the masked-g
// branch as it stood before the lines at funICGNQuadtree.m:184-205 were
// commented out (Feb 2024): tempf, DfDx, DfDy are re-cropped at the current
// window, masked by tempg_BW2, and H, meanf, bottomf recomputed — the form that
// produced the reference's shipped result file (created Nov 2023).  It exists
// only to pin this restatement against that file.
static int icgn6_one(const Frame& fr, double U0x, double U0y, long x0, long y0, int ws, double tol,
                     double P[6], double Hpk[21], int variant) {
  const int ws0 = ws;
  const int maxIterNum = 100;
  for (int k = 0; k < 21; ++k) Hpk[k] = 0;
  P[0] = P[1] = P[2] = P[3] = 0; P[4] = U0x; P[5] = U0y;
  long x1 = x0 - ws / 2, x3 = x0 + ws / 2, y1 = y0 - ws / 2, y3 = y0 + ws / 2;
  if (!mask_crop_ok(fr, x1, x3, y1, y3) || !crop_ok(fr, x1, x3, y1, y3)) return -1;
  Tile T;
  T.load(fr, x1, y1, ws + 1, ws + 1);
  int n = T.mx * T.my;
  long cntf = 0;
  for (int k = 0; k < n; ++k) {
    if (std::isnan(T.f[k])) return -1;  // logical(NaN) throws
    if (T.f[k] == 0) ++cntf;
  }
  const double npx0 = (double)((ws + 1) * (ws + 1));
  if (!((double)cntf < 0.4 * npx0)) {
    for (int k = 0; k < 4; ++k) P[k] = 0;
    return maxIterNum + 2;
  }
  if ((double)cntf > 0.0 * npx0) {
    ws = 2 * (int)std::ceil(std::sqrt(npx0 / (npx0 - (double)cntf)) * ws / 2);
    x1 = x0 - ws / 2; x3 = x0 + ws / 2; y1 = y0 - ws / 2; y3 = y0 + ws / 2;
    if (!mask_crop_ok(fr, x1, x3, y1, y3) || !crop_ok(fr, x1, x3, y1, y3)) return -1;
    T.load(fr, x1, y1, ws + 1, ws + 1);
    n = T.mx * T.my;
  }
  int c = (ws + 1) / 2;  // floor((winsize+1)/2)
  std::vector<uint8_t> bwf(n), bwg(n, 0), tmp(n);
  bwselect_tile(T.m.data(), T.mx, T.my, c, c, 4, bwf.data());
  for (int k = 0; k < n; ++k) {
    const double s = (double)bwf[k];
    T.f[k] *= s; T.gx[k] *= s; T.gy[k] *= s;
  }
  // Hessian H = sum J J^T with J = [dx gx, dx gy, dy gx, dy gy, gx, gy]
  double H[36] = {0};
  auto hessian = [&]() {
    double acc[21] = {0};
    for (int j = 0; j < T.my; ++j)
      for (int i = 0; i < T.mx; ++i) {
        const int k = i + j * T.mx;
        const double dx = (double)(x1 + i - x0), dy = (double)(y1 + j - y0);
        const double J[6] = {dx * T.gx[k], dx * T.gy[k], dy * T.gx[k], dy * T.gy[k], T.gx[k], T.gy[k]};
        int q = 0;
        for (int a = 0; a < 6; ++a)
          for (int b = a; b < 6; ++b) acc[q++] += J[a] * J[b];
      }
    int q = 0;
    for (int a = 0; a < 6; ++a)
      for (int b = a; b < 6; ++b) { H[a * 6 + b] = acc[q]; H[b * 6 + a] = acc[q]; ++q; }
  };
  hessian();
  double meanf, bottomf;
  masked_mean_bottom(T.f.data(), n, &meanf, &bottomf);

  double normNew = 1, normAbs = 1, normInit = 0;
  double sabs_old = -1;
  int step = 0;
  std::vector<double> tg(n);
  while (step <= maxIterNum && normNew > tol && normAbs > tol) {
    ++step;
    if (step > 1 && (double)cntf > 0.0 * npx0) {
      long cg = 0;
      for (int k = 0; k < (int)bwg.size(); ++k) cg += bwg[k];
      const double r = std::sqrt((double)((ws0 + 1) * (ws0 + 1)) / (double)cg) * ws / 2;
      if (!std::isfinite(r)) return -1;  // division by an empty selection
      const int nws = 2 * (int)std::ceil(r);
      if (nws != ws && variant == 1) {
        // tempf keeps its old size until the masked branch below re-crops it;
        // only the code-103 test can still see the old tile (bounds break).
        sabs_old = 0;
        for (int k = 0; k < n; ++k) sabs_old += std::fabs(T.f[k]);
        ws = nws;
        x1 = x0 - ws / 2; x3 = x0 + ws / 2; y1 = y0 - ws / 2; y3 = y0 + ws / 2;
        if (!mask_crop_ok(fr, x1, x3, y1, y3)) return -1;
        T.load(fr, x1, y1, ws + 1, ws + 1);
        n = T.mx * T.my;
        c = (ws + 1) / 2;
        bwg.assign(n, 0); tmp.resize(n); tg.resize(n);
      } else if (nws != ws) {
        // MATLAB re-crops the mask at the new size and later fails on the
        // size mismatch between tempf and the new tempg, unless the warped
        // window leaves the image first (then the loop breaks with 101).
        const long nx1 = x0 - nws / 2, nx3 = x0 + nws / 2, ny1 = y0 - nws / 2, ny3 = y0 + nws / 2;
        if (!mask_crop_ok(fr, nx1, nx3, ny1, ny3)) return -1;
        if (any_out_of_bounds(fr, P, x0, y0, nx1, ny1, nws + 1, nws + 1)) {
          normNew = 1e6;
          break;
        }
        return -1;
      }
    }
    if (any_out_of_bounds(fr, P, x0, y0, x1, y1, T.mx, T.my)) {
      normNew = 1e6;
      break;
    }
    warp_sample(fr, P, x0, y0, x1, y1, T.mx, T.my, tg.data());
    long cntg0 = 0;
    for (int k = 0; k < n; ++k) {
      if (std::isnan(tg[k])) return -1;
      if (tg[k] == 0) ++cntg0;
    }
    if ((double)cntf > 0.0 * npx0 || (double)cntg0 > 0.0 * npx0) {
      for (int k = 0; k < n; ++k) tmp[k] = tg[k] != 0;
      bwselect_tile(tmp.data(), T.mx, T.my, c, c, 8, bwg.data());
      bool anyzero = false;
      for (int k = 0; k < n; ++k)
        if (!bwg[k]) { anyzero = true; break; }
      if (!anyzero) bwselect_tile(T.m.data(), T.mx, T.my, c, c, 8, bwg.data());
      for (int k = 0; k < n; ++k) tg[k] *= (double)bwg[k];
      if (variant == 1) {
        if (!crop_ok(fr, x1, x3, y1, y3)) return -1;
        sabs_old = -1;
        for (int j = 0; j < T.my; ++j)
          for (int i = 0; i < T.mx; ++i) {
            const int k = i + j * T.mx;
            const double s = (double)bwg[k];
            T.f[k] = fr.F(x1 + i, y1 + j) * fr.M(x1 + i, y1 + j) * s;
            T.gx[k] = fr.GX(x1 + i, y1 + j) * s;
            T.gy[k] = fr.GY(x1 + i, y1 + j) * s;
          }
        hessian();
        masked_mean_bottom(T.f.data(), n, &meanf, &bottomf);
      }
    }
    double meang, bottomg;
    masked_mean_bottom(tg.data(), n, &meang, &bottomg);
    double b2[6] = {0};
    for (int j = 0; j < T.my; ++j)
      for (int i = 0; i < T.mx; ++i) {
        const int k = i + j * T.mx;
        const double dx = (double)(x1 + i - x0), dy = (double)(y1 + j - y0);
        const double r = (T.f[k] - meanf) / bottomf - (tg[k] - meang) / bottomg;
        b2[0] += dx * T.gx[k] * r;
        b2[1] += dx * T.gy[k] * r;
        b2[2] += dy * T.gx[k] * r;
        b2[3] += dy * T.gy[k] * r;
        b2[4] += T.gx[k] * r;
        b2[5] += T.gy[k] * r;
      }
    double b[6], nb = 0;
    for (int a = 0; a < 6; ++a) { b[a] = bottomf * b2[a]; nb += b[a] * b[a]; }
    normNew = std::sqrt(nb);
    normAbs = normNew;
    if (step == 1) normInit = normNew;
    if (normInit > tol) normNew = normNew / normInit;
    else normNew = 0;
    if (normNew < tol || normAbs < tol) break;
    double D[6];
    small_solve(H, b, 6, D);
    for (int a = 0; a < 6; ++a) D[a] = -D[a];
    if (!compose_update(P, D)) break;
  }
  if (!(normNew < tol || normAbs < tol)) step = maxIterNum + 1;
  if (std::isnan(normNew)) step = maxIterNum + 1;
  double sabs = 0;
  for (int k = 0; k < n; ++k) sabs += std::fabs(T.f[k]);
  if (sabs_old >= 0) sabs = sabs_old;
  if (sabs < 1e-6) step = maxIterNum + 3;
  // HGlobal = [H(1:6) H(8:12) H(15:18) H(22:24) H(29:30) H(36)]
  int q = 0;
  for (int col = 0; col < 6; ++col)
    for (int row = col; row < 6; ++row) Hpk[q++] = H[row * 6 + col];
  return step;
}

// LocalICGNQuadtree's per-node loop (LocalICGNQuadtree.m:108-147) plus the
// markCoordHoleStrain flag (:112-123).  ws_list (optional) gives a subset size
// per node; NULL means the single DICpara.winsize of the reference.  coords is N x 2 column-major; U0 and U
// interleaved; F = [F11 F21 F12 F22] per node; Hpk N x 21 column-major.
extern "C" void orc_icgn6(const double* f, const double* g, const uint8_t* mask, const double* dfdx,
               const double* dfdy, long W, long H, const double* U0, const double* coords, long N,
               int ws_all, const int32_t* ws_list, double tol, double* U, double* F, double* Hpk,
               int32_t* conv, uint8_t* mark_hole, int variant) {
  Frame fr{f, g, mask, dfdx, dfdy, W, H};
#pragma omp parallel for schedule(dynamic, 4)
  for (long j = 0; j < N; ++j) {
    const long x0 = std::lround(coords[j]), y0 = std::lround(coords[N + j]);
    const int ws = ws_list ? ws_list[j] : ws_all;
    {
      const long x1 = x0 - ws / 2, x3 = x0 + ws / 2, y1 = y0 - ws / 2, y3 = y0 + ws / 2;
      uint8_t mk = 0;
      if (!mask_crop_ok(fr, x1, x3, y1, y3)) mk = 1;
      else {
        for (long yy = y1; yy <= y3 && !mk; ++yy)
          for (long xx = x1; xx <= x3; ++xx)
            if (fr.F(xx, yy) * fr.M(xx, yy) == 0) { mk = 1; break; }
      }
      if (mark_hole) mark_hole[j] = mk;
    }
    double P[6], Hl[21];
    const int code = icgn6_one(fr, U0[2 * j], U0[2 * j + 1], x0, y0, ws, tol, P, Hl, variant);
    conv[j] = code;
    if (code == -1) {
      U[2 * j] = U[2 * j + 1] = NAN;
      for (int a = 0; a < 4; ++a) F[4 * j + a] = NAN;
      for (int a = 0; a < 21; ++a) Hpk[a * N + j] = 0;  // HtempPar keeps its zero init
    } else {
      U[2 * j] = P[4]; U[2 * j + 1] = P[5];
      F[4 * j + 0] = P[0]; F[4 * j + 1] = P[1]; F[4 * j + 2] = P[2]; F[4 * j + 3] = P[3];
      for (int a = 0; a < 21; ++a) Hpk[a * N + j] = Hl[a];
    }
  }
}

// ---------------------------------------------------------------------------
// funICGN_Subpb1 (2-DOF augmented-Lagrangian IC-GN) for one node.
// Returns the ConvItPerEle code; code 0 with NaN U mirrors the catch branch of
// Subpb1Quadtree.m:96-99 (the reference leaves ConvItPerEle at its zero init).
// ---------------------------------------------------------------------------
static int icgn2_one(const Frame& fr, long x0, long y0, int wx, int wy, double mu,
                     const double vdual[2], const double UOld[2], const double FOld[4], double tol,
                     double Uout[2]) {
  const int maxIterNum = 100;
  double P[6] = {FOld[0], FOld[1], FOld[2], FOld[3], UOld[0], UOld[1]};
  long x1 = x0 - wx / 2, x3 = x0 + wx / 2, y1 = y0 - wy / 2, y3 = y0 + wy / 2;
  if ((wx & 1) || (wy & 1)) { Uout[0] = Uout[1] = NAN; return 0; }
  if (!mask_crop_ok(fr, x1, x3, y1, y3) || !crop_ok(fr, x1, x3, y1, y3)) {
    Uout[0] = Uout[1] = NAN;
    return 0;
  }
  Tile T;
  T.load(fr, x1, y1, wx + 1, wy + 1);
  int n = T.mx * T.my;
  long cntf = 0;
  for (int k = 0; k < n; ++k) {
    if (std::isnan(T.f[k])) { Uout[0] = Uout[1] = NAN; return 0; }
    if (T.f[k] == 0) ++cntf;
  }
  const double npx0 = (double)(wx + 1) * (double)(wy + 1);
  if (!((double)cntf < 0.4 * npx0)) {
    Uout[0] = P[4]; Uout[1] = P[5];
    return 102;
  }
  if ((double)cntf > 0.0 * npx0) {
    {
      const double a = (double)(wx + 1) * (double)(wy + 1);
      wx = 2 * (int)std::ceil(std::sqrt(a / (a - (double)cntf)) * wx / 2);
    }
    {
      const double a = (double)(wx + 1) * (double)(wy + 1);
      wy = 2 * (int)std::ceil(std::sqrt(a / (a - (double)cntf)) * wy / 2);
    }
    x1 = x0 - wx / 2; x3 = x0 + wx / 2; y1 = y0 - wy / 2; y3 = y0 + wy / 2;
    if (!mask_crop_ok(fr, x1, x3, y1, y3) || !crop_ok(fr, x1, x3, y1, y3)) {
      Uout[0] = Uout[1] = NAN;
      return 0;
    }
    T.load(fr, x1, y1, wx + 1, wy + 1);
    n = T.mx * T.my;
  }
  // bwselect(BW, floor((wx+1)/2), floor((wy+1)/2), n): column then row
  const int sc = (wx + 1) / 2, sr = (wy + 1) / 2;
  std::vector<uint8_t> bwf(n), bwg(n), tmp(n);
  std::vector<double> fraw(n), gxraw(n), gyraw(n);
  for (int k = 0; k < n; ++k) { fraw[k] = T.f[k]; gxraw[k] = T.gx[k]; gyraw[k] = T.gy[k]; }
  bwselect_tile(T.m.data(), T.mx, T.my, sr, sc, 4, bwf.data());
  for (int k = 0; k < n; ++k) {
    const double s = (double)bwf[k];
    T.f[k] *= s; T.gx[k] *= s; T.gy[k] *= s;
  }
  double H11 = 0, H12 = 0, H22 = 0;
  for (int k = 0; k < n; ++k) {
    H11 += T.gx[k] * T.gx[k]; H12 += T.gx[k] * T.gy[k]; H22 += T.gy[k] * T.gy[k];
  }
  double meanf, bottomf;
  masked_mean_bottom(T.f.data(), n, &meanf, &bottomf);
  double A11 = H11 * 2 / (bottomf * bottomf) + mu, A12 = H12 * 2 / (bottomf * bottomf),
         A22 = H22 * 2 / (bottomf * bottomf) + mu;

  double normNew = 1, normAbs = 1, normInit = 0;
  int step = 0;
  std::vector<double> tg(n);
  while (step <= 100 && normNew > tol && normAbs > tol) {
    ++step;
    if (any_out_of_bounds(fr, P, x0, y0, x1, y1, T.mx, T.my)) {
      normNew = 1e6;
      break;
    }
    warp_sample(fr, P, x0, y0, x1, y1, T.mx, T.my, tg.data());
    long cntg0 = 0;
    for (int k = 0; k < n; ++k) {
      if (std::isnan(tg[k])) { Uout[0] = Uout[1] = NAN; return 0; }
      if (tg[k] == 0) ++cntg0;
    }
    if ((double)cntf > 0.0 * npx0 || (double)cntg0 > 0.0 * npx0) {
      for (int k = 0; k < n; ++k) tmp[k] = tg[k] != 0;
      bwselect_tile(tmp.data(), T.mx, T.my, sr, sc, 4, bwg.data());
      bool anyzero = false;
      for (int k = 0; k < n; ++k)
        if (!bwg[k]) { anyzero = true; break; }
      if (!anyzero) bwselect_tile(T.m.data(), T.mx, T.my, sr, sc, 8, bwg.data());
      for (int k = 0; k < n; ++k) {
        const double s = (double)bwg[k];
        tg[k] *= s;
        // tempf, DfDx, DfDy recomputed from the raw crops masked by tempg_BW2
        T.f[k] = fraw[k] * s;
        T.gx[k] = gxraw[k] * s;
        T.gy[k] = gyraw[k] * s;
      }
      H11 = H12 = H22 = 0;
      for (int k = 0; k < n; ++k) {
        H11 += T.gx[k] * T.gx[k]; H12 += T.gx[k] * T.gy[k]; H22 += T.gy[k] * T.gy[k];
      }
      masked_mean_bottom(T.f.data(), n, &meanf, &bottomf);
      A11 = H11 * 2 / (bottomf * bottomf) + mu;
      A12 = H12 * 2 / (bottomf * bottomf);
      A22 = H22 * 2 / (bottomf * bottomf) + mu;
    }
    double meang, bottomg;
    masked_mean_bottom(tg.data(), n, &meang, &bottomg);
    double b0 = 0, b1 = 0;
    for (int k = 0; k < n; ++k) {
      const double r = (T.f[k] - meanf) / bottomf - (tg[k] - meang) / bottomg;
      b0 += T.gx[k] * r;
      b1 += T.gy[k] * r;
    }
    b0 = bottomf * b0;
    b1 = bottomf * b1;
    const double tb0 = b0 * 2 / (bottomf * bottomf) + mu * (P[4] - UOld[0] - vdual[0]);
    const double tb1 = b1 * 2 / (bottomf * bottomf) + mu * (P[5] - UOld[1] - vdual[1]);
    // max(diag(H2)) ignoring NaN like MATLAB's max
    const double dmax = std::isnan(A11) ? A22 : (std::isnan(A22) ? A11 : std::max(A11, A22));
    const double delta = 1e-3;
    double Hm[4] = {A11 + delta * dmax, A12, A12, A22 + delta * dmax};
    double rhs[2] = {tb0, tb1}, dP[2];
    small_solve(Hm, rhs, 2, dP);
    double D[6] = {0, 0, 0, 0, -dP[0], -dP[1]};
    normNew = std::sqrt(tb0 * tb0 + tb1 * tb1);
    normAbs = normNew;
    if (step == 1) normInit = normNew;
    if (normInit > tol) normNew = normNew / normInit;
    else normNew = 0;
    if (normNew < tol || normAbs < tol) break;
    if (!compose_update(P, D)) break;
  }
  if (!(normNew < tol || normAbs < tol)) step = maxIterNum + 1;
  if (std::isnan(normNew)) step = maxIterNum + 1;
  double sabs = 0;
  for (int k = 0; k < n; ++k) sabs += std::fabs(T.f[k]);
  if (sabs < 1e-6) step = maxIterNum + 3;
  Uout[0] = P[4];
  Uout[1] = P[5];
  return step;
}

// Subpb1Quadtree's per-node loop.  winsize_list N x 2 column-major (x, y);
// udual 4N (unused by the kernel, as in the reference), vdual 2N.
extern "C" void orc_icgn2(const double* f, const double* g, const uint8_t* mask, const double* dfdx,
               const double* dfdy, long W, long H, const double* UOld, const double* FOld,
               const double* vdual, const double* coords, long N, const int32_t* winsize_list,
               double mu, double tol, double* U, int32_t* conv) {
  Frame fr{f, g, mask, dfdx, dfdy, W, H};
#pragma omp parallel for schedule(dynamic, 4)
  for (long j = 0; j < N; ++j) {
    const long x0 = std::lround(coords[j]), y0 = std::lround(coords[N + j]);
    double Uo[2];
    conv[j] = icgn2_one(fr, x0, y0, winsize_list[j], winsize_list[N + j], mu, vdual + 2 * j,
                        UOld + 2 * j, FOld + 4 * j, tol, Uo);
    U[2 * j] = Uo[0];
    U[2 * j + 1] = Uo[1];
  }
}

// ---------------------------------------------------------------------------
// Subpb2Quadtree element loop.  Produces the global system in triplet form
// over FEMSize + 8 DOFs (1-based indices, as MATLAB's sparse() would get them)
// and b (dense, FEMSize + 8).  The triplets of element e occupy
// [256 e, 256 e + 256); b is accumulated here.
// ---------------------------------------------------------------------------
static inline double sgn(double x) { return (x > 0) - (x < 0); }

static void shape_derivs(double ksi, double eta, const double dp[4], double dNdksi[8],
                         double dNdeta[8]) {
  const double d5 = dp[0], d6 = dp[1], d7 = dp[2], d8 = dp[3];
  const double N5k = d5 * 0.5 * (1 - std::fabs(eta)), N5e = d5 * 0.5 * (1 + ksi) * sgn(-eta);
  const double N6k = d6 * 0.5 * (1 + eta) * sgn(-ksi), N6e = d6 * 0.5 * (1 - std::fabs(ksi));
  const double N7k = d7 * 0.5 * (-1) * (1 - std::fabs(eta)), N7e = d7 * 0.5 * (1 - ksi) * sgn(-eta);
  const double N8k = d8 * 0.5 * (1 - eta) * sgn(-ksi), N8e = d8 * 0.5 * (-1) * (1 - std::fabs(ksi));
  dNdksi[0] = -0.25 * (1 - eta) - 0.5 * (N7k + N8k);
  dNdeta[0] = -0.25 * (1 - ksi) - 0.5 * (N7e + N8e);
  dNdksi[1] = 0.25 * (1 - eta) - 0.5 * (N8k + N5k);
  dNdeta[1] = -0.25 * (1 + ksi) - 0.5 * (N8e + N5e);
  dNdksi[2] = 0.25 * (1 + eta) - 0.5 * (N5k + N6k);
  dNdeta[2] = 0.25 * (1 + ksi) - 0.5 * (N5e + N6e);
  dNdksi[3] = -0.25 * (1 + eta) - 0.5 * (N6k + N7k);
  dNdeta[3] = 0.25 * (1 - ksi) - 0.5 * (N6e + N7e);
  dNdksi[4] = N5k; dNdeta[4] = N5e;
  dNdksi[5] = N6k; dNdeta[5] = N6e;
  dNdksi[6] = N7k; dNdeta[6] = N7e;
  dNdksi[7] = N8k; dNdeta[7] = N8e;
}

static void shape_fns(double ksi, double eta, const double dp[4], double Nv[8]) {
  const double N5 = dp[0] * 0.5 * (1 + ksi) * (1 - std::fabs(eta));
  const double N6 = dp[1] * 0.5 * (1 + eta) * (1 - std::fabs(ksi));
  const double N7 = dp[2] * 0.5 * (1 - ksi) * (1 - std::fabs(eta));
  const double N8 = dp[3] * 0.5 * (1 - eta) * (1 - std::fabs(ksi));
  Nv[0] = (1 - ksi) * (1 - eta) * 0.25 - 0.5 * (N7 + N8);
  Nv[1] = (1 + ksi) * (1 - eta) * 0.25 - 0.5 * (N8 + N5);
  Nv[2] = (1 + ksi) * (1 + eta) * 0.25 - 0.5 * (N5 + N6);
  Nv[3] = (1 - ksi) * (1 + eta) * 0.25 - 0.5 * (N6 + N7);
  Nv[4] = N5; Nv[5] = N6; Nv[6] = N7; Nv[7] = N8;
}

// gauss_order 2..5 as in Subpb2Quadtree.m:47-64.
static int gauss_rule(int order, double* pt, double* wt) {
  switch (order) {
    case 2: pt[0] = -1 / std::sqrt(3.0); pt[1] = 1 / std::sqrt(3.0); wt[0] = wt[1] = 1; return 2;
    case 3:
      pt[0] = 0; pt[1] = std::sqrt(3.0 / 5); pt[2] = -std::sqrt(3.0 / 5);
      wt[0] = 8.0 / 9; wt[1] = 5.0 / 9; wt[2] = 5.0 / 9; return 3;
    case 4:
      pt[0] = 0.339981; pt[1] = -0.339981; pt[2] = 0.861136; pt[3] = -0.861136;
      wt[0] = 0.652145; wt[1] = 0.652145; wt[2] = 0.347855; wt[3] = 0.347855; return 4;
    case 5:
      pt[0] = 0; pt[1] = 0.538469; pt[2] = -0.538469; pt[3] = 0.90618; pt[4] = -0.90618;
      wt[0] = 0.568889; wt[1] = 0.478629; wt[2] = 0.478629; wt[3] = 0.236927; wt[4] = 0.236927;
      return 5;
  }
  return 0;
}

extern "C" int orc_subpb2_assemble(const double* coords, long N, const int32_t* elems, long E,
                        int gauss_order, double beta, double mu, double alpha, const double* U,
                        const double* F, int32_t* I, int32_t* J, double* V, double* b) {
  double gpt[5], gwt[5];
  const int ng = gauss_rule(gauss_order, gpt, gwt);
  if (!ng) return -1;
  const long FEMSize = 2 * N;
  const long nb = FEMSize + 8;
  // padded U and F: zeros beyond the last node (dummy node N+1)
  auto Uat = [&](long idx1) -> double { return idx1 <= FEMSize ? U[idx1 - 1] : 0.0; };
  auto Fat = [&](long idx1) -> double { return idx1 <= 4 * N ? F[idx1 - 1] : 0.0; };
  for (long k = 0; k < nb; ++k) b[k] = 0;
  std::vector<double> bpart((size_t)E * 16);
  std::vector<long> bidx((size_t)E * 16);
#pragma omp parallel for schedule(static)
  for (long e = 0; e < E; ++e) {
    long nd[8];
    for (int a = 0; a < 8; ++a) nd[a] = elems[a * E + e];
    double ptx[8], pty[8], dp[4];
    for (int a = 0; a < 8; ++a) {
      if (a < 4 || nd[a] != 0) { ptx[a] = coords[nd[a] - 1]; pty[a] = coords[N + nd[a] - 1]; }
      else { ptx[a] = 0; pty[a] = 0; }
    }
    for (int a = 0; a < 4; ++a) dp[a] = nd[4 + a] != 0 ? 1.0 : 0.0;
    long iu[16], iF[16][4];
    for (int a = 0; a < 8; ++a) {
      long node = nd[a];
      if (a >= 4 && node == 0) node = N + 1;  // dummy node
      iu[2 * a] = 2 * node - 1; iu[2 * a + 1] = 2 * node;
      // tempIndexF columns: [4n-3, 4n-1, 4n-2, 4n] = [F11, F12, F21, F22]
      for (int r = 0; r < 2; ++r) {
        iF[2 * a + r][0] = 4 * node - 3; iF[2 * a + r][1] = 4 * node - 1;
        iF[2 * a + r][2] = 4 * node - 2; iF[2 * a + r][3] = 4 * node;
      }
    }
    double A[16][16] = {{0}}, be[16] = {0};
    for (int gi = 0; gi < ng * ng; ++gi) {
      // [ksiAll, etaAll] = ndgrid(pts, pts): ksi varies fastest
      const double ksi = gpt[gi % ng], eta = gpt[gi / ng];
      const double wk = gwt[gi % ng], we = gwt[gi / ng];
      double Nv[8], dk[8], de[8];
      shape_fns(ksi, eta, dp, Nv);
      shape_derivs(ksi, eta, dp, dk, de);
      double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
      for (int a = 0; a < 8; ++a) {
        J11 += dk[a] * ptx[a]; J12 += dk[a] * pty[a];
        J21 += de[a] * ptx[a]; J22 += de[a] * pty[a];
      }
      const double Jac = J11 * J22 - J12 * J21;
      const double i11 = 1 / Jac * J22, i12 = 1 / Jac * (-J12), i21 = 1 / Jac * (-J21),
                   i22 = 1 / Jac * J11;
      // DN is 4 x 16: rows [d/dx u; d/dy u; d/dx v; d/dy v]
      double DN[4][16] = {{0}};
      double NN[2][16] = {{0}};
      for (int a = 0; a < 8; ++a) {
        const double dx = i11 * dk[a] + i12 * de[a];
        const double dy = i21 * dk[a] + i22 * de[a];
        DN[0][2 * a] = dx; DN[1][2 * a] = dy;
        DN[2][2 * a + 1] = dx; DN[3][2 * a + 1] = dy;
        NN[0][2 * a] = Nv[a]; NN[1][2 * a + 1] = Nv[a];
      }
      const double w = Jac * wk * we;
      double Ui[16];
      for (int p = 0; p < 16; ++p) Ui[p] = Uat(iu[p]);
      for (int p = 0; p < 16; ++p) {
        for (int q = 0; q < 16; ++q) {
          double dd = 0, nn = 0;
          for (int r = 0; r < 4; ++r) dd += DN[r][p] * DN[r][q];
          for (int r = 0; r < 2; ++r) nn += NN[r][p] * NN[r][q];
          A[p][q] += w * ((beta + alpha) * dd + mu * nn);
        }
        double fd = 0;  // diag(DN' * FMinusW(tempIndexF)')
        for (int r = 0; r < 4; ++r) fd += DN[r][p] * Fat(iF[p][r]);
        double nnU = 0, ddU = 0;
        for (int q = 0; q < 16; ++q) {
          double dd = 0, nn = 0;
          for (int r = 0; r < 4; ++r) dd += DN[r][p] * DN[r][q];
          for (int r = 0; r < 2; ++r) nn += NN[r][p] * NN[r][q];
          nnU += nn * Ui[q];
          ddU += dd * Ui[q];
        }
        be[p] += w * (beta * fd + mu * nnU + alpha * ddU);
      }
    }
    for (int p = 0; p < 16; ++p)
      for (int q = 0; q < 16; ++q) {
        // [IndexAXX, IndexAYY] = ndgrid(tempIndexU, tempIndexU); (:) -> p fastest
        const long t = e * 256 + q * 16 + p;
        I[t] = (int32_t)iu[p];
        J[t] = (int32_t)iu[q];
        V[t] = A[p][q];
      }
    for (int p = 0; p < 16; ++p) { bpart[e * 16 + p] = be[p]; bidx[e * 16 + p] = iu[p]; }
  }
  for (long e = 0; e < E; ++e)
    for (int p = 0; p < 16; ++p) b[bidx[e * 16 + p] - 1] += bpart[e * 16 + p];
  return 0;
}


// ---------------------------------------------------------------------------
// funIntegerSearch, whole-field mode (tempNoOfInitPt = 0).
// Grid shrink of funIntegerSearch.m:14-25, then for every grid point the
// normalised cross-correlation of C = f(ii:ii+ws, jj:jj+ws) inside
// D = g(ii-S:ii+ws+S, jj-S:jj+ws+S), cropped to (2S+3)^2 lags
// (funIntegerSearch.m:121-134) and passed to findpeak(.., 1).
// Outputs are ny x nx column-major (row = y index) like the reference.
// peak_rc holds the 1-based integer argmax (row, col) of the cropped map as two
// ny x nx planes; 0 marks a grid point where normxcorr2 threw.
// ---------------------------------------------------------------------------
extern "C" void orc_intsearch_grid(long W, long H, int Sx, int Sy, const double gridx_in[2],
                        const double gridy_in[2], int wsx, int wsy, int stepx, int stepy,
                        double gridx_out[2], double gridy_out[2], long* nx, long* ny) {
  double gx0 = gridx_in[0], gx1 = gridx_in[1], gy0 = gridy_in[0], gy1 = gridy_in[1];
  while (gx0 - Sx - 0.5 * wsx < 1) gx0 += 1;
  while (gy0 - Sy - 0.5 * wsy < 1) gy0 += 1;
  while (gx1 + 1.5 * wsx + Sx > (double)W) gx1 -= 1;
  while (gy1 + 1.5 * wsy + Sy > (double)H) gy1 -= 1;
  gridx_out[0] = gx0; gridx_out[1] = gx1; gridy_out[0] = gy0; gridy_out[1] = gy1;
  // XList = gridx(1) : step : gridx(2)-step
  *nx = (gx1 - stepx >= gx0) ? (long)std::floor((gx1 - stepx - gx0) / stepx) + 1 : 0;
  *ny = (gy1 - stepy >= gy0) ? (long)std::floor((gy1 - stepy - gy0) / stepy) + 1 : 0;
}

// One grid point.  Returns false when normxcorr2 would throw.
static bool ncc_peak(const double* f, const double* g, long W, long ii, long jj, int Sx, int Sy,
                     int wsx, int wsy, double* uo, double* vo, double* cco, int* pr, int* pc) {
  const int m = wsx + 1, n = wsy + 1, am = wsx + 1 + 2 * Sx, an = wsy + 1 + 2 * Sy;
  const double mn = (double)m * (double)n;
  std::vector<double> T((size_t)m * n), A((size_t)am * an);
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < m; ++a) T[a + b * m] = f[(jj - 1 + b) * W + (ii - 1 + a)];
  for (int q = 0; q < an; ++q)
    for (int p = 0; p < am; ++p) A[p + q * am] = g[(jj - 1 - Sy + q) * W + (ii - 1 - Sx + p)];
  for (double t : T) if (!std::isfinite(t)) return false;
  for (double t : A) if (!std::isfinite(t)) return false;
  double sumT = 0;
  for (double t : T) sumT += t;
  const double meanT = sumT / mn;
  double q2 = 0;
  for (double t : T) { const double d = t - meanT; q2 += d * d; }
  const double stdT = std::sqrt(q2 / (mn - 1));
  if (!(stdT != 0)) return false;  // "TEMPLATE cannot have all the same values"
  const double denomT = std::sqrt(mn - 1) * stdT;
  const int nr = 2 * Sx + 3, nc = 2 * Sy + 3;
  std::vector<double> num((size_t)nr * nc), den((size_t)nr * nc);
  double dmax = 0;
  for (int j = 0; j < nc; ++j)
    for (int i = 0; i < nr; ++i) {
      const int dp = i - 1, dq = j - 1;
      double xc = 0, sA = 0, sA2 = 0;
      for (int b = 0; b < n; ++b) {
        const int qq = b + dq;
        if (qq < 0 || qq >= an) continue;
        for (int a = 0; a < m; ++a) {
          const int pp = a + dp;
          if (pp < 0 || pp >= am) continue;
          const double av = A[pp + qq * am];
          xc += T[a + b * m] * av;
          sA += av;
          sA2 += av * av;
        }
      }
      const double nm = xc - sA * sumT / mn;
      const double dl = sA2 - (sA * sA) / mn;
      const double dA = std::sqrt(dl > 0 ? dl : 0.0);
      num[i + j * nr] = nm;
      den[i + j * nr] = denomT * dA;
      if (std::fabs(den[i + j * nr]) > dmax) dmax = std::fabs(den[i + j * nr]);
    }
  const double tolc = std::sqrt(matlab_eps(dmax));
  const double clip = std::sqrt(matlab_eps(1.0));
  std::vector<double> C((size_t)nr * nc);
  double cmax = -INFINITY;
  for (int k = 0; k < nr * nc; ++k) {
    double cv = den[k] > tolc ? num[k] / den[k] : 0.0;
    if ((std::fabs(cv) - 1) > clip) cv = 0;
    C[k] = cv;
    if (cv > cmax) cmax = cv;
  }
  // the first column-major lag within kPeakTie of the maximum: findpeak's
  // first maximum, with lags that tie up to rounding taken as equal
  int imax = 0;
  while (imax < nr * nc - 1 && !(C[imax] >= cmax - kPeakTie)) ++imax;
  const int yp = imax % nr + 1, xp = imax / nr + 1;  // 1-based row / col
  *pr = yp; *pc = xp;
  double ypeak = yp, xpeak = xp, maxf = C[imax];
  if (!(xp == 1 || xp == nc || yp == 1 || yp == nr)) {
    // u = f(ypeak-1:ypeak+1, xpeak-1:xpeak+1)(:), x = column offset, y = row offset
    double uu[9], xs[9], ys[9];
    int t = 0;
    for (int dc = -1; dc <= 1; ++dc)
      for (int dr = -1; dr <= 1; ++dr) {
        uu[t] = C[(yp - 1 + dr) + (xp - 1 + dc) * nr];
        xs[t] = dc; ys[t] = dr; ++t;
      }
    // Least-squares fit of [1 x y xy x^2 y^2] on the 3x3 stencil (X\u), using
    // the closed-form normal equations of that fixed design.
    double s0 = 0, sx = 0, sy = 0, sxy = 0, sxx = 0, syy = 0;
    for (int k = 0; k < 9; ++k) {
      s0 += uu[k]; sx += xs[k] * uu[k]; sy += ys[k] * uu[k]; sxy += xs[k] * ys[k] * uu[k];
      sxx += xs[k] * xs[k] * uu[k]; syy += ys[k] * ys[k] * uu[k];
    }
    const double A2 = sx / 6, A3 = sy / 6, A4 = sxy / 4;
    const double S = (sxx + syy) / 2 - (2.0 / 3.0) * s0;
    const double Dd = (sxx - syy) / 2;
    const double A5 = (S + Dd) / 2, A6 = (S - Dd) / 2;
    const double A1 = (s0 - 6 * S) / 9;
    double xo = (-A3 * A4 + 2 * A6 * A2) / (A4 * A4 - 4 * A5 * A6);
    double yo = -1 / (A4 * A4 - 4 * A5 * A6) * (A4 * A2 - 2 * A5 * A3);
    if (!(std::fabs(xo) > 1 || std::fabs(yo) > 1)) {
      xo = std::round(1000 * xo) / 1000;
      yo = std::round(1000 * yo) / 1000;
      xpeak += xo;
      ypeak += yo;
      maxf = A1 + xo * A2 + yo * A3 + xo * yo * A4 + xo * xo * A5 + yo * yo * A6;
    }
  }
  *uo = ypeak - std::ceil(nr / 2.0);
  *vo = xpeak - std::ceil(nc / 2.0);
  *cco = maxf;
  return true;
}

extern "C" void orc_integer_search(const double* f, const double* g, long W, long H, int Sx, int Sy,
                        const double gridx[2], const double gridy[2], int wsx, int wsy, int stepx,
                        int stepy, double* x, double* y, double* u, double* v, double* cc,
                        int32_t* peak_rc) {
  double gx[2], gy[2];
  long nx, ny;
  orc_intsearch_grid(W, H, Sx, Sy, gridx, gridy, wsx, wsy, stepx, stepy, gx, gy, &nx, &ny);
  const long npt = nx * ny;
#pragma omp parallel for schedule(dynamic, 2)
  for (long t = 0; t < npt; ++t) {
    const long ix = t % nx, iy = t / nx;  // ndgrid(XList, YList)(:)
    const long ii = (long)gx[0] + ix * stepx, jj = (long)gy[0] + iy * stepy;
    const long o = iy + ix * ny;  // (cj1, ci1) in an ny x nx column-major matrix
    double uu, vv, cm;
    int pr = 0, pc = 0;
    if (ncc_peak(f, g, W, ii, jj, Sx, Sy, wsx, wsy, &uu, &vv, &cm, &pr, &pc)) {
      u[o] = uu; v[o] = vv; cc[o] = cm;
    } else {
      u[o] = v[o] = cc[o] = NAN;
    }
    peak_rc[o] = pr;
    peak_rc[npt + o] = pc;
    x[o] = (double)(ii + ii + wsx) / 2;
    y[o] = (double)(jj + jj + wsy) / 2;
  }
}

// ---------------------------------------------------------------------------
// cc.qfactors of funIntegerSearch (funIntegerSearch.m:129-131, 156, 175-176,
// compute_qFactor :211-264): for each grid point the full normxcorr2 map
// (every lag with an overlap), cc_min = cc - min(cc), peak = max(cc_min),
// PCE = peak^2 / mean(cc_min^2) and PPE = 1 / entropy of histcounts(cc_min,30)
// (30 uniform bins over [0, peak], the last closed); [Inf Inf] where
// normxcorr2 throws.  Each column is then shifted by its minimum and divided
// by its largest shifted value (NaN ignored, as MATLAB's min and max do).
// Rows follow the reference's point sequence (x fastest).  qf is npt x 2.
// ---------------------------------------------------------------------------
static void qfactor_point(const double* f, const double* g, long W, long ii, long jj, int Sx, int Sy, int wsx,
                          int wsy, double* pce, double* ppe) {
  const int m = wsx + 1, n = wsy + 1, am = wsx + 1 + 2 * Sx, an = wsy + 1 + 2 * Sy;
  const double mn = (double)m * (double)n;
  std::vector<double> T((size_t)m * n), A((size_t)am * an);
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < m; ++a) T[a + b * m] = f[(jj - 1 + b) * W + (ii - 1 + a)];
  for (int q = 0; q < an; ++q)
    for (int p = 0; p < am; ++p) A[p + q * am] = g[(jj - 1 - Sy + q) * W + (ii - 1 - Sx + p)];
  bool fin = true;
  for (double t : T) fin = fin && std::isfinite(t);
  for (double t : A) fin = fin && std::isfinite(t);
  double sumT = 0;
  for (double t : T) sumT += t;
  const double meanT = sumT / mn;
  double q2 = 0;
  for (double t : T) { const double d = t - meanT; q2 += d * d; }
  const double stdT = std::sqrt(q2 / (mn - 1));
  if (!fin || !(stdT != 0)) { *pce = INFINITY; *ppe = INFINITY; return; }
  const double denomT = std::sqrt(mn - 1) * stdT;
  const int R = m + am - 1, C = n + an - 1;
  std::vector<double> num((size_t)R * C), den((size_t)R * C);
  double dmax = 0;
  for (int j = 0; j < C; ++j)
    for (int i = 0; i < R; ++i) {
      const int dr = i - (m - 1), dc = j - (n - 1);
      double xc = 0, sA = 0, sA2 = 0;
      for (int b = 0; b < n; ++b) {
        const int qq = b + dc;
        if (qq < 0 || qq >= an) continue;
        for (int a = 0; a < m; ++a) {
          const int pp = a + dr;
          if (pp < 0 || pp >= am) continue;
          const double av = A[pp + qq * am];
          xc += T[a + b * m] * av;
          sA += av;
          sA2 += av * av;
        }
      }
      const double dl = sA2 - (sA * sA) / mn;
      num[i + j * R] = xc - sA * sumT / mn;
      den[i + j * R] = denomT * std::sqrt(dl > 0 ? dl : 0.0);
      if (std::fabs(den[i + j * R]) > dmax) dmax = std::fabs(den[i + j * R]);
    }
  const double tolc = std::sqrt(matlab_eps(dmax));
  const double clip = std::sqrt(matlab_eps(1.0));
  const size_t nl = (size_t)R * C;
  double cmin = INFINITY, cmax = -INFINITY;
  for (size_t k = 0; k < nl; ++k) {
    double cv = den[k] > tolc ? num[k] / den[k] : 0.0;
    if ((std::fabs(cv) - 1) > clip) cv = 0;
    num[k] = cv;
    cmin = std::min(cmin, cv);
    cmax = std::max(cmax, cv);
  }
  const double peak = cmax - cmin, bw = peak / 30.0;
  double e2 = 0;
  long hist[30] = {0};
  for (size_t k = 0; k < nl; ++k) {
    const double x = num[k] - cmin;
    e2 += x * x;
    int bin = 0;
    if (peak > 0) {
      // the last edge whose value is <= x, the 30th bin closed at peak
      bin = 29;
      for (int e = 1; e < 30; ++e)
        if (x < e * bw) { bin = e - 1; break; }
    }
    ++hist[bin];
  }
  *pce = peak * peak / (e2 / (double)nl);
  double ent = 0;
  for (int b = 0; b < 30; ++b) {
    const double pb = (double)hist[b] / (double)nl;
    if (pb != 0) ent += pb * std::log(1.0 / pb);
  }
  *ppe = 1.0 / ent;
}

extern "C" void orc_integer_search_qfactors(const double* f, const double* g, long W, long H, int Sx, int Sy,
                                            const double gridx[2], const double gridy[2], int wsx, int wsy,
                                            int stepx, int stepy, double* qraw, double* qf) {
  double gx[2], gy[2];
  long nx, ny;
  orc_intsearch_grid(W, H, Sx, Sy, gridx, gridy, wsx, wsy, stepx, stepy, gx, gy, &nx, &ny);
  const long npt = nx * ny;
#pragma omp parallel for schedule(dynamic, 1)
  for (long t = 0; t < npt; ++t) {
    const long ix = t % nx, iy = t / nx;
    const long ii = (long)gx[0] + ix * stepx, jj = (long)gy[0] + iy * stepy;
    qfactor_point(f, g, W, ii, jj, Sx, Sy, wsx, wsy, &qraw[t], &qraw[npt + t]);
  }
  for (int k = 0; k < 2; ++k) {
    const double* q = qraw + k * npt;
    double mn = INFINITY;
    for (long t = 0; t < npt; ++t)
      if (!std::isnan(q[t])) mn = std::min(mn, q[t]);
    double mx = -INFINITY;
    for (long t = 0; t < npt; ++t) {
      const double d = q[t] - mn;
      if (!std::isnan(d)) mx = std::max(mx, d);
    }
    for (long t = 0; t < npt; ++t) qf[k * npt + t] = (q[t] - mn) / mx;
  }
}

// ---------------------------------------------------------------------------
// Adjoint of the subset ZNSSD cost (no counterpart in the reference).  The cost
// is the criterion funICGNQuadtree.m minimises, taken on the square window:
//   C_n = sum_i (a_i - b_i)^2,   a = (f - fbar) / |f - fbar|,
//   b = (t - tbar) / |t - tbar|,  t_i = ba_interp2 cubic of ImgDef at the warp
//   of funICGNQuadtree.m:151-152 with P = [F11 F21 F12 F22 u v] of the node.
// Window pixels with mask 0 or outside the image are left out.  With
// rho = sum a b, C = 2 - 2 rho and dC/dt_i = -2 (a_i - rho b_i) / |t - tbar|;
// the chain through the Keys weights (ba_interp2.cpp:184-234, clamped taps)
// gives dC/dP and dC/dg.  A subset with fewer than 2 pixels or a constant f or
// t window has cost NaN and no gradient.
// ---------------------------------------------------------------------------
static inline void keys_weights(double d, double w[4], double dw[4]) {
  const double dd = d * d, ddd = dd * d;
  w[0] = 0.5 * (-d + 2.0 * dd - ddd);
  w[1] = 0.5 * (2.0 - 5.0 * dd + 3.0 * ddd);
  w[2] = 0.5 * (d + 4.0 * dd - 3.0 * ddd);
  w[3] = 0.5 * (-dd + ddd);
  dw[0] = 0.5 * (-1.0 + 4.0 * d - 3.0 * dd);
  dw[1] = 0.5 * (-10.0 * d + 9.0 * dd);
  dw[2] = 0.5 * (1.0 + 8.0 * d - 9.0 * dd);
  dw[3] = 0.5 * (-2.0 * d + 3.0 * dd);
}

// Bicubic value and its derivatives along dim 1 (x) and dim 2 (y) at the
// 1-based point (xc, yc); tap k = a + 4 b has index idx[k] and weight wt[k].
static double cubic_with_grad(const double* G, long W, long H, double xc, double yc, double* gx,
                              double* gy, long idx[16], double wt[16]) {
  const double xf = std::floor(xc), yf = std::floor(yc);
  double wx[4], dwx[4], wy[4], dwy[4];
  keys_weights(xc - xf, wx, dwx);
  keys_weights(yc - yf, wy, dwy);
  double t = 0, tx = 0, ty = 0;
  for (int b = 0; b < 4; ++b) {
    long cy = (long)yf - 2 + b;
    cy = cy < 0 ? 0 : (cy >= H ? H - 1 : cy);
    for (int a = 0; a < 4; ++a) {
      long cx = (long)xf - 2 + a;
      cx = cx < 0 ? 0 : (cx >= W ? W - 1 : cx);
      const long k = cx + W * cy;
      const double v = G[k];
      t += wx[a] * wy[b] * v;
      tx += dwx[a] * wy[b] * v;
      ty += wx[a] * dwy[b] * v;
      idx[a + 4 * b] = k;
      wt[a + 4 * b] = wx[a] * wy[b];
    }
  }
  *gx = tx;
  *gy = ty;
  return t;
}

static double adjoint_one(const double* f, const double* g, const uint8_t* mask, long W, long H,
                          long x0, long y0, int ws, const double P[6], double dP[6], double* dg) {
  const int h = ws / 2;
  std::vector<double> fv, tv, gxv, gyv, wtv;
  std::vector<long> dxv, dyv, idxv;
  for (int j = -h; j <= h; ++j)
    for (int i = -h; i <= h; ++i) {
      const long x = x0 + i, y = y0 + j;
      if (x < 1 || x > W || y < 1 || y > H) continue;
      if (mask && !mask[(x - 1) + W * (y - 1)]) continue;
      const double xw = (double)x0 + i + P[0] * i + P[2] * j + P[4];
      const double yw = (double)y0 + j + P[1] * i + P[3] * j + P[5];
      long idx[16];
      double wt[16], gx, gy;
      const double t = cubic_with_grad(g, W, H, xw, yw, &gx, &gy, idx, wt);
      fv.push_back(f[(x - 1) + W * (y - 1)]);
      tv.push_back(t);
      gxv.push_back(gx);
      gyv.push_back(gy);
      dxv.push_back(i);
      dyv.push_back(j);
      idxv.insert(idxv.end(), idx, idx + 16);
      wtv.insert(wtv.end(), wt, wt + 16);
    }
  for (int k = 0; k < 6; ++k) dP[k] = 0;
  const size_t n = fv.size();
  if (n < 2) return NAN;
  double fm = 0, tm = 0;
  for (size_t i = 0; i < n; ++i) { fm += fv[i]; tm += tv[i]; }
  fm /= (double)n;
  tm /= (double)n;
  double sf = 0, st = 0, sft = 0;
  for (size_t i = 0; i < n; ++i) {
    const double a = fv[i] - fm, b = tv[i] - tm;
    sf += a * a;
    st += b * b;
    sft += a * b;
  }
  if (!(sf > 0) || !(st > 0) || !std::isfinite(st)) return NAN;
  const double df = std::sqrt(sf), dt = std::sqrt(st);
  const double rho = sft / (df * dt);
  double cost = 0;
  for (size_t i = 0; i < n; ++i) {
    const double a = (fv[i] - fm) / df, b = (tv[i] - tm) / dt;
    cost += (a - b) * (a - b);
    const double w = -2.0 * (a - rho * b) / dt;
    const double wx = w * gxv[i], wy = w * gyv[i];
    dP[0] += wx * dxv[i];
    dP[1] += wy * dxv[i];
    dP[2] += wx * dyv[i];
    dP[3] += wy * dyv[i];
    dP[4] += wx;
    dP[5] += wy;
    if (dg)
      for (int k = 0; k < 16; ++k) dg[idxv[16 * i + k]] += w * wtv[16 * i + k];
  }
  return cost;
}

// cost (N), dU (2N), dF (4N) and dg (W x H, accumulated) may be NULL except cost.
extern "C" void orc_adjoint(const double* f, const double* g, const uint8_t* mask, long W, long H,
                            const double* coords, long N, int ws_all, const int32_t* ws_list,
                            const double* U, const double* F, double* cost, double* dU, double* dF,
                            double* dg) {
#pragma omp parallel for schedule(dynamic, 16) if (!dg)
  for (long n = 0; n < N; ++n) {
    const long x0 = (long)std::round(coords[n]), y0 = (long)std::round(coords[N + n]);
    const int ws = ws_list ? ws_list[n] : ws_all;
    const double P[6] = {F[4 * n], F[4 * n + 1], F[4 * n + 2], F[4 * n + 3], U[2 * n], U[2 * n + 1]};
    double dP[6];
    cost[n] = adjoint_one(f, g, mask, W, H, x0, y0, ws, P, dP, dg);
    if (dF)
      for (int k = 0; k < 4; ++k) dF[4 * n + k] = dP[k];
    if (dU) { dU[2 * n] = dP[4]; dU[2 * n + 1] = dP[5]; }
  }
}

// ---------------------------------------------------------------------------
// Nodal strain (local replacement of the reference's strain step).  The Gauss
// point strains follow funGlobalNodalStrainQuadtree.m:80-257: at the Gauss
// points of each element (GaussPtOrder^2, points ordered x-major), DN U with
// the hanging-node shape functions gives [du/dx du/dy dv/dx dv/dy].  The
// quadtree elements are axis-aligned rectangles, for which the routine's
// bilinear inverse map returns ksi, eta equal to the Gauss abscissae.  The
// reference then interpolates the Gauss-point values to the nodes with a
// natural-neighbour scatteredInterpolant (:266-276); here every node takes the
// mean, over the elements that contain it, of each element's Gauss point
// nearest to it (on a regular mesh the natural-neighbour weights of those
// points).  Components are stored as the active ADMM loop's strain step stores
// them (funGlobalNodalStrainRBF.m:52-62): F = [du/dx dv/dx du/dy dv/dy].
// A node in no element gets NaN.
// ---------------------------------------------------------------------------
extern "C" void orc_nodal_strain(const double* coords, long N, const int32_t* elems, long E,
                                 const double* U, int gauss_order, double* F) {
  double gpt[5], gwt[5];
  const int ng = gauss_rule(gauss_order, gpt, gwt);
  std::vector<double> sum(4 * (size_t)N, 0.0);
  std::vector<int> cnt(N, 0);
  for (long e = 0; e < E; ++e) {
    int nd[8];
    double px[8], py[8], uu[8], vv[8], dp[4];
    for (int c = 0; c < 8; ++c) {
      nd[c] = elems[c * E + e];
      const bool ok = nd[c] >= 1 && nd[c] <= N;
      px[c] = ok ? coords[nd[c] - 1] : 0.0;
      py[c] = ok ? coords[N + nd[c] - 1] : 0.0;
      uu[c] = ok ? U[2 * (nd[c] - 1)] : 0.0;
      vv[c] = ok ? U[2 * (nd[c] - 1) + 1] : 0.0;
    }
    for (int c = 0; c < 4; ++c) dp[c] = nd[4 + c] != 0 ? 1.0 : 0.0;
    const double x1 = px[0], x3 = px[2], y1 = py[0], y3 = py[2];
    std::vector<double> gs(4 * ng * ng), gxv(ng * ng), gyv(ng * ng);
    for (int ti = 0; ti < ng; ++ti)
      for (int tj = 0; tj < ng; ++tj) {
        const int g = ng * ti + tj;
        const double ksi = gpt[ti], eta = gpt[tj];
        gxv[g] = gpt[ti] * 0.5 * (x3 - x1) + 0.5 * (x3 + x1);
        gyv[g] = gpt[tj] * 0.5 * (y3 - y1) + 0.5 * (y3 + y1);
        double dk[8], de[8];
        shape_derivs(ksi, eta, dp, dk, de);
        double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
        for (int c = 0; c < 8; ++c) {
          J11 += dk[c] * px[c]; J12 += dk[c] * py[c];
          J21 += de[c] * px[c]; J22 += de[c] * py[c];
        }
        const double det = J11 * J22 - J12 * J21;
        const double i11 = J22 / det, i12 = -J12 / det, i21 = -J21 / det, i22 = J11 / det;
        double dudx = 0, dudy = 0, dvdx = 0, dvdy = 0;
        for (int c = 0; c < 8; ++c) {
          const double gx = i11 * dk[c] + i12 * de[c], gy = i21 * dk[c] + i22 * de[c];
          dudx += gx * uu[c]; dudy += gy * uu[c];
          dvdx += gx * vv[c]; dvdy += gy * vv[c];
        }
        gs[4 * g] = dudx; gs[4 * g + 1] = dvdx; gs[4 * g + 2] = dudy; gs[4 * g + 3] = dvdy;
      }
    for (int c = 0; c < 8; ++c) {
      if (nd[c] < 1 || nd[c] > N) continue;
      const long n = nd[c] - 1;
      int best = 0;
      double bd = 1e300;
      for (int g = 0; g < ng * ng; ++g) {
        const double dx = gxv[g] - coords[n], dy = gyv[g] - coords[N + n];
        const double d2 = dx * dx + dy * dy;
        // distances within 1e-9 relative are ties (the first Gauss point
        // wins): a hanging node at an edge midpoint is equidistant from two
        if (d2 < bd * (1.0 - 1e-9)) { bd = d2; best = g; }
      }
      for (int k = 0; k < 4; ++k) sum[4 * n + k] += gs[4 * best + k];
      cnt[n] += 1;
    }
  }
  for (long n = 0; n < N; ++n)
    for (int k = 0; k < 4; ++k) F[4 * n + k] = cnt[n] ? sum[4 * n + k] / cnt[n] : NAN;
}

// NaN fill (local replacement of the reference's thin-plate RBF fill,
// Subpb1Quadtree.m:193-259): sweeps in which every node whose displacement is
// NaN and which shares an element with finite nodes takes the mean of those
// neighbours' values of the previous sweep (neighbours in increasing node
// order), until no NaN node has a finite neighbour.
extern "C" void orc_fill_nans(const double* coords, long N, const int32_t* elems, long E, double* U) {
  (void)coords;
  std::vector<std::vector<long>> nb(N);
  for (long e = 0; e < E; ++e)
    for (int a = 0; a < 8; ++a) {
      const long p = elems[a * E + e];
      if (p < 1 || p > N) continue;
      for (int b = 0; b < 8; ++b) {
        const long q = elems[b * E + e];
        if (q < 1 || q > N || q == p) continue;
        nb[p - 1].push_back(q - 1);
      }
    }
  for (auto& v : nb) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  std::vector<double> old(U, U + 2 * N);
  for (;;) {
    bool changed = false;
    for (long n = 0; n < N; ++n) {
      if (!std::isnan(old[2 * n])) continue;
      double su = 0, sv = 0;
      int k = 0;
      for (long m : nb[n])
        if (!std::isnan(old[2 * m])) { su += old[2 * m]; sv += old[2 * m + 1]; ++k; }
      if (k) { U[2 * n] = su / k; U[2 * n + 1] = sv / k; changed = true; }
    }
    if (!changed) break;
    std::copy(U, U + 2 * N, old.begin());
  }
}

extern "C" int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

extern "C" void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

