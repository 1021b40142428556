// Multigrid integer search (func/funIntegerSearchMg.m:3-343 with
// func/findpeak.m:27-68 and the 'springs' fit of func/gridfit.m) on the device.
//
// Level 1 correlates the whole ROI of f with the same ROI of g: normxcorr2's
// full (2m-1) x (2n-1) map, whose numerator is one FFT correlation (FP64
// complex transforms of fft.cu; A and the flipped zero-mean template packed as
// the real and imaginary parts of one transform).  Every later level splits
// each block in halves (x, y or both, by the aspect of the reference's nominal
// widths) and searches each child within +-5 px of its parent's shift: only
// the 13 x 14 lags that findpeak reads (funIntegerSearchMg.m:182) are formed,
// as direct FP64 sums over template tiles.  Window sums of A and A^2 (the
// normxcorr2 denominators) come from FP64 integral images of g and g^2, one
// pair per call; the tolerance sqrt(eps(max |den|)) is taken over each
// block's FULL map, as normxcorr2 does.  Block geometry (splits, the border
// clamps and the odd-width fix of :31-42, :258-296) is integer arithmetic on
// the device, one thread per block.
//
// The block-centre displacements are then fitted to the node grid by gridfit
// with the springs regularizer: the normal equations of the stacked least-
// squares system form a 9-point stencil on the ny x nx node grid (triangle
// interpolation couples the corners of one cell, springs couple the 8
// neighbours), solved for u, v and cc.max at once by a cooperative
// Jacobi-PCG in FP64 with bounded grid barriers.
//
// Scope: cc.qfactors of the reference's Mg search (PCE and PPE of every
// final-level block's full map, fitted to the grid) are not produced; the
// reference's caller on this path (IntegerSearch.m:125) does not read them.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "coop.cuh"
#include "device_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

constexpr int kTX = 64, kTY = 16;      // template tile of a block search
constexpr int kLagR = 13, kLagC = 14;  // lags findpeak reads: XC(w1:end-w1+1, w2:end-w2+2)
constexpr int kLags = kLagR * kLagC;
constexpr int kMargin = 5;             // D = g(xg-5:xg+5, yg-5:yg+5) (:176)
constexpr long long kGfSpin = 1ll << 24;

struct MgBlock {  // 1-based inclusive pixel ranges, as the reference keeps them
  double xf0, xf1, yf0, yf1;  // template C = f(xf0:xf1, yf0:yf1)
  double xg0, xg1, yg0, yg1;  // window D = g(xg0-5:xg1+5, yg0-5:yg1+5) (level 1: no margin)
  double u, v;                // displacement the block starts from (its parent's, ceil'd)
};
struct MgRes {
  double u, v, phi;
};
struct MgStat {
  double meanT, denT;
  int ok;
  int pad;
};
struct MgImg {
  const double* f;
  const double* g;
  int W, H;
  const double* I1;  // (W+1) x (H+1): sums of g (non-finite taken as 0)
  const double* I2;  // sums of g^2
  const int* In;     // counts of non-finite g
};

// ---------------------------------------------------------------------------
// integral images
// ---------------------------------------------------------------------------
// Row prefix sums: I[(y+1)(W+1) + x+1] = sum_{x' <= x} g(x', y); one CTA per
// row, a contiguous segment per thread, the segment totals scanned by thread 0.
__global__ void __launch_bounds__(256) ii_rows_kernel(const double* __restrict__ g, int W, double* I1, double* I2,
                                                      int* In) {
  __shared__ double s1[256], s2[256];
  __shared__ int sn[256];
  const int y = blockIdx.x;
  const int W1 = W + 1;
  const double* row = g + (size_t)y * W;
  const int per = (W + blockDim.x - 1) / blockDim.x;
  const int b0 = min(W, (int)threadIdx.x * per), b1 = min(W, b0 + per);
  double a1 = 0, a2 = 0;
  int an = 0;
  for (int x = b0; x < b1; ++x) {
    const double v = row[x];
    const bool fin = isfinite(v);
    const double w = fin ? v : 0.0;
    a1 += w;
    a2 += w * w;
    an += fin ? 0 : 1;
  }
  s1[threadIdx.x] = a1;
  s2[threadIdx.x] = a2;
  sn[threadIdx.x] = an;
  __syncthreads();
  if (threadIdx.x == 0) {
    double c1 = 0, c2 = 0;
    int cn = 0;
    for (int k = 0; k < (int)blockDim.x; ++k) {
      const double t1 = s1[k], t2 = s2[k];
      const int tn = sn[k];
      s1[k] = c1; s2[k] = c2; sn[k] = cn;
      c1 += t1; c2 += t2; cn += tn;
    }
  }
  __syncthreads();
  double c1 = s1[threadIdx.x], c2 = s2[threadIdx.x];
  int cn = sn[threadIdx.x];
  double* o1 = I1 + (size_t)(y + 1) * W1;
  double* o2 = I2 + (size_t)(y + 1) * W1;
  int* on = In + (size_t)(y + 1) * W1;
  if (threadIdx.x == 0) { o1[0] = 0; o2[0] = 0; on[0] = 0; }
  for (int x = b0; x < b1; ++x) {
    const double v = row[x];
    const bool fin = isfinite(v);
    const double w = fin ? v : 0.0;
    c1 += w;
    c2 += w * w;
    cn += fin ? 0 : 1;
    o1[x + 1] = c1; o2[x + 1] = c2; on[x + 1] = cn;
  }
}

// Column prefix sums of the row sums (row 0 is zero): a 32 x 32 CTA takes 32
// columns, each of its 32 thread rows a chunk of rows; the chunk totals are
// scanned in shared memory and added back.
__global__ void __launch_bounds__(1024) ii_cols_kernel(int W, int H, double* I1, double* I2, int* In) {
  __shared__ double t1[32][33], t2[32][33];
  __shared__ int tn[32][33];
  const int x = blockIdx.x * 32 + threadIdx.x, ch = threadIdx.y;
  const int W1 = W + 1;
  const int per = (H + 31) / 32;
  const int y0 = 1 + ch * per, y1 = min(H, y0 + per - 1);
  double a1 = 0, a2 = 0;
  int an = 0;
  if (x <= W) {
    if (ch == 0) { I1[x] = 0; I2[x] = 0; In[x] = 0; }
    for (int y = y0; y <= y1; ++y) {
      const size_t k = (size_t)y * W1 + x;
      a1 += I1[k]; a2 += I2[k]; an += In[k];
    }
  }
  t1[ch][threadIdx.x] = a1; t2[ch][threadIdx.x] = a2; tn[ch][threadIdx.x] = an;
  __syncthreads();
  if (ch == 0) {
    double c1 = 0, c2 = 0;
    int cn = 0;
    for (int k = 0; k < 32; ++k) {
      const double u1 = t1[k][threadIdx.x], u2 = t2[k][threadIdx.x];
      const int un = tn[k][threadIdx.x];
      t1[k][threadIdx.x] = c1; t2[k][threadIdx.x] = c2; tn[k][threadIdx.x] = cn;
      c1 += u1; c2 += u2; cn += un;
    }
  }
  __syncthreads();
  if (x > W) return;
  double c1 = t1[ch][threadIdx.x], c2 = t2[ch][threadIdx.x];
  int cn = tn[ch][threadIdx.x];
  for (int y = y0; y <= y1; ++y) {
    const size_t k = (size_t)y * W1 + x;
    c1 += I1[k]; c2 += I2[k]; cn += In[k];
    I1[k] = c1; I2[k] = c2; In[k] = cn;
  }
}

// sum over the 0-based inclusive image rectangle [xa, xb] x [ya, yb]
template <class T>
STDIC_DEV T rect_sum(const T* I, int W1, int xa, int xb, int ya, int yb) {
  return I[(size_t)(yb + 1) * W1 + xb + 1] - I[(size_t)ya * W1 + xb + 1] - I[(size_t)(yb + 1) * W1 + xa] +
         I[(size_t)ya * W1 + xa];
}

// normxcorr2's denominator at one lag: the template (m x n) placed with its
// first pixel at offset (ox, oy) of the window A (Mw x Nw, first pixel at
// 0-based image position (ax0, ay0), zero outside).
STDIC_DEV double lag_den(const MgImg& im, int ax0, int ay0, int Mw, int Nw, int m, int n, int ox, int oy,
                         double denT, double mn) {
  const int xa = max(ox, 0), xb = min(ox + m - 1, Mw - 1), ya = max(oy, 0), yb = min(oy + n - 1, Nw - 1);
  if (xa > xb || ya > yb) return 0.0;
  const int W1 = im.W + 1;
  const double s1 = rect_sum(im.I1, W1, ax0 + xa, ax0 + xb, ay0 + ya, ay0 + yb);
  const double s2 = rect_sum(im.I2, W1, ax0 + xa, ax0 + xb, ay0 + ya, ay0 + yb);
  const double dl = s2 - s1 * s1 / mn;
  return denT * sqrt(dl > 0 ? dl : 0.0);
}

STDIC_DEV double ncc_value(double num, double den, double tol, double clip) {
  double c = den > tol ? num / den : 0.0;
  if ((fabs(c) - 1) > clip) c = 0;
  return c;
}

STDIC_DEV double eps_of_d(double x) {
  x = fabs(x);
  if (!(x > 0)) return 4.9406564584124654e-324;
  int e;
  frexp(x, &e);
  const int p = e - 53;
  return p < -1074 ? 4.9406564584124654e-324 : ldexp(1.0, p);
}

STDIC_DEV bool whole(double v) { return isfinite(v) && floor(v) == v; }

// The template and window rectangles of a block (0-based image positions)
// when the reference's crops succeed; false where MATLAB's indexing throws.
STDIC_DEV bool block_rects(const MgBlock& b, int W, int H, bool level1, int* tx0, int* ty0, int* m, int* n, int* ax0,
                           int* ay0, int* Mw, int* Nw) {
  if (!(whole(b.xf0) && whole(b.xf1) && whole(b.yf0) && whole(b.yf1) && whole(b.xg0) && whole(b.xg1) &&
        whole(b.yg0) && whole(b.yg1)))
    return false;
  const int mg = level1 ? 0 : kMargin;
  const double gx0 = b.xg0 - mg, gx1 = b.xg1 + mg, gy0 = b.yg0 - mg, gy1 = b.yg1 + mg;
  if (b.xf0 < 1 || b.yf0 < 1 || b.xf1 > W || b.yf1 > H || b.xf1 < b.xf0 || b.yf1 < b.yf0) return false;
  if (gx0 < 1 || gy0 < 1 || gx1 > W || gy1 > H || gx1 < gx0 || gy1 < gy0) return false;
  *tx0 = (int)b.xf0 - 1; *ty0 = (int)b.yf0 - 1;
  *m = (int)(b.xf1 - b.xf0) + 1; *n = (int)(b.yf1 - b.yf0) + 1;
  *ax0 = (int)gx0 - 1; *ay0 = (int)gy0 - 1;
  *Mw = (int)(gx1 - gx0) + 1; *Nw = (int)(gy1 - gy0) + 1;
  return *Mw >= *m && *Nw >= *n;  // normxcorr2 needs the template inside A
}

// ---------------------------------------------------------------------------
// per-block template statistics: crops valid, no non-finite value in C or D,
// meanT and denT = sqrt(mn-1) std(T); ok = 0 where the reference's try block
// fails (bad crop, normxcorr2 error: non-finite data, constant template)
// ---------------------------------------------------------------------------
// Pass 1 (pass = 0) and pass 2 (pass = 1) of the template statistics: nct
// CTAs per block add the template's values (pass 1) or squared deviations from
// its mean (pass 2) over a strided share of its pixels; part[block][cta]
// receives the CTA's sum, bad[block][cta] whether it saw a non-finite value.
__global__ void __launch_bounds__(256) mg_tsum_kernel(MgImg im, const MgBlock* __restrict__ blocks, int level1,
                                                      int nct, int pass, const MgStat* __restrict__ st,
                                                      double* __restrict__ part, int* __restrict__ bad) {
  __shared__ double red[8];
  const int bi = blockIdx.x / nct, cta = blockIdx.x % nct;
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  const bool rects = block_rects(blocks[bi], im.W, im.H, level1 != 0, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  double acc = 0;
  int nf = 0;
  if (rects && (pass == 0 || st[bi].ok)) {
    const double mean = pass ? st[bi].meanT : 0.0;
    const int np = m * n;
    for (int q = cta * blockDim.x + threadIdx.x; q < np; q += nct * blockDim.x) {
      const int i = q % m, j = q / m;
      const double v = im.f[(size_t)(ty0 + j) * im.W + tx0 + i];
      if (pass == 0) {
        if (!isfinite(v)) nf = 1;
        acc += v;
      } else {
        const double d = v - mean;
        acc += d * d;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  nf = __syncthreads_or(nf);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    part[blockIdx.x] = t;
    if (pass == 0) bad[blockIdx.x] = nf;
  }
}

// Per block, after pass 1 (pass = 0): the crops' validity, meanT and the
// non-finite checks of C and D; after pass 2: denT = sqrt(mn-1) std(T) and
// ok = 0 where the reference's try block fails (bad crop, normxcorr2 error:
// non-finite data, constant template).  The partial sums are added in CTA
// order, so the result does not depend on scheduling.
__global__ void mg_tstat_kernel(MgImg im, const MgBlock* __restrict__ blocks, int nb, int level1, int nct, int pass,
                                const double* __restrict__ part, const int* __restrict__ bad,
                                MgStat* __restrict__ st) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x;
  if (bi >= nb) return;
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  const bool rects = block_rects(blocks[bi], im.W, im.H, level1 != 0, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  const double mn = (double)m * (double)n;
  if (pass == 0) {
    if (!rects) {
      st[bi] = MgStat{0.0, 0.0, 0, 0};
      return;
    }
    double sum = 0;
    int nf = 0;
    for (int c = 0; c < nct; ++c) {
      sum += part[(size_t)bi * nct + c];
      nf |= bad[(size_t)bi * nct + c];
    }
    const bool finiteA = rect_sum(im.In, im.W + 1, ax0, ax0 + Mw - 1, ay0, ay0 + Nw - 1) == 0;
    st[bi] = MgStat{sum / mn, 0.0, (finiteA && !nf) ? 1 : 0, 0};
  } else {
    if (!st[bi].ok) return;
    double q = 0;
    for (int c = 0; c < nct; ++c) q += part[(size_t)bi * nct + c];
    const double stdT = sqrt(q / (mn - 1));
    st[bi].denT = sqrt(mn - 1) * stdT;
    st[bi].ok = stdT != 0 ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// level 1: the full map by FFT
// ---------------------------------------------------------------------------
// z[y][x] = A(x, y) + i Tz(m-1-x, n-1-y), zero padded to Fx x Fy
__global__ void mg_fill_kernel(MgImg im, const MgBlock* __restrict__ blk, const MgStat* __restrict__ st,
                               double2* __restrict__ z, int Fx, int Fy) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= Fx) return;
  const size_t k = (size_t)y * Fx + x;
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  block_rects(blk[0], im.W, im.H, true, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  double a = 0, t = 0;
  if (x < Mw && y < Nw) a = im.g[(size_t)(ay0 + y) * im.W + ax0 + x];
  if (x < m && y < n) t = im.f[(size_t)(ty0 + n - 1 - y) * im.W + tx0 + m - 1 - x] - st[0].meanT;
  z[k] = make_double2(a, t);
}

// P = FFT(A) FFT(Tflip) from Z = FFT(A + i Tflip), in the transposed layout
// Zt[kx][ky]: FFT(A) = (Z(k) + conj Z(-k)) / 2, FFT(Tflip) = (Z(k) - conj Z(-k)) / 2i
__global__ void mg_product_kernel(const double2* __restrict__ Zt, double2* __restrict__ Pt, int Fx, int Fy) {
  const int ky = blockIdx.x * blockDim.x + threadIdx.x, kx = blockIdx.y;
  if (ky >= Fy) return;
  const size_t k = (size_t)kx * Fy + ky;
  const int mx = kx == 0 ? 0 : Fx - kx, my = ky == 0 ? 0 : Fy - ky;
  const double2 z1 = Zt[k], z2 = Zt[(size_t)mx * Fy + my];
  const double ar = 0.5 * (z1.x + z2.x), ai = 0.5 * (z1.y - z2.y);  // (z1 + conj z2) / 2
  const double br = 0.5 * (z1.y + z2.y), bi = -0.5 * (z1.x - z2.x);  // (z1 - conj z2) / 2i
  Pt[k] = make_double2(ar * br - ai * bi, ar * bi + ai * br);
}

// max |den| over the full (Mw+m-1) x (Nw+n-1) map of each block, as the bits
// of a non-negative double (integer order = value order)
__global__ void __launch_bounds__(256) mg_denmax_kernel(MgImg im, const MgBlock* __restrict__ blocks,
                                                        const MgStat* __restrict__ st, int level1,
                                                        unsigned long long* __restrict__ dmax) {
  const int bi = blockIdx.y;
  if (!st[bi].ok) return;
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  block_rects(blocks[bi], im.W, im.H, level1 != 0, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  const int R = Mw + m - 1, C = Nw + n - 1;
  const double mn = (double)m * n, denT = st[bi].denT;
  if (!level1) {
    // The tolerance only decides lags whose denominator is at most
    // sqrt(eps(max |den|)), and every denominator of the map is at most
    // denT sqrt(sum of A^2 over the window D).  When every lag of the 13 x 14
    // crop lies above the tolerance that bound implies (doubled, against
    // rounding), the values findpeak reads do not depend on the map's maximum
    // and the scan is skipped (dmax stays 0, the smallest tolerance).
    __shared__ int s_need;
    const double ub = 2.0 * denT * sqrt(fmax(rect_sum(im.I2, im.W + 1, ax0, ax0 + Mw - 1, ay0, ay0 + Nw - 1), 0.0));
    const double tmax = sqrt(eps_of_d(ub));
    int low = 0;
    for (int l = threadIdx.x; l < kLags; l += blockDim.x)
      if (!(lag_den(im, ax0, ay0, Mw, Nw, m, n, l % kLagR - 1, l / kLagR - 1, denT, mn) > tmax)) low = 1;
    low = __syncthreads_or(low);
    if (threadIdx.x == 0) s_need = low;
    __syncthreads();
    if (!s_need) return;
  }
  double best = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R * C; k += gridDim.x * blockDim.x) {
    const int r = k % R, c = k / R;
    best = fmax(best, lag_den(im, ax0, ay0, Mw, Nw, m, n, r - m + 1, c - n + 1, denT, mn));
  }
  for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_down_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(dmax + bi, (unsigned long long)__double_as_longlong(best));
}

// level 1, pass 1: the largest value of each CTA's lags
__global__ void __launch_bounds__(256) mg_l1_max_kernel(MgImg im, const MgBlock* __restrict__ blk,
                                                        const MgStat* __restrict__ st, const double2* __restrict__ q,
                                                        int Fx, const unsigned long long* __restrict__ dmax,
                                                        double scale, double* __restrict__ pv) {
  __shared__ double sv[32];
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  block_rects(blk[0], im.W, im.H, true, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  const long long R = Mw + m - 1, C = Nw + n - 1;
  const double mn = (double)m * n, denT = st[0].denT;
  const double tol = sqrt(eps_of_d(__longlong_as_double((long long)dmax[0])));
  const double clip = sqrt(eps_of_d(1.0));
  double bv = -INFINITY;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < (int)(R * C); k += gridDim.x * blockDim.x) {
    const int r = k % (int)R, c = k / (int)R;
    const double num = q[(size_t)c * Fx + r].x * scale;
    bv = fmax(bv, ncc_value(num, lag_den(im, ax0, ay0, Mw, Nw, m, n, r - m + 1, c - n + 1, denT, mn), tol, clip));
  }
  for (int o = 16; o > 0; o >>= 1) bv = fmax(bv, __shfl_down_sync(0xffffffffu, bv, o));
  if ((threadIdx.x & 31) == 0) sv[threadIdx.x >> 5] = bv;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) bv = fmax(bv, sv[w]);
    pv[blockIdx.x] = bv;
  }
}

// level 1, pass 2: the first lag (column-major) within kPeakTie of the
// map's maximum, per CTA
__global__ void __launch_bounds__(256) mg_l1_first_kernel(MgImg im, const MgBlock* __restrict__ blk,
                                                          const MgStat* __restrict__ st, const double2* __restrict__ q,
                                                          int Fx, const unsigned long long* __restrict__ dmax,
                                                          double scale, const double* __restrict__ pv, int np,
                                                          long long* __restrict__ pi) {
  __shared__ long long si[32];
  __shared__ double sm;
  if (threadIdx.x == 0) {
    double m0 = -INFINITY;
    for (int k = 0; k < np; ++k) m0 = fmax(m0, pv[k]);
    sm = m0;
  }
  __syncthreads();
  const double gmax = sm;
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  block_rects(blk[0], im.W, im.H, true, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  const long long R = Mw + m - 1, C = Nw + n - 1;
  const double mn = (double)m * n, denT = st[0].denT;
  const double tol = sqrt(eps_of_d(__longlong_as_double((long long)dmax[0])));
  const double clip = sqrt(eps_of_d(1.0));
  long long bi = 0x7fffffffffffffffLL;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < (int)(R * C); k += gridDim.x * blockDim.x) {
    const int r = k % (int)R, c = k / (int)R;
    const double num = q[(size_t)c * Fx + r].x * scale;
    const double v = ncc_value(num, lag_den(im, ax0, ay0, Mw, Nw, m, n, r - m + 1, c - n + 1, denT, mn), tol, clip);
    if (v >= gmax - kPeakTie) { bi = k; break; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const long long oi = __shfl_down_sync(0xffffffffu, bi, o);
    bi = oi < bi ? oi : bi;
  }
  if ((threadIdx.x & 31) == 0) si[threadIdx.x >> 5] = bi;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) bi = si[w] < bi ? si[w] : bi;
    pi[blockIdx.x] = bi;
  }
}

// findpeak (findpeak.m:27-68) on a map C (nr x nc, column-major) read through
// val(r, c): the first maximum at linear index imax, the least-squares
// quadratic of its 3 x 3 neighbourhood unless it lies on the edge or the fit
// moves it by more than one sample, offsets rounded to 1/1000.
template <class F>
STDIC_DEV void findpeak_at(const F& val, int nr, int nc, long long imax, double* ypeak, double* xpeak, double* maxf) {
  const int yp = (int)(imax % nr) + 1, xp = (int)(imax / nr) + 1;
  *ypeak = yp;
  *xpeak = xp;
  *maxf = val(yp - 1, xp - 1);
  if (xp == 1 || xp == nc || yp == 1 || yp == nr) return;
  double v9[9];
  for (int dc = -1; dc <= 1; ++dc)
    for (int dr = -1; dr <= 1; ++dr) v9[(dr + 1) + 3 * (dc + 1)] = val(yp - 1 + dr, xp - 1 + dc);
  double xo, yo, mf;
  if (findpeak_fit3(v9, &xo, &yo, &mf)) {
    *xpeak += xo;
    *ypeak += yo;
    *maxf = mf;
  }
}

// level 1: the global maximum, findpeak, u = ypeak - zero_disp(1), v = xpeak - zero_disp(2)
__global__ void mg_l1_peak_kernel(MgImg im, const MgBlock* __restrict__ blk, const MgStat* __restrict__ st,
                                  const double2* __restrict__ q, int Fx, const unsigned long long* __restrict__ dmax,
                                  double scale, const double* __restrict__ pv, const long long* __restrict__ pi,
                                  int np, MgRes* __restrict__ res) {
  if (threadIdx.x != 0) return;
  long long bi = 0x7fffffffffffffffLL;
  for (int k = 0; k < np; ++k) bi = pi[k] < bi ? pi[k] : bi;
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  block_rects(blk[0], im.W, im.H, true, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  const int R = Mw + m - 1, C = Nw + n - 1;
  const double mn = (double)m * n, denT = st[0].denT;
  const double tol = sqrt(eps_of_d(__longlong_as_double((long long)dmax[0])));
  const double clip = sqrt(eps_of_d(1.0));
  auto val = [&](int r, int c) {
    const double num = q[(size_t)c * Fx + r].x * scale;
    return ncc_value(num, lag_den(im, ax0, ay0, Mw, Nw, m, n, r - m + 1, c - n + 1, denT, mn), tol, clip);
  };
  double yp, xp, mf;
  findpeak_at(val, R, C, bi, &yp, &xp, &mf);
  res[0] = MgRes{yp - ceil((R + 1) / 2.0), xp - ceil((C + 1) / 2.0), mf};
}

// ---------------------------------------------------------------------------
// levels >= 2
// ---------------------------------------------------------------------------
// children of block p (funIntegerSearchMg.m:71-150): mode 0 splits x, 1 splits
// y, 2 both (children (xa,ya), (xb,ya), (xa,yb), (xb,yb)); a block not wider
// than winsize along a split side is copied instead
__global__ void mg_split_kernel(const MgBlock* __restrict__ cur, MgBlock* __restrict__ nxt, int ncur, int mode,
                                double winsize) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ncur) return;
  const MgBlock b = cur[p];
  const double mxf = 0.5 * (b.xf0 + b.xf1), mxg = 0.5 * (b.xg0 + b.xg1);
  const double myf = 0.5 * (b.yf0 + b.yf1), myg = 0.5 * (b.yg0 + b.yg1);
  if (mode == 0 || mode == 1) {
    MgBlock c0 = b, c1 = b;
    if (mode == 0 && b.xf1 - b.xf0 > winsize) {
      c0.xf1 = mxf; c0.xg1 = mxg;
      c1.xf0 = mxf; c1.xg0 = mxg;
    } else if (mode == 1 && b.yf1 - b.yf0 > winsize) {
      c0.yf1 = myf; c0.yg1 = myg;
      c1.yf0 = myf; c1.yg0 = myg;
    }
    nxt[2 * p] = c0;
    nxt[2 * p + 1] = c1;
  } else {
    MgBlock c[4] = {b, b, b, b};
    if (b.xf1 - b.xf0 > winsize && b.yf1 - b.yf0 > winsize) {
      c[0].xf1 = mxf; c[0].xg1 = mxg; c[0].yf1 = myf; c[0].yg1 = myg;
      c[1].xf0 = mxf; c[1].xg0 = mxg; c[1].yf1 = myf; c[1].yg1 = myg;
      c[2].xf1 = mxf; c[2].xg1 = mxg; c[2].yf0 = myf; c[2].yg0 = myg;
      c[3].xf0 = mxf; c[3].xg0 = mxg; c[3].yf0 = myf; c[3].yg0 = myg;
    }
    for (int k = 0; k < 4; ++k) nxt[4 * p + k] = c[k];
  }
}

// Direct sums of the numerator at the 13 x 14 lags for the template tiles of
// each block: nct CTAs per block, each taking tiles t = cta, cta + nct, ...;
// thread l < 182 owns lag (l % 13, l / 13), i.e. the template's first pixel
// at offset (l % 13 - 1, l / 13 - 1) of the window A.
__global__ void __launch_bounds__(192) mg_tiles_kernel(MgImg im, const MgBlock* __restrict__ blocks,
                                                       const MgStat* __restrict__ st, int nct,
                                                       double* __restrict__ part) {
  __shared__ double T[kTY][kTX];
  __shared__ double A[kTY + kLagC - 1][kTX + kLagR - 1];
  const int bi = blockIdx.x / nct, cta = blockIdx.x % nct;
  const int l = threadIdx.x;
  double acc = 0;
  if (st[bi].ok) {
    int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
    block_rects(blocks[bi], im.W, im.H, false, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
    const double meanT = st[bi].meanT;
    const int ntx = (m + kTX - 1) / kTX, nty = (n + kTY - 1) / kTY;
    const int lr = l % kLagR, lc = l / kLagR;
    for (int t = cta; t < ntx * nty; t += nct) {
      const int i0 = (t % ntx) * kTX, j0 = (t / ntx) * kTY;
      __syncthreads();
      for (int k = threadIdx.x; k < kTX * kTY; k += blockDim.x) {
        const int i = k % kTX, j = k / kTX;
        T[j][i] = (i0 + i < m && j0 + j < n) ? im.f[(size_t)(ty0 + j0 + j) * im.W + tx0 + i0 + i] - meanT : 0.0;
      }
      // A window of the tile: A(x, y) for x = i0 - 1 .. i0 + kTX + 10, y = j0 - 1 .. j0 + kTY + 11
      for (int k = threadIdx.x; k < (kTX + kLagR - 1) * (kTY + kLagC - 1); k += blockDim.x) {
        const int a = k % (kTX + kLagR - 1), b = k / (kTX + kLagR - 1);
        const int x = i0 - 1 + a, y = j0 - 1 + b;
        A[b][a] = (x >= 0 && x < Mw && y >= 0 && y < Nw) ? im.g[(size_t)(ay0 + y) * im.W + ax0 + x] : 0.0;
      }
      __syncthreads();
      if (l < kLags) {
        const int jn = min(kTY, n - j0), in_ = min(kTX, m - i0);
        for (int j = 0; j < jn; ++j) {
          const double* tr = T[j];
          const double* ar = A[j + lc] + lr;
          for (int i = 0; i < in_; ++i) acc = fma(tr[i], ar[i], acc);
        }
      }
    }
  }
  if (l < kLags) part[(size_t)blockIdx.x * kLags + l] = acc;
}

// Per block: the numerators (partials summed in CTA order), the values with
// the block's full-map tolerance, findpeak on the 13 x 14 crop and the
// displacement u = parent u + (ypeak - 7), v = parent v + (xpeak - 7)
// (zero_disp of the 13 x 13 crop, :183-188); NaN, NaN, 0 where the try fails.
__global__ void __launch_bounds__(192) mg_finish_kernel(MgImg im, const MgBlock* __restrict__ blocks,
                                                        const MgStat* __restrict__ st, int nct,
                                                        const double* __restrict__ part,
                                                        const unsigned long long* __restrict__ dmax,
                                                        MgRes* __restrict__ res) {
  __shared__ double C[kLags];
  const int bi = blockIdx.x;
  const MgBlock b = blocks[bi];
  if (!st[bi].ok) {
    if (threadIdx.x == 0) res[bi] = MgRes{nan(""), nan(""), 0.0};
    return;
  }
  int tx0, ty0, m, n, ax0, ay0, Mw, Nw;
  block_rects(b, im.W, im.H, false, &tx0, &ty0, &m, &n, &ax0, &ay0, &Mw, &Nw);
  const double mn = (double)m * n, denT = st[bi].denT;
  const double tol = sqrt(eps_of_d(__longlong_as_double((long long)dmax[bi])));
  const double clip = sqrt(eps_of_d(1.0));
  const int l = threadIdx.x;
  if (l < kLags) {
    double num = 0;
    for (int c = 0; c < nct; ++c) num += part[((size_t)bi * nct + c) * kLags + l];
    const int lr = l % kLagR, lc = l / kLagR;
    C[l] = ncc_value(num, lag_den(im, ax0, ay0, Mw, Nw, m, n, lr - 1, lc - 1, denT, mn), tol, clip);
  }
  __syncthreads();
  const int bidx = cta_first_near_max(C, kLags);
  if (threadIdx.x != 0) return;
  auto val = [&](int r, int c) { return C[r + kLagR * c]; };
  double yp, xp, mf;
  findpeak_at(val, kLagR, kLagC, bidx, &yp, &xp, &mf);
  res[bi] = MgRes{b.u + (yp - 7.0), b.v + (xp - 7.0), mf};
}

}  // namespace

// Window of g after a search (:31-42 for level 1, :258-296 after each level):
// xg = xf + ceil(u), clamped to the border gaps (moving xf by the same amount),
// then the widths made even; the block carries ceil(u), ceil(v) on.
static __host__ __device__ void mg_clamp(double* xf, double* yf, double* xg, double* yg, double u, double v, int W, int H,
                                  double bgx, double bgy) {
  const double cu = ceil(u), cv = ceil(v);
  xg[0] = xf[0] + cu; xg[1] = xf[1] + cu;
  yg[0] = yf[0] + cv; yg[1] = yf[1] + cv;
  if (xg[0] < bgx) { const double t = xg[0]; xg[0] = bgx; xf[0] = xf[0] + bgx - t; }
  if (yg[0] < bgy) { const double t = yg[0]; yg[0] = bgy; yf[0] = yf[0] + bgy - t; }
  if (xg[1] > W - bgx) { const double t = xg[1]; xg[1] = W - bgx; xf[1] = xf[1] + ((W - bgx) - t); }
  if (yg[1] > H - bgy) { const double t = yg[1]; yg[1] = H - bgy; yf[1] = yf[1] + ((H - bgy) - t); }
  if (fmod(xf[1] - xf[0], 2.0) == 1) { xf[1] -= 1; xg[1] -= 1; }
  if (fmod(yf[1] - yf[0], 2.0) == 1) { yf[1] -= 1; yg[1] -= 1; }
}

namespace {

__global__ void mg_clamp_kernel(MgBlock* __restrict__ blocks, const MgRes* __restrict__ res, int nb, int W, int H,
                                double bgx, double bgy) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  MgBlock b = blocks[k];
  const MgRes r = res[k];
  double xf[2] = {b.xf0, b.xf1}, yf[2] = {b.yf0, b.yf1}, xg[2], yg[2];
  mg_clamp(xf, yf, xg, yg, r.u, r.v, W, H, bgx, bgy);
  b.xf0 = xf[0]; b.xf1 = xf[1]; b.yf0 = yf[0]; b.yf1 = yf[1];
  b.xg0 = xg[0]; b.xg1 = xg[1]; b.yg0 = yg[0]; b.yg1 = yg[1];
  b.u = ceil(r.u);
  b.v = ceil(r.v);
  blocks[k] = b;
}

// final level: block centres and their results
__global__ void mg_collect_kernel(const MgBlock* __restrict__ blocks, const MgRes* __restrict__ res, int nb,
                                  double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  out[k] = 0.5 * (blocks[k].xf0 + blocks[k].xf1);
  out[nb + k] = 0.5 * (blocks[k].yf0 + blocks[k].yf1);
  out[2 * (size_t)nb + k] = res[k].u;
  out[3 * (size_t)nb + k] = res[k].v;
  out[4 * (size_t)nb + k] = res[k].phi;
}

// ---------------------------------------------------------------------------
// gridfit (springs): normal equations as a 9-point stencil, k = (dj+1) + 3(di+1)
// ---------------------------------------------------------------------------
struct GfArgs {
  int nx, ny, nd;
  int nz;            // right-hand sides (data columns after x, y), 1..3
  const double* xn;  // nx node positions
  const double* yn;  // ny
  const double* dat; // nd x (2 + nz) column-major: x, y, then the data values
  double xscale, yscale;
  double* K;         // ngrid x 9
  double* colA;      // ngrid: column sums of |A|
  double* rhs;       // nz x ngrid
  unsigned long long* nmax;  // [0] max colA, [1] max column sum of |Areg|
  double* x;         // nz x ngrid solution
  double* r;
  double* z;
  double* p;
  double* Ap;
  double* part;      // 16 x 1024 partial sums
  int* misc;         // [0] barrier count, [1] generation
  int* status;       // 0 ok, 1 not converged, 2 wait gave up
  int* iters;
  double tol;
  int maxit;
  long long spin;
};

STDIC_DEV double gf_dx(const GfArgs& a, int i) { return a.xn[i + 1] - a.xn[i]; }
STDIC_DEV double gf_dy(const GfArgs& a, int j) { return a.yn[j + 1] - a.yn[j]; }

// the triangle interpolation row of data point d (gridfit.m 'triangle')
STDIC_DEV void gf_row(const GfArgs& a, int d, int c[3], double w[3]) {
  const double x = a.dat[d], y = a.dat[a.nd + d];
  // histc: the cell whose left node is the last node <= x, the last node folded
  int lo = 0, hi = a.nx;
  while (lo < hi) { const int mid = (lo + hi) >> 1; if (a.xn[mid] <= x) lo = mid + 1; else hi = mid; }
  int ix = lo;  // 1-based cell index
  if (ix >= a.nx) ix = a.nx - 1;
  if (ix < 1) ix = 1;
  lo = 0; hi = a.ny;
  while (lo < hi) { const int mid = (lo + hi) >> 1; if (a.yn[mid] <= y) lo = mid + 1; else hi = mid; }
  int iy = lo;
  if (iy >= a.ny) iy = a.ny - 1;
  if (iy < 1) iy = 1;
  double tx = (x - a.xn[ix - 1]) / gf_dx(a, ix - 1);
  double ty = (y - a.yn[iy - 1]) / gf_dy(a, iy - 1);
  tx = fmin(fmax(tx, 0.0), 1.0);
  ty = fmin(fmax(ty, 0.0), 1.0);
  const int n0 = (iy - 1) + a.ny * (ix - 1);
  const int L = tx > ty ? a.ny : 1;
  const double t1 = fmin(tx, ty), t2 = fmax(tx, ty);
  c[0] = n0; c[1] = n0 + a.ny + 1; c[2] = n0 + L;
  w[0] = 1 - t2; w[1] = t1; w[2] = t2 - t1;
}

__global__ void gf_data_kernel(GfArgs a) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= a.nd) return;
  const int ng = a.nx * a.ny;
  int c[3];
  double w[3];
  gf_row(a, d, c, w);
  for (int p = 0; p < 3; ++p) {
    const int jp = c[p] % a.ny, ip = c[p] / a.ny;
    for (int q = 0; q < 3; ++q) {
      const int jq = c[q] % a.ny, iq = c[q] / a.ny;
      atomicAdd(a.K + (size_t)c[p] * 9 + (jq - jp + 1) + 3 * (iq - ip + 1), w[p] * w[q]);
    }
    atomicAdd(a.colA + c[p], fabs(w[p]));
    for (int s = 0; s < a.nz; ++s) atomicAdd(a.rhs + (size_t)s * ng + c[p], w[p] * a.dat[(size_t)(2 + s) * a.nd + d]);
  }
}

// spring weight between node (j, i) and its neighbour (j + dj, i + di), 0 if none
STDIC_DEV double gf_spring(const GfArgs& a, int j, int i, int dj, int di) {
  const int j2 = j + dj, i2 = i + di;
  if (j2 < 0 || j2 >= a.ny || i2 < 0 || i2 >= a.nx || (dj == 0 && di == 0)) return 0.0;
  if (di == 0) return 1.0 / (gf_dy(a, min(j, j2)) / a.yscale);
  if (dj == 0) return 1.0 / (gf_dx(a, min(i, i2)) / a.xscale);
  const double ex = gf_dx(a, min(i, i2)) / a.xscale, ey = gf_dy(a, min(j, j2)) / a.yscale;
  return 1.0 / sqrt(ex * ex + ey * ey);
}

__global__ void gf_norms_kernel(GfArgs a) {
  const int nd = blockIdx.x * blockDim.x + threadIdx.x;
  if (nd >= a.nx * a.ny) return;
  const int j = nd % a.ny, i = nd / a.ny;
  double s = 0;
  for (int di = -1; di <= 1; ++di)
    for (int dj = -1; dj <= 1; ++dj) s += gf_spring(a, j, i, dj, di);
  atomicMax(a.nmax + 1, (unsigned long long)__double_as_longlong(s));
  atomicMax(a.nmax, (unsigned long long)__double_as_longlong(a.colA[nd]));
}

// K += lambda^2 Areg' Areg with lambda = ||A||_1 / ||Areg||_1 (smoothness 1)
__global__ void gf_assemble_kernel(GfArgs a) {
  const int nd = blockIdx.x * blockDim.x + threadIdx.x;
  if (nd >= a.nx * a.ny) return;
  const double NA = __longlong_as_double((long long)a.nmax[0]), NR = __longlong_as_double((long long)a.nmax[1]);
  const double lam = NA / NR;
  const int j = nd % a.ny, i = nd / a.ny;
  double diag = 0;
  for (int di = -1; di <= 1; ++di)
    for (int dj = -1; dj <= 1; ++dj) {
      const double st = gf_spring(a, j, i, dj, di);
      if (st == 0) continue;
      const double s2 = (lam * st) * (lam * st);
      diag += s2;
      a.K[(size_t)nd * 9 + (dj + 1) + 3 * (di + 1)] -= s2;
    }
  a.K[(size_t)nd * 9 + 4] += diag;
}

// Jacobi-PCG on the nz right-hand sides at once, cooperative; each stops at
// |r| <= tol |b|
__global__ void __launch_bounds__(256) gf_cg_kernel(GfArgs a) {
  __shared__ double red[32 * 4];
  const int ng = a.nx * a.ny;
  const int nz = a.nz;
  const int nb = gridDim.x;
  const int tid0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  int* cnt = &a.misc[0];
  int* gen = &a.misc[1];
  double* pz = a.part;               // r.z (3 slots), then |b|^2 (3)
  double* pq = a.part + 6 * 1024;    // p.Ap (3)
  double* pr = a.part + 9 * 1024;    // r.z (3), then |r|^2 (3)
  auto matvec = [&](const double* v, int s, int n) {
    const int j = n % a.ny, i = n / a.ny;
    const double* k9 = a.K + (size_t)n * 9;
    double acc = 0;
    for (int di = -1; di <= 1; ++di) {
      const int i2 = i + di;
      if (i2 < 0 || i2 >= a.nx) continue;
      for (int dj = -1; dj <= 1; ++dj) {
        const int j2 = j + dj;
        if (j2 < 0 || j2 >= a.ny) continue;
        acc += k9[(dj + 1) + 3 * (di + 1)] * v[(size_t)s * ng + j2 + a.ny * i2];
      }
    }
    return acc;
  };
  double v[4] = {0, 0, 0, 0}, w4[4] = {0, 0, 0, 0};
  for (int n = tid0; n < ng; n += stride) {
    const double id = 1.0 / a.K[(size_t)n * 9 + 4];
    for (int s = 0; s < nz; ++s) {
      const size_t k = (size_t)s * ng + n;
      const double b = a.rhs[k];
      a.x[k] = 0;
      a.r[k] = b;
      a.z[k] = b * id;
      a.p[k] = b * id;
      v[s] += b * b * id;
      w4[s] += b * b;
    }
  }
  block_partials(v, nz, pz, red);
  block_partials(w4, nz, pz + 3 * 1024, red);
  if (!grid_barrier(cnt, gen, nb, a.status, a.spin)) return;
  double t0[4], t1[4];
  totals(pz, nz, t0, red);
  totals(pz + 3 * 1024, nz, t1, red);
  double rz[3] = {0, 0, 0}, bn[3] = {0, 0, 0};
  bool conv[3] = {true, true, true};
  for (int s = 0; s < nz; ++s) {
    rz[s] = t0[s];
    bn[s] = sqrt(t1[s]);
    conv[s] = !(bn[s] > 0);
  }
  int it = 0;
  while (!(conv[0] && conv[1] && conv[2]) && it < a.maxit) {
    ++it;
    double q[4] = {0, 0, 0, 0};
    for (int n = tid0; n < ng; n += stride)
      for (int s = 0; s < nz; ++s) {
        const double y = matvec(a.p, s, n);
        a.Ap[(size_t)s * ng + n] = y;
        q[s] += a.p[(size_t)s * ng + n] * y;
      }
    block_partials(q, nz, pq, red);
    if (!grid_barrier(cnt, gen, nb, a.status, a.spin)) return;
    double pAp[4];
    totals(pq, nz, pAp, red);
    double al[3] = {0, 0, 0};
    for (int s = 0; s < nz; ++s) al[s] = conv[s] ? 0.0 : rz[s] / pAp[s];
    double s1[4] = {0, 0, 0, 0}, s2[4] = {0, 0, 0, 0};
    for (int n = tid0; n < ng; n += stride) {
      const double id = 1.0 / a.K[(size_t)n * 9 + 4];
      for (int s = 0; s < nz; ++s) {
        const size_t k = (size_t)s * ng + n;
        a.x[k] += al[s] * a.p[k];
        a.r[k] -= al[s] * a.Ap[k];
        a.z[k] = a.r[k] * id;
        s1[s] += a.r[k] * a.z[k];
        s2[s] += a.r[k] * a.r[k];
      }
    }
    block_partials(s1, nz, pr, red);
    block_partials(s2, nz, pr + 3 * 1024, red);
    if (!grid_barrier(cnt, gen, nb, a.status, a.spin)) return;
    double t2[4], t3[4];
    totals(pr, nz, t2, red);
    totals(pr + 3 * 1024, nz, t3, red);
    double be[3] = {0, 0, 0};
    for (int s = 0; s < nz; ++s) {
      be[s] = conv[s] ? 0.0 : t2[s] / rz[s];
      rz[s] = t2[s];
      if (!conv[s] && sqrt(t3[s]) <= a.tol * bn[s]) conv[s] = true;
    }
    for (int n = tid0; n < ng; n += stride)
      for (int s = 0; s < nz; ++s) {
        const size_t k = (size_t)s * ng + n;
        a.p[k] = a.z[k] + be[s] * a.p[k];
      }
    if (!grid_barrier(cnt, gen, nb, a.status, a.spin)) return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *a.iters = it;
    if (!(conv[0] && conv[1] && conv[2])) atomicCAS(a.status, 0, 1);
  }
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Carver {
  char* base;
  size_t off = 0;
  template <class T>
  T* take(size_t count) {
    T* p = base ? (T*)(base + off) : nullptr;
    off += al256(sizeof(T) * count);
    return p;
  }
};

int ceil_pow2(long long v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

struct GridfitOut {
  std::vector<double> xn, yn;  // the nodes (extended to the data, gridfit.m)
  std::vector<double> z;       // nz x (ny nx), each column-major ny x nx
  int iters = 0;
};

// gridfit(x, y, z, xnodes, ynodes, 'regularizer', 'springs') for nz <= 3 data
// columns sharing x and y (func/gridfit.m with its defaults: triangle
// interpolation, smoothness 1, autoscale): rows with a NaN in any column are
// dropped, the nodes are extended to the data, and the normal equations of
// [A; lambda Areg] z = [data; 0] with lambda = ||A||_1 / ||Areg||_1 are solved
// by the cooperative PCG.  Returns 0, -1 (too few data), -3 (allocation),
// -5 (a barrier wait gave up) or -6 (not converged).
int gridfit_springs(const std::vector<double>& xnodes, const std::vector<double>& ynodes,
                    const std::vector<double>& x, const std::vector<double>& y,
                    const std::vector<std::vector<double>>& zs, const std::function<void*(size_t)>& grow,
                    cudaStream_t s, long long* nl, GridfitOut* out, const char** err) {
  const int nz = (int)zs.size();
  std::vector<double> px, py, pz;
  for (size_t k = 0; k < x.size(); ++k) {
    bool bad = std::isnan(x[k]) || std::isnan(y[k]);
    for (int c = 0; c < nz; ++c) bad = bad || std::isnan(zs[c][k]);
    if (bad) continue;
    px.push_back(x[k]);
    py.push_back(y[k]);
  }
  const int nd = (int)px.size();
  if (nd < 3) {
    *err = "gridfit: insufficient data for surface estimation";
    return -1;
  }
  std::vector<double> hd((size_t)(2 + nz) * nd);
  {
    int q = 0;
    for (size_t k = 0; k < x.size(); ++k) {
      bool bad = std::isnan(x[k]) || std::isnan(y[k]);
      for (int c = 0; c < nz; ++c) bad = bad || std::isnan(zs[c][k]);
      if (bad) continue;
      hd[q] = x[k];
      hd[nd + q] = y[k];
      for (int c = 0; c < nz; ++c) hd[(size_t)(2 + c) * nd + q] = zs[c][k];
      ++q;
    }
  }
  std::vector<double> xn = xnodes, yn = ynodes;
  xn.front() = std::min(xn.front(), *std::min_element(px.begin(), px.end()));
  xn.back() = std::max(xn.back(), *std::max_element(px.begin(), px.end()));
  yn.front() = std::min(yn.front(), *std::min_element(py.begin(), py.end()));
  yn.back() = std::max(yn.back(), *std::max_element(py.begin(), py.end()));
  const int nx = (int)xn.size(), ny = (int)yn.size();
  const long long ng = (long long)nx * ny;
  double xs = 0, ys = 0;
  for (int i = 0; i + 1 < nx; ++i) xs += xn[i + 1] - xn[i];
  for (int j = 0; j + 1 < ny; ++j) ys += yn[j + 1] - yn[j];
  xs /= (nx - 1);
  ys /= (ny - 1);
  Carver cz{nullptr};
  cz.take<double>(nx); cz.take<double>(ny); cz.take<double>(hd.size());
  cz.take<double>(9 * (size_t)ng); cz.take<double>(ng); cz.take<unsigned long long>(2);
  for (int k = 0; k < 6; ++k) cz.take<double>((size_t)nz * ng);
  cz.take<double>(16 * 1024); cz.take<int>(8);
  void* w = grow(cz.off);
  if (!w) {
    *err = "device allocation for gridfit failed";
    return -3;
  }
  Carver c{(char*)w};
  GfArgs ga{};
  ga.nx = nx; ga.ny = ny; ga.nd = nd; ga.nz = nz;
  double* dxn = c.take<double>(nx);
  double* dyn = c.take<double>(ny);
  double* ddat = c.take<double>(hd.size());
  ga.xn = dxn; ga.yn = dyn; ga.dat = ddat;
  ga.xscale = xs; ga.yscale = ys;
  ga.K = c.take<double>(9 * (size_t)ng);
  ga.colA = c.take<double>(ng);
  ga.nmax = c.take<unsigned long long>(2);
  ga.rhs = c.take<double>((size_t)nz * ng);
  ga.x = c.take<double>((size_t)nz * ng);
  ga.r = c.take<double>((size_t)nz * ng);
  ga.z = c.take<double>((size_t)nz * ng);
  ga.p = c.take<double>((size_t)nz * ng);
  ga.Ap = c.take<double>((size_t)nz * ng);
  ga.part = c.take<double>(16 * 1024);
  int* ints = c.take<int>(8);
  ga.misc = ints;
  ga.status = ints + 4;
  ga.iters = ints + 5;
  ga.tol = 1e-12;
  ga.maxit = (int)std::min<long long>(200000, 20 * ng + 1000);
  ga.spin = kGfSpin;
  auto chk = [&](cudaError_t e) {
    if (e != cudaSuccess) *err = cudaGetErrorString(e);
    return e == cudaSuccess;
  };
  if (!chk(cudaMemcpyAsync(dxn, xn.data(), sizeof(double) * nx, cudaMemcpyHostToDevice, s)) ||
      !chk(cudaMemcpyAsync(dyn, yn.data(), sizeof(double) * ny, cudaMemcpyHostToDevice, s)) ||
      !chk(cudaMemcpyAsync(ddat, hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice, s)) ||
      !chk(cudaMemsetAsync(ga.K, 0, sizeof(double) * 9 * ng, s)) ||
      !chk(cudaMemsetAsync(ga.colA, 0, sizeof(double) * ng, s)) ||
      !chk(cudaMemsetAsync(ga.nmax, 0, sizeof(unsigned long long) * 2, s)) ||
      !chk(cudaMemsetAsync(ga.rhs, 0, sizeof(double) * nz * ng, s)) ||
      !chk(cudaMemsetAsync(ints, 0, sizeof(int) * 8, s)))
    return -2;
  gf_data_kernel<<<(nd + 255) / 256, 256, 0, s>>>(ga); ++*nl;
  gf_norms_kernel<<<(int)((ng + 255) / 256), 256, 0, s>>>(ga); ++*nl;
  gf_assemble_kernel<<<(int)((ng + 255) / 256), 256, 0, s>>>(ga); ++*nl;
  if (!chk(cudaGetLastError())) return -2;
  int dev = 0, nsm = 0, per_sm = 0;
  if (!chk(cudaGetDevice(&dev)) || !chk(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) ||
      !chk(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gf_cg_kernel, 256, 0)))
    return -2;
  int nbk = (int)std::min<long long>((long long)nsm * std::max(per_sm, 1), (ng + 255) / 256);
  nbk = std::max(1, std::min(nbk, 1024));
  void* args[] = {&ga};
  if (!chk(cudaLaunchCooperativeKernel((const void*)gf_cg_kernel, dim3(nbk), dim3(256), args, 0, s))) return -2;
  ++*nl;
  int hs[8];
  out->z.assign((size_t)nz * ng, 0.0);
  if (!chk(cudaMemcpyAsync(hs, ints, sizeof(int) * 8, cudaMemcpyDeviceToHost, s)) ||
      !chk(cudaMemcpyAsync(out->z.data(), ga.x, sizeof(double) * nz * ng, cudaMemcpyDeviceToHost, s)) ||
      !chk(cudaStreamSynchronize(s)))
    return -2;
  out->iters = hs[5];
  out->xn = xn;
  out->yn = yn;
  if (hs[4] == 2) {
    *err = "gridfit: a grid-barrier wait of the conjugate-gradient kernel gave up";
    return -5;
  }
  if (hs[4] == 1) {
    *err = "gridfit: the conjugate-gradient solve did not reach its tolerance";
    return -6;
  }
  return 0;
}

#define MG_TRY(expr)                                  \
  do {                                                \
    cudaError_t e_ = (expr);                          \
    if (e_ != cudaSuccess) {                          \
      *err = cudaGetErrorString(e_);                  \
      return -2;                                      \
    }                                                 \
  } while (0)

}  // namespace

size_t mg_fixed_workspace_bytes(int W, int H) {
  const size_t n = (size_t)(W + 1) * (H + 1);
  return al256(n * 8) * 2 + al256(n * 4) + 4096;
}

int integer_search_mg(const double* f, const double* g, int W, int H, const double gridx_in[2],
                      const double gridy_in[2], int winsize, const double step[2], void* fixed_ws,
                      const std::function<void*(size_t)>& grow, cudaStream_t s, long long* launches, MgSearchOut* out,
                      const char** err) {
  long long nl = 0;
  // integral images of g, g^2 and of the non-finite count
  Carver fw{(char*)fixed_ws};
  const size_t nI = (size_t)(W + 1) * (H + 1);
  double* I1 = fw.take<double>(nI);
  double* I2 = fw.take<double>(nI);
  int* In = fw.take<int>(nI);
  MgImg im{f, g, W, H, I1, I2, In};
  ii_rows_kernel<<<H, 256, 0, s>>>(g, W, I1, I2, In); ++nl;
  ii_cols_kernel<<<(W + 1 + 31) / 32, dim3(32, 32), 0, s>>>(W, H, I1, I2, In); ++nl;
  MG_TRY(cudaGetLastError());

  // ROI and border gaps (:5-9)
  const double bg = 1 + std::floor(0.75 * winsize + 0.5);
  double gx[2] = {gridx_in[0], gridx_in[1]}, gy[2] = {gridy_in[0], gridy_in[1]};
  if (gx[0] < bg) gx[0] = bg;
  if (gy[0] < bg) gy[0] = bg;
  if (gx[1] > W - bg) gx[1] = W - bg;
  if (gy[1] > H - bg) gy[1] = H - bg;
  if (!(gx[1] > gx[0]) || !(gy[1] > gy[0]) || gx[0] != std::floor(gx[0]) || gx[1] != std::floor(gx[1]) ||
      gy[0] != std::floor(gy[0]) || gy[1] != std::floor(gy[1])) {
    *err = "the search region is empty after the border gaps, or not whole pixels";
    return -1;
  }
  const int m = (int)(gx[1] - gx[0]) + 1, n = (int)(gy[1] - gy[0]) + 1;
  const long long R = 2ll * m - 1, Cc = 2ll * n - 1;
  const int Fx = ceil_pow2(R), Fy = ceil_pow2(Cc);
  if (Fx > kFftMaxLen || Fy > kFftMaxLen) {
    *err = "the search region exceeds 4096 pixels a side";
    return -1;
  }
  // level 1 (:16-28) on scratch of the first grow
  const int npart1 = 1024;
  size_t need1 = 0;
  {
    Carver cz{nullptr};
    cz.take<double2>((size_t)Fx * Fy);
    cz.take<double2>((size_t)Fx * Fy);
    cz.take<double2>(Fx / 2);
    cz.take<double2>(Fy / 2);
    cz.take<MgBlock>(1);
    cz.take<MgStat>(1);
    cz.take<MgRes>(1);
    cz.take<unsigned long long>(1);
    cz.take<double>(npart1);
    cz.take<long long>(npart1);
    cz.take<int>(npart1);
    need1 = cz.off;
  }
  void* w1 = grow(need1);
  if (!w1) {
    *err = "device allocation for the level-1 transforms failed";
    return -3;
  }
  Carver c1{(char*)w1};
  double2* z = c1.take<double2>((size_t)Fx * Fy);
  double2* zt = c1.take<double2>((size_t)Fx * Fy);
  double2* twx = c1.take<double2>(Fx / 2);
  double2* twy = c1.take<double2>(Fy / 2);
  MgBlock* b1 = c1.take<MgBlock>(1);
  MgStat* st1 = c1.take<MgStat>(1);
  MgRes* r1 = c1.take<MgRes>(1);
  unsigned long long* dm1 = c1.take<unsigned long long>(1);
  double* pv = c1.take<double>(npart1);
  long long* pi = c1.take<long long>(npart1);
  int* pbad = c1.take<int>(npart1);
  MgBlock hb{gx[0], gx[1], gy[0], gy[1], gx[0], gx[1], gy[0], gy[1], 0.0, 0.0};
  MG_TRY(cudaMemcpyAsync(b1, &hb, sizeof(MgBlock), cudaMemcpyHostToDevice, s));
  MG_TRY(cudaMemsetAsync(dm1, 0, sizeof(unsigned long long), s));
  // template statistics of the whole region: 1024 CTAs, two passes
  mg_tsum_kernel<<<npart1, 256, 0, s>>>(im, b1, 1, npart1, 0, st1, pv, pbad); ++nl;
  mg_tstat_kernel<<<1, 32, 0, s>>>(im, b1, 1, 1, npart1, 0, pv, pbad, st1); ++nl;
  mg_tsum_kernel<<<npart1, 256, 0, s>>>(im, b1, 1, npart1, 1, st1, pv, pbad); ++nl;
  mg_tstat_kernel<<<1, 32, 0, s>>>(im, b1, 1, 1, npart1, 1, pv, pbad, st1); ++nl;
  MgStat hst;
  MG_TRY(cudaMemcpyAsync(&hst, st1, sizeof(MgStat), cudaMemcpyDeviceToHost, s));
  MG_TRY(cudaStreamSynchronize(s));
  if (!hst.ok) {
    *err = "normxcorr2 of the whole region fails (constant or non-finite template, or non-finite image)";
    return -1;
  }
  mg_fill_kernel<<<dim3((Fx + 255) / 256, Fy), 256, 0, s>>>(im, b1, st1, z, Fx, Fy); ++nl;
  MG_TRY(launch_fft_twiddles(twx, Fx, s)); ++nl;
  MG_TRY(launch_fft_twiddles(twy, Fy, s)); ++nl;
  MG_TRY(launch_fft_rows(z, Fy, Fx, twx, false, s)); ++nl;
  MG_TRY(launch_transpose_c(z, zt, Fy, Fx, s)); ++nl;
  MG_TRY(launch_fft_rows(zt, Fx, Fy, twy, false, s)); ++nl;
  mg_product_kernel<<<dim3((Fy + 255) / 256, Fx), 256, 0, s>>>(zt, z, Fx, Fy); ++nl;
  MG_TRY(launch_fft_rows(z, Fx, Fy, twy, true, s)); ++nl;
  MG_TRY(launch_transpose_c(z, zt, Fx, Fy, s)); ++nl;
  MG_TRY(launch_fft_rows(zt, Fy, Fx, twx, true, s)); ++nl;
  const double scale = 1.0 / ((double)Fx * (double)Fy);
  {
    const long long lags = R * Cc;
    const int gxb = (int)std::min<long long>(1024, std::max<long long>(1, (lags + 255) / 256));
    mg_denmax_kernel<<<dim3(gxb, 1), 256, 0, s>>>(im, b1, st1, 1, dm1); ++nl;
    mg_l1_max_kernel<<<npart1, 256, 0, s>>>(im, b1, st1, zt, Fx, dm1, scale, pv); ++nl;
    mg_l1_first_kernel<<<npart1, 256, 0, s>>>(im, b1, st1, zt, Fx, dm1, scale, pv, npart1, pi); ++nl;
    mg_l1_peak_kernel<<<1, 32, 0, s>>>(im, b1, st1, zt, Fx, dm1, scale, pv, pi, npart1, r1); ++nl;
  }
  MG_TRY(cudaGetLastError());
  MgRes hr1;
  MG_TRY(cudaMemcpyAsync(&hr1, r1, sizeof(MgRes), cudaMemcpyDeviceToHost, s));
  MG_TRY(cudaStreamSynchronize(s));
  out->level1_u = hr1.u;
  out->level1_v = hr1.v;

  // level-1 window of g (:31-42)
  {
    double xf[2] = {gx[0], gx[1]}, yf[2] = {gy[0], gy[1]}, xg[2], yg[2];
    mg_clamp(xf, yf, xg, yg, hr1.u, hr1.v, W, H, bg, bg);
    hb = MgBlock{xf[0], xf[1], yf[0], yf[1], xg[0], xg[1], yg[0], yg[1], std::ceil(hr1.u), std::ceil(hr1.v)};
  }
  // the level plan (:53-69): split modes from the nominal widths
  std::vector<int> modes;
  std::vector<double> wxs, wys;
  {
    double wx = hb.xf1 - hb.xf0, wy = hb.yf1 - hb.yf0;
    for (int guard = 0; guard < 64 && wx / wy > 0; ++guard) {
      const double ratio = wx / wy;
      const int mode = ratio > 2 ? 0 : (ratio < 0.5 ? 1 : 2);
      if (mode == 0) wx /= 2;
      else if (mode == 1) wy /= 2;
      else { wx /= 2; wy /= 2; }
      modes.push_back(mode);
      wxs.push_back(wx);
      wys.push_back(wy);
      if (wx < winsize && wy < winsize) break;
    }
  }
  if (modes.empty() || !(wxs.back() < winsize && wys.back() < winsize)) {
    *err = "the search region has no multigrid levels (a zero or non-finite width)";
    return -1;
  }
  std::vector<long long> nbs;
  long long nb = 1;
  for (int md : modes) {
    nb *= md == 2 ? 4 : 2;
    nbs.push_back(nb);
  }
  if (nb > 65535) {
    *err = "too many multigrid blocks (more than 65535 at the last level)";
    return -1;
  }
  std::vector<int> ncts;
  for (size_t k = 0; k < modes.size(); ++k) {
    const double px = (wxs[k] + 1) * (wys[k] + 1);
    const long long tiles = (long long)std::ceil((wxs[k] + 1) / kTX) * (long long)std::ceil((wys[k] + 1) / kTY);
    int nct = (int)std::min<long long>(std::max<long long>(1, tiles), std::max<long long>(1, (long long)(px / 1024)));
    nct = std::max(1, std::min(nct, 1024));
    ncts.push_back(nct);
  }
  size_t part_max = 0;
  size_t tsum_max = 1;
  for (size_t k = 0; k < modes.size(); ++k) {
    part_max = std::max(part_max, (size_t)nbs[k] * ncts[k] * kLags);
    tsum_max = std::max(tsum_max, (size_t)nbs[k] * ncts[k]);
  }
  // the levels' scratch (a second grow: level 1's transforms are no longer needed)
  size_t need2 = 0;
  {
    Carver cz{nullptr};
    cz.take<MgBlock>(nb);
    cz.take<MgBlock>(nb);
    cz.take<MgStat>(nb);
    cz.take<MgRes>(nb);
    cz.take<unsigned long long>(nb);
    cz.take<double>(part_max);
    cz.take<double>(5 * (size_t)nb);
    cz.take<double>(tsum_max);
    cz.take<int>(tsum_max);
    need2 = cz.off;
  }
  void* w2 = grow(need2);
  if (!w2) {
    *err = "device allocation for the multigrid levels failed";
    return -3;
  }
  Carver c2{(char*)w2};
  MgBlock* cur = c2.take<MgBlock>(nb);
  MgBlock* nxt = c2.take<MgBlock>(nb);
  MgStat* st = c2.take<MgStat>(nb);
  MgRes* res = c2.take<MgRes>(nb);
  unsigned long long* dmax = c2.take<unsigned long long>(nb);
  double* part = c2.take<double>(part_max);
  double* coll = c2.take<double>(5 * (size_t)nb);
  double* tpart = c2.take<double>(tsum_max);
  int* tbad = c2.take<int>(tsum_max);
  MG_TRY(cudaMemcpyAsync(cur, &hb, sizeof(MgBlock), cudaMemcpyHostToDevice, s));
  long long ncur = 1;
  for (size_t k = 0; k < modes.size(); ++k) {
    const long long nn = nbs[k];
    const int nct = ncts[k];
    mg_split_kernel<<<(int)((ncur + 255) / 256), 256, 0, s>>>(cur, nxt, (int)ncur, modes[k], (double)winsize); ++nl;
    const unsigned nt = (unsigned)(nn * nct);
    const int sb = (int)((nn + 127) / 128);
    mg_tsum_kernel<<<nt, 256, 0, s>>>(im, nxt, 0, nct, 0, st, tpart, tbad); ++nl;
    mg_tstat_kernel<<<sb, 128, 0, s>>>(im, nxt, (int)nn, 0, nct, 0, tpart, tbad, st); ++nl;
    mg_tsum_kernel<<<nt, 256, 0, s>>>(im, nxt, 0, nct, 1, st, tpart, tbad); ++nl;
    mg_tstat_kernel<<<sb, 128, 0, s>>>(im, nxt, (int)nn, 0, nct, 1, tpart, tbad, st); ++nl;
    MG_TRY(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long) * nn, s));
    {
      // lags of a block's full map: about (2 wx + 11)(2 wy + 11); 8 lags per thread
      const double lags = (2 * wxs[k] + 12) * (2 * wys[k] + 12);
      const int gxb = (int)std::max(1.0, std::min(64.0, std::ceil(lags / (256.0 * 8))));
      mg_denmax_kernel<<<dim3(gxb, (unsigned)nn), 256, 0, s>>>(im, nxt, st, 0, dmax); ++nl;
    }
    mg_tiles_kernel<<<(unsigned)(nn * nct), 192, 0, s>>>(im, nxt, st, nct, part); ++nl;
    mg_finish_kernel<<<(unsigned)nn, 192, 0, s>>>(im, nxt, st, nct, part, dmax, res); ++nl;
    MG_TRY(cudaGetLastError());
    if (k + 1 < modes.size()) {
      mg_clamp_kernel<<<(int)((nn + 255) / 256), 256, 0, s>>>(nxt, res, (int)nn, W, H, bg, bg); ++nl;
      std::swap(cur, nxt);
    }
    ncur = nn;
  }
  // final level -> block centres and results on the host (:300-308)
  mg_collect_kernel<<<(int)((nb + 255) / 256), 256, 0, s>>>(nxt, res, (int)nb, coll); ++nl;
  std::vector<double> hc(5 * (size_t)nb);
  MG_TRY(cudaMemcpyAsync(hc.data(), coll, sizeof(double) * hc.size(), cudaMemcpyDeviceToHost, s));
  MG_TRY(cudaStreamSynchronize(s));
  const double* tx = hc.data();
  const double* ty = tx + nb;
  const double* tu = ty + nb;
  const double* tv = tu + nb;
  const double* tp = tv + nb;
  out->blocks.assign(hc.begin(), hc.end());
  out->nblocks = nb;

  // the node grid (:310-328)
  auto argmin = [&](const double* a, bool mx) {
    long long b = 0;
    for (long long k = 1; k < nb; ++k)
      if (mx ? a[k] > a[b] : a[k] < a[b]) b = k;
    return b;
  };
  const long long ix1 = argmin(tx, false), ix2 = argmin(tx, true), iy1 = argmin(ty, false), iy2 = argmin(ty, true);
  const double bx1 = std::ceil(1 + 1.25 * winsize + tu[ix1]), bx2 = std::ceil(1 + 1.25 * winsize + tu[ix2]);
  const double by1 = std::ceil(1 + 1.25 * winsize + tv[iy1]), by2 = std::ceil(1 + 1.25 * winsize + tv[iy2]);
  double gxx[2] = {gx[0], gx[1]}, gyy[2] = {gy[0], gy[1]};
  if (gxx[0] < bx1) gxx[0] = bx1;
  if (gyy[0] < by1) gyy[0] = by1;
  if (gxx[1] > W - bx2 + 1) gxx[1] = W - bx2 + 1;
  if (gyy[1] > H - by2 + 1) gyy[1] = H - by2 + 1;
  std::vector<double> xl, yl;
  for (double v = gxx[0]; v <= gxx[1] + 1e-9 * std::fabs(step[0]); v += step[0]) xl.push_back(v);
  for (double v = gyy[0]; v <= gyy[1] + 1e-9 * std::fabs(step[1]); v += step[1]) yl.push_back(v);
  if (xl.size() < 2 || yl.size() < 2) {
    *err = "the node grid after the border gaps has fewer than 2 x 2 nodes";
    return -1;
  }
  const double xmin = xl.front(), xmax = xl.back(), ymin = yl.front(), ymax = yl.back();
  std::vector<double> dx_, dy_, du, dv, dp;
  for (long long k = 0; k < nb; ++k) {
    if (!(tx[k] > xmin && tx[k] < xmax && ty[k] > ymin && ty[k] < ymax)) continue;
    dx_.push_back(tx[k]); dy_.push_back(ty[k]); du.push_back(tu[k]); dv.push_back(tv[k]); dp.push_back(tp[k]);
  }
  // gridfit (:329-336): u and v from the blocks with a finite displacement,
  // cc.max from all selected blocks (gridfit drops the NaN rows of each call;
  // a failed block has NaN u, v but cc.max 0)
  std::vector<double> xu, yu, uu, vu;
  for (size_t k = 0; k < dx_.size(); ++k)
    if (!std::isnan(du[k]) && !std::isnan(dv[k])) {
      xu.push_back(dx_[k]); yu.push_back(dy_[k]); uu.push_back(du[k]); vu.push_back(dv[k]);
    }
  const bool same = xu.size() == dx_.size();
  GridfitOut g1, g2;
  int rc = 0;
  if (same) {
    rc = gridfit_springs(xl, yl, dx_, dy_, {du, dv, dp}, grow, s, &nl, &g1, err);
  } else {
    rc = gridfit_springs(xl, yl, xu, yu, {uu, vu}, grow, s, &nl, &g1, err);
    if (rc == 0) rc = gridfit_springs(xl, yl, dx_, dy_, {dp}, grow, s, &nl, &g2, err);
  }
  if (launches) *launches += nl;
  if (rc) return rc;
  out->nx = (int)g1.xn.size();
  out->ny = (int)g1.yn.size();
  out->xnodes = g1.xn;
  out->ynodes = g1.yn;
  const size_t ng = (size_t)out->nx * out->ny;
  out->x3.assign(3 * ng, 0.0);
  std::copy(g1.z.begin(), g1.z.begin() + 2 * ng, out->x3.begin());
  if (same) std::copy(g1.z.begin() + 2 * ng, g1.z.begin() + 3 * ng, out->x3.begin() + 2 * ng);
  else std::copy(g2.z.begin(), g2.z.begin() + ng, out->x3.begin() + 2 * ng);
  out->cg_iters = std::max(g1.iters, same ? 0 : g2.iters);
  return 0;
}

}  // namespace stdic
