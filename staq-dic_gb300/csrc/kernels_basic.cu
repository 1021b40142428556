// Gather/stencil kernels of the STAQ-DIC hot path and the small helpers the
// solvers share.
//   interp_kernel      ba_interp2.cpp:184-234 (bit-identical, see device_common.cuh)
//   gradient_kernel    func/funImgGradient.m:53-78
//   intsearch_kernel   func/funIntegerSearch.m:110-170 + func/findpeak.m:27-68 with
//                      normxcorr2 restated from its published definition
//   badpoints_kernel   LocalICGNQuadtree.m:153-177 / Subpb1Quadtree.m:173-191
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <mutex>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "device_common.cuh"
#include "kernels.h"

namespace stdic {

// ---------------------------------------------------------------------------
// ba_interp2: one thread per output sample, P layers.
// ---------------------------------------------------------------------------
template <class REAL>
__global__ void interp_kernel(const REAL* __restrict__ F, long long M, long long N, long long P,
                              const REAL* __restrict__ X, const REAL* __restrict__ Y, long long n,
                              REAL* __restrict__ out) {
  const long long LO = M * N;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const REAL x = X[k], y = Y[k];
    for (long long j = 0; j < P; ++j) {
      if constexpr (sizeof(REAL) == 8)
        out[k + j * n] = ba_cubic_exact((const double*)F + j * LO, M, N, x, y);
      else
        out[k + j * n] = ba_cubic_exact_f32((const float*)F + j * LO, M, N, x, y);
    }
  }
}

cudaError_t launch_interp(const void* F, long long M, long long N, long long P, const void* X,
                          const void* Y, long long n, void* out, int dtype, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int threads = 256;
  long long blocks = (n + threads - 1) / threads;
  const long long cap = 32ll * current_sm_count();
  if (blocks > cap) blocks = cap;
  if (dtype == 0)
    interp_kernel<double><<<(int)blocks, threads, 0, s>>>((const double*)F, M, N, P,
                                                          (const double*)X, (const double*)Y, n,
                                                          (double*)out);
  else
    interp_kernel<float><<<(int)blocks, threads, 0, s>>>((const float*)F, M, N, P, (const float*)X,
                                                         (const float*)Y, n, (float*)out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// funImgGradient: 7-tap correlation [-1/60 3/20 -3/4 0 3/4 -3/20 1/60] along x
// and y, crop 3 on each side, times the mask.  A 32 x 8 output tile with its
// 3-pixel halo is staged in shared memory by coalesced row loads; the sums are
// rounded in the order of a left-to-right loop over the taps.
// ---------------------------------------------------------------------------
template <class REAL>
__global__ void __launch_bounds__(256) gradient_kernel(const REAL* __restrict__ img,
                                                       const uint8_t* __restrict__ mask, int W,
                                                       int H, REAL* __restrict__ dfdx,
                                                       REAL* __restrict__ dfdy) {
  constexpr int TX = 32, TY = 8, R = 3;
  __shared__ REAL t[TY + 2 * R][TX + 2 * R + 1];
  const int Wo = W - 6, Ho = H - 6;
  const int bx = blockIdx.x * TX, by = blockIdx.y * TY;  // output tile origin
  // output (i, j) sits on image pixel (i + 3, j + 3); tile covers image
  // x in [bx, bx + TX + 6), y in [by, by + TY + 6)
  for (int q = threadIdx.x; q < (TY + 2 * R) * (TX + 2 * R); q += blockDim.x) {
    const int ly = q / (TX + 2 * R), lx = q % (TX + 2 * R);
    const int gx = bx + lx, gy = by + ly;
    t[ly][lx] = (gx < W && gy < H) ? img[(long long)gy * W + gx] : REAL(0);
  }
  __syncthreads();
  const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
  const int i = bx + lx, j = by + ly;
  if (i >= Wo || j >= Ho) return;
  const REAL h[7] = {REAL(-1.0 / 60), REAL(3.0 / 20), REAL(-3.0 / 4), REAL(0.0),
                     REAL(3.0 / 4), REAL(-3.0 / 20), REAL(1.0 / 60)};
  REAL sx = 0, sy = 0;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    if constexpr (sizeof(REAL) == 8) {
      sx = da(sx, dm(h[k], t[ly + R][lx + k]));
      sy = da(sy, dm(h[k], t[ly + k][lx + R]));
    } else {
      sx = __fadd_rn(sx, __fmul_rn(h[k], t[ly + R][lx + k]));
      sy = __fadd_rn(sy, __fmul_rn(h[k], t[ly + k][lx + R]));
    }
  }
  const REAL m = (REAL)mask[(long long)(j + 3) * W + (i + 3)];
  dfdx[(long long)j * Wo + i] = sx * m;
  dfdy[(long long)j * Wo + i] = sy * m;
}

// The same stencil with the input tile (32 x 8 outputs plus the 3-pixel halo,
// 40 x 14 elements) brought into shared memory by one TMA 2-D tile copy
// completing on an mbarrier.  The copy starts at the tile origin, whose x is a
// multiple of 32 elements (TMA's 16-byte rule); elements beyond the image are
// filled with zeros by the copy.  The wait is bounded: after 2^24 polls the
// CTA sets *err, polls once more for a bounded interval so that it does not
// exit with the copy in flight, and leaves its outputs unwritten.
template <class REAL>
__global__ void __launch_bounds__(256) gradient_tma_kernel(const __grid_constant__ CUtensorMap tmap,
                                                           const uint8_t* __restrict__ mask, int W,
                                                           int H, REAL* __restrict__ dfdx,
                                                           REAL* __restrict__ dfdy, int* err) {
  constexpr int TX = 32, TY = 8, R = 3, BX = 40, BY = TY + 2 * R;
  __shared__ __align__(128) REAL t[BY][BX];
  __shared__ __align__(8) uint64_t bar;
  const int Wo = W - 6, Ho = H - 6;
  const int bx = blockIdx.x * TX, by = blockIdx.y * TY;
  const unsigned sbar = (unsigned)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned bytes = (unsigned)(BX * BY * sizeof(REAL));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sbar), "r"(bytes) : "memory");
    const unsigned dst = (unsigned)__cvta_generic_to_shared(&t[0][0]);
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<unsigned long long>(&tmap)), "r"(bx), "r"(by), "r"(sbar)
        : "memory");
  }
  auto wait = [&](int polls) {
    bool d = false;
    for (int it = 0; it < polls && !d; ++it) {
      unsigned done;
      asm volatile(
          "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
          : "=r"(done) : "r"(sbar), "r"(0u) : "memory");
      d = done != 0;
    }
    return d;
  };
  if (!wait(1 << 24)) {
    // Last resort: the copy has not landed after 2^24 polls.  The error is
    // recorded, and the CTA keeps polling for a second bounded interval so
    // that it does not leave while the copy may still be writing its shared
    // memory; its outputs stay unwritten either way.
    if (threadIdx.x == 0 && err) atomicExch(err, 1);
    wait(1 << 24);
    return;
  }
  const int lx = threadIdx.x % TX, ly = threadIdx.x / TX;
  const int i = bx + lx, j = by + ly;
  if (i >= Wo || j >= Ho) return;
  const REAL h[7] = {REAL(-1.0 / 60), REAL(3.0 / 20), REAL(-3.0 / 4), REAL(0.0),
                     REAL(3.0 / 4), REAL(-3.0 / 20), REAL(1.0 / 60)};
  REAL sx = 0, sy = 0;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    if constexpr (sizeof(REAL) == 8) {
      sx = da(sx, dm(h[k], t[ly + R][lx + k]));
      sy = da(sy, dm(h[k], t[ly + k][lx + R]));
    } else {
      sx = __fadd_rn(sx, __fmul_rn(h[k], t[ly + R][lx + k]));
      sy = __fadd_rn(sy, __fmul_rn(h[k], t[ly + k][lx + R]));
    }
  }
  const REAL m = (REAL)mask[(long long)(j + 3) * W + (i + 3)];
  dfdx[(long long)j * Wo + i] = sx * m;
  dfdy[(long long)j * Wo + i] = sy * m;
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    else
      cudaGetLastError();
  });
  return fn;
}

// 2-D tensor map of a W x H image (x = dim 1 contiguous) with a 40 x 14 box;
// false when TMA cannot describe it (pitch or base not 16-byte aligned).
bool image_tensor_map(const void* img, int W, int H, int dtype, CUtensorMap* m) {
  const size_t es = dtype == 0 ? 8 : 4;
  if (((uintptr_t)img & 15) != 0 || ((size_t)W * es) % 16 != 0) return false;
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
  const cuuint64_t strides[1] = {(cuuint64_t)W * es};
  const cuuint32_t box[2] = {40, 14};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, dtype == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
             const_cast<void*>(img), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

bool encode_image_map_f32(const void* base, long long W, long long rows, int box, CUtensorMap* m) {
  if (((uintptr_t)base & 15) != 0 || (W * 4) % 16 != 0 || box < 4 || box > 256 || (box * 4) % 16 != 0) return false;
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)W * 4};
  const cuuint32_t bx[2] = {(cuuint32_t)box, (cuuint32_t)box};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, bx, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t launch_gradient(const void* img, const uint8_t* mask, int W, int H, void* dfdx,
                            void* dfdy, int dtype, cudaStream_t s, int* err) {
  const int Wo = W - 6, Ho = H - 6;
  if (Wo <= 0 || Ho <= 0) return cudaErrorInvalidValue;
  dim3 grid((Wo + 31) / 32, (Ho + 7) / 8);
  CUtensorMap tm;
  if (image_tensor_map(img, W, H, dtype, &tm)) {
    if (dtype == 0)
      gradient_tma_kernel<double><<<grid, 256, 0, s>>>(tm, mask, W, H, (double*)dfdx, (double*)dfdy, err);
    else
      gradient_tma_kernel<float><<<grid, 256, 0, s>>>(tm, mask, W, H, (float*)dfdx, (float*)dfdy, err);
    return cudaGetLastError();
  }
  if (dtype == 0)
    gradient_kernel<double><<<grid, 256, 0, s>>>((const double*)img, mask, W, H, (double*)dfdx,
                                                 (double*)dfdy);
  else
    gradient_kernel<float><<<grid, 256, 0, s>>>((const float*)img, mask, W, H, (float*)dfdx,
                                                (float*)dfdy);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Integer search: one CTA per grid point.  The template C (m x n) and search
// window D (am x an) are staged in shared memory; each thread owns lags of the
// cropped (2S+3)^2 normalised cross-correlation map.  normxcorr2's numerics:
//   num = sum(T.A) - sum(A) sum(T)/mn,  den = sqrt(mn-1) std(T) sqrt(max(sum(A^2)
//   - sum(A)^2/mn, 0)) over the zero-padded window, C = num/den where
//   den > sqrt(eps(max den)), and C = 0 where |C| - 1 > sqrt(eps(1)).
// ---------------------------------------------------------------------------
STDIC_DEV double eps_of(double x) {
  x = fabs(x);
  if (!(x > 0)) return 4.9406564584124654e-324;
  int e;
  frexp(x, &e);
  const int p = e - 53;
  return p < -1074 ? 4.9406564584124654e-324 : ldexp(1.0, p);
}

__global__ void __launch_bounds__(256) intsearch_kernel(const double* __restrict__ f,
                                                        const double* __restrict__ g, int W, int Sx,
                                                        int Sy, double gx0, double gy0, int nx,
                                                        int ny, int wsx, int wsy, int stepx,
                                                        int stepy, double* x, double* y, double* u,
                                                        double* v, double* cc, int32_t* peak) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ double red[32 * 2];
  __shared__ int best_idx;
  const int t = blockIdx.x;
  const int ix = t % nx, iy = t / nx;
  const long long ii = (long long)gx0 + (long long)ix * stepx;
  const long long jj = (long long)gy0 + (long long)iy * stepy;
  const int m = wsx + 1, n = wsy + 1, am = wsx + 1 + 2 * Sx, an = wsy + 1 + 2 * Sy;
  const int nr = 2 * Sx + 3, nc = 2 * Sy + 3, nl = nr * nc;
  const double mn = (double)m * (double)n;
  double* T = (double*)dsm;
  double* A = T + m * n;
  double* num = A + am * an;
  double* den = num + nl;
  const long long o = iy + (long long)ix * ny;
  int bad = 0;
  for (int q = threadIdx.x; q < m * n; q += blockDim.x) {
    const int a = q % m, b = q / m;
    const double val = f[(jj - 1 + b) * W + (ii - 1 + a)];
    T[q] = val;
    if (!isfinite(val)) bad = 1;
  }
  for (int q = threadIdx.x; q < am * an; q += blockDim.x) {
    const int p = q % am, r = q / am;
    const double val = g[(jj - 1 - Sy + r) * W + (ii - 1 - Sx + p)];
    A[q] = val;
    if (!isfinite(val)) bad = 1;
  }
  bad = __syncthreads_or(bad);
  double s[1] = {0};
  for (int q = threadIdx.x; q < m * n; q += blockDim.x) s[0] += T[q];
  block_sum<1>(s, red);
  const double sumT = s[0];
  const double meanT = sumT / mn;
  double q2[1] = {0};
  for (int q = threadIdx.x; q < m * n; q += blockDim.x) {
    const double d = T[q] - meanT;
    q2[0] += d * d;
  }
  block_sum<1>(q2, red);
  const double stdT = sqrt(q2[0] / (mn - 1));
  if (bad || !(stdT != 0)) {
    if (threadIdx.x == 0) {
      u[o] = v[o] = cc[o] = nan("");
      if (peak) { peak[o] = 0; peak[(long long)nx * ny + o] = 0; }
      x[o] = (double)(ii + ii + wsx) / 2;
      y[o] = (double)(jj + jj + wsy) / 2;
    }
    return;
  }
  const double denomT = sqrt(mn - 1) * stdT;
  double dmax = 0;
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    const int dp = k % nr - 1, dq = k / nr - 1;
    const int a0 = dp < 0 ? -dp : 0, a1 = (am - dp) < m ? (am - dp) : m;
    const int b0 = dq < 0 ? -dq : 0, b1 = (an - dq) < n ? (an - dq) : n;
    double xc = 0, sA = 0, sA2 = 0;
    for (int b = b0; b < b1; ++b) {
      const double* Tr = T + b * m;
      const double* Ar = A + (b + dq) * am + dp;
      for (int a = a0; a < a1; ++a) {
        const double av = Ar[a];
        xc = fma(Tr[a], av, xc);
        sA += av;
        sA2 = fma(av, av, sA2);
      }
    }
    const double nm = xc - sA * sumT / mn;
    const double dl = sA2 - (sA * sA) / mn;
    const double dA = sqrt(dl > 0 ? dl : 0.0);
    num[k] = nm;
    den[k] = denomT * dA;
    dmax = fmax(dmax, fabs(den[k]));
  }
  // block max of |den|
  for (int off = 16; off > 0; off >>= 1) dmax = fmax(dmax, __shfl_down_sync(0xffffffffu, dmax, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dmax;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t2 = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) t2 = fmax(t2, __shfl_down_sync(0xffffffffu, t2, off));
    if (threadIdx.x == 0) red[0] = t2;
  }
  __syncthreads();
  const double tolc = sqrt(eps_of(red[0]));
  const double clip = sqrt(eps_of(1.0));
  __syncthreads();
  // C into num[], then first (column-major) argmax
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    double cv = den[k] > tolc ? num[k] / den[k] : 0.0;
    if ((fabs(cv) - 1) > clip) cv = 0;
    num[k] = cv;
  }
  __syncthreads();
  // findpeak's first maximum, with lags tied up to rounding taken as equal
  const int first = cta_first_near_max(num, nl);
  if (threadIdx.x == 0) best_idx = first;
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double* C = num;
  const int imax = best_idx;
  const double cmax = C[imax];
  const int yp = imax % nr + 1, xp = imax / nr + 1;
  double ypeak = yp, xpeak = xp, maxf = cmax;
  if (!(xp == 1 || xp == nc || yp == 1 || yp == nr)) {
    double v9[9];
    for (int dc = -1; dc <= 1; ++dc)
      for (int dr = -1; dr <= 1; ++dr) v9[(dr + 1) + 3 * (dc + 1)] = C[(yp - 1 + dr) + (xp - 1 + dc) * nr];
    double xo, yo, mf;
    if (findpeak_fit3(v9, &xo, &yo, &mf)) {
      xpeak += xo;
      ypeak += yo;
      maxf = mf;
    }
  }
  u[o] = ypeak - ceil(nr / 2.0);
  v[o] = xpeak - ceil(nc / 2.0);
  cc[o] = maxf;
  if (peak) { peak[o] = yp; peak[(long long)nx * ny + o] = xp; }
  x[o] = (double)(ii + ii + wsx) / 2;
  y[o] = (double)(jj + jj + wsy) / 2;
}

cudaError_t launch_intsearch(const double* f, const double* g, int W, int H, int Sx, int Sy,
                             double gx0, double gy0, int nx, int ny, int wsx, int wsy, int stepx,
                             int stepy, double* x, double* y, double* u, double* v, double* cc,
                             int32_t* peak, cudaStream_t s) {
  (void)H;
  if (nx <= 0 || ny <= 0) return cudaSuccess;
  const size_t m = wsx + 1, n = wsy + 1, am = wsx + 1 + 2 * Sx, an = wsy + 1 + 2 * Sy;
  const size_t nl = (size_t)(2 * Sx + 3) * (2 * Sy + 3);
  const size_t smem = sizeof(double) * (m * n + am * an + 2 * nl);
  if (smem > 200 * 1024) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(intsearch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  intsearch_kernel<<<nx * ny, 256, smem, s>>>(f, g, W, Sx, Sy, gx0, gy0, nx, ny, wsx, wsy, stepx,
                                              stepy, x, y, u, v, cc, peak);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Quality factors of the integer search (funIntegerSearch.m:129-131, 211-264):
// for each grid point the FULL normxcorr2 map (every lag with any overlap,
// (m + am - 1) x (n + an - 1)), then
//   cc_min = cc - min(cc), peak = max(cc_min),
//   PCE = peak^2 / mean(cc_min^2),
//   PPE = 1 / entropy of the 30-bin histogram of cc_min (p log(1/p) summed
//         over the non-empty bins),
// and [Inf Inf] where normxcorr2 throws (constant or non-finite template or
// window).  The histogram takes 30 bins of uniform width over [0, peak], the
// last one closed, which is the documented behaviour of histcounts(X, 30);
// MATLAB's own placement of those edges is internal to it.  One CTA per grid
// point; the map is written to scratch (R x C doubles per point) between the
// two passes.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) intsearch_qfactor_kernel(
    const double* __restrict__ f, const double* __restrict__ g, int W, int Sx, int Sy, double gx0, double gy0,
    int nx, int ny, int wsx, int wsy, int stepx, int stepy, double* __restrict__ maps, double* __restrict__ qraw) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ double red[32 * 4];
  __shared__ int hist[30];
  const int t = blockIdx.x;
  const int ix = t % nx, iy = t / nx;
  const long long ii = (long long)gx0 + (long long)ix * stepx;
  const long long jj = (long long)gy0 + (long long)iy * stepy;
  const int m = wsx + 1, n = wsy + 1, am = wsx + 1 + 2 * Sx, an = wsy + 1 + 2 * Sy;
  const int R = m + am - 1, Cn = n + an - 1, nl = R * Cn;
  const double mn = (double)m * (double)n;
  double* T = (double*)dsm;
  double* A = T + m * n;
  // the point's map, column-major R x Cn (the cc of the full lag range),
  // with room for the numerators after it
  double* map = maps + (long long)t * 2 * nl;
  // row of cc.qfactors: the reference's point sequence, x fastest
  // (PtPosSeq from ndgrid(XList, YList), funIntegerSearch.m:90-95)
  const long long o = ix + (long long)iy * nx;
  const long long npt = (long long)nx * ny;
  int bad = 0;
  for (int q = threadIdx.x; q < m * n; q += blockDim.x) {
    const int a = q % m, b = q / m;
    const double val = f[(jj - 1 + b) * W + (ii - 1 + a)];
    T[q] = val;
    if (!isfinite(val)) bad = 1;
  }
  for (int q = threadIdx.x; q < am * an; q += blockDim.x) {
    const int pp = q % am, r = q / am;
    const double val = g[(jj - 1 - Sy + r) * W + (ii - 1 - Sx + pp)];
    A[q] = val;
    if (!isfinite(val)) bad = 1;
  }
  bad = __syncthreads_or(bad);
  double s[1] = {0};
  for (int q = threadIdx.x; q < m * n; q += blockDim.x) s[0] += T[q];
  block_sum<1>(s, red);
  const double sumT = s[0];
  const double meanT = sumT / mn;
  double q2[1] = {0};
  for (int q = threadIdx.x; q < m * n; q += blockDim.x) {
    const double d = T[q] - meanT;
    q2[0] += d * d;
  }
  block_sum<1>(q2, red);
  const double stdT = sqrt(q2[0] / (mn - 1));
  if (bad || !(stdT != 0)) {
    if (threadIdx.x == 0) {
      qraw[o] = INFINITY;
      qraw[npt + o] = INFINITY;
    }
    return;
  }
  const double denomT = sqrt(mn - 1) * stdT;
  // pass 1: numerator and denominator of every lag; lag (dr, dc) puts the
  // template's first element on A(dr, dc) (0-based, may be negative)
  double dmax = 0;
  double* den = map;  // the denominators first, then the values in place
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    const int dr = k % R - (m - 1), dc = k / R - (n - 1);
    const int a0 = dr < 0 ? -dr : 0, a1 = (am - dr) < m ? (am - dr) : m;
    const int b0 = dc < 0 ? -dc : 0, b1 = (an - dc) < n ? (an - dc) : n;
    double xc = 0, sA = 0, sA2 = 0;
    for (int b = b0; b < b1; ++b) {
      const double* Tr = T + b * m;
      const double* Ar = A + (b + dc) * am + dr;
      for (int a = a0; a < a1; ++a) {
        const double av = Ar[a];
        xc = fma(Tr[a], av, xc);
        sA += av;
        sA2 = fma(av, av, sA2);
      }
    }
    const double nm = xc - sA * sumT / mn;
    const double dl = sA2 - (sA * sA) / mn;
    const double dv = denomT * sqrt(dl > 0 ? dl : 0.0);
    // keep the numerator in the upper half of the slot pair: den[k], then the
    // numerator after all denominators
    den[k] = dv;
    map[nl + k] = nm;
    dmax = fmax(dmax, fabs(dv));
  }
  for (int off = 16; off > 0; off >>= 1) dmax = fmax(dmax, __shfl_down_sync(0xffffffffu, dmax, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dmax;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t2 = threadIdx.x < (blockDim.x + 31) / 32 ? red[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) t2 = fmax(t2, __shfl_down_sync(0xffffffffu, t2, off));
    if (threadIdx.x == 0) red[0] = t2;
  }
  __syncthreads();
  const double tolc = sqrt(eps_of(red[0]));
  const double clip = sqrt(eps_of(1.0));
  __syncthreads();
  // pass 2: the values, their min and max
  double vmin = INFINITY, vmax = -INFINITY;
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    const double dv = den[k];
    double cv = dv > tolc ? map[nl + k] / dv : 0.0;
    if ((fabs(cv) - 1) > clip) cv = 0;
    map[k] = cv;
    vmin = fmin(vmin, cv);
    vmax = fmax(vmax, cv);
  }
  for (int off = 16; off > 0; off >>= 1) {
    vmin = fmin(vmin, __shfl_down_sync(0xffffffffu, vmin, off));
    vmax = fmax(vmax, __shfl_down_sync(0xffffffffu, vmax, off));
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = vmin; red[32 + (threadIdx.x >> 5)] = vmax; }
  if (threadIdx.x < 30) hist[threadIdx.x] = 0;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = (blockDim.x + 31) / 32;
    double a = threadIdx.x < nw ? red[threadIdx.x] : INFINITY;
    double b = threadIdx.x < nw ? red[32 + threadIdx.x] : -INFINITY;
    for (int off = 16; off > 0; off >>= 1) {
      a = fmin(a, __shfl_down_sync(0xffffffffu, a, off));
      b = fmax(b, __shfl_down_sync(0xffffffffu, b, off));
    }
    if (threadIdx.x == 0) { red[64] = a; red[65] = b; }
  }
  __syncthreads();
  const double cmin = red[64];
  const double peak = red[65] - cmin;
  const double bw = peak / 30.0;
  // pass 3: sum of cc_min^2 and the histogram
  double e2[1] = {0};
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    const double x = map[k] - cmin;
    e2[0] = fma(x, x, e2[0]);
    int bin = 0;
    if (peak > 0) {
      bin = (int)floor(x / bw);
      bin = bin < 0 ? 0 : (bin > 29 ? 29 : bin);
      // edges k * bw (k < 30) and peak: move across an edge the division rounded past
      if (bin > 0 && x < bin * bw) --bin;
      if (bin < 29 && x >= (bin + 1) * bw) ++bin;
    }
    atomicAdd(&hist[bin], 1);
  }
  block_sum<1>(e2, red);
  if (threadIdx.x == 0) {
    const double pce = peak * peak / (e2[0] / (double)nl);
    double ent = 0;
    for (int b = 0; b < 30; ++b) {
      const double pb = (double)hist[b] / (double)nl;
      if (pb != 0) ent += pb * log(1.0 / pb);
    }
    qraw[o] = pce;
    qraw[npt + o] = 1.0 / ent;
  }
}

// cc.qfactors(:,k) = (q - min q) / max(q - min q) over all grid points, with
// MATLAB's min and max (NaN ignored); one CTA.
__global__ void __launch_bounds__(256) qfactor_normalise_kernel(const double* __restrict__ qraw, long long npt,
                                                                 double* __restrict__ qf) {
  __shared__ double red[32];
  for (int k = 0; k < 2; ++k) {
    const double* q = qraw + k * npt;
    double mn = INFINITY;
    for (long long i = threadIdx.x; i < npt; i += blockDim.x)
      if (!isnan(q[i])) mn = fmin(mn, q[i]);
    for (int off = 16; off > 0; off >>= 1) mn = fmin(mn, __shfl_down_sync(0xffffffffu, mn, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mn;
    __syncthreads();
    if (threadIdx.x == 0) {
      double v = INFINITY;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmin(v, red[w]);
      red[0] = v;
    }
    __syncthreads();
    const double qmin = red[0];
    __syncthreads();
    double mx = -INFINITY;
    for (long long i = threadIdx.x; i < npt; i += blockDim.x) {
      const double d = q[i] - qmin;
      if (!isnan(d)) mx = fmax(mx, d);
    }
    for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      double v = -INFINITY;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmax(v, red[w]);
      red[0] = v;
    }
    __syncthreads();
    const double dmax = red[0];
    __syncthreads();
    for (long long i = threadIdx.x; i < npt; i += blockDim.x) qf[k * npt + i] = (q[i] - qmin) / dmax;
  }
}

size_t intsearch_qfactor_scratch_bytes(int nx, int ny, int Sx, int Sy, int wsx, int wsy) {
  const size_t R = (size_t)2 * wsx + 2 * Sx + 1, C = (size_t)2 * wsy + 2 * Sy + 1;
  return ((size_t)nx * ny * (2 * R * C + 2)) * sizeof(double);
}

cudaError_t launch_intsearch_qfactors(const double* f, const double* g, int W, int Sx, int Sy, double gx0,
                                      double gy0, int nx, int ny, int wsx, int wsy, int stepx, int stepy,
                                      double* scratch, double* qf, cudaStream_t s) {
  if (nx <= 0 || ny <= 0) return cudaSuccess;
  const size_t m = wsx + 1, n = wsy + 1, am = wsx + 1 + 2 * Sx, an = wsy + 1 + 2 * Sy;
  const size_t smem = sizeof(double) * (m * n + am * an);
  if (smem > 200 * 1024) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(intsearch_qfactor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  const long long npt = (long long)nx * ny;
  const size_t nl = (m + am - 1) * (n + an - 1);
  double* qraw = scratch;
  double* maps = scratch + 2 * npt;
  intsearch_qfactor_kernel<<<(int)npt, 256, smem, s>>>(f, g, W, Sx, Sy, gx0, gy0, nx, ny, (int)wsx, (int)wsy,
                                                       stepx, stepy, maps, qraw);
  (void)nl;
  qfactor_normalise_kernel<<<1, 256, 0, s>>>(qraw, npt, qf);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Bad-subset filter after the per-node loop.  LocalICGNQuadtree: bad =
// conv<0 | conv>99, then also conv > max(mean+std, 6) of the good codes;
// Subpb1Quadtree: max(mean+0.25 std, 10).  U (and F for the first pass) become
// NaN at bad nodes; badnum is #bad - #(conv==102).  A grid adds the
// statistics of the good codes exactly in 64-bit integers; a second grid
// derives the threshold in every block (the codes are integers, so
// c > thr <=> c > floor(thr)) and writes the NaNs.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) badpoints_stats_kernel(const int32_t* __restrict__ conv, int N,
                                                              unsigned long long* sums) {
  __shared__ long long red[5][8];
  long long v[5] = {0, 0, 0, 0, 0};  // sum c, sum c^2, #good, #bad, #(c == 102)
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    const long long c = conv[k];
    const bool bad = c < 0 || c > kMaxIter - 1;
    if (!bad) { v[0] += c; v[1] += c * c; ++v[2]; }
    v[3] += bad;
    v[4] += (c == kMaxIter + 2);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 5; ++q) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if (lane == 0) red[q][warp] = v[q];
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
    if (t) atomicAdd(&sums[threadIdx.x], (unsigned long long)t);
  }
}

__global__ void __launch_bounds__(256) badpoints_apply_kernel(const int32_t* __restrict__ conv, int N, double* U,
                                                              double* F, int two_dof,
                                                              const unsigned long long* __restrict__ sums,
                                                              int* badnum) {
  __shared__ int cmax_s;
  if (threadIdx.x == 0) {
    const long long t0 = (long long)sums[0], t1 = (long long)sums[1], t2 = (long long)sums[2];
    const double n = (double)t2;
    const double mean = (double)t0 / n;
    // sum (c - mean)^2 = (n sum c^2 - (sum c)^2) / n, the numerator exact in integers
    const long long num = t2 * t1 - t0 * t0;
    const double sd = t2 > 1 ? sqrt((double)num / n / (n - 1.0)) : (t2 == 1 ? 0.0 : nan(""));
    const double cand = two_dof ? mean + 0.25 * sd : mean + 1.0 * sd;
    const double floorv = two_dof ? 10.0 : 6.0;
    const double thr = isnan(cand) ? floorv : fmax(cand, floorv);
    cmax_s = thr >= (double)kMaxIter ? kMaxIter : (int)floor(thr);
    if (blockIdx.x == 0 && badnum) *badnum = (int)((long long)sums[3] - (long long)sums[4]);
  }
  __syncthreads();
  const int thr = cmax_s;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    const int c = conv[k];
    if (c < 0 || c > kMaxIter - 1 || c > thr) {
      U[2 * k] = nan("");
      U[2 * k + 1] = nan("");
      if (F && !two_dof)
        for (int a = 0; a < 4; ++a) F[4 * k + a] = nan("");
    }
  }
}

cudaError_t launch_badpoints(int32_t* conv, int N, double* U, double* F, int two_dof,
                             int* badnum_dev, unsigned long long* tmp_dev, cudaStream_t s) {
  if (N <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(tmp_dev, 0, 5 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const int blocks = (int)std::min<long long>(((long long)N + 255) / 256, 4ll * current_sm_count());
  badpoints_stats_kernel<<<blocks, 256, 0, s>>>(conv, N, tmp_dev);
  badpoints_apply_kernel<<<blocks, 256, 0, s>>>(conv, N, U, F, two_dof, tmp_dev, badnum_dev);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
__global__ void to_f32_kernel(const double* __restrict__ in, float* __restrict__ out, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x)
    out[k] = (float)in[k];
}

int current_sm_count() {
  static int cached[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 152;
  }
  if (dev >= 0 && dev < 64 && cached[dev] > 0) return cached[dev];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    n = 152;
  }
  if (dev >= 0 && dev < 64) cached[dev] = n;
  return n;
}

cudaError_t launch_to_f32(const double* in, float* out, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 255) / 256;
  const long long cap = 16ll * current_sm_count();
  if (blocks > cap) blocks = cap;
  to_f32_kernel<<<(int)blocks, 256, 0, s>>>(in, out, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Work queue of the batched solver: nodes ordered by subset size, a counting
// sort over the subset edge length in three grid-wide steps (per-block
// histograms merged into 256 global bins, a scan of the bins, then a scatter
// in which each block reserves its range of every bin with one atomic).
// ---------------------------------------------------------------------------
struct QueueKey {
  const int32_t* ws_list;
  const int32_t* wsl2;
  int ws_all, N, ascending, bw;
  // row bands (NB > 1): the y coordinates of the nodes and the frame's rows
  const double* coord_y;
  int H;
  // order 0: larger subsets first; 1: smaller first; 2: subsets of at least
  // bw pixels a side first (larger first), then the rest smaller first
  STDIC_DEV int size_bin(int w) const {
    const int b = min(max(w, 0), 255);
    if (ascending == 2) return b >= bw ? 255 - b : 256 - bw + b;
    return ascending ? b : 255 - b;
  }
  STDIC_DEV int edge(int k) const {
    int w = ws_all;
    if (wsl2) w = max(wsl2[k], wsl2[N + k]);
    else if (ws_list) w = ws_list[k];
    return w;
  }
  // the first of NB bands (band b ends at row (b + 1) H / NB) whose rows
  // cover every row the node's set-up may read: its window grown to the
  // largest size the mask can cause (grown_tile_pixels), around the rounded
  // centre (1-based rows y0 - wg / 2 .. y0 + wg / 2)
  template <int NB>
  STDIC_DEV int band(int k, int w) const {
    if (NB == 1) return 0;
    const int wg = 2 * (int)((1.2910 * w) / 2 + 1) + 2;
    const long long need = llround(coord_y[k]) + wg / 2;  // 0-based rows [0, need)
    int b = 0;
    while (b < NB - 1 && (long long)(b + 1) * H / NB < need) ++b;
    return b;
  }
  template <int NB>
  STDIC_DEV int operator()(int k) const {
    const int w = edge(k);
    return band<NB>(k, w) * 256 + size_bin(w);
  }
};

constexpr int kQueueBlockItems = 2048;  // items per block of the histogram and scatter steps

template <int NB>
__global__ void __launch_bounds__(256) queue_hist_kernel(QueueKey key, int* __restrict__ ghist) {
  __shared__ int hist[256 * NB];
  for (int b = threadIdx.x; b < 256 * NB; b += 256) hist[b] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int k0 = blockIdx.x * kQueueBlockItems;
  const int k1 = min(key.N, k0 + kQueueBlockItems);
  // the trip count is the same for every thread, so all lanes of a warp take
  // part in each match, whether or not they hold an item
  for (int k = k0 + threadIdx.x; k - threadIdx.x < k1; k += blockDim.x) {
    const int kk = k < k1 ? key.template operator()<NB>(k) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, kk);
    if (kk >= 0 && lane == __ffs(grp) - 1) atomicAdd(&hist[kk], __popc(grp));
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 256 * NB; b += 256)
    if (hist[b]) atomicAdd(&ghist[b], hist[b]);
}

// exclusive scan of the 256 NB bins into cursor (thread t scans bins t NB ..
// t NB + NB - 1), the number of items of at least big_ws pixels a side, and
// (when given) each band's first position (band_off, NB + 1 ints) and its
// items of at least big_ws pixels a side (band_big)
template <int NB>
__global__ void __launch_bounds__(256) queue_scan_kernel(const int* __restrict__ ghist, int* cursor,
                                                         int ascending, int big_ws, int* n_big, int* band_off,
                                                         int* band_big) {
  __shared__ int wsum[8], wbig[8][NB];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  int h[NB], tot = 0;
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    h[j] = ghist[t * NB + j];
    tot += h[j];
  }
  int inc = tot;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  // bin b holds subsets of edge w in band b / 256, with b % 256 = 255 - w
  // (orders 0 and 2 for w >= big_ws) or w (order 1)
  int big[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) big[j] = 0;
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    const int bin = t * NB + j, sb = bin & 255;
    const int w = ascending == 2 ? 255 - sb : (ascending ? sb : 255 - sb);
    const int v = w >= max(big_ws, 0) ? h[j] : 0;
    // band of this bin, accumulated per band slot (NB is small)
#pragma unroll
    for (int q = 0; q < NB; ++q)
      if (q == bin / 256) big[q] += v;
  }
#pragma unroll
  for (int q = 0; q < NB; ++q)
    for (int o = 16; o > 0; o >>= 1) big[q] += __shfl_xor_sync(0xffffffffu, big[q], o);
  if (lane == 31) wsum[warp] = inc;
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NB; ++q) wbig[warp][q] = big[q];
  }
  __syncthreads();
  int off = 0;
  for (int q = 0; q < warp; ++q) off += wsum[q];
  int run = off + inc - tot;
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    const int bin = t * NB + j;
    cursor[bin] = run;
    if (band_off && (bin & 255) == 0) band_off[bin / 256] = run;
    run += h[j];
  }
  if (t == 255 && band_off) band_off[NB] = run;
  if (t == 0) {
    int all = 0;
    for (int q = 0; q < NB; ++q) {
      int nb = 0;
      for (int w8 = 0; w8 < 8; ++w8) nb += wbig[w8][q];
      if (band_big) band_big[q] = nb;
      all += nb;
    }
    if (n_big) *n_big = all;
  }
}

template <int NB>
__global__ void __launch_bounds__(256) queue_scatter_kernel(QueueKey key, int* cursor, int32_t* __restrict__ order) {
  __shared__ int cnt[256 * NB], base[256 * NB];
  for (int b = threadIdx.x; b < 256 * NB; b += 256) cnt[b] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int k0 = blockIdx.x * kQueueBlockItems;
  const int k1 = min(key.N, k0 + kQueueBlockItems);
  for (int k = k0 + threadIdx.x; k - threadIdx.x < k1; k += blockDim.x) {
    const int kk = k < k1 ? key.template operator()<NB>(k) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, kk);
    if (kk >= 0 && lane == __ffs(grp) - 1) atomicAdd(&cnt[kk], __popc(grp));
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 256 * NB; b += 256) base[b] = cnt[b] ? atomicAdd(&cursor[b], cnt[b]) : 0;
  __syncthreads();
  for (int k = k0 + threadIdx.x; k - threadIdx.x < k1; k += blockDim.x) {
    const int kk = k < k1 ? key.template operator()<NB>(k) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, kk);
    const int leader = __ffs(grp) - 1;
    int pos = 0;
    if (kk >= 0 && lane == leader) pos = atomicAdd(&base[kk], __popc(grp));
    pos = __shfl_sync(0xffffffffu, pos, leader);
    if (kk >= 0) order[pos + __popc(grp & ((1u << lane) - 1u))] = k;
  }
}

template <int NB>
cudaError_t build_queue_nb(const QueueKey& key, int big_ws, int32_t* order, int* n_big, int* ghist, int* cursor,
                           int* band_off, int* band_big, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(ghist, 0, 256 * NB * sizeof(int), s);
  if (e != cudaSuccess) return e;
  const int blocks = (key.N + kQueueBlockItems - 1) / kQueueBlockItems;
  queue_hist_kernel<NB><<<blocks, 256, 0, s>>>(key, ghist);
  queue_scan_kernel<NB><<<1, 256, 0, s>>>(ghist, cursor, key.ascending, big_ws, n_big, band_off, band_big);
  queue_scatter_kernel<NB><<<blocks, 256, 0, s>>>(key, cursor, order);
  return cudaGetLastError();
}

cudaError_t launch_build_queue(const int32_t* ws_list, const int32_t* wsl2, int ws_all, int N,
                               int32_t* order, int* n_big, int* scratch, cudaStream_t s, int ascending,
                               int big_ws) {
  if (N <= 0) return cudaSuccess;
  QueueKey key{ws_list, wsl2, ws_all, N, ascending, min(max(big_ws, 1), 255), nullptr, 0};
  return build_queue_nb<1>(key, big_ws, order, n_big, scratch, scratch + 256, nullptr, nullptr, s);
}

cudaError_t launch_build_band_queue(const int32_t* ws_list, int ws_all, int N, const double* coord_y, int H, int nb,
                                    int32_t* order, int* n_big, int* band_off, int* band_big, int* scratch,
                                    cudaStream_t s, int ascending, int big_ws) {
  if (N <= 0) return cudaSuccess;
  QueueKey key{ws_list, nullptr, ws_all, N, ascending, min(max(big_ws, 1), 255), coord_y, H};
  int* ghist = scratch;
  int* cursor = scratch + 256 * kQueueMaxBands;
  switch (nb) {
    case 1: return build_queue_nb<1>(key, big_ws, order, n_big, ghist, cursor, band_off, band_big, s);
    case 2: return build_queue_nb<2>(key, big_ws, order, n_big, ghist, cursor, band_off, band_big, s);
    case 4: return build_queue_nb<4>(key, big_ws, order, n_big, ghist, cursor, band_off, band_big, s);
    case 8: return build_queue_nb<8>(key, big_ws, order, n_big, ghist, cursor, band_off, band_big, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace stdic
