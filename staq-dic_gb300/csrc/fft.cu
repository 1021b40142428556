// FP64 complex FFTs of power-of-two length, for the full normalised
// cross-correlation map of the multigrid integer search's first level
// (normxcorr2 of the whole ROI, func/funIntegerSearchMg.m:19).
//
// A 2-D transform is done as row transforms in shared memory, a tiled
// transpose, and row transforms again; the caller keeps the spectrum in the
// transposed layout, since the correlation only multiplies spectra pointwise.
//
//   fft_rows_kernel      one CTA per row of L <= 8192 points (L x 16 bytes of
//                        shared memory): bit-reversed load, log2(L) radix-2
//                        decimation-in-time stages, store.  Twiddles come from
//                        a table exp(-2 pi i k / L), k < L/2, made once per
//                        length with CUDA's sincospi.  The inverse uses the
//                        conjugate twiddles and leaves the 1/L scaling to the
//                        caller.
//   transpose_c_kernel   32 x 32 tiles through shared memory, both sides
//                        coalesced.
#include "device_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

__global__ void fft_twiddle_kernel(double2* __restrict__ tw, int L) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= L / 2) return;
  double s, c;
  sincospi(-2.0 * (double)k / (double)L, &s, &c);
  tw[k] = make_double2(c, s);
}

template <bool INV>
__global__ void __launch_bounds__(512) fft_rows_kernel(double2* __restrict__ data, int L, int lg,
                                                       const double2* __restrict__ tw) {
  extern __shared__ __align__(16) double2 sfft[];
  double2* row = data + (size_t)blockIdx.x * L;
  for (int i = threadIdx.x; i < L; i += blockDim.x) sfft[__brev((unsigned)i) >> (32 - lg)] = row[i];
  __syncthreads();
  const int half = L >> 1;
  for (int h = 1, tstep = half; h < L; h <<= 1, tstep >>= 1) {
    for (int b = threadIdx.x; b < half; b += blockDim.x) {
      const int pos = b & (h - 1);
      const int i0 = ((b - pos) << 1) + pos, i1 = i0 + h;
      double2 w = __ldg(tw + pos * tstep);
      if (INV) w.y = -w.y;
      const double2 a = sfft[i0], c = sfft[i1];
      const double tr = w.x * c.x - w.y * c.y, ti = w.x * c.y + w.y * c.x;
      sfft[i0] = make_double2(a.x + tr, a.y + ti);
      sfft[i1] = make_double2(a.x - tr, a.y - ti);
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < L; i += blockDim.x) row[i] = sfft[i];
}

__global__ void __launch_bounds__(256) transpose_c_kernel(const double2* __restrict__ in, double2* __restrict__ out,
                                                          int rows, int cols) {
  __shared__ double2 t[32][33];
  const int x = blockIdx.x * 32 + threadIdx.x;
  const int y0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int y = y0 + j;
    if (x < cols && y < rows) t[j][threadIdx.x] = in[(size_t)y * cols + x];
  }
  __syncthreads();
  const int ox = y0 + threadIdx.x;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int oy = blockIdx.x * 32 + j;
    if (ox < rows && oy < cols) out[(size_t)oy * rows + ox] = t[threadIdx.x][j];
  }
}

int log2_exact(int L) {
  int lg = 0;
  while ((1 << lg) < L) ++lg;
  return (1 << lg) == L ? lg : -1;
}

}  // namespace

cudaError_t launch_fft_twiddles(double2* tw, int L, cudaStream_t s) {
  if (L < 2 || L > kFftMaxLen || log2_exact(L) < 0) return cudaErrorInvalidValue;
  fft_twiddle_kernel<<<(L / 2 + 255) / 256, 256, 0, s>>>(tw, L);
  return cudaGetLastError();
}

cudaError_t launch_fft_rows(double2* data, long long rows, int L, const double2* tw, bool inverse, cudaStream_t s) {
  const int lg = log2_exact(L);
  if (L < 2 || L > kFftMaxLen || lg < 0 || rows <= 0 || rows > 0x7fffffffLL) return cudaErrorInvalidValue;
  const int threads = L / 2 < 512 ? (L / 2 < 32 ? 32 : L / 2) : 512;
  const size_t smem = sizeof(double2) * (size_t)L;
  cudaError_t e;
  if (inverse) {
    e = cudaFuncSetAttribute(fft_rows_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) fft_rows_kernel<true><<<(unsigned)rows, threads, smem, s>>>(data, L, lg, tw);
  } else {
    e = cudaFuncSetAttribute(fft_rows_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) fft_rows_kernel<false><<<(unsigned)rows, threads, smem, s>>>(data, L, lg, tw);
  }
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t launch_transpose_c(const double2* in, double2* out, int rows, int cols, cudaStream_t s) {
  if (rows <= 0 || cols <= 0 || (rows + 31) / 32 > 65535) return cudaErrorInvalidValue;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  transpose_c_kernel<<<grid, block, 0, s>>>(in, out, rows, cols);
  return cudaGetLastError();
}

}  // namespace stdic
