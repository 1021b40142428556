// Batched IC-GN, host side: launch dispatch over the team widths (each
// instantiated in icgn_batched_tw{1,2,4,8}.cu), launch-shape sizes, and the
// FP64 factor kernel between the set-up and iteration stages.
#include <algorithm>

#include "icgn_batched.cuh"

namespace stdic {

int batched_tile_px_bytes(bool two) { return tile_px_bytes(two); }

size_t batched_team_bytes(int sm_px, bool two, int tw, int gtile) {
  return team_bytes(sm_px, two, tw, gtile);
}

size_t batched_scratch_bytes(int npx_max, bool two, long long warps) {
  return slice_bytes(npx_max, two) * (size_t)warps + 256;
}

int batched_small_px(int sm_px, bool two, int tw, int gtile) {
  const size_t sub = (team_bytes(sm_px, two, tw, gtile) / tw) & ~(size_t)127;
  const int gs = gtile / tw;
  const long long fixed = (long long)(gtile_bytes(gs) + sizeof(TeamCtl) + sizeof(float) * 32 + 16 + 64 + 15);
  long long px = ((long long)sub - fixed) / tile_px_bytes(two);
  while (px > 0 && team_bytes((int)px, two, 1, gs) > sub) --px;
  return (int)(px > 0 ? px : 0);
}

// FP64 inverse of each subset's 6x6 Hessian, one thread per subset (between
// the set-up and iteration stages): by Cholesky, or, when that fails, by LU
// with partial pivoting as MATLAB's mldivide falls back for such a matrix (a
// singular matrix gives a non-finite inverse, as H \ b gives non-finite steps).
// Inverse of the packed symmetric 6x6 H (lower, row-major) by Gauss-Jordan
// elimination of [H | I] with partial pivoting (the row operations of LU with
// partial pivoting, applied to the six unit right-hand sides at once); a zero
// pivot gives a non-finite inverse.  Out of line so that its local arrays
// exist only on this rare path.
__device__ __noinline__ void lu_inverse6(const double* __restrict__ H, double* __restrict__ out) {
  double A[6][12];
  for (int r = 0; r < 6; ++r)
    for (int c2 = 0; c2 < 6; ++c2) {
      A[r][c2] = r >= c2 ? H[r * (r + 1) / 2 + c2] : H[c2 * (c2 + 1) / 2 + r];
      A[r][6 + c2] = r == c2 ? 1.0 : 0.0;
    }
  for (int k = 0; k < 6; ++k) {
    int p = k;
    double amax = fabs(A[k][k]);
    for (int i = k + 1; i < 6; ++i)
      if (fabs(A[i][k]) > amax) { amax = fabs(A[i][k]); p = i; }
    if (p != k)
      for (int j = 0; j < 12; ++j) { const double t = A[k][j]; A[k][j] = A[p][j]; A[p][j] = t; }
    const double inv = 1.0 / A[k][k];
    for (int j = 0; j < 12; ++j) A[k][j] *= inv;
    for (int i = 0; i < 6; ++i) {
      if (i == k) continue;
      const double f = A[i][k];
      for (int j = 0; j < 12; ++j) A[i][j] -= f * A[k][j];
    }
  }
  for (int r = 0; r < 6; ++r)
    for (int c2 = 0; c2 < 6; ++c2) out[r * 6 + c2] = A[r][6 + c2];
}

__global__ void __launch_bounds__(64) factor6_kernel(const SubsetState6* __restrict__ st,
                                                      const double* __restrict__ H6,
                                                      double* __restrict__ Hinv6, int n,
                                                      const int32_t* __restrict__ list,
                                                      const int* __restrict__ counts) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (list) {
    // the subsets the iterations take, packed at the front of the grid (in
    // node order the subsets decided in the set-up come in runs, which left
    // the busiest SM at 1.5x the mean)
    const int nw = counts[0], ns = counts[1];
    if (t >= nw + ns) return;
    t = t < nw ? list[t] : list[2 * (size_t)n - ns + (t - nw)];
  }
  if (t >= n || st[t].code != 0) return;
  // packed lower Cholesky factor L (row-major), all indices compile-time
  double l[21];
#pragma unroll
  for (int k = 0; k < 21; ++k) l[k] = H6[(size_t)t * 21 + k];
  // GB300 issues FP64 at a small fraction of the FP32 rate, so each pivot
  // takes one reciprocal square root (l_jj = d rsqrt(d), 1/l_jj = rsqrt(d))
  // instead of a square root and a division
  bool ok = true;
  double rl[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double d = l[j * (j + 1) / 2 + j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= l[j * (j + 1) / 2 + k] * l[j * (j + 1) / 2 + k];
    ok = ok && (d > 0);
    const double dd = d > 0 ? d : 1.0;
    const double inv = rsqrt(dd);
    rl[j] = inv;
    l[j * (j + 1) / 2 + j] = dd * inv;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double s2 = l[i * (i + 1) / 2 + j];
#pragma unroll
      for (int k = 0; k < j; ++k) s2 -= l[i * (i + 1) / 2 + k] * l[j * (j + 1) / 2 + k];
      l[i * (i + 1) / 2 + j] = s2 * inv;
    }
  }
  // the inverse is handed to the iteration stage as FP32 pairs (hi, lo) whose
  // sum carries its FP64 value to about 2^-48: the split costs FP64
  // instructions, which GB300 issues slowly, so it is done once here rather
  // than by every team that takes the subset
  float2* outp = reinterpret_cast<float2*>(Hinv6) + (size_t)t * 36;
  if (!ok) {
    // the rare LU path has its own array, so that the Cholesky path's
    // result (out below) is never addressed and stays in registers
    double lu[36];
    lu_inverse6(H6 + (size_t)t * 21, lu);
    for (int k = 0; k < 36; ++k) {
      const float hi = (float)lu[k];
      outp[k] = make_float2(hi, (float)(lu[k] - (double)hi));
    }
    return;
  }
  double out[36];
  // M = L^-1 (lower, packed), then H^-1 = M^T M
  double m[21];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double inv = rl[i];
    m[i * (i + 1) / 2 + i] = inv;
#pragma unroll
    for (int j = 0; j < i; ++j) {
      double s2 = 0.0;
#pragma unroll
      for (int k = j; k < i; ++k) s2 += l[i * (i + 1) / 2 + k] * m[k * (k + 1) / 2 + j];
      m[i * (i + 1) / 2 + j] = -s2 * inv;
    }
  }
#pragma unroll
  for (int r = 0; r < 6; ++r) {
#pragma unroll
    for (int c2 = r; c2 < 6; ++c2) {
      double s2 = 0.0;
#pragma unroll
      for (int k = c2; k < 6; ++k) s2 += m[k * (k + 1) / 2 + r] * m[k * (k + 1) / 2 + c2];
      out[r * 6 + c2] = s2;
      out[c2 * 6 + r] = s2;
    }
  }
#pragma unroll
  for (int k = 0; k < 36; ++k) {
    const float hi = (float)out[k];
    outp[k] = make_float2(hi, (float)(out[k] - (double)hi));
  }
}

cudaError_t launch_factor6(const SubsetState6* st, const double* H6, double* Hinv6, int n,
                           const int32_t* list, const int* counts, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  // 64-thread blocks: four times as many blocks as SMs even for ~20k
  // subsets, so that the FP64-bound work spreads evenly
  factor6_kernel<<<(n + 63) / 64, 64, 0, s>>>(st, H6, Hinv6, n, list, counts);
  return cudaGetLastError();
}

cudaError_t launch_icgn_batched(const BatchedArgs& b, int blocks, int threads, cudaStream_t s) {
  const bool stg = b.stage != 1 && (b.gtile > 0 || b.gtile_small > 0);
  switch (b.warps_per_subset) {
    case 1: return stg ? launch_icgn_batched_tw1s(b, blocks, threads, s) : launch_icgn_batched_tw1u(b, blocks, threads, s);
    case 2: return stg ? launch_icgn_batched_tw2s(b, blocks, threads, s) : launch_icgn_batched_tw2u(b, blocks, threads, s);
    case 4: return stg ? launch_icgn_batched_tw4s(b, blocks, threads, s) : launch_icgn_batched_tw4u(b, blocks, threads, s);
    case 8: return stg ? launch_icgn_batched_tw8s(b, blocks, threads, s) : launch_icgn_batched_tw8u(b, blocks, threads, s);
  }
  return cudaErrorInvalidValue;
}

// Resident blocks per SM of one configuration (for grid sizing and the
// autotuner): of the 6-DOF set-up stage (stage 1), or of the iteration stage
// (any other stage) and the fused 2-DOF form.
int batched_blocks_per_sm(int tw, bool two, int threads, int smem_px, int gtile, int stage) {
  const int teams = threads / (tw * 32);
  const size_t smem = batched_team_bytes(smem_px, two, tw, gtile) * teams + 128;
  if (smem > 227 * 1024) return 0;
  const bool stg = (two || stage != 1) && gtile > 0;
  switch (tw) {
    case 1: return stg ? batched_blocks_per_sm_tw1s(two, threads, smem, stage) : batched_blocks_per_sm_tw1u(two, threads, smem, stage);
    case 2: return stg ? batched_blocks_per_sm_tw2s(two, threads, smem, stage) : batched_blocks_per_sm_tw2u(two, threads, smem, stage);
    case 4: return stg ? batched_blocks_per_sm_tw4s(two, threads, smem, stage) : batched_blocks_per_sm_tw4u(two, threads, smem, stage);
    case 8: return stg ? batched_blocks_per_sm_tw8s(two, threads, smem, stage) : batched_blocks_per_sm_tw8u(two, threads, smem, stage);
  }
  return 0;
}

}  // namespace stdic
