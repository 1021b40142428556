// Helpers of the cooperative persistent kernels (the Subpb2 PCG and the
// gridfit CG of the multigrid integer search): a bounded grid barrier and
// deterministic grid-wide sums.
#pragma once
#include "device_common.cuh"

namespace stdic {

// Bounded grid barrier: a block that waits longer than `limit` polls sets
// *status = 2 and every block leaves at its next barrier check.
STDIC_DEV bool grid_barrier(int* count, volatile int* gen, int nblocks, int* status, long long limit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const int g = *gen;
    __threadfence();
    if (atomicAdd(count, 1) == nblocks - 1) {
      *count = 0;
      __threadfence();
      atomicAdd((int*)gen, 1);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > limit) { atomicExch(status, 2); break; }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int*)status == 0;
}

// per-block partial sums of up to 4 values into part[slot*1024 + block]; the
// totals are read back by every block in a fixed order (deterministic)
STDIC_DEV void block_partials(double v[4], int nv, double* part, double* red) {
  for (int k = 0; k < nv; ++k) {
    double t = v[k];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[k * 32 + (threadIdx.x >> 5)] = t;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double s = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[threadIdx.x * 32 + q];
    part[threadIdx.x * 1024 + blockIdx.x] = s;
  }
  __syncthreads();
}

STDIC_DEV void totals(const double* part, int nv, double* out, double* red) {
  if (threadIdx.x < 32) {
    for (int k = 0; k < nv; ++k) {
      double s = 0;
      for (int q = threadIdx.x; q < (int)gridDim.x; q += 32) s += part[k * 1024 + q];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) red[k] = s;
    }
  }
  __syncthreads();
  for (int k = 0; k < nv; ++k) out[k] = red[k];
  __syncthreads();
}

}  // namespace stdic
