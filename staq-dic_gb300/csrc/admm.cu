// Steps of the AL-DIC ADMM loop around Subpb1 and Subpb2
// (main_ALDIC_Quadtree_v2.m:337-395): nodal strain of the global displacement,
// NaN fill of the local displacement, the hole copies and the dual update.
//
// Nodal strain: the Gauss-point strains are those of
// funGlobalNodalStrainQuadtree.m:80-257 (DN U with the hanging-node shape
// functions; the quadtree elements are axis-aligned rectangles, for which the
// routine's bilinear inverse map gives ksi, eta equal to the Gauss abscissae).
// The reference maps them to the nodes with a natural-neighbour interpolant
// over all Gauss points; here a node takes the mean, over the elements that
// contain it (in increasing element order), of each element's Gauss point
// nearest to it.  F is stored as [du/dx dv/dx du/dy dv/dy], the order of the
// strain step the active loop calls (funGlobalNodalStrainRBF.m:52-62).
//
// NaN fill: the reference refills the bad local subsets with a thin-plate RBF
// over all finite nodes of a mask region (a dense solve) and a natural
// scatteredInterpolant (Subpb1Quadtree.m:193-259).  Here NaN nodes take, in
// sweeps, the mean of their finite mesh neighbours of the previous sweep
// (neighbours in increasing node order) until no NaN node has a finite
// neighbour; the NaN nodes are listed first and one CTA sweeps the list.
#include <algorithm>

#include "device_common.cuh"
#include "fem_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

constexpr int kMaxElemPerNode = 16;

__global__ void k_topo_count(const int32_t* __restrict__ elems, int E, int N, int* deg) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x)
    for (int c = 0; c < 8; ++c) {
      const int nd = elems[(size_t)c * E + e];
      if (nd >= 1 && nd <= N) atomicAdd(&deg[nd - 1], 1);
    }
}

// exclusive scan of n ints (one CTA); out has n + 1 entries
__global__ void __launch_bounds__(1024) k_topo_scan(const int* in, int* out, int n) {
  cta_exclusive_scan(in, out, n);
}

__global__ void k_topo_fill(const int32_t* __restrict__ elems, int E, int N, const int* ptr, int* cur,
                            int* list) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x)
    for (int c = 0; c < 8; ++c) {
      const int nd = elems[(size_t)c * E + e];
      if (nd < 1 || nd > N) continue;
      list[ptr[nd - 1] + atomicAdd(&cur[nd - 1], 1)] = e;
    }
}

// each node's element list in increasing order (insertion sort; lists are short)
__global__ void k_topo_sort(int N, const int* ptr, int* list) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    const int a = ptr[n], b = ptr[n + 1];
    for (int i = a + 1; i < b; ++i) {
      const int v = list[i];
      int j = i - 1;
      while (j >= a && list[j] > v) { list[j + 1] = list[j]; --j; }
      list[j + 1] = v;
    }
  }
}

__global__ void k_nodal_strain(const double* __restrict__ coords, int N, const int32_t* __restrict__ elems,
                               int E, const double* __restrict__ U, int gauss_order, const int* ptr,
                               const int* list, double* __restrict__ F) {
  double gpt[5], gwt[5];
  const int ng = gauss_rule(gauss_order, gpt, gwt);
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
    double acc[4] = {0, 0, 0, 0};
    const int a = ptr[n], b = ptr[n + 1];
    const double xn = coords[n], yn = coords[N + n];
    for (int k = a; k < b; ++k) {
      const int e = list[k];
      int nd[8];
      double px[8], py[8], uu[8], vv[8], dp[4];
      for (int c = 0; c < 8; ++c) {
        nd[c] = elems[(size_t)c * E + e];
        const bool ok = nd[c] >= 1 && nd[c] <= N;
        px[c] = ok ? coords[nd[c] - 1] : 0.0;
        py[c] = ok ? coords[N + nd[c] - 1] : 0.0;
        uu[c] = ok ? U[2 * (nd[c] - 1)] : 0.0;
        vv[c] = ok ? U[2 * (nd[c] - 1) + 1] : 0.0;
      }
      for (int c = 0; c < 4; ++c) dp[c] = nd[4 + c] != 0 ? 1.0 : 0.0;
      const double x1 = px[0], x3 = px[2], y1 = py[0], y3 = py[2];
      // the element's Gauss point nearest to the node (x-major order, first on
      // ties).  A hanging node at an edge midpoint is exactly as far from two
      // Gauss points; distances within 1e-9 relative count as equal, so that
      // rounding (and the contraction of the distance into FMAs) never decides
      // which one it takes.
      int bi = 0, bj = 0;
      double bd = 1e300;
      for (int ti = 0; ti < ng; ++ti)
        for (int tj = 0; tj < ng; ++tj) {
          const double gx = gpt[ti] * 0.5 * (x3 - x1) + 0.5 * (x3 + x1);
          const double gy = gpt[tj] * 0.5 * (y3 - y1) + 0.5 * (y3 + y1);
          const double dx = gx - xn, dy = gy - yn;
          const double d2 = dx * dx + dy * dy;
          if (d2 < bd * (1.0 - 1e-9)) { bd = d2; bi = ti; bj = tj; }
        }
      double Nv[8], dk[8], de[8];
      shape(gpt[bi], gpt[bj], dp, Nv, dk, de);
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
      acc[0] += dudx; acc[1] += dvdx; acc[2] += dudy; acc[3] += dvdy;
    }
    const int cnt = b - a;
    for (int q = 0; q < 4; ++q) F[4 * n + q] = cnt ? acc[q] / cnt : nan("");
  }
}

// NaN fill, step 1: the NaN nodes that lie in some element (the others have
// no neighbour and stay NaN), in any order
__global__ void k_nan_nodes(int N, const int* __restrict__ ptr, const double* __restrict__ U, int* cnt,
                            int* nodes) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
    if (isnan(U[2 * n]) && ptr[n + 1] > ptr[n]) nodes[atomicAdd(cnt, 1)] = n;
}

// the mean of the finite mesh neighbours of node n (sorted unique neighbour
// order); false when none is finite
STDIC_DEV bool neighbour_mean(int n, int N, const int32_t* __restrict__ elems, int E, const int* ptr,
                              const int* list, const double* U, double* mu, double* mv) {
  int cand[8 * kMaxElemPerNode];
  int nc = 0;
  const int a = ptr[n], b = min(ptr[n + 1], ptr[n] + kMaxElemPerNode);
  for (int k = a; k < b; ++k) {
    const int e = list[k];
    for (int c = 0; c < 8; ++c) {
      const int q = elems[(size_t)c * E + e];
      if (q < 1 || q > N || q - 1 == n) continue;
      const int val = q - 1;
      bool dup = false;
      for (int t = 0; t < nc && !dup; ++t) dup = cand[t] == val;
      if (dup || nc >= 8 * kMaxElemPerNode) continue;
      int j = nc - 1;
      while (j >= 0 && cand[j] > val) { cand[j + 1] = cand[j]; --j; }
      cand[j + 1] = val;
      ++nc;
    }
  }
  double su = 0, sv = 0;
  int cnt = 0;
  for (int t = 0; t < nc; ++t) {
    const int m = cand[t];
    if (!isnan(U[2 * m])) { su += U[2 * m]; sv += U[2 * m + 1]; ++cnt; }
  }
  if (!cnt) return false;
  *mu = su / cnt;
  *mv = sv / cnt;
  return true;
}

// NaN fill, step 2: Jacobi sweeps over the listed nodes in one CTA.  A sweep
// computes every still-NaN node's neighbour mean from the values before the
// sweep, then writes them; sweeps stop when one fills nothing.
__global__ void __launch_bounds__(1024) k_fill_nans(int N, const int32_t* __restrict__ elems, int E,
                                                    const int* ptr, const int* list, double* U,
                                                    const int* cnt, const int* __restrict__ nodes,
                                                    double* vals) {
  __shared__ int changed;
  const int m = *cnt;
  for (int sweep = 0; sweep <= m; ++sweep) {
    if (threadIdx.x == 0) changed = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      const int n = nodes[i];
      double u = nan(""), v = nan("");
      if (isnan(U[2 * n]) && neighbour_mean(n, N, elems, E, ptr, list, U, &u, &v)) changed = 1;
      vals[2 * i] = u;
      vals[2 * i + 1] = v;
    }
    __syncthreads();
    const int ch = changed;
    for (int i = threadIdx.x; i < m; i += blockDim.x)
      if (!isnan(vals[2 * i])) {
        const int n = nodes[i];
        U[2 * n] = vals[2 * i];
        U[2 * n + 1] = vals[2 * i + 1];
      }
    __syncthreads();
    if (!ch) break;
  }
}

// dst[k] = src[k] at the flagged nodes (width values per node)
__global__ void k_copy_marked(const uint8_t* __restrict__ mark, int N, int width, const double* __restrict__ src,
                              double* __restrict__ dst) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x)
    if (mark[n])
      for (int q = 0; q < width; ++q) dst[(size_t)width * n + q] = src[(size_t)width * n + q];
}

// out = a - b (n values)
__global__ void k_sub(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                      long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    out[k] = a[k] - b[k];
}

int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  return (int)std::max<long long>(1, std::min<long long>(b, 8ll * current_sm_count()));
}

}  // namespace

size_t topo_workspace_bytes(int N, int E) {
  return sizeof(int) * ((size_t)N * 3 + 1 + 8 * (size_t)E) + 256;
}

cudaError_t build_topology(const int32_t* elems, int E, int N, void* ws, int** ptr, int** list,
                           cudaStream_t s) {
  int* deg = (int*)ws;
  int* p = deg + N;       // N + 1
  int* cur = p + N + 1;   // N
  int* l = cur + N;       // 8E
  cudaError_t e = cudaMemsetAsync(deg, 0, sizeof(int) * (size_t)N, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(cur, 0, sizeof(int) * (size_t)N, s);
  if (e != cudaSuccess) return e;
  if (E > 0) k_topo_count<<<grid_for(E, 256), 256, 0, s>>>(elems, E, N, deg);
  k_topo_scan<<<1, 1024, 0, s>>>(deg, p, N);
  if (E > 0) k_topo_fill<<<grid_for(E, 256), 256, 0, s>>>(elems, E, N, p, cur, l);
  k_topo_sort<<<grid_for(N, 256), 256, 0, s>>>(N, p, l);
  *ptr = p;
  *list = l;
  return cudaGetLastError();
}

cudaError_t launch_nodal_strain(const double* coords, int N, const int32_t* elems, int E, const double* U,
                                int gauss_order, const int* ptr, const int* list, double* F, cudaStream_t s) {
  if (N <= 0) return cudaSuccess;
  k_nodal_strain<<<grid_for(N, 128), 128, 0, s>>>(coords, N, elems, E, U, gauss_order, ptr, list, F);
  return cudaGetLastError();
}

size_t fill_tmp_doubles(int N) { return 2 * (size_t)N + ((size_t)N + 1) / 2 + 2; }

cudaError_t launch_fill_nans(int N, const int32_t* elems, int E, const int* ptr, const int* list, double* U,
                             double* tmp, cudaStream_t s) {
  if (N <= 0) return cudaSuccess;
  double* vals = tmp;
  int* nodes = (int*)(tmp + 2 * (size_t)N);
  int* cnt = nodes + N + 1;
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  k_nan_nodes<<<grid_for(N, 256), 256, 0, s>>>(N, ptr, U, cnt, nodes);
  k_fill_nans<<<1, 1024, 0, s>>>(N, elems, E, ptr, list, U, cnt, nodes, vals);
  return cudaGetLastError();
}

cudaError_t launch_copy_marked(const uint8_t* mark, int N, int width, const double* src, double* dst,
                               cudaStream_t s) {
  if (N <= 0 || !mark) return cudaSuccess;
  k_copy_marked<<<grid_for(N, 256), 256, 0, s>>>(mark, N, width, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_sub(const double* a, const double* b, double* out, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_sub<<<grid_for(n, 256), 256, 0, s>>>(a, b, out, n);
  return cudaGetLastError();
}

}  // namespace stdic
