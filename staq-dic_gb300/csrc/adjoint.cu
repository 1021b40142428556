// Adjoint of the subset ZNSSD cost (no counterpart in the reference).
//
// For node n with warp parameters P = [F11 F21 F12 F22 u v] (its F and U) and
// the (ws+1)^2 window around round(x_n), the cost is the criterion
// funICGNQuadtree.m minimises, on the window pixels whose mask is set:
//   C_n = sum_i (a_i - b_i)^2,  a = (f - fbar)/|f - fbar|,  b = (t - tbar)/|t - tbar|,
//   t_i = bicubic (Keys, a = -1/2, clamped taps, as ba_interp2.cpp) of g at
//   x_i' = x0 + dx + F11 dx + F12 dy + u,  y_i' = y0 + dy + F21 dx + F22 dy + v.
// With rho = sum a b, dC/dt_i = -2 (a_i - rho b_i) / |t - tbar|; the chain
// through the warp gives dC/dP and through the tap weights dC/dg.
//
// One warp per subset, pulled from a work counter.  Pass A interpolates the
// window and forms the statistics; pass B forms the adjoint weight of every
// pixel, its contribution to dC/dP, and scatters w * weight into dg.  In the
// store mode pass A keeps t and its two position derivatives in shared memory
// for pass B; in the recompute mode pass B interpolates again, so a subset
// needs no per-pixel storage at all.  The dg scatter goes to a per-warp
// shared-memory tile over the subset's tap footprint (shared atomics), which
// is then added to dg with one global atomic per touched element; a footprint
// larger than the tile (a strongly stretched warp) falls back to global
// atomics.  T = double is the FP64 form, T = float the FP32 form (positions as
// an integer base plus a T offset).
#include "device_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

template <class T>
STDIC_DEV T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Keys weights and their derivatives at fraction d.
template <class T>
STDIC_DEV void keys(T d, T w[4], T dw[4]) {
  const T dd = d * d, ddd = dd * d;
  w[0] = T(0.5) * (-d + T(2) * dd - ddd);
  w[1] = T(0.5) * (T(2) - T(5) * dd + T(3) * ddd);
  w[2] = T(0.5) * (d + T(4) * dd - T(3) * ddd);
  w[3] = T(0.5) * (-dd + ddd);
  dw[0] = T(0.5) * (T(-1) + T(4) * d - T(3) * dd);
  dw[1] = T(0.5) * (T(-10) * d + T(9) * dd);
  dw[2] = T(0.5) * (T(1) + T(8) * d - T(9) * dd);
  dw[3] = T(0.5) * (T(-2) * d + T(3) * dd);
}

// Bicubic value and derivatives at 1-based (x0 + ox, y0 + oy); clamped taps.
template <class T>
STDIC_DEV T sample_grad(const T* __restrict__ g, int W, int H, int x0, T ox, int y0, T oy, T& gx,
                        T& gy) {
  const T fx = floor(ox), fy = floor(oy);
  T wx[4], dwx[4], wy[4], dwy[4];
  keys<T>(ox - fx, wx, dwx);
  keys<T>(oy - fy, wy, dwy);
  const int bx = x0 + (int)fx - 2, by = y0 + (int)fy - 2;  // 0-based first tap
  T t = 0, tx = 0, ty = 0;
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    const int cy = min(max(by + b, 0), H - 1);
    T r = 0, rd = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int cx = min(max(bx + a, 0), W - 1);
      const T v = __ldg(g + (long long)cy * W + cx);
      r += wx[a] * v;
      rd += dwx[a] * v;
    }
    t += wy[b] * r;
    tx += wy[b] * rd;
    ty += dwy[b] * r;
  }
  gx = tx;
  gy = ty;
  return t;
}

template <class T>
STDIC_DEV void atomic_add_t(T* p, T v) {
  atomicAdd(p, v);
}

struct AdjArgs {
  const void* f;
  const void* g;
  const uint8_t* mask;  // may be null (every pixel)
  int W, H, N;
  const double* coords;
  const double* U;
  const double* F;
  int ws_all;
  const int32_t* ws_list;
  int ws_max;
  double* cost_n;
  double* dU;
  double* dF;
  void* dg;  // may be null
  int* head;
  int acc_side;  // side of the per-warp dg tile (0: global atomics only)
  int store;     // shared-memory pixels per warp for the store mode (0: recompute)
};

template <class T, bool STORE>
__global__ void __launch_bounds__(128) adjoint_kernel(AdjArgs A) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T* __restrict__ f = (const T*)A.f;
  const T* __restrict__ g = (const T*)A.g;
  T* dg = (T*)A.dg;
  const int W = A.W, H = A.H;
  const size_t acc_n = (size_t)A.acc_side * A.acc_side;
  const size_t per_warp = acc_n * sizeof(T) + (STORE ? (size_t)3 * A.store * sizeof(T) : 0);
  unsigned char* mine = dsm + per_warp * warp;
  T* acc = (T*)mine;
  T* st = (T*)(mine + acc_n * sizeof(T));  // t, tx, ty planes of A.store pixels
  for (size_t k = lane; k < acc_n; k += 32) acc[k] = T(0);
  __syncwarp();

  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(A.head, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= A.N) break;
    const int x0 = (int)llround(A.coords[item]), y0 = (int)llround(A.coords[A.N + item]);
    const int ws = A.ws_list ? A.ws_list[item] : A.ws_all;
    const int h = ws / 2, m = ws + 1, npx = m * m;
    const T P0 = (T)A.F[4 * item], P1 = (T)A.F[4 * item + 1], P2 = (T)A.F[4 * item + 2],
            P3 = (T)A.F[4 * item + 3], P4 = (T)A.U[2 * item], P5 = (T)A.U[2 * item + 1];
    // shift of the one-pass sums: f at the node (0 if outside the image)
    const bool cin = x0 >= 1 && x0 <= W && y0 >= 1 && y0 <= H;
    const T sh = cin ? f[(long long)(y0 - 1) * W + (x0 - 1)] : T(0);
    auto valid_px = [&](int i, int j, T& fv) {
      const int x = x0 - h + i, y = y0 - h + j;
      if (x < 1 || x > W || y < 1 || y > H) return false;
      const long long o = (long long)(y - 1) * W + (x - 1);
      if (A.mask && !A.mask[o]) return false;
      fv = f[o];
      return true;
    };
    // ---------------- pass A: statistics ----------------
    T sf = 0, st_ = 0, sff = 0, stt = 0, sft = 0;
    int n = 0;
    const bool use_store = STORE && npx <= A.store;
    for (int p = lane; p < npx; p += 32) {
      const int i = p % m, j = p / m;
      T fv;
      if (!valid_px(i, j, fv)) continue;
      const T dx = (T)(i - h), dy = (T)(j - h);
      const T ox = dx + P0 * dx + P2 * dy + P4, oy = dy + P1 * dx + P3 * dy + P5;
      T gx, gy;
      const T t = sample_grad<T>(g, W, H, x0, ox, y0, oy, gx, gy);
      if (use_store) { st[p] = t; st[A.store + p] = gx; st[2 * A.store + p] = gy; }
      const T a = fv - sh, b = t - sh;
      sf += a; st_ += b; sff += a * a; stt += b * b; sft += a * b;
      ++n;
    }
    sf = warp_sum(sf); st_ = warp_sum(st_); sff = warp_sum(sff); stt = warp_sum(stt);
    sft = warp_sum(sft);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    const T nn = (T)n;
    const T fm = sf / nn, tm = st_ / nn;
    const T vf = sff - nn * fm * fm, vt = stt - nn * tm * tm, cft = sft - nn * fm * tm;
    const bool ok = n >= 2 && vf > T(0) && vt > T(0) && isfinite((double)vt);
    if (!ok) {
      if (lane == 0) {
        A.cost_n[item] = nan("");
        if (A.dU) { A.dU[2 * item] = 0.0; A.dU[2 * item + 1] = 0.0; }
        if (A.dF)
          for (int k = 0; k < 4; ++k) A.dF[4 * item + k] = 0.0;
      }
      continue;
    }
    const T df = sqrt(vf), dtn = sqrt(vt);
    const T idf = T(1) / df, idt = T(1) / dtn;
    const T rho = cft * idf * idt;
    // dg tile over the tap footprint (corners of the affine warp, 1-pixel margin)
    int ax = 0, ay = 0;
    bool tile = false;
    if (dg && A.acc_side > 0) {
      T omin = T(1e30), omax = T(-1e30), pmin = T(1e30), pmax = T(-1e30);
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const T dx = (T)((c & 1) ? h : -h), dy = (T)((c & 2) ? h : -h);
        const T ox = dx + P0 * dx + P2 * dy + P4, oy = dy + P1 * dx + P3 * dy + P5;
        omin = fmin(omin, ox); omax = fmax(omax, ox); pmin = fmin(pmin, oy); pmax = fmax(pmax, oy);
      }
      if (omin > T(-1e6) && omax < T(1e6) && pmin > T(-1e6) && pmax < T(1e6)) {
        const long long lx0 = (long long)x0 + (long long)floor(omin) - 3;
        const long long lx1 = (long long)x0 + (long long)floor(omax) + 2;
        const long long ly0 = (long long)y0 + (long long)floor(pmin) - 3;
        const long long ly1 = (long long)y0 + (long long)floor(pmax) + 2;
        const long long cx0 = lx0 < 0 ? 0 : lx0, cy0 = ly0 < 0 ? 0 : ly0;
        const long long cx1 = lx1 > W - 1 ? W - 1 : lx1, cy1 = ly1 > H - 1 ? H - 1 : ly1;
        if (cx1 - cx0 + 1 <= A.acc_side && cy1 - cy0 + 1 <= A.acc_side && cx1 >= cx0 && cy1 >= cy0) {
          ax = (int)cx0; ay = (int)cy0;
          tile = true;
        }
      }
    }
    // ---------------- pass B: adjoint ----------------
    T cost = 0, d0 = 0, d1 = 0, d2 = 0, d3 = 0, d4 = 0, d5 = 0;
    for (int p = lane; p < npx; p += 32) {
      const int i = p % m, j = p / m;
      T fv;
      if (!valid_px(i, j, fv)) continue;
      const T dx = (T)(i - h), dy = (T)(j - h);
      const T ox = dx + P0 * dx + P2 * dy + P4, oy = dy + P1 * dx + P3 * dy + P5;
      T t, gx, gy;
      if (use_store) { t = st[p]; gx = st[A.store + p]; gy = st[2 * A.store + p]; }
      else t = sample_grad<T>(g, W, H, x0, ox, y0, oy, gx, gy);
      const T a = (fv - sh - fm) * idf, b = (t - sh - tm) * idt;
      const T r = a - b;
      cost += r * r;
      const T w = T(-2) * (a - rho * b) * idt;
      const T wx_ = w * gx, wy_ = w * gy;
      d0 += wx_ * dx; d1 += wy_ * dx; d2 += wx_ * dy; d3 += wy_ * dy; d4 += wx_; d5 += wy_;
      if (dg) {
        const T fx = floor(ox), fy = floor(oy);
        T kx[4], dkx[4], ky[4], dky[4];
        keys<T>(ox - fx, kx, dkx);
        keys<T>(oy - fy, ky, dky);
        const int bx = x0 + (int)fx - 2, by = y0 + (int)fy - 2;
#pragma unroll
        for (int bb = 0; bb < 4; ++bb) {
          const int cy = min(max(by + bb, 0), H - 1);
#pragma unroll
          for (int aa = 0; aa < 4; ++aa) {
            const int cx = min(max(bx + aa, 0), W - 1);
            const T v = w * kx[aa] * ky[bb];
            const int lx = cx - ax, ly = cy - ay;
            if (tile && lx >= 0 && lx < A.acc_side && ly >= 0 && ly < A.acc_side)
              atomic_add_t(acc + (size_t)ly * A.acc_side + lx, v);
            else
              atomic_add_t(dg + (long long)cy * W + cx, v);
          }
        }
      }
    }
    cost = warp_sum(cost);
    d0 = warp_sum(d0); d1 = warp_sum(d1); d2 = warp_sum(d2);
    d3 = warp_sum(d3); d4 = warp_sum(d4); d5 = warp_sum(d5);
    if (lane == 0) {
      A.cost_n[item] = (double)cost;
      if (A.dF) {
        A.dF[4 * item] = (double)d0; A.dF[4 * item + 1] = (double)d1;
        A.dF[4 * item + 2] = (double)d2; A.dF[4 * item + 3] = (double)d3;
      }
      if (A.dU) { A.dU[2 * item] = (double)d4; A.dU[2 * item + 1] = (double)d5; }
    }
    if (tile) {
      // add the tile to dg and clear it for the next subset
      __syncwarp();
      for (int k = lane; k < A.acc_side * A.acc_side; k += 32) {
        const T v = acc[k];
        if (v != T(0)) {
          const int lx = k % A.acc_side, ly = k / A.acc_side;
          if (ax + lx < W && ay + ly < H) atomic_add_t(dg + (long long)(ay + ly) * W + (ax + lx), v);
          acc[k] = T(0);
        }
      }
      __syncwarp();
    }
  }
}

// J = sum of the finite subset costs, in a fixed order (one block).
__global__ void __launch_bounds__(1024) cost_sum_kernel(const double* __restrict__ c, int N, double* out) {
  __shared__ double part[1024];
  double s = 0;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const double v = c[k];
    if (isfinite(v)) s += v;
  }
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

template <class T, bool STORE>
cudaError_t launch_adj(const AdjArgs& a, int nsm, cudaStream_t s) {
  const size_t acc_n = (size_t)a.acc_side * a.acc_side;
  const size_t per_warp = acc_n * sizeof(T) + (STORE ? (size_t)3 * a.store * sizeof(T) : 0);
  int warps = 4;
  while (warps > 1 && per_warp * warps > 200 * 1024) --warps;
  const size_t smem = per_warp * warps;
  if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(adjoint_kernel<T, STORE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_kernel<T, STORE>, warps * 32, smem);
  if (e != cudaSuccess) return e;
  int blocks = nsm * (per_sm > 0 ? per_sm : 1);
  blocks = min(blocks, (a.N + warps - 1) / warps);
  if (blocks < 1) blocks = 1;
  adjoint_kernel<T, STORE><<<blocks, warps * 32, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_adjoint(const AdjointArgs& x, cudaStream_t s, long long* launches) {
  AdjArgs a{};
  a.f = x.f; a.g = x.g; a.mask = x.mask; a.W = x.W; a.H = x.H; a.N = x.N;
  a.coords = x.coords; a.U = x.U; a.F = x.F; a.ws_all = x.ws_all; a.ws_list = x.ws_list;
  a.ws_max = x.ws_max; a.cost_n = x.cost_n; a.dU = x.dU; a.dF = x.dF; a.dg = x.dg; a.head = x.head;
  // per-warp shared memory: the dg tile, then (store mode) three planes of
  // the window; either is dropped when a warp's share would not fit
  const size_t es_ = x.f64 ? 8 : 4;
  a.acc_side = x.dg ? x.ws_max + 12 : 0;
  a.store = x.store ? (x.ws_max + 1) * (x.ws_max + 1) : 0;
  if ((size_t)a.acc_side * a.acc_side * es_ + (size_t)3 * a.store * es_ > 200 * 1024) a.store = 0;
  if ((size_t)a.acc_side * a.acc_side * es_ > 200 * 1024) a.acc_side = 0;
  long long nl = 0;
  const size_t es = x.f64 ? 8 : 4;
  cudaError_t e = cudaMemsetAsync(x.head, 0, sizeof(int), s);
  if (e == cudaSuccess && x.dg) e = cudaMemsetAsync(x.dg, 0, es * (size_t)x.W * x.H, s);
  if (e != cudaSuccess) return e;
  if (x.N > 0) {
    if (x.f64) e = a.store ? launch_adj<double, true>(a, x.nsm, s) : launch_adj<double, false>(a, x.nsm, s);
    else e = a.store ? launch_adj<float, true>(a, x.nsm, s) : launch_adj<float, false>(a, x.nsm, s);
    if (e != cudaSuccess) return e;
    ++nl;
  }
  if (x.cost) {
    cost_sum_kernel<<<1, 1024, 0, s>>>(x.cost_n, x.N, x.cost);
    e = cudaGetLastError();
    ++nl;
  }
  if (launches) *launches += nl;
  return e;
}

}  // namespace stdic
