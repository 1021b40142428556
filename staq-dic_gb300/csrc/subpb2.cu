// Subproblem 2 of the AL-DIC ADMM: global FEM solve on the quadtree mesh
// (func_quadtree/Subpb2Quadtree.m).
//
//   A = sum_e sum_gp |J| w ((beta+alpha) DN'DN + mu N'N)       (:259)
//   b = sum_e sum_gp |J| w (beta diag(DN' F_e') + mu N'N U_e + alpha DN'DN U_e)   (:262)
//   Uhat(Dirichlet) = U(Dirichlet); Uhat(Free) = A(Free,Free) \ (b - A Uhat)(Free)  (:332-339)
//
// DN maps u-DOFs to rows 1-2 and v-DOFs to rows 3-4 and N maps them to rows 1 and
// 2, so A never couples u with v: A = K (x) I2 with one scalar node matrix
//   K_ab = sum |J| w ((beta+alpha) grad N_a . grad N_b + mu N_a N_b).
// The solver assembles K once in CSR (node graph built on the device) and runs
// Jacobi-preconditioned CG on both right-hand sides together in FP64.  The CG
// is one cooperative persistent kernel whose grid barriers are bounded spins
// (an exhausted wait sets a status the host reads; nothing traps).
#include <algorithm>

#include "device_common.cuh"
#include "coop.cuh"
#include "fem_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

constexpr int kMaxElemPerNode = 16;
constexpr long long kSpinLimit = 1ll << 24;  // bounded grid-barrier wait
// per hanging-node pattern: Sxx, Syy, M (8x8 each), Gx, Gy (8 each)
constexpr int kTabStride = 3 * 64 + 16;

struct Ws {  // carved from the caller's workspace
  int* deg;        // N+1
  int* eptr;       // N+1
  int* elist;      // 8E
  int* cursor;     // N
  int* rowlen;     // N+1
  int* rowptr;     // N+1
  int* col;        // 64E
  double* val;     // 64E
  double* diag;    // N
  double* b;       // 2N (u, v planes)
  double* x;       // 2N
  double* r;       // 2N
  double* z;       // 2N
  double* p;       // 2N
  double* Ap;      // 2N
  uint8_t* freen;  // N
  uint8_t* dirn;   // N
  int* misc;       // 16 ints: [0] any zero entry, [1] min node, [2] barrier count, [3] barrier gen
  double* part;    // partial sums: 10 slots x 1024 blocks (one region per CG phase)
  double* tab;     // reference-element tables: 16 hanging patterns x kTabStride
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

Ws carve(void* base, int N, int E, size_t* total) {
  Ws w;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    void* p = (char*)base + o;
    o += align256(bytes);
    return p;
  };
  w.deg = (int*)take(sizeof(int) * (N + 1));
  w.eptr = (int*)take(sizeof(int) * (N + 1));
  w.elist = (int*)take(sizeof(int) * 8 * (size_t)E);
  w.cursor = (int*)take(sizeof(int) * N);
  w.rowlen = (int*)take(sizeof(int) * (N + 1));
  w.rowptr = (int*)take(sizeof(int) * (N + 1));
  w.col = (int*)take(sizeof(int) * 64 * (size_t)E);
  w.val = (double*)take(sizeof(double) * 64 * (size_t)E);
  w.diag = (double*)take(sizeof(double) * N);
  w.b = (double*)take(sizeof(double) * 2 * N);
  w.x = (double*)take(sizeof(double) * 2 * N);
  w.r = (double*)take(sizeof(double) * 2 * N);
  w.z = (double*)take(sizeof(double) * 2 * N);
  w.p = (double*)take(sizeof(double) * 2 * N);
  w.Ap = (double*)take(sizeof(double) * 2 * N);
  w.freen = (uint8_t*)take(N);
  w.dirn = (uint8_t*)take(N);
  w.misc = (int*)take(sizeof(int) * 16);
  w.part = (double*)take(sizeof(double) * 10 * 1024);
  w.tab = (double*)take(sizeof(double) * 16 * kTabStride);
  if (total) *total = o;
  return w;
}

// ---- mesh graph --------------------------------------------------------------
__global__ void k_init(Ws w, int N) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n <= N; n += gridDim.x * blockDim.x) {
    w.deg[n] = 0;
    if (n < N) { w.freen[n] = 0; w.dirn[n] = 0; w.cursor[n] = 0; }
  }
  if (blockIdx.x == 0 && threadIdx.x < 16) w.misc[threadIdx.x] = threadIdx.x == 1 ? 0x7fffffff : 0;
}

__global__ void k_degree(Subpb2Args a, Ws w) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.E; e += gridDim.x * blockDim.x) {
    for (int c = 0; c < 8; ++c) {
      const int nd = a.elems[(size_t)c * a.E + e];
      if (nd == 0) { atomicOr(&w.misc[0], 1); continue; }
      if (nd < 1 || nd > a.N) { atomicOr(&w.misc[4], 1); continue; }  // invalid index
      atomicAdd(&w.deg[nd - 1], 1);
      atomicMin(&w.misc[1], nd);
      w.freen[nd - 1] = 1;  // involved
    }
  }
}

// exclusive scan of n+1 ints in one CTA (n up to a few million)
__global__ void __launch_bounds__(1024) k_scan(const int* in, int* out, int n) {
  cta_exclusive_scan(in, out, n);
}

__global__ void k_fill_elist(Subpb2Args a, Ws w) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < a.E; e += gridDim.x * blockDim.x) {
    for (int c = 0; c < 8; ++c) {
      const int nd = a.elems[(size_t)c * a.E + e];
      if (nd < 1 || nd > a.N) continue;
      const int pos = atomicAdd(&w.cursor[nd - 1], 1);
      w.elist[w.eptr[nd - 1] + pos] = e;
    }
  }
}

// Sorted unique neighbour nodes (0-based) of node n.  Returns the count; the
// list is written to out when out != nullptr.
STDIC_DEV int neighbours(const Subpb2Args& a, const Ws& w, int n, int* out) {
  int cand[8 * kMaxElemPerNode];
  int nc = 0;
  const int e0 = w.eptr[n], e1 = min(w.eptr[n + 1], e0 + kMaxElemPerNode);
  for (int k = e0; k < e1; ++k) {
    const int e = w.elist[k];
    for (int c = 0; c < 8; ++c) {
      const int nd = a.elems[(size_t)c * a.E + e];
      if (nd >= 1 && nd <= a.N) cand[nc++] = nd - 1;
    }
  }
  // insertion sort + unique
  for (int i = 1; i < nc; ++i) {
    const int v = cand[i];
    int j = i - 1;
    while (j >= 0 && cand[j] > v) { cand[j + 1] = cand[j]; --j; }
    cand[j + 1] = v;
  }
  int u = 0;
  for (int i = 0; i < nc; ++i)
    if (i == 0 || cand[i] != cand[i - 1]) {
      if (out) out[u] = cand[i];
      ++u;
    }
  return u;
}

__global__ void k_rowlen(Subpb2Args a, Ws w) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += gridDim.x * blockDim.x) {
    if (w.eptr[n + 1] - w.eptr[n] > kMaxElemPerNode) atomicOr(&w.misc[5], 1);
    w.rowlen[n] = neighbours(a, w, n, nullptr);
  }
}

__global__ void k_fill_cols(Subpb2Args a, Ws w) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += gridDim.x * blockDim.x) {
    neighbours(a, w, n, w.col + w.rowptr[n]);
  }
}

// ---- element integration (Subpb2Quadtree.m:94-262) -----------------------------
STDIC_DEV int find_col(const Ws& w, int row, int c) {
  int lo = w.rowptr[row], hi = w.rowptr[row + 1] - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const int v = w.col[mid];
    if (v == c) return mid;
    if (v < c) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

// Reference-square integrals of each hanging-node pattern (bit c of the
// pattern: hanging node 5 + c present), over the Gauss rule of the call:
//   Sxx_pq = sum w dN_p/dksi dN_q/dksi,  Syy_pq = sum w dN_p/deta dN_q/deta,
//   M_pq = sum w N_p N_q,  Gx_p = sum w dN_p/dksi,  Gy_p = sum w dN_p/deta.
// An axis-aligned rectangle with edges hx = x2 - x1, hy = y4 - y1 (and any
// hanging node at its edge midpoint) has the constant Jacobian diag(hx, hy)/2,
// so its element integrals are these tables scaled by hx and hy.
__global__ void k_ref_tables(int gauss_order, Ws w) {
  const int pat = blockIdx.x, p = threadIdx.x >> 3, q = threadIdx.x & 7;
  double gpt[5], gwt[5];
  const int ng = gauss_rule(gauss_order, gpt, gwt);
  double dp[4];
  for (int c = 0; c < 4; ++c) dp[c] = (pat >> c) & 1 ? 1.0 : 0.0;
  double sxx = 0, syy = 0, m = 0, gx = 0, gy = 0;
  for (int gi = 0; gi < ng * ng; ++gi) {
    const double ksi = gpt[gi % ng], eta = gpt[gi / ng];
    const double wgt = gwt[gi % ng] * gwt[gi / ng];
    double Nv[8], dk[8], de[8];
    shape(ksi, eta, dp, Nv, dk, de);
    double np = 0, nq = 0, kp = 0, kq = 0, ep = 0, eq = 0;
    for (int c = 0; c < 8; ++c) {
      if (c == p) { np = Nv[c]; kp = dk[c]; ep = de[c]; }
      if (c == q) { nq = Nv[c]; kq = dk[c]; eq = de[c]; }
    }
    sxx += wgt * kp * kq;
    syy += wgt * ep * eq;
    m += wgt * np * nq;
    gx += wgt * kp;
    gy += wgt * ep;
  }
  double* t = w.tab + pat * kTabStride;
  t[p * 8 + q] = sxx;
  t[64 + p * 8 + q] = syy;
  t[128 + p * 8 + q] = m;
  if (q == 0) { t[192 + p] = gx; t[200 + p] = gy; }
}

// Element integration, eight lanes per element: lane p assembles row p of the
// element matrix and right-hand side.  Rectangles take the reference tables;
// any other element integrates its Gauss points directly.
__global__ void __launch_bounds__(256) k_element(Subpb2Args a, Ws w) {
  const int p = threadIdx.x & 7;
  const long long g0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
  const long long gs = ((long long)gridDim.x * blockDim.x) >> 3;
  for (long long e = g0; e < a.E; e += gs) {
    int nd[8];
    double px[8], py[8], dp[4];
    bool corners = true;
    for (int c = 0; c < 8; ++c) {
      nd[c] = a.elems[(size_t)c * a.E + e];
      const bool ok = nd[c] >= 1 && nd[c] <= a.N;
      if (c < 4) corners &= ok;
      px[c] = ok ? a.coords[nd[c] - 1] : 0.0;
      py[c] = ok ? a.coords[a.N + nd[c] - 1] : 0.0;
    }
    int pat = 0;
    for (int c = 0; c < 4; ++c) {
      dp[c] = nd[4 + c] != 0 ? 1.0 : 0.0;
      pat |= nd[4 + c] != 0 ? 1 << c : 0;
    }
    const double hx = px[1] - px[0], hy = py[3] - py[0];
    bool rect = corners && py[1] == py[0] && px[2] == px[1] && py[2] == py[3] && px[3] == px[0] && hx != 0 &&
                hy != 0;
    // hanging nodes at their edge midpoints: 5 on 2-3, 6 on 3-4, 7 on 4-1, 8 on 1-2
    const int ea[4] = {1, 2, 3, 0}, eb[4] = {2, 3, 0, 1};
    for (int c = 0; c < 4; ++c)
      if (nd[4 + c] != 0)
        rect &= nd[4 + c] >= 1 && nd[4 + c] <= a.N && px[4 + c] == 0.5 * (px[ea[c]] + px[eb[c]]) &&
                py[4 + c] == 0.5 * (py[ea[c]] + py[eb[c]]);
    const bool okp = nd[p] >= 1 && nd[p] <= a.N;
    double Uu[8], Uv[8];
    for (int c = 0; c < 8; ++c) {
      const bool ok = nd[c] >= 1 && nd[c] <= a.N;
      Uu[c] = ok ? a.U[2 * (nd[c] - 1)] : 0.0;
      Uv[c] = ok ? a.U[2 * (nd[c] - 1) + 1] : 0.0;
    }
    double F11 = 0, F21 = 0, F12 = 0, F22 = 0;
    if (okp) {
      const double* Fp = a.F + 4 * (size_t)(nd[p] - 1);
      F11 = Fp[0]; F21 = Fp[1]; F12 = Fp[2]; F22 = Fp[3];
    }
    double Kr[8], bu = 0, bv = 0;
    if (rect) {
      const double* t = w.tab + pat * kTabStride;
      const double ryx = hy / hx, rxy = hx / hy, cm = a.mu * (0.25 * hx * hy), cs = a.beta + a.alpha;
      for (int q = 0; q < 8; ++q) {
        const double sd = ryx * t[p * 8 + q] + rxy * t[64 + p * 8 + q];
        const double mm = cm * t[128 + p * 8 + q];
        Kr[q] = cs * sd + mm;
        const double r = mm + a.alpha * sd;
        bu += r * Uu[q];
        bv += r * Uv[q];
      }
      const double gxp = 0.5 * hy * t[192 + p], gyp = 0.5 * hx * t[200 + p];
      bu += a.beta * (gxp * F11 + gyp * F12);
      bv += a.beta * (gxp * F21 + gyp * F22);
    } else {
      double gpt[5], gwt[5];
      const int ng = gauss_rule(a.gauss_order, gpt, gwt);
      for (int q = 0; q < 8; ++q) Kr[q] = 0;
      for (int gi = 0; gi < ng * ng; ++gi) {
        const double ksi = gpt[gi % ng], eta = gpt[gi / ng];
        const double wgt = gwt[gi % ng] * gwt[gi / ng];
        double Nv[8], dk[8], de[8];
        shape(ksi, eta, dp, Nv, dk, de);
        double J11 = 0, J12 = 0, J21 = 0, J22 = 0;
        for (int c = 0; c < 8; ++c) {
          J11 += dk[c] * px[c]; J12 += dk[c] * py[c];
          J21 += de[c] * px[c]; J22 += de[c] * py[c];
        }
        const double Jac = J11 * J22 - J12 * J21;
        const double i11 = 1 / Jac * J22, i12 = 1 / Jac * (-J12), i21 = 1 / Jac * (-J21),
                     i22 = 1 / Jac * J11;
        double gx[8], gy[8], gxp = 0, gyp = 0, np = 0;
        for (int c = 0; c < 8; ++c) {
          gx[c] = i11 * dk[c] + i12 * de[c];
          gy[c] = i21 * dk[c] + i22 * de[c];
          if (c == p) { gxp = gx[c]; gyp = gy[c]; np = Nv[c]; }
        }
        const double wj = Jac * wgt;
        double nnu = 0, nnv = 0, ddu = 0, ddv = 0;
        for (int q = 0; q < 8; ++q) {
          const double dd = gxp * gx[q] + gyp * gy[q];
          const double nn = np * Nv[q];
          Kr[q] += wj * ((a.beta + a.alpha) * dd + a.mu * nn);
          nnu += nn * Uu[q]; nnv += nn * Uv[q];
          ddu += dd * Uu[q]; ddv += dd * Uv[q];
        }
        bu += wj * (a.beta * (gxp * F11 + gyp * F12) + a.mu * nnu + a.alpha * ddu);
        bv += wj * (a.beta * (gxp * F21 + gyp * F22) + a.mu * nnv + a.alpha * ddv);
      }
    }
    if (!okp) continue;
    const int row = nd[p] - 1;
    atomicAdd(&w.b[row], bu);
    atomicAdd(&w.b[a.N + row], bv);
    for (int q = 0; q < 8; ++q) {
      if (nd[q] < 1 || nd[q] > a.N) continue;
      const int k = find_col(w, row, nd[q] - 1);
      if (k >= 0) atomicAdd(&w.val[k], Kr[q]);
      if (nd[q] == nd[p]) atomicAdd(&w.diag[row], Kr[q]);
    }
  }
}

// zero the matrix values, diagonal and right-hand sides of an assembled structure
__global__ void k_zero_values(Subpb2Args a, Ws w) {
  if (blockIdx.x == 0 && threadIdx.x == 0) w.misc[2] = 0;  // grid-barrier count
  const int nnz = w.rowptr[a.N];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) w.val[k] = 0.0;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += gridDim.x * blockDim.x) {
    w.diag[n] = 0.0;
    w.b[n] = 0.0;
    w.b[a.N + n] = 0.0;
  }
}

// Neumann rows (Subpb2Quadtree.m:323-329): BCForce = -F / winstepsize
__global__ void k_neumann(Subpb2Args a, Ws w) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < a.nn; t += gridDim.x * blockDim.x) {
    const int n1 = (int)a.neumann[t], n2 = (int)a.neumann[a.nn + t];
    const double nx = a.neumann[2 * a.nn + t], ny = a.neumann[3 * a.nn + t];
    if (n1 < 1 || n1 > a.N || n2 < 1 || n2 > a.N) continue;
    const double dxl = a.coords[n1 - 1] - a.coords[n2 - 1];
    const double dyl = a.coords[a.N + n1 - 1] - a.coords[a.N + n2 - 1];
    const double ln = 0.5 * sqrt(dxl * dxl + dyl * dyl);
    const int nds[2] = {n1 - 1, n2 - 1};
    for (int k = 0; k < 2; ++k) {
      const int n = nds[k];
      const double* Fn = a.F + 4 * n;
      const double s = -1.0 / a.winstepsize;
      atomicAdd(&w.b[n], ln * (s * Fn[0] * nx + s * Fn[2] * ny));
      atomicAdd(&w.b[a.N + n], ln * (s * Fn[1] * nx + s * Fn[3] * ny));
    }
  }
}

// Dirichlet flags; free = involved (unique(elementsFEM(:,1:8)) without its
// first entry) minus Dirichlet.
__global__ void k_dirichlet(Subpb2Args a, Ws w) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < a.nd; t += gridDim.x * blockDim.x) {
    const int n = a.dirichlet[t];
    if (n >= 1 && n <= a.N) w.dirn[n - 1] = 1;
  }
}

__global__ void k_free_and_lift(Subpb2Args a, Ws w) {
  // unique() sorts, and the reference drops the first entry (the 0 of absent
  // hanging nodes); without any 0 that drops the smallest node instead.
  const int drop = w.misc[0] ? -1 : w.misc[1] - 1;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += gridDim.x * blockDim.x) {
    bool fr = w.freen[n] && n != drop && !w.dirn[n];
    w.freen[n] = fr;
    // Uhat lift vector: U at Dirichlet nodes, 0 elsewhere (kept in x)
    w.x[n] = w.dirn[n] ? a.U[2 * n] : 0.0;
    w.x[a.N + n] = w.dirn[n] ? a.U[2 * n + 1] : 0.0;
  }
}

// b -= K * x_lift on free rows; x reset to the lifted values elsewhere later
__global__ void k_lift_rhs(Subpb2Args a, Ws w) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < a.N; n += gridDim.x * blockDim.x) {
    double su = 0, sv = 0;
    for (int k = w.rowptr[n]; k < w.rowptr[n + 1]; ++k) {
      const int c = w.col[k];
      su += w.val[k] * w.x[c];
      sv += w.val[k] * w.x[a.N + c];
    }
    w.b[n] -= su;
    w.b[a.N + n] -= sv;
  }
}

// ---- PCG ---------------------------------------------------------------------------
struct PcgArgs {
  Subpb2Args a;
  Ws w;
  int* iters;
  double* resid;
  int* status;
};

__global__ void __launch_bounds__(256) k_pcg(PcgArgs P) {
  __shared__ double red[32 * 4];
  const Subpb2Args& a = P.a;
  const Ws& w = P.w;
  const int N = a.N;
  const int nb = gridDim.x;
  int* cnt = &w.misc[2];
  int* gen = &w.misc[3];
  const long long spin_limit = a.spin_limit > 0 ? a.spin_limit : kSpinLimit;
  const int tid0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  // invalid node index (misc[4]) or a node in more than kMaxElemPerNode
  // elements (misc[5]): report and stop before any barrier
  if (w.misc[4] | w.misc[5]) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(P.status, 3);
    return;
  }
  double* part0 = w.part;             // set-up sums (4 slots)
  double* part1 = w.part + 4 * 1024;  // p.Ap (2 slots)
  double* part2 = w.part + 6 * 1024;  // r.z, |r|^2 (4 slots)
  // r = b on free rows, x = 0 there; z = r / diag; p = z
  double v[4] = {0, 0, 0, 0};
  for (int n = tid0; n < N; n += stride) {
    const bool f = w.freen[n];
    const double ru = f ? w.b[n] : 0.0, rv = f ? w.b[N + n] : 0.0;
    const double id = f ? 1.0 / w.diag[n] : 0.0;
    if (f) { w.x[n] = 0; w.x[N + n] = 0; }
    w.r[n] = ru; w.r[N + n] = rv;
    w.z[n] = ru * id; w.z[N + n] = rv * id;
    w.p[n] = ru * id; w.p[N + n] = rv * id;
    v[0] += ru * ru * id; v[1] += rv * rv * id;  // r.z
    v[2] += ru * ru; v[3] += rv * rv;            // |b|^2
  }
  block_partials(v, 4, part0, red);
  if (!grid_barrier(cnt, gen, nb, P.status, spin_limit)) return;
  double t0[4];
  totals(part0, 4, t0, red);
  double rz[2] = {t0[0], t0[1]};
  const double bn[2] = {sqrt(t0[2]), sqrt(t0[3])};
  const double tol = a.tol;
  bool conv[2] = {!(bn[0] > 0), !(bn[1] > 0)};
  int it = 0;
  double rn[2] = {bn[0], bn[1]};
  while (!(conv[0] && conv[1]) && it < a.maxit) {
    ++it;
    // Ap = K p (free rows), partial p.Ap
    double q[4] = {0, 0, 0, 0};
    for (int n = tid0; n < N; n += stride) {
      double su = 0, sv = 0;
      if (w.freen[n]) {
        for (int k = w.rowptr[n]; k < w.rowptr[n + 1]; ++k) {
          const int c = w.col[k];
          const double kv = w.val[k];
          su += kv * w.p[c];
          sv += kv * w.p[N + c];
        }
      }
      w.Ap[n] = su; w.Ap[N + n] = sv;
      q[0] += w.p[n] * su; q[1] += w.p[N + n] * sv;
    }
    block_partials(q, 2, part1, red);
    if (!grid_barrier(cnt, gen, nb, P.status, spin_limit)) return;
    double pAp[2];
    totals(part1, 2, pAp, red);
    double al[2];
    for (int c = 0; c < 2; ++c) al[c] = conv[c] ? 0.0 : rz[c] / pAp[c];
    double s[4] = {0, 0, 0, 0};
    for (int n = tid0; n < N; n += stride) {
      if (!w.freen[n]) continue;
      const double id = 1.0 / w.diag[n];
      for (int c = 0; c < 2; ++c) {
        const int k = c * N + n;
        w.x[k] += al[c] * w.p[k];
        w.r[k] -= al[c] * w.Ap[k];
        w.z[k] = w.r[k] * id;
        s[c] += w.r[k] * w.z[k];
        s[2 + c] += w.r[k] * w.r[k];
      }
    }
    block_partials(s, 4, part2, red);
    if (!grid_barrier(cnt, gen, nb, P.status, spin_limit)) return;
    double t[4];
    totals(part2, 4, t, red);
    double be[2];
    for (int c = 0; c < 2; ++c) {
      rn[c] = sqrt(t[2 + c]);
      be[c] = conv[c] ? 0.0 : t[c] / rz[c];
      rz[c] = t[c];
      if (!conv[c] && rn[c] <= tol * bn[c]) conv[c] = true;
    }
    for (int n = tid0; n < N; n += stride) {
      if (!w.freen[n]) continue;
      for (int c = 0; c < 2; ++c) {
        const int k = c * N + n;
        w.p[k] = w.z[k] + be[c] * w.p[k];
      }
    }
    if (!grid_barrier(cnt, gen, nb, P.status, spin_limit)) return;
  }
  // Uhat: solution on free nodes, U on Dirichlet nodes, 0 elsewhere
  for (int n = tid0; n < N; n += stride) {
    const bool f = w.freen[n], d = w.dirn[n];
    a.Uhat[2 * n] = f ? w.x[n] : (d ? a.U[2 * n] : 0.0);
    a.Uhat[2 * n + 1] = f ? w.x[N + n] : (d ? a.U[2 * n + 1] : 0.0);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *P.iters = it;
    const double r0 = bn[0] > 0 ? rn[0] / bn[0] : 0.0, r1 = bn[1] > 0 ? rn[1] / bn[1] : 0.0;
    *P.resid = fmax(r0, r1);
    if (!(conv[0] && conv[1])) atomicCAS(P.status, 0, 1);
  }
}

}  // namespace

size_t subpb2_workspace_bytes(int N, int E) {
  size_t total = 0;
  carve(nullptr, N, E, &total);
  return total + 256;
}

cudaError_t run_subpb2(const Subpb2Args& a, void* workspace, int* iters_dev, double* resid_dev,
                       int* status_dev, cudaStream_t s, long long* launches, int phase) {
  if (a.N <= 0) return cudaSuccess;
  Ws w = carve(workspace, a.N, a.E, nullptr);
  const int T = 256;
  const long long max_blocks = 8ll * current_sm_count();
  auto blocks = [&](long long n) { return (int)std::min<long long>((n + T - 1) / T, max_blocks); };
  long long nl = 0;
  if (phase & kSubpb2Structure) {
    // node graph, CSR pattern, Dirichlet flags and reference tables: they
    // depend on the mesh, the Dirichlet set and the Gauss order only
    k_init<<<blocks(a.N + 1), T, 0, s>>>(w, a.N); ++nl;
    if (a.E > 0) { k_degree<<<blocks(a.E), T, 0, s>>>(a, w); ++nl; }
    k_scan<<<1, 1024, 0, s>>>(w.deg, w.eptr, a.N); ++nl;
    if (a.E > 0) { k_fill_elist<<<blocks(a.E), T, 0, s>>>(a, w); ++nl; }
    k_rowlen<<<blocks(a.N), T, 0, s>>>(a, w); ++nl;
    k_scan<<<1, 1024, 0, s>>>(w.rowlen, w.rowptr, a.N); ++nl;
    k_fill_cols<<<blocks(a.N), T, 0, s>>>(a, w); ++nl;
    if (a.nd > 0) { k_dirichlet<<<blocks(a.nd), T, 0, s>>>(a, w); ++nl; }
    k_ref_tables<<<16, 64, 0, s>>>(a.gauss_order, w); ++nl;
  }
  if (!(phase & kSubpb2Solve)) {
    if (launches) *launches += nl;
    return cudaGetLastError();
  }
  cudaMemsetAsync(status_dev, 0, sizeof(int), s);
  k_zero_values<<<blocks(64ll * a.E > a.N ? 64ll * a.E : a.N), T, 0, s>>>(a, w); ++nl;
  if (a.E > 0) { k_element<<<blocks(8ll * a.E), T, 0, s>>>(a, w); ++nl; }
  if (a.nn > 0) { k_neumann<<<blocks(a.nn), T, 0, s>>>(a, w); ++nl; }
  k_free_and_lift<<<blocks(a.N), T, 0, s>>>(a, w); ++nl;
  k_lift_rhs<<<blocks(a.N), T, 0, s>>>(a, w); ++nl;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // cooperative persistent PCG: every block must be resident
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, T, 0);
  if (e != cudaSuccess) return e;
  int nb = std::min(nsm * std::max(per_sm, 1), (a.N + T - 1) / T);
  nb = std::max(1, std::min(nb, 1024));
  PcgArgs P{a, w, iters_dev, resid_dev, status_dev};
  void* args[] = {&P};
  e = cudaLaunchCooperativeKernel((const void*)k_pcg, dim3(nb), dim3(T), args, 0, s);
  ++nl;
  if (launches) *launches += nl;
  return e;
}

}  // namespace stdic
