// Quadtree mesh generation (func_quadtree/GenerateQuadtreeMesh.m:18-133 with
// func/MeshSetUp.m, func_quadtree/funMarkEdge.m, func_quadtree/funMarkInside.m
// and func_quadtree/refinement/QrefineR.m + provideGeometricData.m).
//
// The mask tests over every element's bounding box (its value range for the
// refinement marks, its sum for the removal of elements inside the mask) run
// on the GPU, one warp per element.  The refinement itself -- the sorted edge
// list, the closure that keeps one hanging node per edge, red refinement and
// the node numbering -- is graph bookkeeping over a few hundred thousand
// integers per pass and runs on the host, in the reference's order, so that
// node and element numbers come out exactly as the reference numbers them.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "../../include/staqdic.h"
#include "device_common.cuh"
#include "kernels.h"

namespace stdic {
namespace {

// Min, max and sum of the mask over each element box [x0, x1] x [y0, y1]
// (1-based, inclusive; W x H column-major mask).  One warp per box.
__global__ void __launch_bounds__(256) mask_box_kernel(const uint8_t* __restrict__ mask, int W, int H,
                                                       const int4* __restrict__ boxes, int n,
                                                       int* __restrict__ range, long long* __restrict__ sum) {
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int e = blockIdx.x * wpb + (threadIdx.x >> 5); e < n; e += gridDim.x * wpb) {
    const int4 b = boxes[e];
    const int x0 = max(b.x, 1), x1 = min(b.y, W), y0 = max(b.z, 1), y1 = min(b.w, H);
    const int bw = x1 - x0 + 1, bh = y1 - y0 + 1;
    int mn = 255, mx = 0;
    long long s = 0;
    if (bw > 0 && bh > 0) {
      for (int q = lane; q < bw * bh; q += 32) {
        const int i = q % bw, j = q / bw;
        const int v = mask[(long long)(y0 - 1 + j) * W + (x0 - 1 + i)];
        mn = min(mn, v);
        mx = max(mx, v);
        s += v;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if (lane == 0) {
      range[e] = (bw > 0 && bh > 0) ? mx - mn : 0;
      sum[e] = s;
    }
  }
}

using Quad = std::array<int, 4>;
using Tri = std::array<int, 3>;

struct Mesh {
  std::vector<double> x, y;  // node coordinates (node k at index k - 1)
  std::vector<Quad> el;
  std::vector<Tri> irr;      // [node_a node_b midnode], node_a < node_b
};

// provideGeometricData.m with the irregular list as its triangles: the edge
// list sorted as unique(sort(edges, 2), 'rows') orders it, and each row's
// edges.  Rows of the edge list come triangle edges first (edge k of every
// triangle, k = 1..3), then quadrilateral edges (edge k of every element).
struct EdgeData {
  std::vector<std::array<int, 2>> nodes;          // edge -> (a, b), a < b
  std::vector<std::array<int, 3>> irr2edges;      // coarse edge, then the two half edges
  std::vector<std::array<int, 4>> el2edges;
};

EdgeData geometric_data(const Mesh& m) {
  const size_t nI = m.irr.size(), nE = m.el.size();
  std::vector<std::array<long long, 3>> rows;  // (a, b, row)
  rows.reserve(3 * nI + 4 * nE);
  long long r = 0;
  for (int k = 0; k < 3; ++k)
    for (size_t i = 0; i < nI; ++i, ++r) {
      const int a = m.irr[i][k], b = m.irr[i][(k + 1) % 3];
      rows.push_back({std::min(a, b), std::max(a, b), r});
    }
  for (int k = 0; k < 4; ++k)
    for (size_t i = 0; i < nE; ++i, ++r) {
      const int a = m.el[i][k], b = m.el[i][(k + 1) % 4];
      rows.push_back({std::min(a, b), std::max(a, b), r});
    }
  std::sort(rows.begin(), rows.end());
  EdgeData d;
  std::vector<int> ie(rows.size());
  for (size_t k = 0; k < rows.size(); ++k) {
    if (k == 0 || rows[k][0] != rows[k - 1][0] || rows[k][1] != rows[k - 1][1])
      d.nodes.push_back({(int)rows[k][0], (int)rows[k][1]});
    ie[rows[k][2]] = (int)d.nodes.size() - 1;
  }
  d.irr2edges.resize(nI);
  for (int k = 0; k < 3; ++k)
    for (size_t i = 0; i < nI; ++i) d.irr2edges[i][k] = ie[k * nI + i];
  d.el2edges.resize(nE);
  for (int k = 0; k < 4; ++k)
    for (size_t i = 0; i < nE; ++i) d.el2edges[i][k] = ie[3 * nI + k * nE + i];
  return d;
}

// QrefineR.m: red refinement of the marked elements (0-based ids) with the
// closure that refines every element with three marked edges or a marked
// edge that already holds a hanging node, so no edge gets a second one.
void qrefine(Mesh& m, const std::vector<int>& marked) {
  const EdgeData d = geometric_data(m);
  const size_t nE = m.el.size(), nI = m.irr.size(), nEd = d.nodes.size();
  std::vector<long long> e2n(nEd, 0);
  for (int e : marked)
    for (int k = 0; k < 4; ++k) e2n[d.el2edges[e][k]] = 1;
  for (size_t i = 0; i < nI; ++i) e2n[d.irr2edges[i][0]] = 1;
  for (;;) {
    // elements not fully marked with three marked edges or an edge of -1,
    // taken from one snapshot, then all their edges marked
    std::vector<int> kdx;
    for (size_t e = 0; e < nE; ++e) {
      int s = 0;
      long long mn = 1;
      for (int k = 0; k < 4; ++k) {
        const long long v = e2n[d.el2edges[e][k]];
        s += v != 0;
        mn = std::min(mn, v);
      }
      if (s < 4 && (s > 2 || mn < 0)) kdx.push_back((int)e);
    }
    for (int e : kdx)
      for (int k = 0; k < 4; ++k)
        if (e2n[d.el2edges[e][k]] == 0) e2n[d.el2edges[e][k]] = 1;
    // a coarse edge whose half edge is marked: its own element must refine
    std::vector<int> flag;
    for (size_t i = 0; i < nI; ++i)
      if (e2n[d.irr2edges[i][1]] != 0 || e2n[d.irr2edges[i][2]] != 0) flag.push_back(d.irr2edges[i][0]);
    size_t nswap = 0;
    std::vector<int> swap;
    for (int f : flag)
      if (e2n[f] != -1) swap.push_back(f);
    for (int f : swap) e2n[f] = -1;
    nswap = swap.size();
    if (kdx.empty() && nswap == 0) break;
  }
  for (size_t i = 0; i < nI; ++i) e2n[d.irr2edges[i][0]] = -1;
  // new midpoint nodes in edge order
  long long next = (long long)m.x.size();
  for (size_t ed = 0; ed < nEd; ++ed)
    if (e2n[ed] > 0) {
      e2n[ed] = ++next;
      const int a = d.nodes[ed][0], b = d.nodes[ed][1];
      m.x.push_back((m.x[a - 1] + m.x[b - 1]) / 2);
      m.y.push_back((m.y[a - 1] + m.y[b - 1]) / 2);
    }
  for (size_t i = 0; i < nI; ++i) e2n[d.irr2edges[i][0]] = m.irr[i][2];
  std::vector<Quad> nn(nE);
  std::vector<int> reftyp(nE);
  for (size_t e = 0; e < nE; ++e) {
    int t = 0;
    for (int k = 0; k < 4; ++k) {
      nn[e][k] = (int)e2n[d.el2edges[e][k]];
      t |= (nn[e][k] != 0) << k;
    }
    reftyp[e] = t;
  }
  // centre nodes of the red elements, in element order
  std::vector<int> mid(nE, 0);
  for (size_t e = 0; e < nE; ++e)
    if (reftyp[e] == 15) {
      mid[e] = (int)m.x.size() + 1;
      const Quad& c = m.el[e];
      m.x.push_back((m.x[c[0] - 1] + m.x[c[1] - 1] + m.x[c[2] - 1] + m.x[c[3] - 1]) / 4);
      m.y.push_back((m.y[c[0] - 1] + m.y[c[1] - 1] + m.y[c[2] - 1] + m.y[c[3] - 1]) / 4);
    }
  std::vector<Quad> out;
  out.reserve(nE * 2);
  for (size_t e = 0; e < nE; ++e) {
    const Quad& c = m.el[e];
    if (reftyp[e] < 15) {
      out.push_back(c);
    } else {
      const Quad& n = nn[e];
      out.push_back({c[0], n[0], mid[e], n[3]});
      out.push_back({c[1], n[1], mid[e], n[0]});
      out.push_back({c[2], n[2], mid[e], n[1]});
      out.push_back({c[3], n[3], mid[e], n[2]});
    }
  }
  // the new hanging nodes: edges of the elements kept whole (edge by edge),
  // then the half edges of the old hanging edges that were split again
  std::vector<Tri> irr;
  for (int k = 0; k < 4; ++k)
    for (size_t e = 0; e < nE; ++e)
      if (reftyp[e] > 0 && reftyp[e] < 15 && nn[e][k] != 0) {
        const auto& ab = d.nodes[d.el2edges[e][k]];
        irr.push_back({ab[0], ab[1], nn[e][k]});
      }
  for (int k = 0; k < 2; ++k)
    for (size_t i = 0; i < nI; ++i) {
      const long long v0 = e2n[d.irr2edges[i][1]], v1 = e2n[d.irr2edges[i][2]];
      const long long v = k == 0 ? v0 : v1;
      if (v0 + v1 != 0 && v != 0) {
        const auto& ab = d.nodes[d.irr2edges[i][1 + k]];
        irr.push_back({ab[0], ab[1], (int)v});
      }
    }
  m.el.swap(out);
  m.irr.swap(irr);
}

}  // namespace

// Element boxes on the device -> value range and sum of the mask in each.
cudaError_t launch_mask_boxes(const uint8_t* mask, int W, int H, const int4* boxes, int n, int* range,
                              long long* sum, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int wpb = 8;
  int blocks = (n + wpb - 1) / wpb;
  blocks = std::min(blocks, 32 * current_sm_count());
  mask_box_kernel<<<blocks, 32 * wpb, 0, s>>>(mask, W, H, boxes, n, range, sum);
  return cudaGetLastError();
}

int quadtree_mesh_generate(const uint8_t* mask, int W, int H, const double* gx, const double* gy, int ny, int nx,
                           double winstepsize, double element_min_size, QuadtreeMeshOut* out,
                           const std::function<void*(size_t)>& grow, cudaStream_t s, long long* launches,
                           const char** err) {
  *err = nullptr;
  Mesh m;
  // MeshSetUp.m: node i of the transposed grids (x fastest), elements row by row
  const int M = nx, N = ny;
  m.x.resize((size_t)M * N);
  m.y.resize((size_t)M * N);
  for (int b = 0; b < N; ++b)
    for (int a = 0; a < M; ++a) {
      m.x[(size_t)b * M + a] = gx[(size_t)a * N + b];
      m.y[(size_t)b * M + a] = gy[(size_t)a * N + b];
    }
  for (int j = 1; j < N; ++j)
    for (int i = 1; i < M; ++i)
      m.el.push_back({(j - 1) * M + i, (j - 1) * M + i + 1, j * M + i + 1, j * M + i});
  double xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY;
  for (size_t k = 0; k < m.x.size(); ++k) {
    xmin = std::min(xmin, m.x[k]); xmax = std::max(xmax, m.x[k]);
    ymin = std::min(ymin, m.y[k]); ymax = std::max(ymax, m.y[k]);
  }
  // boxes of the current elements -> (range, sum) from the device
  std::vector<int4> boxes;
  std::vector<int> range;
  std::vector<long long> sum;
  auto box_of = [&](const Quad& c, double* bx) {
    double a = INFINITY, b = -INFINITY, cc = INFINITY, dd = -INFINITY;
    for (int k = 0; k < 4; ++k) {
      a = std::min(a, m.x[c[k] - 1]); b = std::max(b, m.x[c[k] - 1]);
      cc = std::min(cc, m.y[c[k] - 1]); dd = std::max(dd, m.y[c[k] - 1]);
    }
    bx[0] = a; bx[1] = b; bx[2] = cc; bx[3] = dd;
  };
  auto mask_stats = [&]() -> int {
    const size_t n = m.el.size();
    boxes.resize(n);
    for (size_t e = 0; e < n; ++e) {
      double bx[4];
      box_of(m.el[e], bx);
      // MATLAB's colon a:b over the mask: every integer from a up to b
      boxes[e] = make_int4((int)std::ceil(bx[0]), (int)std::floor(bx[1]), (int)std::ceil(bx[2]),
                           (int)std::floor(bx[3]));
    }
    range.assign(n, 0);
    sum.assign(n, 0);
    if (n == 0) return 0;
    const size_t bytes = n * (sizeof(int4) + sizeof(int) + sizeof(long long)) + 64;
    unsigned char* ws = (unsigned char*)grow(bytes);
    if (!ws) { *err = "workspace allocation failed"; return STDIC_E_NOMEM; }
    int4* db = (int4*)ws;
    long long* ds = (long long*)(((uintptr_t)(db + n) + 15) & ~(uintptr_t)15);
    int* dr = (int*)(ds + n);
    cudaError_t e = cudaMemcpyAsync(db, boxes.data(), n * sizeof(int4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_mask_boxes(mask, W, H, db, (int)n, dr, ds, s);
    if (e == cudaSuccess) ++*launches;
    if (e == cudaSuccess) e = cudaMemcpyAsync(range.data(), dr, n * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sum.data(), ds, n * sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { *err = cudaGetErrorString(e); return STDIC_E_CUDA; }
    return 0;
  };
  // GenerateQuadtreeMesh.m:24-36: refine until no element is marked
  for (;;) {
    int rc = mask_stats();
    if (rc) return rc;
    std::vector<int> marked;
    for (size_t e = 0; e < m.el.size(); ++e) {
      double bx[4];
      box_of(m.el[e], bx);
      const double size = std::min(std::fabs(bx[1] - bx[0]), std::fabs(bx[3] - bx[2]));
      if (range[e] > 0 && size > element_min_size) marked.push_back((int)e);
    }
    qrefine(m, marked);
    if (marked.empty()) break;
  }
  // :45-54: corners from the one at (min x, min y): rank by (x - xmin)^2 +
  // 2 (y - ymin)^2 (stable) and take the ranks in the order 1 2 4 3
  for (auto& c : m.el) {
    double xs[4], ys[4], t[4];
    for (int k = 0; k < 4; ++k) { xs[k] = m.x[c[k] - 1]; ys[k] = m.y[c[k] - 1]; }
    const double x0 = *std::min_element(xs, xs + 4), y0 = *std::min_element(ys, ys + 4);
    for (int k = 0; k < 4; ++k) t[k] = (xs[k] - x0) * (xs[k] - x0) + 2 * ((ys[k] - y0) * (ys[k] - y0));
    int r[4] = {0, 1, 2, 3};
    std::stable_sort(r, r + 4, [&](int a, int b) { return t[a] < t[b]; });
    const Quad old = c;
    c = {old[r[0]], old[r[1]], old[r[3]], old[r[2]]};
  }
  // :57-75: hanging-node columns 5 (edge 2-3), 6 (3-4), 7 (4-1), 8 (1-2) of
  // the first element holding each irregular edge, in the reference's order
  // of orientation checks
  const size_t nE = m.el.size();
  std::vector<std::array<int, 8>> el8(nE);
  for (size_t e = 0; e < nE; ++e) {
    for (int k = 0; k < 4; ++k) el8[e][k] = m.el[e][k];
    for (int k = 4; k < 8; ++k) el8[e][k] = 0;
  }
  static const int chk[8][3] = {{0, 1, 7}, {1, 2, 4}, {2, 3, 5}, {3, 0, 6}, {1, 0, 7}, {2, 1, 4}, {3, 2, 5}, {0, 3, 6}};
  for (int c = 0; c < 8; ++c) {
    std::unordered_map<unsigned long long, int> first;
    first.reserve(nE * 2);
    for (size_t e = 0; e < nE; ++e) {
      const unsigned long long key = ((unsigned long long)(unsigned)m.el[e][chk[c][0]] << 32) |
                                     (unsigned)m.el[e][chk[c][1]];
      first.emplace(key, (int)e);
    }
    // every (element, column) is written at most once (an irregular edge is
    // listed once, and both orientations of one element's edge go to one
    // column), so the order of the checks does not matter
    for (const auto& t : m.irr) {
      const unsigned long long key = ((unsigned long long)(unsigned)t[0] << 32) | (unsigned)t[1];
      auto it = first.find(key);
      if (it != first.end()) el8[it->second][chk[c][2]] = t[2];
    }
  }
  // funMarkInside.m: remove the elements whose box holds fewer than half of
  // (xmax - xmin)(ymax - ymin) mask ones
  int rc = mask_stats();
  if (rc) return rc;
  std::vector<std::array<int, 8>> kept;
  for (size_t e = 0; e < nE; ++e) {
    double bx[4];
    box_of(m.el[e], bx);
    if (!((double)sum[e] < 0.5 * (bx[1] - bx[0]) * (bx[3] - bx[2]))) kept.push_back(el8[e]);
  }
  // :79-133: the refined elements and the border band, grown twice by
  // element adjacency
  std::vector<char> in(m.x.size() + 1, 0);
  const double step = winstepsize;
  for (const auto& c : kept) {
    const double x1 = m.x[c[0] - 1], y1 = m.y[c[0] - 1], x3 = m.x[c[2] - 1], y3 = m.y[c[2] - 1];
    const double diag = std::sqrt((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3));
    const bool sel = diag < 0.99 * std::sqrt(2.0) * step || x1 < xmin + 1.01 * step || x3 > xmax - 1.01 * step ||
                     y1 < ymin + 1.01 * step || y3 > ymax - 1.01 * step;
    if (sel)
      for (int k = 0; k < 8; ++k)
        if (c[k] > 0) in[c[k]] = 1;
  }
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<char> nin(in.size(), 0);
    for (const auto& c : kept) {
      bool hit = false;
      for (int k = 0; k < 8 && !hit; ++k) hit = c[k] > 0 && in[c[k]];
      if (hit)
        for (int k = 0; k < 8; ++k)
          if (c[k] > 0) nin[c[k]] = 1;
    }
    in.swap(nin);
  }
  out->x = m.x;
  out->y = m.y;
  out->elems = kept;
  out->irregular = m.irr;
  out->dirichlet.clear();
  for (size_t k = 1; k < in.size(); ++k)
    if (in[k]) out->dirichlet.push_back((int)k);
  return 0;
}

}  // namespace stdic
