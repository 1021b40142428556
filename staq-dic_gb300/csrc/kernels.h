// Internal kernel interface of libstaqdic (not part of the public C ABI).
#pragma once
#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

namespace stdic {

// SM count of the current device (queried once per device ordinal; 152 on
// GB300), for grid-stride launches sized as a multiple of the SMs.
int current_sm_count();

// Arguments of the IC-GN kernels (6-DOF first pass and 2-DOF Subpb1).
struct IcgnArgs {
  const void* f;
  const void* g;
  const uint8_t* mask;
  const void* dfdx;
  const void* dfdy;
  int W, H;
  int N;
  const double* coords;  // N x 2 column-major, 1-based
  // 6-DOF
  const double* U0;
  int ws_all;
  const int32_t* ws_list;  // optional
  double* F;
  double* Hpk;      // N x 21, optional
  uint8_t* mark;    // optional
  // 2-DOF
  const double* UOld;
  const double* FOld;
  const double* vdual;
  const int32_t* wsl2;  // N x 2
  double mu;
  // common
  double tol;
  double* U;
  int32_t* conv;
  int ws_max;   // largest requested subset size
  int npx_max;  // largest tile (pixels) after window growth
};

// Largest tile after the reference's window growth for a subset size ws.
inline int grown_tile_pixels(int ws) {
  // growth factor < sqrt(1/0.6) because fewer than 40 % of the pixels are masked
  const int wg = 2 * (int)((1.2910 * ws) / 2 + 1) + 2;
  return (wg + 1) * (wg + 1);
}

// Square box sizes (floats a side) of the TMA copies that stage the warped g
// footprint of a subset in shared memory; a subset takes the smallest box that
// holds its footprint with a 2-pixel margin (a multiple of 8: TMA's 16-byte
// rule for the inner dimension).
constexpr int kGBoxes = 9;
__host__ __device__ constexpr int gbox_side(int k) {  // 16, 24, 32, 40, 48, 64, 80, 96, 128
  return k < 5 ? 16 + 8 * k : (k == 5 ? 64 : (k == 6 ? 80 : (k == 7 ? 96 : 128)));
}

// 2-D tiled tensor map of a rows x W float image (W contiguous) with a box x
// box tile; false when TMA cannot describe it (base or pitch not 16-byte
// aligned, or the driver entry point is missing).
bool encode_image_map_f32(const void* base, long long W, long long rows, int box, CUtensorMap* m);

// Batched FP32 queue entry, precomputed per call on the device.
struct BatchedArgs {
  IcgnArgs a;
  const float* f32;
  const float* g32;
  const float* dfdx32;
  const float* dfdy32;
  const int32_t* order;   // node order of the work queue
  int* queue_head;        // two global work counters (team phase, single-warp phase)
  const int* n_big;       // split: number of queue entries of the team phase (device)
  int split;              // 1: large subsets on teams of warps_per_subset, the rest on single warps
  int smem_px_small;      // split: tile pixels of a single warp's share of the team slot
  // 6-DOF: the set-up stage appends every subset it leaves to the iterations
  // to one of two lists (order2[0..) for the wide teams, order2[N..) for single
  // warps; counts in n2[0], n2[1]), which the iteration stage then pulls
  int32_t* order2;
  int* n2;
  int split_ws;           // subsets at least this size (or masked) go to the wide-team list
  int gtile;              // floats of the staged g footprint per team (0: gather from global)
  int gtile_small;        // split: the same for a single warp's share
  int warps_per_subset;
  int two_dof;
  int frames;             // number of frame pairs stacked in g32 (multi-frame)
  long long g_stride;     // elements between stacked deformed frames
  unsigned char* scratch; // per-team global slices for tiles that exceed the shared slot
  int smem_px;            // tile pixels each team keeps in shared memory
  // 6-DOF split: stage 1 = per-subset set-up (writes st6, H6), stage 2 =
  // iterations (reads st6, Hinv6); the 2-DOF form runs fused (stage 0)
  int stage;
  void* st6;              // SubsetState6 per item
  double* H6;             // 21 per item: packed lower Hessian (row-major)
  double* Hinv6;          // 36 per item: the FP64 inverse Hessian (row-major) as FP32 pairs (hi, lo)
  // TMA staging of the warped g footprint: gbox_n tensor maps of g32 (W x
  // H*frames floats), gmap[k] with gbox_side(k)-square boxes; gbox_n = 0 stages
  // per element (cp.async) or gathers from global memory instead
  int gbox_n;
  int* tma_err;           // set to 1 when a footprint copy's bounded wait gives up
  // 6-DOF set-up stage over one band of a frame uploaded in row bands
  // (band_list set): the queue's nodes regrouped by the band whose rows they
  // need (band_list, with band_off[band] .. band_off[band + 1]), of which the
  // first band_nbig[band] go to the wide teams of the split form; band_list
  // null: the whole queue
  const int32_t* band_list;
  const int* band_off;
  const int* band_nbig;
  int band;
  CUtensorMap gmap[kGBoxes];
};

// Per-subset state handed from the 6-DOF set-up stage to the iterations.
struct SubsetState6 {
  int code;      // 0: iterate; otherwise the final ConvItPerEle (outputs already written)
  int ws;        // subset size after window growth
  int cntf;      // zero pixels of tempf in the original window
  int masked;    // 1 when the mask tile has a zero (tempf/DfDx/DfDy use the 4-conn selection)
  float meanf, bottomf, sabs, pad;
  // f-side parts of the b-vector, constant over the iterations:
  // Jf = sum J (tempf - meanf), J1 = sum J, with J the steepest-descent images
  float Jf[6], J1[6];
};

// list/counts (optional): the iteration stage's work lists of the set-up
// stage (list[0..counts[0]) and list[2n - counts[1]..2n)); only those subsets
// are factorised, packed at the front of the grid so that they spread evenly
// over the SMs
cudaError_t launch_factor6(const SubsetState6* st, const double* H6, double* Hinv6, int n,
                           const int32_t* list, const int* counts, cudaStream_t s);


// Size of one team's shared slot / global slice of the batched kernel.
// bytes per tile pixel of the per-subset arrays
int batched_tile_px_bytes(bool two);
size_t batched_team_bytes(int sm_px, bool two, int tw, int gtile);
size_t batched_scratch_bytes(int npx_max, bool two, long long warps);
int batched_blocks_per_sm(int tw, bool two, int threads, int smem_px, int gtile, int stage);

cudaError_t launch_interp(const void* F, long long M, long long N, long long P, const void* X,
                          const void* Y, long long n, void* out, int dtype, cudaStream_t s);
// err (optional, device) is set to 1 when a tile copy's bounded wait gives up.
cudaError_t launch_gradient(const void* img, const uint8_t* mask, int W, int H, void* dfdx,
                            void* dfdy, int dtype, cudaStream_t s, int* err = nullptr);
cudaError_t launch_intsearch(const double* f, const double* g, int W, int H, int Sx, int Sy,
                             double gx0, double gy0, int nx, int ny, int wsx, int wsy, int stepx,
                             int stepy, double* x, double* y, double* u, double* v, double* cc,
                             int32_t* peak, cudaStream_t s);
// Plain FP64 IC-GN, one CTA per node, in subset-size classes (CTA size and
// shared memory per class).  order: N device ints; qscratch: 512 device ints
// (the queue histogram and cursors); ranges: 12 device ints (class ranges, then one work counter per class).
// *kernels receives the number of kernels launched.
// cc.qfactors of the integer search: PCE and PPE of each grid point's full
// normxcorr2 map, normalised over the points; qf is npt x 2 (column-major),
// scratch holds intsearch_qfactor_scratch_bytes(...) bytes.
size_t intsearch_qfactor_scratch_bytes(int nx, int ny, int Sx, int Sy, int wsx, int wsy);
cudaError_t launch_intsearch_qfactors(const double* f, const double* g, int W, int Sx, int Sy, double gx0,
                                      double gy0, int nx, int ny, int wsx, int wsy, int stepx, int stepy,
                                      double* scratch, double* qf, cudaStream_t s);
// Streams and events on which the size classes run concurrently (nullptr:
// one after another on s): class 0 on s, class k on side[k-1], forked from s
// after the class ranges are known and joined back into s at the end.
struct PlainStreams {
  cudaStream_t side[3];
  cudaEvent_t fork;
  cudaEvent_t join[3];
};
cudaError_t launch_icgn6_plain(const IcgnArgs& a, int32_t* order, int* qscratch, int* ranges, cudaStream_t s,
                               int* kernels, const PlainStreams* ps = nullptr);
cudaError_t launch_icgn2_plain(const IcgnArgs& a, int32_t* order, int* qscratch, int* ranges, cudaStream_t s,
                               int* kernels, const PlainStreams* ps = nullptr);
// tmp_dev: five device 64-bit integers of scratch (the code statistics)
cudaError_t launch_badpoints(int32_t* conv, int N, double* U, double* F, int two_dof,
                             int* badnum_dev, unsigned long long* tmp_dev, cudaStream_t s);
cudaError_t launch_to_f32(const double* in, float* out, long long n, cudaStream_t s);
// Counting sort of the nodes by subset size into order: ascending 0 sorts by
// decreasing size, 1 by increasing size, 2 puts the subsets of at least big_ws
// pixels a side first (decreasing) and the rest after them (increasing).
// n_big (optional) receives the number of nodes whose size is at least big_ws.
// scratch: 512 device ints
cudaError_t launch_build_queue(const int32_t* ws_list, const int32_t* wsl2, int ws_all, int N,
                               int32_t* order, int* n_big, int* scratch, cudaStream_t s, int ascending = 0,
                               int big_ws = 0);
// The same sort of a 6-DOF queue (sizes ws_list or ws_all) with the nodes
// first grouped by row band, for a frame of H rows uploaded in nb bands
// (1, 2, 4 or 8; band b ends at row (b + 1) H / nb, the last at H): a node
// goes to the first band whose rows cover every row its set-up may read (its
// window grown to the largest size the mask can cause, around its rounded y
// coordinate coord_y).  band_off (nb + 1 ints) receives each band's first
// position and the total, band_big (nb ints) each band's nodes of at least
// big_ws pixels a side; n_big the total of those.  scratch: 2 * 256 *
// kQueueMaxBands device ints.
constexpr int kQueueMaxBands = 8;
cudaError_t launch_build_band_queue(const int32_t* ws_list, int ws_all, int N, const double* coord_y, int H, int nb,
                                    int32_t* order, int* n_big, int* band_off, int* band_big, int* scratch,
                                    cudaStream_t s, int ascending, int big_ws);
// Largest tile of a single warp's share of a split team slot.
int batched_small_px(int sm_px, bool two, int tw, int gtile);
cudaError_t launch_icgn_batched(const BatchedArgs& b, int blocks, int threads, cudaStream_t s);

// Adjoint of the subset ZNSSD cost (device pointers; f, g in FP64 when f64,
// else FP32; dg of the same type; mask, dU, dF, dg, cost may be null).
struct AdjointArgs {
  const void* f;
  const void* g;
  const uint8_t* mask;
  int W, H, N;
  const double* coords;
  const double* U;
  const double* F;
  int ws_all;
  const int32_t* ws_list;
  int ws_max;
  double* cost_n;  // N
  double* cost;    // 1: sum of the finite subset costs
  double* dU;
  double* dF;
  void* dg;
  int* head;       // work counter (scratch)
  int f64;
  int store;       // 1: keep interpolated subsets in shared memory between the passes
  int nsm;
};
cudaError_t launch_adjoint(const AdjointArgs& a, cudaStream_t s, long long* launches);

// Node -> element lists of a mesh (sorted per node), in ws of
// topo_workspace_bytes(N, E); *ptr (N + 1) and *list point into ws.
size_t topo_workspace_bytes(int N, int E);
cudaError_t build_topology(const int32_t* elems, int E, int N, void* ws, int** ptr, int** list,
                           cudaStream_t s);
// F (4N) = nodal strain of U (2N); NaN at nodes in no element.
cudaError_t launch_nodal_strain(const double* coords, int N, const int32_t* elems, int E, const double* U,
                                int gauss_order, const int* ptr, const int* list, double* F, cudaStream_t s);
// Fills the NaN nodes of U (2N) from their mesh neighbours; tmp holds
// fill_tmp_doubles(N) doubles.
size_t fill_tmp_doubles(int N);
cudaError_t launch_fill_nans(int N, const int32_t* elems, int E, const int* ptr, const int* list, double* U,
                             double* tmp, cudaStream_t s);
cudaError_t launch_copy_marked(const uint8_t* mark, int N, int width, const double* src, double* dst,
                               cudaStream_t s);
cudaError_t launch_sub(const double* a, const double* b, double* out, long long n, cudaStream_t s);

// FP64 complex FFTs (fft.cu): tw holds L/2 twiddles exp(-2 pi i k / L) made
// by launch_fft_twiddles; rows transforms of length L (a power of two, at most
// kFftMaxLen) in place, the inverse unscaled; out = in^T (rows x cols in).
constexpr int kFftMaxLen = 8192;
cudaError_t launch_fft_twiddles(double2* tw, int L, cudaStream_t s);
cudaError_t launch_fft_rows(double2* data, long long rows, int L, const double2* tw, bool inverse, cudaStream_t s);
cudaError_t launch_transpose_c(const double2* in, double2* out, int rows, int cols, cudaStream_t s);

// Multigrid integer search (funIntegerSearchMg.m).  fixed_ws holds
// mg_fixed_workspace_bytes(W, H) bytes (the integral images); grow(bytes)
// returns device scratch of at least that size (it may move between calls).
// Returns 0, -1 (argument or a MATLAB error of the reference, *err says
// which), -2 (CUDA), -3 (allocation), -5 (a bounded wait gave up) or -6 (the
// gridfit solve did not converge).
struct MgSearchOut {
  int nx = 0, ny = 0;                // node grid
  std::vector<double> xnodes, ynodes;
  std::vector<double> x3;            // u, v, cc.max on the grid, each ny x nx column-major
  std::vector<double> blocks;        // 5 x nblocks: final-level block centre x, y and u, v, cc.max
  long long nblocks = 0;
  double level1_u = 0, level1_v = 0; // the whole-region shift of level 1
  int cg_iters = 0;
};
size_t mg_fixed_workspace_bytes(int W, int H);
int integer_search_mg(const double* f, const double* g, int W, int H, const double gridx[2], const double gridy[2],
                      int winsize, const double step[2], void* fixed_ws, const std::function<void*(size_t)>& grow,
                      cudaStream_t s, long long* launches, MgSearchOut* out, const char** err);

// Quadtree mesh generation (GenerateQuadtreeMesh.m with MeshSetUp.m).
struct QuadtreeMeshOut {
  std::vector<double> x, y;                       // node coordinates
  std::vector<std::array<int, 8>> elems;          // elementsFEM rows
  std::vector<std::array<int, 3>> irregular;      // [node_a node_b midnode]
  std::vector<int> dirichlet;                     // markCoordHoleEdge, ascending
};
// mask: W x H device memory (0/1); gx, gy: the ny x nx search grids (host,
// column-major, row = y) as MeshSetUp receives them; grow(bytes) returns
// device scratch of at least that size.  Returns 0 or a STDIC_E_* code with
// *err set.
int quadtree_mesh_generate(const uint8_t* mask, int W, int H, const double* gx, const double* gy, int ny, int nx,
                           double winstepsize, double element_min_size, QuadtreeMeshOut* out,
                           const std::function<void*(size_t)>& grow, cudaStream_t s, long long* launches,
                           const char** err);

// funPOR_GPR: T (nT x np) and u_pred (nT1 x np) device, column-major; t_train,
// t_pre and the scalar outputs host; ws holds por_workspace_bytes(np, nT, nB).
size_t por_workspace_bytes(long long np, int nT, int nB);
int por_gpr(const double* T, int nT, long long np, const double* t_train, const double* t_pre, int nT1, int nB,
            double* u_pred, double* alpha, double* beta_pod, double* beta_gpr, void* ws, cudaStream_t s,
            long long* launches, const char** err);

// Subpb2 (FEM).  All pointers are device pointers.
struct Subpb2Args {
  const double* coords;
  int N;
  const int32_t* elems;
  int E;
  const int32_t* dirichlet;
  int nd;
  const double* neumann;
  int nn;
  int gauss_order;
  double beta, mu, alpha, winstepsize;
  const double* U;
  const double* F;
  double tol;
  int maxit;
  double* Uhat;
  // polls a PCG block waits at a grid barrier before it gives up with status
  // 2 (STDIC_E_TIMEOUT); 0 takes the default of 2^24
  long long spin_limit;
};
// workspace: caller-provided device memory of subpb2_workspace_bytes(N, E)
size_t subpb2_workspace_bytes(int N, int E);
// phase: kSubpb2Structure builds the node graph, CSR pattern, Dirichlet flags
// and reference-element tables in the workspace; kSubpb2Solve assembles the
// values for a.U and a.F on that structure and runs the PCG.  A solve-only call
// needs an earlier structure call on the same workspace, mesh, Dirichlet set
// and Gauss order.
constexpr int kSubpb2Structure = 1, kSubpb2Solve = 2, kSubpb2All = 3;
cudaError_t run_subpb2(const Subpb2Args& a, void* workspace, int* iters_dev, double* resid_dev,
                       int* status_dev, cudaStream_t s, long long* launches, int phase = kSubpb2All);

}  // namespace stdic
