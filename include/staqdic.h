/* staqdic.h — C ABI of the GB300 (sm_103a) STAQ-DIC augmented-Lagrangian hot path.
 *
 * Each entry point replaces one routine of the reference (paths relative to the
 * STAQ-DIC repository) and keeps its argument meaning, so a MEX gateway can call
 * it with the arrays MATLAB already holds:
 *
 *   stdic_interp_bicubic   ba_interp2.cpp:318-335 (mexFunction) / :184-234
 *   stdic_img_gradient     func/funImgGradient.m:1-88
 *   stdic_integer_search   func/funIntegerSearch.m:3-203 + func/findpeak.m:1-68
 *   stdic_integer_search_mg func/funIntegerSearchMg.m:3-343 (+ findpeak.m, gridfit.m 'springs')
 *   stdic_icgn_subsets     func_quadtree/funICGNQuadtree.m:1-451 (N nodes at once)
 *   stdic_icgn_local       func_quadtree/LocalICGNQuadtree.m:1-177
 *   stdic_subpb1_subsets   func/funICGN_Subpb1.m:1-474 (N nodes at once)
 *   stdic_subpb1           func_quadtree/Subpb1Quadtree.m:1-191
 *   stdic_subpb2           func_quadtree/Subpb2Quadtree.m:1-413
 *   stdic_quadtree_mesh    func_quadtree/GenerateQuadtreeMesh.m:18-133 (+ MeshSetUp.m,
 *                          refinement/QrefineR.m)
 *   stdic_por_gpr          func/funPOR_GPR.m:1-99
 *   stdic_icgn_adjoint     no counterpart in the reference (gradient of the
 *                          ZNSSD cost of the IC-GN subsets)
 *
 * Conventions (MATLAB's):
 *   - arrays are column-major, first index contiguous; an image is W x H with
 *     x = dim 1 (the reference stores images transposed, Img(x, y));
 *   - node coordinates are 1-based pixel positions (N x 2, x column first);
 *   - U is interleaved [u1 v1 u2 v2 ...]; F is [F11 F21 F12 F22] per node;
 *   - packed Hessians are N x 21 (lower triangle, column by column);
 *   - elementsFEM is E x 8 int32, 1-based, 0 = no hanging node.
 *
 * Memory: every pointer may be host memory (MATLAB's arrays) or device memory
 * of the context's GPU.  Host buffers are staged through a context-owned device
 * workspace and the call returns after the results are copied back.  When every
 * pointer of a call is device memory the call is asynchronous on the context's
 * stream (per-node codes are ready after stream synchronisation).  Pinned host
 * memory (cudaHostAlloc, cudaHostRegister) lets the batched LocalICGNQuadtree
 * calls overlap copies with kernels: the deformed frame is uploaded on a
 * context-owned second stream during the set-up kernels, and HtempPar is
 * downloaded during the iterations; in stdic_icgn_local the reference frame,
 * its gradients and the mask are uploaded in row bands (STDIC_UPLOAD_BANDS:
 * 0, 1, 2, 4 or 8, default 4), each band's set-up kernel starting when its
 * rows arrive.  Pageable memory gives the same results with the copies in
 * order.
 *
 * Errors: 0 on success, a negative STDIC_E_* code otherwise (stdic_last_error
 * gives text).  Per-node failures never raise: they are reported through the
 * ConvItPerEle codes exactly as the reference writes them (1..100 converged at
 * that iteration, 101 not converged / NaN / warp out of image, 102 >= 40 % of
 * the subset masked, 103 empty subset, -1 MATLAB run-time error in
 * funICGNQuadtree; 0 with NaN U for a run-time error inside Subpb1Quadtree).
 *
 * Threading: a context owns one CUDA stream and a workspace; calls on one
 * context must not overlap.  Distinct contexts are independent.
 */
#ifndef STAQDIC_H
#define STAQDIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  STDIC_OK = 0,
  STDIC_E_ARG = -1,         /* invalid argument (sizes, odd subset size, ...) */
  STDIC_E_CUDA = -2,        /* CUDA runtime error */
  STDIC_E_NOMEM = -3,       /* device allocation failed */
  STDIC_E_UNSUPPORTED = -4, /* option the reference path cannot take */
  STDIC_E_TIMEOUT = -5,     /* a bounded device wait gave up */
  STDIC_E_NOTCONV = -6      /* iterative solver did not reach its tolerance */
};

enum { STDIC_F64 = 0, STDIC_F32 = 1 };

/* precision/form of the IC-GN solvers */
enum {
  STDIC_PLAIN_F64 = 0,   /* one subset per CTA, FP64, reproduces the reference */
  STDIC_BATCHED_F32 = 1  /* persistent kernel over a size-sorted queue: FP32
                            interpolation and residuals, per-lane FP32 FMA sums
                            reduced across lanes in FP32, the 6x6 (2x2) system
                            factorised and inverted in FP64 and applied in
                            double-float arithmetic */
};

typedef struct stdic_ctx stdic_ctx;

/* One reference/deformed frame pair as funICGNQuadtree sees it:
 * ImgRef (f), ImgDef (g), Df.ImgRefMask, Df.DfDx, Df.DfDy ((W-6) x (H-6)).
 * dtype applies to f, g, dfdx and dfdy.  STDIC_PLAIN_F64 needs STDIC_F64 data;
 * STDIC_BATCHED_F32 takes either (FP64 data is converted once per call). */
typedef struct {
  const void* f;
  const void* g;
  const uint8_t* mask;
  const void* dfdx;
  const void* dfdy;
  int W, H;
  int dtype;
} stdic_frame;

/* Context on CUDA device `device`.  Its own stream is a blocking stream:
 * work on it is ordered with the legacy default stream, so device buffers
 * produced or consumed there (the default stream of most frameworks) need no
 * extra synchronisation.  A call that stages host buffers returns after its
 * results are on the host; a call on device buffers only returns after its
 * work is queued on the context's stream. */
int stdic_ctx_create(stdic_ctx** ctx, int device);
int stdic_ctx_destroy(stdic_ctx* ctx);
/* Use an external cudaStream_t (NULL restores the context's own stream). */
int stdic_ctx_set_stream(stdic_ctx* ctx, void* cuda_stream);
const char* stdic_last_error(const stdic_ctx* ctx);
/* Number of kernels this context launched since creation (instrumentation;
 * no counterpart in the reference). */
long long stdic_kernel_launches(const stdic_ctx* ctx);
/* Bound, in polls, of every grid-barrier wait of the cooperative Subpb2 PCG
 * run by this context (stdic_subpb2, stdic_admm); 0 restores the default of
 * 2^24.  A wait that runs out makes the call return STDIC_E_TIMEOUT and leaves
 * the context usable.  Instrumentation and failure-detection testing; no
 * counterpart in the reference. */
int stdic_ctx_set_wait_limit(stdic_ctx* ctx, long long polls);
/* Device time in ms of the last IC-GN solver kernel (plain or batched), from
 * CUDA events on the launching stream; -1 if none ran.  Waits for that kernel.
 * Instrumentation; no counterpart in the reference. */
double stdic_last_solver_ms(stdic_ctx* ctx);

/* Z = ba_interp2(F, X, Y, 'cubic').  F is M x N x P (P layers), X/Y hold n
 * points (X indexes dim 2, Y dim 1, 1-based); out is n x P.  dtype STDIC_F64 or
 * STDIC_F32 for all of F, X, Y, out.  Bit-identical to the reference's
 * compiled ba_interp2.cpp on x86-64 (no fused multiply-add). */
int stdic_interp_bicubic(stdic_ctx* ctx, const void* F, int64_t M, int64_t N, int64_t P,
                         const void* X, const void* Y, int64_t n, void* out, int dtype);

/* Df = funImgGradient(ImgRef, ImgDef, ImgRefMask): dfdx, dfdy are (W-6) x (H-6).
 * dtype is the element type of img, dfdx and dfdy. */
int stdic_img_gradient(stdic_ctx* ctx, const void* img, const uint8_t* mask, int W, int H,
                       void* dfdx, void* dfdy, int dtype);

/* Grid of funIntegerSearch after its border shrink (funIntegerSearch.m:14-25):
 * returns nx, ny of the ny x nx outputs. */
int stdic_integer_search_grid(int W, int H, const int S[2], const double gridx[2],
                              const double gridy[2], const int winsize[2],
                              const int winstepsize[2], int* nx, int* ny);

/* [x,y,u,v,cc] = funIntegerSearch(f, g, S, gridx, gridy, winsize, winstepsize, 0, ..).
 * f, g are W x H double.  Outputs are ny x nx (row = y index) column-major;
 * cc is cc.max.  peak_rc (optional, 2 x ny x nx planes) receives the 1-based
 * integer argmax (row, col) of each cropped (2S+3)^2 correlation map; 0 where
 * normxcorr2 throws (constant template), where u, v, cc are NaN.  qfactors
 * (optional, (ny nx) x 2 column-major, rows in the reference's point order,
 * x fastest) receives cc.qfactors (funIntegerSearch.m:129-131,156,175-176,
 * 211-264): the peak-to-correlation-energy and peak-to-entropy ratios of each
 * point's full normxcorr2 map, each column shifted to start at 0 and divided
 * by its largest value, Inf before the normalisation where normxcorr2 throws. */
int stdic_integer_search(stdic_ctx* ctx, const double* f, const double* g, int W, int H,
                         const int S[2], const double gridx[2], const double gridy[2],
                         const int winsize[2], const int winstepsize[2], double* x, double* y,
                         double* u, double* v, double* cc, int32_t* peak_rc, double* qfactors);

/* [xGrid, yGrid, uGrid, vGrid, cc] = funIntegerSearchMg(f, g, gridx, gridy, winsize,
 * winstepsize) (func/funIntegerSearchMg.m:3-343, the multigrid search that
 * IntegerSearch.m:125 calls for large displacements): normxcorr2 of the whole
 * region, then blocks halved level by level, each searched within +-5 px of
 * its parent's shift, and the block-centre displacements fitted to the node
 * grid by gridfit with the springs regularizer.  f, g are W x H double;
 * gridx, gridy the [first last] region (1-based); winstepsize [x y].  The node
 * grid is chosen inside the routine: counts receives [nx ny], and x, y, u, v,
 * cc (cc.max; each optional) receive ny x nx column-major arrays (row = y).
 * capacity is the number of elements each given output holds;
 * (floor((gridx[1]-gridx[0])/winstepsize[0]) + 1) *
 * (floor((gridy[1]-gridy[0])/winstepsize[1]) + 1) always suffices.  The
 * reference's cc.qfactors (quality factors of the last level's maps) are not
 * produced: its caller on this path does not read them.  Errors where the
 * reference raises: a region too small for the border gaps or wider than 4096
 * px, a constant or non-finite region at level 1, fewer than 3 blocks for
 * gridfit (STDIC_E_ARG); STDIC_E_NOTCONV if the gridfit solve misses its
 * tolerance.  blocks (optional, nblocks x 5 column-major, block_capacity rows)
 * receives the last level's blocks before the fit -- centre x, centre y, u,
 * v and cc.max, the reference's tempx, tempy, tempu, tempv, tempPhi
 * (:300-306), NaN u, v and cc.max 0 where a block's search failed; nblocks
 * (optional) receives their number. */
int stdic_integer_search_mg(stdic_ctx* ctx, const double* f, const double* g, int W, int H,
                            const double gridx[2], const double gridy[2], int winsize,
                            const double winstepsize[2], double* x, double* y, double* u, double* v,
                            double* cc, int64_t capacity, int32_t counts[2], double* blocks,
                            int64_t block_capacity, int64_t* nblocks);

/* LocalICGNQuadtree(U0, coordinatesFEM, Df, ImgRef, ImgDef, DICpara, 'GaussNewton', tol)
 * without its NaN-fill tail (out of this path): U (2N) and F (4N) carry NaN at
 * the bad subsets the reference marks.  winsize is DICpara.winsize; ws_list
 * (optional, N int32) gives a subset size per node instead.  Hpk is HtempPar
 * (N x 21), conv is ConvItPerEle, mark_hole (optional, N) flags the nodes of
 * markCoordHoleStrain, badnum (optional) receives LocalICGNBadPtNum.
 * Only 'GaussNewton' exists: the reference's 'LevenbergMarquardt' branch calls
 * ImgDef.eval on a spline object and cannot run on image arrays. */
int stdic_icgn_local(stdic_ctx* ctx, const stdic_frame* fr, const double* U0,
                     const double* coords, int N, int winsize, const int32_t* ws_list, double tol,
                     double* U, double* F, double* Hpk, int32_t* conv, uint8_t* mark_hole,
                     int* badnum, int precision);

/* [U,F,stepwithinwhile,HGlobal] = funICGNQuadtree(U0, x0, y0, Df, ImgRef, ImgDef,
 * winsize, tol, 'GaussNewton') for N nodes at once (x0, y0 = round(coords)):
 * the per-node loop of LocalICGNQuadtree without its bad-subset filter.  A
 * MATLAB run-time error of the routine gives code -1 and NaN outputs.
 * Replaces func_quadtree/funICGNQuadtree.m:1-451. */
int stdic_icgn_subsets(stdic_ctx* ctx, const stdic_frame* fr, const double* U0,
                       const double* coords, int N, int winsize, const int32_t* ws_list,
                       double tol, double* U, double* F, double* Hpk, int32_t* conv,
                       int precision);

/* [U,~,stepwithinwhile] = funICGN_Subpb1(x0, y0, Df, ImgRef, ImgDef, winsize_x,
 * winsize_y, H, beta, mu, udual, vdual, UOld, FOld, tol, 'GaussNewton') for N
 * nodes (func/funICGN_Subpb1.m:1-474): the per-node loop of Subpb1Quadtree
 * without its bad-subset filter; a run-time error gives code 0 and NaN U. */
int stdic_subpb1_subsets(stdic_ctx* ctx, const stdic_frame* fr, const double* UOld,
                         const double* FOld, const double* vdual, const double* coords, int N,
                         const int32_t* winsize_list, double mu, double tol, double* U,
                         int32_t* conv, int precision);

/* Subpb1Quadtree(UOld, FOld, udual, vdual, coordinatesFEM, Df, ImgRef, ImgDef,
 * mu, beta, HPar, ALSolveStep, DICpara, 'GaussNewton', tol) for ALSolveStep > 1
 * without its NaN-fill tail.  winsize_list is DICpara.winsize_List (N x 2).
 * udual, beta and HPar do not change the result in the reference
 * (funICGN_Subpb1.m overwrites H and never reads udual or beta); they are
 * accepted for signature parity and may be NULL/0. */
int stdic_subpb1(stdic_ctx* ctx, const stdic_frame* fr, const double* UOld, const double* FOld,
                 const double* udual, const double* vdual, const double* coords, int N,
                 const int32_t* winsize_list, double mu, double beta, double tol, double* U,
                 int32_t* conv, int* badnum, int precision);

/* Uhat = Subpb2Quadtree(DICmesh, GaussPtOrder, beta, mu, U, F, udual, vdual,
 * alpha, winstepsize, ~).  The duals enter the reference multiplied by zero
 * (Subpb2Quadtree.m:42-44), so they are not taken.  neumann is nn x 4 (node1,
 * node2, nx, ny; column-major, may be NULL).  The system is solved by
 * Jacobi-preconditioned CG in FP64 to relative residual tol (<= 0 -> 1e-10),
 * at most maxit iterations (<= 0 -> 10000); iters receives the count. */
int stdic_subpb2(stdic_ctx* ctx, const double* coords, int N, const int32_t* elems, int E,
                 const int32_t* dirichlet, int nd, const double* neumann, int nn,
                 int gauss_order, double beta, double mu, const double* U, const double* F,
                 double alpha, double winstepsize, double tol, int maxit, double* Uhat,
                 int* iters);

/* [DICmesh] of GenerateQuadtreeMesh.m:18-133 (func_quadtree/), started from
 * the uniform mesh MeshSetUp.m builds on the search grid and refined with
 * QrefineR.m (func_quadtree/refinement/): elements whose bounding box holds
 * both mask values are split into four until their smaller side is at most
 * element_min_size (DICmesh.elementMinSize), with at most one hanging node per
 * edge; corners are reordered, hanging nodes stored in columns 5-8, elements
 * with less than half their box in the mask removed, and the Dirichlet set
 * markCoordHoleEdge built (refined and border elements, grown twice).  mask
 * is DICpara.ImgRefMask (W x H, 0/1); x0, y0 are the ny x nx grids passed to
 * MeshSetUp (row = y, whole pixels); winstepsize is max(DICpara.winstepsize).
 * Outputs (each may be NULL; capacity[k] gives the rows each holds) are
 * column-major: coords N x 2 (coordinatesFEM), elems E x 8 (elementsFEM),
 * irregular nI x 3 (DICmesh.irregular) and dirichlet nd (ascending).  counts
 * (host, 4) always receives N, E, nI and nd, so a call with NULL outputs sizes
 * them.  Node and element numbering is the reference's. */
int stdic_quadtree_mesh(stdic_ctx* ctx, const uint8_t* mask, int W, int H, const double* x0,
                        const double* y0, int ny, int nx, double winstepsize,
                        double element_min_size, double* coords, int32_t* elems,
                        int32_t* irregular, int32_t* dirichlet, const int64_t* capacity,
                        int64_t* counts);

/* [u_pred, alpha, beta_POD, beta_GPR] = funPOR_GPR(T_snap, t_train, t_pre, nB)
 * (func/funPOR_GPR.m:1-99), the initial guess of the next frame that
 * main_ALDIC_Quadtree_v2.m:185-196 predicts from the last five frames (once
 * for u, once for v).  T_snap is nT x np (one snapshot per row), u_pred
 * nT1 x np, both column-major; t_train (nT), t_pre (nT1), alpha, beta_pod and
 * beta_gpr (nT1) are host memory (the scalars may be NULL).  The proper
 * orthogonal decomposition is the reference's (its trapezoid inner product,
 * nB leading modes); the regression of each mode coefficient over time
 * follows fitrgp's documented model ('linear' basis, exact fit and
 * prediction, squared-exponential kernel, noise sigma >= 2e-5, the documented
 * starting point) with hyperparameters from a Nelder-Mead search of the
 * exact marginal likelihood; MATLAB's optimiser itself is not reproduced. */
int stdic_por_gpr(stdic_ctx* ctx, const double* T_snap, int nT, int64_t np, const double* t_train,
                  const double* t_pre, int nT1, int nB, double* u_pred, double* alpha,
                  double* beta_pod, double* beta_gpr);

/* No reference counterpart (the batching of the chosen form across frame
 * pairs): funICGNQuadtree over N nodes for `frames` deformed frames at once,
 * all sharing the reference frame of fr (f, its gradients and mask) and one
 * mesh, in one persistent kernel.  fr->g holds the frames' W x H images one
 * after another.  U0, U (2N per frame), F (4N per frame) and conv (N per frame)
 * hold the frames one after another; Hpk (optional) is (N frames) x 21.  Each
 * frame's results are those of stdic_icgn_subsets on that frame alone, up to
 * the FP32 summation order of the launch shape.  STDIC_BATCHED_F32 only. */
int stdic_icgn_subsets_frames(stdic_ctx* ctx, const stdic_frame* fr, int frames, const double* U0,
                              const double* coords, int N, int winsize, const int32_t* ws_list,
                              double tol, double* U, double* F, double* Hpk, int32_t* conv,
                              int precision);

/* The strain step of the ADMM loop (a local replacement; the active loop
 * calls funGlobalNodalStrainRBF.m).  The Gauss-point strains DN U of every
 * element are those of funGlobalNodalStrainQuadtree.m:80-257; each node takes
 * the mean, over the elements containing it, of each element's Gauss point
 * nearest to it (the reference interpolates with a natural-neighbour
 * scatteredInterpolant).  F (4N) = [du/dx dv/dx du/dy dv/dy] per node, the
 * order of the active loop's strain step; NaN at nodes in no element. */
int stdic_nodal_strain(stdic_ctx* ctx, const double* coords, int N, const int32_t* elems, int E,
                       const double* U, int gauss_order, double* F);

/* The NaN fill after the local step (a local replacement of the thin-plate RBF
 * fill of Subpb1Quadtree.m:193-259): in sweeps, every node whose U (2N,
 * in/out) is NaN takes the mean of its finite mesh neighbours of the previous
 * sweep, until no NaN node has a finite neighbour. */
int stdic_fill_nans(stdic_ctx* ctx, const double* coords, int N, const int32_t* elems, int E,
                    double* U);

/* `steps` ADMM iterations of main_ALDIC_Quadtree_v2.m:337-395 on one frame:
 *   U1 = Subpb1(U2, F2, vdual) with its bad-subset filter, NaN fill
 *   (stdic_fill_nans) and U1(hole) = U2(hole); F1 = F2;
 *   U2 = Subpb2(U1, F1) (GaussPtOrder 2, alpha 0, PCG tol 1e-10);
 *   F2 = nodal strain of U2 (stdic_nodal_strain); F2(hole) = F1(hole),
 *   U2(hole) = U1(hole); udual = F2 - F1; vdual = U2 - U1.
 * winsize_list is N x 2; mark_hole (N, may be NULL) is markCoordHoleStrain.
 * U2 (2N), F2 (4N), udual (4N), vdual (2N) are read and updated; U1 (2N) is
 * the last local solution; badnum and pcg_iters (steps each) the per-step
 * LocalICGNBadPtNum and CG counts (each may be NULL).  With use_graph the
 * first iteration runs directly and the others replay one CUDA graph of the
 * iteration; graph_used (may be NULL) says whether the capture succeeded.
 * The strain and fill steps are local replacements of the reference's global
 * ones, so the iterates follow the reference's scheme, not its exact values. */
int stdic_admm(stdic_ctx* ctx, const stdic_frame* fr, const double* coords, int N,
               const int32_t* elems, int E, const int32_t* dirichlet, int nd,
               const int32_t* winsize_list, const uint8_t* mark_hole, double mu, double beta,
               double tol, int steps, int precision, int use_graph, double* U2, double* F2,
               double* udual, double* vdual, double* U1, int* badnum, int* pcg_iters,
               int* graph_used);

/* modes of stdic_icgn_adjoint */
enum {
  STDIC_ADJ_RECOMPUTE = 0, /* interpolate each subset again in the backward pass */
  STDIC_ADJ_STORE = 1      /* keep it in shared memory between the two passes */
};

/* No reference counterpart: the gradient of the subset ZNSSD cost, the
 * criterion funICGNQuadtree.m minimises.  For node n, with P = [F11 F21 F12
 * F22 u v] taken from F (4N) and U (2N) and the (ws+1)^2 window around
 * round(coords_n) (pixels with mask 0 or outside the image left out):
 *   C_n = sum_i (a_i - b_i)^2,  a = (f - fbar)/|f - fbar|,  b = (t - tbar)/|t - tbar|,
 *   t = bicubic of ImgDef (as ba_interp2) at the warp of funICGNQuadtree.m:151-152.
 * Outputs (each may be NULL): cost = sum of the finite C_n; cost_n (N; NaN
 * for a window with fewer than 2 pixels or a constant f or t); dU (2N) and dF
 * (4N), the gradients of C_n with respect to the node's U and F; dg (W x H),
 * the gradient of the total cost with respect to ImgDef.  fr->dfdx/dfdy are
 * not used and mask may be NULL.  precision STDIC_PLAIN_F64 computes in FP64
 * (double frame, double dg); STDIC_BATCHED_F32 in FP32 (dg is float).  mode is
 * STDIC_ADJ_RECOMPUTE or STDIC_ADJ_STORE. */
int stdic_icgn_adjoint(stdic_ctx* ctx, const stdic_frame* fr, const double* coords, int N,
                       int winsize, const int32_t* ws_list, const double* U, const double* F,
                       double* cost, double* cost_n, double* dU, double* dF, void* dg, int mode,
                       int precision);

/* No reference counterpart.  stdic_subpb2 without a context and without any
 * device allocation, for callers that cannot allocate when the global step
 * runs (a caching allocator holding nearly all of HBM, a loop that must not
 * take cudaFree's synchronisation, a host that reserves memory once).  The
 * scratch is a 16 MiB __device__ array in the library (per device, once its
 * module is loaded); a mesh needing more returns STDIC_E_NOMEM.  Every array
 * must be device memory of the current device; the call runs on cuda_stream
 * (NULL: the default stream) and returns after that stream has finished it.
 * iters (host, may be NULL) receives the PCG count; err (may be NULL) receives
 * a message of at most err_len bytes.  Two calls in flight on one device at
 * once race on the shared array: serialise them.  Every call looks the array's
 * address up (cudaGetSymbolAddress) in the current device's context, so a
 * context torn down and created again is followed; the first call on a device
 * may load the module.  The call synchronises its stream, so it is never
 * capturable: on a capturing stream it returns STDIC_E_UNSUPPORTED. */
int stdic_subpb2_noalloc(const double* coords, int N, const int32_t* elems, int E,
                         const int32_t* dirichlet, int nd, const double* neumann, int nn,
                         int gauss_order, double beta, double mu, const double* U,
                         const double* F, double alpha, double winstepsize, double tol,
                         int maxit, double* Uhat, int* iters, void* cuda_stream, char* err,
                         int err_len);

#ifdef __cplusplus
}
#endif

#endif /* STAQDIC_H */
