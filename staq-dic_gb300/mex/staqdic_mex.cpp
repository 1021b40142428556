// staqdic_mex: one MATLAB MEX gateway over the C ABI of libstaqdic
// (include/staqdic.h).  The same-name .m shims in matlab/ call it, so that
// main_ALDIC_Quadtree_v2.m runs unchanged on the GPU path:
//
//   Z = staqdic_mex('ba_interp2', F, X, Y)                         ba_interp2.cpp:318-335
//   [DfDx, DfDy] = staqdic_mex('gradient', ImgRef, ImgRefMask)      func/funImgGradient.m:53-78
//   [x, y, u, v, ccmax, qfactors] = staqdic_mex('integer_search', f, g, S, gridx, gridy,
//                                               winsize, winstepsize)   func/funIntegerSearch.m:82-203
//   [xGrid, yGrid, uGrid, vGrid, ccmax] = staqdic_mex('integer_search_mg', f, g, gridx, gridy,
//                                                     winsize, winstepsize)  func/funIntegerSearchMg.m:3-343
//   [U, F, HtempPar, ConvItPerEle, markCoordHoleStrain, LocalICGNBadPtNum] =
//       staqdic_mex('icgn_local', U0, coordinatesFEM, DfDx, DfDy, ImgRefMask, ImgRef, ImgDef,
//                   winsize, winsize_List, tol, precision)     func_quadtree/LocalICGNQuadtree.m:1-177
//   [U, ConvItPerEle, Subpb1BadPtNum] = staqdic_mex('subpb1', UOld, FOld, udual, vdual,
//       coordinatesFEM, DfDx, DfDy, ImgRefMask, ImgRef, ImgDef, mu, beta, winsize_List, tol,
//       precision)                                              func_quadtree/Subpb1Quadtree.m:1-191
//   Uhat = staqdic_mex('subpb2', coordinatesFEM, elementsFEM, dirichlet, neumann,
//                      GaussPtOrder, beta, mu, U, F, alpha, winstepsize)
//                                                               func_quadtree/Subpb2Quadtree.m:1-413
//
// MATLAB arrays are column-major and 1-based, which is the C ABI's convention,
// so the numeric buffers pass through untouched; only index arrays that MATLAB
// holds as double (elementsFEM, the Dirichlet list, winsize_List) and masks of
// another class are converted, into mxMalloc'd int32 / uint8 copies.  Outputs
// are created with mxCreate* as ba_interp2.cpp:287 does.  A negative return code
// of the library becomes mexErrMsgIdAndTxt with the library's message, the
// way ba_interp2.cpp:321-335 reports its errors; per-node failures are result
// codes, never errors.  One context (CUDA stream + workspace) on device 0 is
// kept for the MATLAB session and released by mexAtExit.
//
// Build (MATLAB):  mex -R2018a -I<repo>/include staqdic_mex.cpp -L<lib dir> -lstaqdic
#include <stdint.h>

#include <cmath>
#include <cstring>

#include "mex.h"
#include "staqdic.h"

namespace {

stdic_ctx* g_ctx = nullptr;

void release_ctx() {
  if (g_ctx) stdic_ctx_destroy(g_ctx);
  g_ctx = nullptr;
}

stdic_ctx* ctx() {
  if (!g_ctx) {
    const int rc = stdic_ctx_create(&g_ctx, 0);
    if (rc != STDIC_OK || !g_ctx)
      mexErrMsgIdAndTxt("staqdic:context", "staqdic_mex: no CUDA device for the library (code %d)", rc);
    mexAtExit(release_ctx);
  }
  return g_ctx;
}

void check(int rc, const char* op) {
  if (rc != STDIC_OK)
    mexErrMsgIdAndTxt("staqdic:call", "staqdic_mex('%s'): %s (code %d)", op, stdic_last_error(g_ctx), rc);
}

void need(bool ok, const char* op, const char* what) {
  if (!ok) mexErrMsgIdAndTxt("staqdic:args", "staqdic_mex('%s'): %s", op, what);
}

size_t numel(const mxArray* a) { return (size_t)mxGetNumberOfElements(a); }

const double* dbl(const mxArray* a, const char* op, const char* name) {
  if (!mxIsDouble(a)) mexErrMsgIdAndTxt("staqdic:args", "staqdic_mex('%s'): %s must be double", op, name);
  return (const double*)mxGetData(a);
}

double scalar(const mxArray* a, const char* op, const char* name) {
  if (!mxIsDouble(a) || numel(a) < 1)
    mexErrMsgIdAndTxt("staqdic:args", "staqdic_mex('%s'): %s must be a double scalar", op, name);
  return ((const double*)mxGetData(a))[0];
}

// double / single / int32 index array -> int32 copy (mxFree after use)
int32_t* to_i32(const mxArray* a) {
  const size_t n = numel(a);
  int32_t* out = (int32_t*)mxMalloc((n ? n : 1) * sizeof(int32_t));
  if (mxIsInt32(a)) {
    std::memcpy(out, mxGetData(a), n * sizeof(int32_t));
  } else if (mxIsDouble(a)) {
    const double* p = (const double*)mxGetData(a);
    for (size_t k = 0; k < n; ++k) out[k] = (int32_t)p[k];
  } else if (mxIsSingle(a)) {
    const float* p = (const float*)mxGetData(a);
    for (size_t k = 0; k < n; ++k) out[k] = (int32_t)p[k];
  } else {
    mxFree(out);
    mexErrMsgIdAndTxt("staqdic:args", "staqdic_mex: index arrays must be double, single or int32");
  }
  return out;
}

// logical / uint8 / double mask -> uint8 copy (mxFree after use)
uint8_t* to_u8(const mxArray* a) {
  const size_t n = numel(a);
  uint8_t* out = (uint8_t*)mxMalloc(n ? n : 1);
  if (mxIsLogical(a) || mxIsUint8(a)) {
    std::memcpy(out, mxGetData(a), n);
  } else if (mxIsDouble(a)) {
    const double* p = (const double*)mxGetData(a);
    for (size_t k = 0; k < n; ++k) out[k] = p[k] != 0.0 ? 1 : 0;
  } else if (mxIsSingle(a)) {
    const float* p = (const float*)mxGetData(a);
    for (size_t k = 0; k < n; ++k) out[k] = p[k] != 0.0f ? 1 : 0;
  } else {
    mxFree(out);
    mexErrMsgIdAndTxt("staqdic:args", "staqdic_mex: masks must be logical, uint8, double or single");
  }
  return out;
}

mxArray* dmat(size_t m, size_t n) { return mxCreateDoubleMatrix((mwSize)m, (mwSize)n, mxREAL); }
double* pr(mxArray* a) { return (double*)mxGetData(a); }

// int32 buffer -> double column (MATLAB's ConvItPerEle is double)
mxArray* i32_to_dcol(const int32_t* v, size_t n) {
  mxArray* a = dmat(n, 1);
  for (size_t k = 0; k < n; ++k) pr(a)[k] = (double)v[k];
  return a;
}

// ---------------------------------------------------------------------------
void op_interp(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const char* op = "ba_interp2";
  need(nrhs == 4, op, "Z = staqdic_mex('ba_interp2', F, X, Y)");
  need(nlhs <= 1, op, "one output");
  const mxArray *F = prhs[1], *X = prhs[2], *Y = prhs[3];
  const bool dbl3 = mxIsDouble(F) && mxIsDouble(X) && mxIsDouble(Y);
  const bool sgl3 = mxIsSingle(F) && mxIsSingle(X) && mxIsSingle(Y);
  need(dbl3 || sgl3, op, "ba_interp2 takes only double or single arguments for IMG,X,Y, and all must have the same class");
  need(numel(X) == numel(Y), op, "X and Y must have the same number of elements");
  const mwSize* fd = mxGetDimensions(F);
  const mwSize fnd = mxGetNumberOfDimensions(F);
  const int64_t M = (int64_t)fd[0], N = fnd > 1 ? (int64_t)fd[1] : 1;
  int64_t P = 1;
  for (mwSize i = 2; i < fnd; ++i) P *= (int64_t)fd[i];
  // output: the shape of X followed by F's dimensions beyond the second
  const mwSize* xd = mxGetDimensions(X);
  const mwSize xnd = mxGetNumberOfDimensions(X);
  mwSize od[16];
  mwSize ond = 0;
  for (mwSize i = 0; i < xnd && ond < 16; ++i) od[ond++] = xd[i];
  for (mwSize i = 2; i < fnd && ond < 16; ++i) od[ond++] = fd[i];
  plhs[0] = mxCreateNumericArray(ond, od, sgl3 ? mxSINGLE_CLASS : mxDOUBLE_CLASS, mxREAL);
  check(stdic_interp_bicubic(ctx(), mxGetData(F), M, N, P, mxGetData(X), mxGetData(Y), (int64_t)numel(X),
                             mxGetData(plhs[0]), sgl3 ? STDIC_F32 : STDIC_F64),
        op);
}

void op_gradient(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const char* op = "gradient";
  need(nrhs == 3 && nlhs <= 2, op, "[DfDx, DfDy] = staqdic_mex('gradient', ImgRef, ImgRefMask)");
  const mxArray* img = prhs[1];
  const double* f = dbl(img, op, "ImgRef");
  need(mxGetNumberOfDimensions(img) == 2, op, "ImgRef must be a 2-D image");
  const int W = (int)mxGetM(img), H = (int)mxGetN(img);
  need(W >= 7 && H >= 7, op, "the image must be at least 7 x 7");
  need(numel(prhs[2]) == (size_t)W * H, op, "ImgRefMask must have the size of ImgRef");
  uint8_t* mask = to_u8(prhs[2]);
  plhs[0] = dmat(W - 6, H - 6);
  plhs[1] = dmat(W - 6, H - 6);
  const int rc = stdic_img_gradient(ctx(), f, mask, W, H, pr(plhs[0]), pr(plhs[1]), STDIC_F64);
  mxFree(mask);
  check(rc, op);
}

void op_integer_search(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const char* op = "integer_search";
  need(nrhs == 8 && nlhs <= 6, op,
       "[x,y,u,v,ccmax,qfactors] = staqdic_mex('integer_search', f, g, S, gridx, gridy, winsize, winstepsize)");
  const double* f = dbl(prhs[1], op, "f");
  const double* g = dbl(prhs[2], op, "g");
  const int W = (int)mxGetM(prhs[1]), H = (int)mxGetN(prhs[1]);
  need(mxGetM(prhs[2]) == (size_t)W && mxGetN(prhs[2]) == (size_t)H, op, "f and g must have one size");
  auto pair_i = [&](const mxArray* a, const char* name, int out[2]) {
    const double* p = dbl(a, op, name);
    need(numel(a) >= 1, op, name);
    out[0] = (int)p[0];
    out[1] = (int)(numel(a) > 1 ? p[1] : p[0]);
  };
  auto pair_d = [&](const mxArray* a, const char* name, double out[2]) {
    const double* p = dbl(a, op, name);
    need(numel(a) >= 2, op, "gridx and gridy hold [first last]");
    out[0] = p[0];
    out[1] = p[numel(a) - 1];
  };
  int S[2], ws[2], st[2];
  double gx[2], gy[2];
  pair_i(prhs[3], "tempSizeOfSearchRegion", S);
  pair_d(prhs[4], "gridx", gx);
  pair_d(prhs[5], "gridy", gy);
  pair_i(prhs[6], "winsize", ws);
  pair_i(prhs[7], "winstepsize", st);
  int nx = 0, ny = 0;
  check(stdic_integer_search_grid(W, H, S, gx, gy, ws, st, &nx, &ny), op);
  for (int k = 0; k < 5; ++k) plhs[k] = dmat(ny, nx);
  double* q = nullptr;
  if (nlhs >= 6) {
    plhs[5] = dmat((size_t)nx * ny, 2);
    q = pr(plhs[5]);
  }
  check(stdic_integer_search(ctx(), f, g, W, H, S, gx, gy, ws, st, pr(plhs[0]), pr(plhs[1]), pr(plhs[2]),
                             pr(plhs[3]), pr(plhs[4]), nullptr, q),
        op);
}

void op_integer_search_mg(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const char* op = "integer_search_mg";
  need(nrhs == 7 && nlhs <= 5, op,
       "[xGrid,yGrid,uGrid,vGrid,ccmax] = staqdic_mex('integer_search_mg', f, g, gridx, gridy, winsize, winstepsize)");
  const double* f = dbl(prhs[1], op, "f");
  const double* g = dbl(prhs[2], op, "g");
  const int W = (int)mxGetM(prhs[1]), H = (int)mxGetN(prhs[1]);
  need(mxGetM(prhs[2]) == (size_t)W && mxGetN(prhs[2]) == (size_t)H, op, "f and g must have one size");
  const double* px = dbl(prhs[3], op, "gridx");
  const double* py = dbl(prhs[4], op, "gridy");
  need(numel(prhs[3]) >= 2 && numel(prhs[4]) >= 2, op, "gridx and gridy hold [first last]");
  const double gx[2] = {px[0], px[numel(prhs[3]) - 1]}, gy[2] = {py[0], py[numel(prhs[4]) - 1]};
  const int ws = (int)scalar(prhs[5], op, "winsize");
  const double* pst = dbl(prhs[6], op, "winstepsize");
  need(numel(prhs[6]) >= 1, op, "winstepsize");
  const double st[2] = {pst[0], numel(prhs[6]) > 1 ? pst[1] : pst[0]};
  need(st[0] > 0 && st[1] > 0, op, "winstepsize must be positive");
  // the node grid is chosen inside the search; its size is bounded by the region
  const int64_t cap = (int64_t)(std::floor((gx[1] - gx[0]) / st[0]) + 1) * (int64_t)(std::floor((gy[1] - gy[0]) / st[1]) + 1);
  need(cap >= 4, op, "the search region holds fewer than 2 x 2 grid steps");
  double* buf[5];
  for (int k = 0; k < 5; ++k) buf[k] = (double*)mxMalloc((size_t)cap * sizeof(double));
  int32_t counts[2] = {0, 0};
  const int rc = stdic_integer_search_mg(ctx(), f, g, W, H, gx, gy, ws, st, buf[0], buf[1], buf[2], buf[3], buf[4],
                                         cap, counts, nullptr, 0, nullptr);
  if (rc != STDIC_OK)
    for (int k = 0; k < 5; ++k) mxFree(buf[k]);
  check(rc, op);
  const size_t nx = (size_t)counts[0], ny = (size_t)counts[1];
  for (int k = 0; k < 5; ++k) {
    plhs[k] = dmat(ny, nx);
    std::memcpy(pr(plhs[k]), buf[k], nx * ny * sizeof(double));
    mxFree(buf[k]);
  }
}

// the frame of an IC-GN call from MATLAB's Df fields and images
stdic_frame frame_of(const mxArray* dfdx, const mxArray* dfdy, const uint8_t* mask, const mxArray* f,
                     const mxArray* g, int precision, const char* op) {
  stdic_frame fr;
  const int W = (int)mxGetM(f), H = (int)mxGetN(f);
  need(mxGetM(g) == (size_t)W && mxGetN(g) == (size_t)H, op, "ImgRef and ImgDef must have one size");
  need(numel(dfdx) == (size_t)(W - 6) * (H - 6) && numel(dfdy) == numel(dfdx), op,
       "Df.DfDx and Df.DfDy must be (W-6) x (H-6)");
  const bool single = mxIsSingle(f) && mxIsSingle(g) && mxIsSingle(dfdx) && mxIsSingle(dfdy);
  const bool dbl4 = mxIsDouble(f) && mxIsDouble(g) && mxIsDouble(dfdx) && mxIsDouble(dfdy);
  need(single || dbl4, op, "images and gradients must all be double or all single");
  need(!(single && precision == STDIC_PLAIN_F64), op, "the plain FP64 form needs double images");
  fr.f = mxGetData(f);
  fr.g = mxGetData(g);
  fr.mask = mask;
  fr.dfdx = mxGetData(dfdx);
  fr.dfdy = mxGetData(dfdy);
  fr.W = W;
  fr.H = H;
  fr.dtype = single ? STDIC_F32 : STDIC_F64;
  return fr;
}

void op_icgn_local(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const char* op = "icgn_local";
  need(nrhs == 12 && nlhs <= 6, op,
       "[U,F,HtempPar,ConvItPerEle,markCoordHoleStrain,BadPtNum] = staqdic_mex('icgn_local', U0, "
       "coordinatesFEM, DfDx, DfDy, ImgRefMask, ImgRef, ImgDef, winsize, winsize_List, tol, precision)");
  const double* U0 = dbl(prhs[1], op, "U0");
  const double* coords = dbl(prhs[2], op, "coordinatesFEM");
  const size_t N = mxGetM(prhs[2]);
  need(mxGetN(prhs[2]) == 2 && numel(prhs[1]) == 2 * N, op, "coordinatesFEM is N x 2 and U0 2N");
  const int winsize = (int)scalar(prhs[8], op, "winsize");
  const double tol = scalar(prhs[10], op, "tol");
  const int precision = (int)scalar(prhs[11], op, "precision");
  const mxArray* wl = prhs[9];
  need(mxIsEmpty(wl) || numel(wl) == N || numel(wl) == 2 * N, op, "winsize_List must be empty, N or N x 2");
  const size_t np = numel(prhs[6]);
  need(numel(prhs[5]) == np, op, "ImgRefMask must have the size of ImgRef");
  uint8_t* mask = to_u8(prhs[5]);
  int32_t* wsl = nullptr;
  int wmax = winsize;
  if (!mxIsEmpty(wl)) {
    // winsize_List: one size per node (its first column when N x 2)
    wsl = to_i32(wl);
    for (size_t k = 0; k < N; ++k) wmax = wsl[k] > wmax ? wsl[k] : wmax;
  }
  const stdic_frame fr = frame_of(prhs[3], prhs[4], mask, prhs[6], prhs[7], precision, op);
  plhs[0] = dmat(2 * N, 1);
  plhs[1] = dmat(4 * N, 1);
  plhs[2] = dmat(N, 21);
  int32_t* conv = (int32_t*)mxMalloc((N ? N : 1) * sizeof(int32_t));
  uint8_t* mark = (uint8_t*)mxMalloc(N ? N : 1);
  int badnum = 0;
  const int rc = stdic_icgn_local(ctx(), &fr, U0, coords, (int)N, wmax, wsl, tol, pr(plhs[0]), pr(plhs[1]),
                                  pr(plhs[2]), conv, mark, &badnum, precision);
  if (rc == STDIC_OK) {
    plhs[3] = i32_to_dcol(conv, N);
    // markCoordHoleStrain: the 1-based indices of the flagged nodes, as find() gives them
    size_t nm = 0;
    for (size_t k = 0; k < N; ++k) nm += mark[k] != 0;
    plhs[4] = dmat(nm, 1);
    for (size_t k = 0, j = 0; k < N; ++k)
      if (mark[k]) pr(plhs[4])[j++] = (double)(k + 1);
    plhs[5] = mxCreateDoubleScalar((double)badnum);
  }
  mxFree(conv);
  mxFree(mark);
  mxFree(mask);
  if (wsl) mxFree(wsl);
  check(rc, op);
}

void op_subpb1(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const char* op = "subpb1";
  need(nrhs == 16 && nlhs <= 3, op,
       "[U, ConvItPerEle, BadPtNum] = staqdic_mex('subpb1', UOld, FOld, udual, vdual, coordinatesFEM, "
       "DfDx, DfDy, ImgRefMask, ImgRef, ImgDef, mu, beta, winsize_List, tol, precision)");
  const double* UOld = dbl(prhs[1], op, "UOld");
  const double* FOld = dbl(prhs[2], op, "FOld");
  const double* udual = mxIsEmpty(prhs[3]) ? nullptr : dbl(prhs[3], op, "udual");
  const double* vdual = dbl(prhs[4], op, "vdual");
  const double* coords = dbl(prhs[5], op, "coordinatesFEM");
  const size_t N = mxGetM(prhs[5]);
  need(mxGetN(prhs[5]) == 2 && numel(prhs[1]) == 2 * N && numel(prhs[2]) == 4 * N && numel(prhs[4]) == 2 * N, op,
       "coordinatesFEM N x 2, UOld 2N, FOld 4N, vdual 2N");
  const double mu = scalar(prhs[11], op, "mu"), beta = scalar(prhs[12], op, "beta");
  need(numel(prhs[13]) == 2 * N, op, "winsize_List must be N x 2");
  const double tol = scalar(prhs[14], op, "tol");
  const int precision = (int)scalar(prhs[15], op, "precision");
  need(numel(prhs[8]) == numel(prhs[9]), op, "ImgRefMask must have the size of ImgRef");
  uint8_t* mask = to_u8(prhs[8]);
  int32_t* wsl = to_i32(prhs[13]);
  const stdic_frame fr = frame_of(prhs[6], prhs[7], mask, prhs[9], prhs[10], precision, op);
  plhs[0] = dmat(2 * N, 1);
  int32_t* conv = (int32_t*)mxMalloc((N ? N : 1) * sizeof(int32_t));
  int badnum = 0;
  const int rc = stdic_subpb1(ctx(), &fr, UOld, FOld, udual, vdual, coords, (int)N, wsl, mu, beta, tol,
                              pr(plhs[0]), conv, &badnum, precision);
  if (rc == STDIC_OK) {
    plhs[1] = i32_to_dcol(conv, N);
    plhs[2] = mxCreateDoubleScalar((double)badnum);
  }
  mxFree(conv);
  mxFree(mask);
  mxFree(wsl);
  check(rc, op);
}

void op_subpb2(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const char* op = "subpb2";
  need(nrhs == 12 && nlhs <= 2, op,
       "[Uhat, iters] = staqdic_mex('subpb2', coordinatesFEM, elementsFEM, dirichlet, neumann, "
       "GaussPtOrder, beta, mu, U, F, alpha, winstepsize)");
  const double* coords = dbl(prhs[1], op, "coordinatesFEM");
  const size_t N = mxGetM(prhs[1]);
  need(mxGetN(prhs[1]) == 2, op, "coordinatesFEM must be N x 2");
  const size_t E = mxGetM(prhs[2]);
  need(E == 0 || mxGetN(prhs[2]) == 8, op, "elementsFEM must be E x 8");
  const mxArray* neu = prhs[4];
  const size_t nn = mxIsEmpty(neu) ? 0 : mxGetM(neu);
  need(nn == 0 || mxGetN(neu) == 4, op, "neumann must be nn x 4");
  const int order = (int)scalar(prhs[5], op, "GaussPtOrder");
  const double beta = scalar(prhs[6], op, "beta"), mu = scalar(prhs[7], op, "mu");
  const double* U = dbl(prhs[8], op, "U");
  const double* F = dbl(prhs[9], op, "F");
  need(numel(prhs[8]) == 2 * N && numel(prhs[9]) == 4 * N, op, "U must be 2N and F 4N");
  const double alpha = scalar(prhs[10], op, "alpha"), step = scalar(prhs[11], op, "winstepsize");
  int32_t* elems = to_i32(prhs[2]);
  const size_t nd = numel(prhs[3]);
  int32_t* dir = nd ? to_i32(prhs[3]) : nullptr;
  const double* neup = nn ? dbl(neu, op, "neumann") : nullptr;
  plhs[0] = dmat(2 * N, 1);
  int iters = 0;
  const int rc = stdic_subpb2(ctx(), coords, (int)N, elems, (int)E, dir, (int)nd, neup, (int)nn, order, beta, mu,
                              U, F, alpha, step, 1e-10, 0, pr(plhs[0]), &iters);
  mxFree(elems);
  if (dir) mxFree(dir);
  if (rc == STDIC_OK && nlhs >= 2) plhs[1] = mxCreateDoubleScalar((double)iters);
  check(rc, op);
}

}  // namespace

extern "C" void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs < 1 || !mxIsChar(prhs[0]))
    mexErrMsgIdAndTxt("staqdic:op", "staqdic_mex: the first argument names the operation");
  char op[32];
  if (mxGetString(prhs[0], op, sizeof op) != 0)
    mexErrMsgIdAndTxt("staqdic:op", "staqdic_mex: operation name too long");
  if (!std::strcmp(op, "ba_interp2")) return op_interp(nlhs, plhs, nrhs, prhs);
  if (!std::strcmp(op, "gradient")) return op_gradient(nlhs, plhs, nrhs, prhs);
  if (!std::strcmp(op, "integer_search")) return op_integer_search(nlhs, plhs, nrhs, prhs);
  if (!std::strcmp(op, "integer_search_mg")) return op_integer_search_mg(nlhs, plhs, nrhs, prhs);
  if (!std::strcmp(op, "icgn_local")) return op_icgn_local(nlhs, plhs, nrhs, prhs);
  if (!std::strcmp(op, "subpb1")) return op_subpb1(nlhs, plhs, nrhs, prhs);
  if (!std::strcmp(op, "subpb2")) return op_subpb2(nlhs, plhs, nrhs, prhs);
  mexErrMsgIdAndTxt("staqdic:op", "staqdic_mex: unknown operation '%s'", op);
}
