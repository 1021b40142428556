// Host driver for the reference's own ba_interp2.cpp (compiled unmodified from
// the reference tree against mexshim/mex.h).  Exposes a C entry point that wraps
// caller buffers as mxArrays and calls mexFunction, so tests can compare the
// oracle and the CUDA kernels with the reference's compiled interpolation.
// Test infrastructure only.
#include "mex.h"
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

const mwSize* mxGetDimensions(const mxArray* a) { return a->dims; }
mwSize mxGetNumberOfDimensions(const mxArray* a) { return a->ndim; }
mwSize mxGetNumberOfElements(const mxArray* a) {
  mwSize n = 1;
  for (mwSize i = 0; i < a->ndim; ++i) n *= a->dims[i];
  return n;
}
bool mxIsDouble(const mxArray* a) { return a->cls == mxDOUBLE_CLASS; }
bool mxIsSingle(const mxArray* a) { return a->cls == mxSINGLE_CLASS; }
void* mxGetData(const mxArray* a) { return a->data; }
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity) {
  mxArray* a = new mxArray();
  a->cls = cls;
  a->ndim = ndim;
  mwSize n = 1;
  for (mwSize i = 0; i < ndim; ++i) { a->dims[i] = dims[i]; n *= dims[i]; }
  const size_t es = cls == mxDOUBLE_CLASS ? 8 : 4;
  a->data = std::calloc(n ? n : 1, es);
  a->owns = true;
  return a;
}
void mexErrMsgTxt(const char* msg) { throw std::runtime_error(msg); }

static mxArray wrap(const void* p, mwSize m, mwSize n, mxClassID cls) {
  mxArray a;
  a.cls = cls;
  a.ndim = 2;
  a.dims[0] = m;
  a.dims[1] = n;
  a.data = const_cast<void*>(p);
  a.owns = false;
  return a;
}

static int run(const void* F, long M, long N, const void* X, const void* Y, long n, void* out,
               mxClassID cls) {
  mxArray aF = wrap(F, (mwSize)M, (mwSize)N, cls);
  mxArray aX = wrap(X, (mwSize)n, 1, cls);
  mxArray aY = wrap(Y, (mwSize)n, 1, cls);
  const mxArray* prhs[3] = {&aF, &aX, &aY};
  mxArray* plhs[1] = {nullptr};
  try {
    mexFunction(1, plhs, 3, prhs);
  } catch (const std::exception&) {
    return -1;
  }
  const size_t es = cls == mxDOUBLE_CLASS ? 8 : 4;
  std::memcpy(out, plhs[0]->data, es * (size_t)n);
  std::free(plhs[0]->data);
  delete plhs[0];
  return 0;
}

extern "C" int ref_ba_interp2_f64(const double* F, long M, long N, const double* X,
                                  const double* Y, long n, double* out) {
  return run(F, M, N, X, Y, n, out, mxDOUBLE_CLASS);
}
extern "C" int ref_ba_interp2_f32(const float* F, long M, long N, const float* X, const float* Y,
                                  long n, float* out) {
  return run(F, M, N, X, Y, n, out, mxSINGLE_CLASS);
}
