// Host implementation of mex.h (see there) and C entry points for tests:
//   * ref_ba_interp2_f64/_f32 wrap caller buffers as mxArrays and call the
//     mexFunction of the reference's ba_interp2.cpp (linked beside this file);
//   * shim_* build and read mxArrays and call whichever mexFunction is linked
//     (the repository's MEX gateway in the gateway test), returning MATLAB's
//     error message instead of unwinding.
// Test infrastructure only.
#include "mex.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

namespace {
void (*g_exit_fn)(void) = nullptr;

size_t class_bytes(mxClassID cls) {
  switch (cls) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxINT32_CLASS: return 4;
    case mxLOGICAL_CLASS:
    case mxUINT8_CLASS:
    case mxCHAR_CLASS: return 1;
    default: return 8;
  }
}
}  // namespace

const mwSize* mxGetDimensions(const mxArray* a) { return a->dims; }
mwSize mxGetNumberOfDimensions(const mxArray* a) { return a->ndim; }
mwSize mxGetNumberOfElements(const mxArray* a) {
  mwSize n = 1;
  for (mwSize i = 0; i < a->ndim; ++i) n *= a->dims[i];
  return n;
}
size_t mxGetM(const mxArray* a) { return a->ndim > 0 ? a->dims[0] : 0; }
size_t mxGetN(const mxArray* a) {
  size_t n = 1;
  for (mwSize i = 1; i < a->ndim; ++i) n *= a->dims[i];
  return a->ndim > 1 ? n : 1;
}
bool mxIsDouble(const mxArray* a) { return a->cls == mxDOUBLE_CLASS; }
bool mxIsSingle(const mxArray* a) { return a->cls == mxSINGLE_CLASS; }
bool mxIsLogical(const mxArray* a) { return a->cls == mxLOGICAL_CLASS; }
bool mxIsUint8(const mxArray* a) { return a->cls == mxUINT8_CLASS; }
bool mxIsInt32(const mxArray* a) { return a->cls == mxINT32_CLASS; }
bool mxIsChar(const mxArray* a) { return a->cls == mxCHAR_CLASS; }
bool mxIsEmpty(const mxArray* a) { return mxGetNumberOfElements(a) == 0; }
mxClassID mxGetClassID(const mxArray* a) { return a->cls; }
void* mxGetData(const mxArray* a) { return a->data; }
int mxGetString(const mxArray* a, char* buf, mwSize buflen) {
  if (!mxIsChar(a) || buflen == 0) return 1;
  const size_t n = mxGetNumberOfElements(a);
  const size_t k = n < buflen - 1 ? n : buflen - 1;
  std::memcpy(buf, a->data, k);
  buf[k] = '\0';
  return n < buflen ? 0 : 1;
}
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity) {
  mxArray* a = new mxArray();
  a->cls = cls;
  a->ndim = ndim;
  mwSize n = 1;
  for (mwSize i = 0; i < ndim; ++i) { a->dims[i] = dims[i]; n *= dims[i]; }
  a->data = std::calloc(n ? n : 1, class_bytes(cls));
  a->owns = true;
  return a;
}
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
  const mwSize d[2] = {m, n};
  return mxCreateNumericArray(2, d, mxDOUBLE_CLASS, c);
}
mxArray* mxCreateDoubleScalar(double v) {
  mxArray* a = mxCreateDoubleMatrix(1, 1, mxREAL);
  ((double*)a->data)[0] = v;
  return a;
}
void* mxMalloc(size_t n) { return std::malloc(n ? n : 1); }
void mxFree(void* p) { std::free(p); }
void mexErrMsgTxt(const char* msg) { throw std::runtime_error(msg); }
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw std::runtime_error(std::string(id) + ": " + buf);
}
int mexAtExit(void (*fn)(void)) {
  g_exit_fn = fn;
  return 0;
}

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

// ---- test driver entry points ----------------------------------------------
extern "C" mxArray* shim_array(int cls, int ndim, const size_t* dims, const void* data) {
  mwSize d[8];
  for (int i = 0; i < ndim && i < 8; ++i) d[i] = dims[i];
  mxArray* a = mxCreateNumericArray((mwSize)ndim, d, (mxClassID)cls, mxREAL);
  const size_t bytes = mxGetNumberOfElements(a) * class_bytes((mxClassID)cls);
  if (data && bytes) std::memcpy(a->data, data, bytes);
  return a;
}
extern "C" mxArray* shim_string(const char* s) {
  const size_t n = std::strlen(s);
  const size_t d[2] = {1, n};
  return shim_array(mxCHAR_CLASS, 2, d, s);
}
extern "C" void* shim_data(const mxArray* a) { return a->data; }
extern "C" int shim_class(const mxArray* a) { return (int)a->cls; }
extern "C" int shim_ndim(const mxArray* a) { return (int)a->ndim; }
extern "C" size_t shim_dim(const mxArray* a, int i) { return i < (int)a->ndim ? a->dims[i] : 1; }
extern "C" void shim_free(mxArray* a) {
  if (!a) return;
  if (a->owns) std::free(a->data);
  delete a;
}
// Calls the linked mexFunction; 0 on success, -1 with MATLAB's message in err.
extern "C" int shim_call(int nlhs, mxArray** plhs, int nrhs, const mxArray** prhs, char* err, int err_len) {
  for (int k = 0; k < nlhs; ++k) plhs[k] = nullptr;
  try {
    mexFunction(nlhs, plhs, nrhs, prhs);
  } catch (const std::exception& e) {
    if (err && err_len > 0) {
      std::strncpy(err, e.what(), (size_t)err_len - 1);
      err[err_len - 1] = '\0';
    }
    return -1;
  }
  return 0;
}
// What MATLAB does when the MEX file is cleared or the session ends.
extern "C" void shim_run_atexit(void) {
  if (g_exit_fn) g_exit_fn();
  g_exit_fn = nullptr;
}
