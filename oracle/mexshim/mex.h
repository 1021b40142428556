// Minimal stand-in for MATLAB's mex.h, written for this repository.  Test
// infrastructure only.  It lets two sources compile as host libraries:
//   * the reference's ba_interp2.cpp, unmodified (the interpolation checker);
//   * this repository's MEX gateway (staq-dic_gb300/mex/staqdic_mex.cpp), so
//     that tests can drive mexFunction as MATLAB would.
// It models numeric, logical and char arrays (column-major, up to 8
// dimensions), mxMalloc/mxFree, and error reporting (an error throws a C++
// exception that the test driver catches, where MATLAB would unwind to the
// prompt).  The class identifiers carry the values of MATLAB's published API.
#pragma once
#include <cstddef>
#include <cstdint>

typedef size_t mwSize;
typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxLOGICAL_CLASS = 3,
  mxCHAR_CLASS = 4,
  mxDOUBLE_CLASS = 6,
  mxSINGLE_CLASS = 7,
  mxUINT8_CLASS = 9,
  mxINT32_CLASS = 12
} mxClassID;
typedef enum { mxREAL = 0 } mxComplexity;

struct mxArray {
  mxClassID cls;
  mwSize ndim;
  mwSize dims[8];
  void* data;
  bool owns;
};

const mwSize* mxGetDimensions(const mxArray* a);
mwSize mxGetNumberOfDimensions(const mxArray* a);
mwSize mxGetNumberOfElements(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
bool mxIsDouble(const mxArray* a);
bool mxIsSingle(const mxArray* a);
bool mxIsLogical(const mxArray* a);
bool mxIsUint8(const mxArray* a);
bool mxIsInt32(const mxArray* a);
bool mxIsChar(const mxArray* a);
bool mxIsEmpty(const mxArray* a);
mxClassID mxGetClassID(const mxArray* a);
void* mxGetData(const mxArray* a);
int mxGetString(const mxArray* a, char* buf, mwSize buflen);
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity c);
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray* mxCreateDoubleScalar(double v);
void* mxMalloc(size_t n);
void mxFree(void* p);
void mexErrMsgTxt(const char* msg);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexAtExit(void (*fn)(void));

extern "C" void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
