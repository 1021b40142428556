// Minimal stand-in for MATLAB's mex.h, written for this repository so that the
// reference's ba_interp2.cpp compiles unmodified as a host library.  It models
// only what that file touches: numeric arrays of double or single, their
// dimensions and data pointers, and error reporting.  Test infrastructure only.
#pragma once
#include <cstddef>

typedef size_t mwSize;
typedef enum { mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7 } mxClassID;
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
bool mxIsDouble(const mxArray* a);
bool mxIsSingle(const mxArray* a);
void* mxGetData(const mxArray* a);
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity c);
void mexErrMsgTxt(const char* msg);

extern "C" void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
