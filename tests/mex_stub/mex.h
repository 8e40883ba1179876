/* Minimal stand-in for MATLAB's MEX API (mex.h / matrix.h), enough to
 * compile, link and call a MEX gateway outside MATLAB: numeric matrices with
 * their dimensions and class, mexPrintf to stdout, mexErrMsgTxt as a C++
 * exception.  Test infrastructure only. */
#ifndef PFDTD_TEST_MEX_H
#define PFDTD_TEST_MEX_H

#include <cstddef>

typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxDOUBLE_CLASS = 6,
  mxSINGLE_CLASS = 7,
  mxUINT32_CLASS = 13
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX } mxComplexity;

typedef struct mxArray_tag mxArray;

mxArray* mxCreateNumericMatrix(size_t m, size_t n, mxClassID cls, mxComplexity flag);
void mxDestroyArray(mxArray* a);
void* mxGetData(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
size_t mxGetNumberOfElements(const mxArray* a);
mxClassID mxGetClassID(const mxArray* a);

int mexPrintf(const char* fmt, ...);
int mexEvalString(const char* cmd);
void mexErrMsgTxt(const char* msg);

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

#endif
