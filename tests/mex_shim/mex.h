/*
 * mex.h -- minimal stand-in for MATLAB's mex.h (TEST INFRASTRUCTURE ONLY).
 * MATLAB is not installed here; this header declares the subset of the MEX /
 * matrix API the gateways in knn-toolbox_gb300/mex use, with MATLAB's names,
 * argument types and class codes, implemented by mex_shim.cpp.
 */
#ifndef KNN_TEST_MEX_SHIM_H
#define KNN_TEST_MEX_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mxArray_tag mxArray;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
void *mxGetData(const mxArray *a);
double *mxGetPr(const mxArray *a);
double mxGetScalar(const mxArray *a);
mxClassID mxGetClassID(const mxArray *a);
mxArray *mxCreateNumericMatrix(size_t m, size_t n, mxClassID c, mxComplexity flag);
mxArray *mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity flag);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);

#ifdef __cplusplus
}
#endif

#endif
