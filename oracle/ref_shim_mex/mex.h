/* Test-only stand-in for MATLAB's mex.h, so that the reference's peak finder
 * (MultiD_fitter/shared/maximumfind2.c) compiles without MATLAB. It declares the
 * few API names that file's gateway function uses; the gateway is never
 * called, only the NMS function (definitions in mex_stubs.c abort if reached). */
#ifndef BSFIT_REF_SHIM_MEX_PEAK_H
#define BSFIT_REF_SHIM_MEX_PEAK_H
#include <stddef.h>
typedef size_t mwSize;
typedef struct bsfit_mx_array mxArray;
typedef enum { mxDOUBLE_CLASS = 6 } mxClassID;
typedef enum { mxREAL = 0 } mxComplexity;
void* mxGetData(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
double mxGetScalar(const mxArray* a);
mxArray* mxCreateNumericMatrix(size_t m, size_t n, mxClassID c, mxComplexity x);
void mexErrMsgTxt(const char* msg);
#endif
