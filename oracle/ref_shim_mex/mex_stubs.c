/* Test-only: the MATLAB API functions named by the reference peak finder's
 * gateway, which the checker never calls. */
#include <stdlib.h>
#include "mex.h"
void* mxGetData(const mxArray* a) { (void)a; abort(); }
size_t mxGetM(const mxArray* a) { (void)a; abort(); }
size_t mxGetN(const mxArray* a) { (void)a; abort(); }
double mxGetScalar(const mxArray* a) { (void)a; abort(); }
mxArray* mxCreateNumericMatrix(size_t m, size_t n, mxClassID c, mxComplexity x) {
  (void)m; (void)n; (void)c; (void)x; abort();
}
void mexErrMsgTxt(const char* msg) { (void)msg; abort(); }
