/* Test-only stand-in for MATLAB's mex.h, so that the reference's CPU fitter
 * sources (CPUmleFit_LM.cpp, CPUsplineLib.cpp, CPUgaussLib.cpp) compile without
 * MATLAB. The fitter functions only use the mwSize type from it. */
#ifndef BSFIT_REF_SHIM_MEX_H
#define BSFIT_REF_SHIM_MEX_H
#include <stddef.h>
typedef size_t mwSize;
#endif
