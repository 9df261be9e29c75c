/* extern "C" entry points over the reference CPU fitter, compiled from the
 * reference sources in place (see build_ref.sh). Each fit entry loops over the
 * ROIs exactly like the reference CPU mex driver
 * (MultiD_bspline/visual code/CPUmleFit_LM/mexFunction.cpp:392-408), passing the
 * coefficient array sizes minus 3. REAL is float for the FP32 build and double
 * for the promoted FP64 build. Test-only. */
#include "CPUmleFit_LM.h"
#include "CPUsplineLib.h"

#ifdef BSFIT_REF_PROMOTE_DOUBLE
#define REF_SUFFIX(name) name##_f64
#else
#define REF_SUFFIX(name) name##_f32
#endif
typedef float REAL; /* becomes double under the promotion macro */

extern "C" {

void REF_SUFFIX(ref_fit6)(const REAL* data, const REAL* coeff, int cx, int cy, int cz,
                          int sz, int iterations, int nfits, REAL* P, REAL* CRLB, REAL* LL) {
  for (int ii = 0; ii < nfits; ii++)
    kernel_bsplineMLEFit_z_EMCCD(ii, data, coeff, cx - 3, cy - 3, cz - 3, sz, iterations,
                                 P, CRLB, LL, nfits, (REAL*)0);
}

void REF_SUFFIX(ref_fit7)(const REAL* data, const REAL* coeff, int cx, int cy, int cz, int cw,
                          int sz, int iterations, const REAL* initP, int nfits, REAL* P,
                          REAL* CRLB, REAL* LL) {
  for (int ii = 0; ii < nfits; ii++)
    kernel_bsplineMLEFit_z_EMCCD_4D(ii, data, coeff, cx - 3, cy - 3, cz - 3, cw - 3, sz,
                                    iterations, initP, P, CRLB, LL, nfits, (REAL*)0);
}

void REF_SUFFIX(ref_fit8)(const REAL* data, const REAL* coeff5, const REAL* coeff3, int cx,
                          int cy, int cz, int cw, int cu, int sz, int iterations,
                          const REAL* initP, int nfits, REAL* P, REAL* CRLB, REAL* LL) {
  for (int ii = 0; ii < nfits; ii++)
    kernel_bsplineMLEFit_z_EMCCD_53D(ii, data, coeff5, coeff3, cx - 3, cy - 3, cz - 3, cw - 3,
                                     cu - 3, sz, iterations, initP, P, CRLB, LL, nfits,
                                     (REAL*)0);
}

REAL REF_SUFFIX(ref_eval_bspline)(REAL xi, int deg) {
  REAL b;
  kernel_evalBSpline(xi, deg, &b);
  return b;
}

void REF_SUFFIX(ref_delta3d)(REAL xs, REAL ys, REAL zs, REAL* f, REAL* dx, REAL* dy, REAL* dz) {
  kernel_computeDelta3D_bSpline(xs, ys, zs, f, dx, dy, dz);
}

void REF_SUFFIX(ref_derivative3d)(REAL xi, REAL yi, REAL zi, int nx, int ny, int nz, REAL* f,
                                  REAL* dx, REAL* dy, REAL* dz, const REAL* coeff, REAL* theta,
                                  REAL* dudt, REAL* model) {
  kernel_Derivative_bSpline1(xi, yi, zi, nx, ny, nz, f, dx, dy, dz, coeff, theta, dudt, model);
}

int REF_SUFFIX(ref_cholesky)(REAL* A, int n, REAL* L, REAL* U) {
  return kernel_cholesky(A, n, L, U);
}

void REF_SUFFIX(ref_lu_evaluate)(REAL* L, REAL* U, REAL* b, int n, REAL* x) {
  kernel_luEvaluate(L, U, b, n, x);
}

}

extern "C" {

void REF_SUFFIX(ref_delta5d)(REAL xs, REAL ys, REAL zs, REAL ws, REAL us, REAL* f, REAL* dx,
                             REAL* dy, REAL* dz, REAL* dw, REAL* du) {
  kernel_computeDelta5D_bSpline(xs, ys, zs, ws, us, f, dx, dy, dz, dw, du);
}

void REF_SUFFIX(ref_derivative5d)(REAL xi, REAL yi, REAL zi, REAL wi, REAL ui, int nx, int ny,
                                  int nz, int nw, int nu, REAL* f, REAL* dx, REAL* dy, REAL* dz,
                                  REAL* dw, REAL* du, const REAL* coeff, REAL* theta, REAL* dudt,
                                  REAL* model) {
  kernel_Derivative_bSpline15D(xi, yi, zi, wi, ui, nx, ny, nz, nw, nu, f, dx, dy, dz, dw, du,
                               coeff, theta, dudt, model);
}

void REF_SUFFIX(ref_lu_evaluate5d)(REAL* L, REAL* U, REAL* b, int n, REAL* x) {
  kernel_luEvaluate5D(L, U, b, n, x);
}

}
