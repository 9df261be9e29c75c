// bsfit oracle: a CPU restatement of the reference B-spline MLE fitter (fit
// types 6, 7 and 8 of CPUmleFit_LM / GPUmleFit_LM_multiD).
//
// THIS IS TEST INFRASTRUCTURE. It is the checker for the CUDA fitter: only the
// tests, the smoke check, the CPU-baseline leg of the benchmark and its
// reference arm load it. No product path links, calls or falls back to it.
//
// Every function restates the reference CPU method step by step, including the
// places where the reference's C++ promotes an expression to double (the
// `-1.0 *` in the derivative sums, `pow(model, 2)`, the `1.5 *` literals, the
// MSVC-style max/min macros against double literals). With T = float the
// restatement is meant to reproduce the reference's FP32 build bit for bit; with
// T = double it reproduces the reference compiled with float promoted to double
// (the FP64 oracle of the reference method). Both claims are pinned by the
// tests against the reference's own sources compiled here and against the
// golden fixtures generated from them.
//
// Reference paths below are relative to the reference project root; VC stands
// for "MultiD_bspline/visual code".
//
// Build: g++ -O2 -ffp-contract=off -fopenmp -shared -fPIC (see build.py); no
// FMA contraction, so x86-64 and aarch64 builds give identical results.

#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

// MSVC-style macros from VC/CPUmleFit_LM/definitions.h:36-43, kept as
// functions with the same selection rule. The argument types follow the C++
// usual arithmetic conversions of the macro expansion, so callers pass already
// promoted values.
template <typename A>
inline A mmax(A a, A b) { return (a > b) ? a : b; }
template <typename A>
inline A mmin(A a, A b) { return (a < b) ? a : b; }

// Float literal PI (VC/CPUmleFit_LM/definitions.h:15).
constexpr float kPI = 3.141592f;
constexpr float kTOL = 1e-6f;   // TOLERANCE, definitions.h:23
constexpr float kTOL1 = 1e-5f;  // TOLERANCE1, definitions.h:24

// log / sqrt / floor resolve to the float overloads for T = float, as in the
// reference built with <cmath> in scope; pow(T, int) resolves to double pow.
inline float xlog(float v) { return std::log(v); }
inline double xlog(double v) { return std::log(v); }

// int(floor(v)) with the x86 conversion rule of the reference's MSVC/x64 build
// (cvttss2si): NaN and values outside the int range give INT_MIN. Stated here
// so that builds on other architectures, and the CUDA kernels, agree on it.
template <typename T>
inline int floor_to_int(T v) {
  T f = std::floor(v);
  if (!(f >= (T)-2147483648.0 && f < (T)2147483648.0)) return (int)(-2147483647 - 1);
  return (int)f;
}

// ---------------------------------------------------------------------------
// Cardinal B-spline basis, VC/CPUmleFit_LM/CPUsplineLib.cpp:1289-1326.
// Degree 3 gives the value weights, degree 2 the derivative weights. Half-open
// intervals; zero outside. The third degree-2 branch promotes to double through
// the `1.5 *` literal (CPUsplineLib.cpp:1305).
template <typename T>
T eval_bspline(T xi, int deg) {
  T b = 0;
  if (deg == 2) {
    T x2 = xi * xi;
    if (xi >= 0.5f && xi < 1.5f) {
      b = 1.125f - 1.5f * xi + 0.5f * x2;
    } else if (xi >= -0.5f && xi < 0.5f) {
      b = 0.75f - x2;
    } else if (xi >= -1.5f && xi < -0.5f) {
      b = (T)((double)(T)1.125f + 1.5 * (double)xi + (double)(T)(0.5f * x2));
    }
  } else if (deg == 3) {
    T x2 = xi * xi;
    T x3 = x2 * xi;
    if (xi >= 1.0f && xi < 2.0f) {
      b = 4.0f / 3.0f - 2.0f * xi + x2 - 1.0f / 6.0f * x3;
    } else if (xi >= 0.0f && xi < 1.0f) {
      b = 2.0f / 3.0f - x2 + 0.5f * x3;
    } else if (xi >= -1.0f && xi < 0.0f) {
      b = 2.0f / 3.0f - x2 - 0.5f * x3;
    } else if (xi >= -2.0f && xi < -1.0f) {
      b = 4.0f / 3.0f + 2.0f * xi + x2 + 1.0f / 6.0f * x3;
    }
  }
  return b;
}

// ---------------------------------------------------------------------------
// Tensor-product weights for the 4^D neighbourhood of one ROI evaluation,
// VC/CPUmleFit_LM/CPUsplineLib.cpp:1129-1197 (3D), :972-1126 (4D),
// :477-758 (5D).
//
// Axis order used throughout this file: 0 = Y (the coefficient array's fastest
// axis, ky), 1 = X (kx), 2 = Z, 3 = W, 4 = U. frac[a] is the fractional part of
// the ROI position along axis a. The loops run U (outermost) .. Y (innermost);
// within one 2^D block, bit a of the term index selects side 1 or side 2 of
// axis a. Value weights per axis: B1 = B3(t + v - 1), B2 = B3(t - v);
// derivative weights: dB1 = B2(t - 1 + v - 1/2), dB2 = B2(t - 1 - v + 1/2),
// v = loop index 1..2. The product runs Y * X * Z * W * U, left to right.
// wf receives the value weights, wd[a] the weights of the derivative along a.
template <typename T, int D>
void compute_delta(const T* frac, T* wf, T* const* wd) {
  const int B = 1 << D;
  T dfrac[5];
  for (int a = 0; a < D; ++a) dfrac[a] = frac[a] - 1.0f;
  // B1/B2/dB1/dB2 per axis per loop index v = 1, 2.
  T b1[5][3], b2[5][3], db1[5][3], db2[5][3];
  for (int a = 0; a < D; ++a)
    for (int v = 1; v <= 2; ++v) {
      b1[a][v] = eval_bspline<T>(frac[a] + v - 1.0f, 3);
      b2[a][v] = eval_bspline<T>(frac[a] - v, 3);
      db1[a][v] = eval_bspline<T>(dfrac[a] + v - 1.0f / 2.0f, 2);
      db2[a][v] = eval_bspline<T>(dfrac[a] - v + 1.0f / 2.0f, 2);
    }
  // Loop indices: lv[a] for axis a; outermost is axis D-1.
  int nloop = 1 << D;
  for (int n = 0; n < nloop; ++n) {
    int lv[5];
    // nIndex = n enumerates (v_{D-1}, ..., v_0) with v_0 (Y) fastest.
    for (int a = 0; a < D; ++a) lv[a] = ((n >> a) & 1) + 1;
    for (int b = 0; b < B; ++b) {
      T val[5], der[5];
      for (int a = 0; a < D; ++a) {
        bool side2 = (b >> a) & 1;
        val[a] = side2 ? b2[a][lv[a]] : b1[a][lv[a]];
        der[a] = side2 ? db2[a][lv[a]] : db1[a][lv[a]];
      }
      T p = val[0];
      for (int a = 1; a < D; ++a) p = p * val[a];
      wf[B * n + b] = p;
      for (int d = 0; d < D; ++d) {
        T q = (d == 0) ? der[0] : val[0];
        for (int a = 1; a < D; ++a) q = q * (a == d ? der[a] : val[a]);
        wd[d][B * n + b] = q;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Per-pixel model and derivatives, VC/CPUmleFit_LM/CPUsplineLib.cpp:1199-1288
// (3D), :761-970 (4D), :43-475 (5D).
//
// pos[a]: the pixel's spline position along axis a; n[a]: nData along a (the
// coefficient size minus 3). Knot: floor(pos) clamped to [1, n-1], or n when
// pos equals n exactly. Coefficient strides follow the reference: the Y row
// length is nData_X + 3 (the two lateral sizes are equal for square ROIs).
// The value sum is T arithmetic; each derivative sum is double arithmetic
// because of the `-1.0 *` factor, rounded to T when added to its accumulator.
// Outputs: dudt[0] = -N * dF/dX, dudt[1] = -N * dF/dY, dudt[2] = F,
// dudt[3] = 1, dudt[4..] = N * dF/dZ, dF/dW, dF/dU; model = bg + N * F.
template <typename T, int D>
void derivative(const T* pos, const int* n, const T* wf, T* const* wd, const T* cmat,
                const T* theta, T* dudt, T* model) {
  const int B = 1 << D;
  int kc[5];
  for (int a = 0; a < D; ++a) {
    int c = floor_to_int(pos[a]);
    c = mmax(c, 1);
    c = mmin(c, n[a] - 1);
    kc[a] = c;
  }
  for (int a = 0; a < D; ++a)
    if (pos[a] == (T)n[a]) kc[a] = n[a];
  long long stride[5];
  // Strides exactly as written in the reference: (nDatax + 3) for the X axis,
  // (nDatax + 3) * (nDatay + 3) for Z, and so on.
  stride[0] = 1;
  stride[1] = n[1] + 3;
  long long acc = (long long)(n[1] + 3) * (n[0] + 3);
  for (int a = 2; a < D; ++a) {
    stride[a] = acc;
    acc *= (n[a] + 3);
  }
  int k[5];
  for (int a = 0; a < D; ++a) k[a] = kc[a] + 1;

  T f = 0;
  T dacc[5] = {0, 0, 0, 0, 0};
  int nloop = 1 << D;
  for (int nIndex = 0; nIndex < nloop; ++nIndex) {
    int lv[5];
    for (int a = 0; a < D; ++a) lv[a] = ((nIndex >> a) & 1) + 1;
    long long node[32];
#pragma GCC unroll 32
    for (int b = 0; b < B; ++b) {
      long long idx = 0;
#pragma GCC unroll 5
      for (int a = 0; a < D; ++a) {
        bool side2 = (b >> a) & 1;
        int kk = side2 ? (k[a] + lv[a] - 1) : (k[a] - lv[a]);
        idx += (long long)kk * stride[a];
      }
      node[b] = idx;
    }
    T s = cmat[node[0]] * wf[B * nIndex];
#pragma GCC unroll 32
    for (int b = 1; b < B; ++b) s = s + cmat[node[b]] * wf[B * nIndex + b];
    f += s;
#pragma GCC unroll 5
    for (int d = 0; d < D; ++d) {
      double sd = 0.0;
#pragma GCC unroll 32
      for (int b = 0; b < B; ++b) {
        long long nd = node[b];
        T w = wd[d][B * nIndex + b];
        if (D == 5 && d == 2 && b == 27) {
          // Reference typo (CPUsplineLib.cpp:313): this term reads
          // delta_dfz[32 * nIndex + 271]. Past the end of the 1024-entry array
          // (nIndex >= 24) the reference's g++ build reads the next array of
          // the caller's frame, the W-derivative weights.
          int widx = B * nIndex + 271;
          w = (widx < 1024) ? wd[2][widx] : wd[3][widx - 1024];
        }
        if (D == 5 && d == 4 && b == 16) {
          // Reference typo (CPUsplineLib.cpp:420-421): the U-derivative term 16
          // differences the side-1 U node (ku - s) although its weight is the
          // side-2 one.
          nd = node[b] - (long long)(k[4] + lv[4] - 1) * stride[4] + (long long)(k[4] - lv[4]) * stride[4];
        }
        double term = (-1.0 * (double)cmat[nd] + (double)cmat[nd + stride[d]]) * (double)w;
        sd = (b == 0) ? term : sd + term;
      }
      dacc[d] = (T)((double)dacc[d] + sd);
    }
  }
  dudt[0] = -1.0f * theta[2] * dacc[1];
  dudt[1] = -1.0f * theta[2] * dacc[0];
  for (int a = 2; a < D; ++a) dudt[a + 2] = theta[2] * dacc[a];
  dudt[2] = f;
  dudt[3] = 1.0f;
  *model = theta[3] + theta[2] * f;
}

// ---------------------------------------------------------------------------
// Initial guesses, VC/CPUmleFit_LM/CPUgaussLib.cpp:172-225. The centroid uses
// the fast index (ii) for x and the slow index (jj) for y; the maximum starts at
// 0 and the minimum at 10e10f.
template <typename T>
void center_of_mass(int sz, const T* data, T* x, T* y) {
  T tx = 0.0f, ty = 0.0f, ts = 0.0f;
  for (int ii = 0; ii < sz; ii++)
    for (int jj = 0; jj < sz; jj++) {
      tx += data[sz * jj + ii] * ii;
      ty += data[sz * jj + ii] * jj;
      ts += data[sz * jj + ii];
    }
  *x = tx / ts;
  *y = ty / ts;
}

template <typename T>
void max_min(int sz, const T* data, T* maxn, T* minbg) {
  *maxn = 0.0f;
  *minbg = 10e10f;
  for (int kk = 0; kk < sz; kk++)
    for (int ll = 0; ll < sz; ll++) {
      *maxn = mmax(*maxn, data[kk * sz + ll]);
      *minbg = mmin(*minbg, data[kk * sz + ll]);
    }
}

// ---------------------------------------------------------------------------
// Unpivoted Cholesky, VC/CPUmleFit_LM/CPUsplineLib.cpp:1363-1390. Fails only on
// a negative pivot. The off-diagonal update is double arithmetic (`1.0 /`).
template <typename T>
int cholesky(const T* A, int n, T* L, T* U) {
  for (int i = 0; i < n; i++)
    for (int j = 0; j < (i + 1); j++) {
      T s = 0;
      for (int kk = 0; kk < j; kk++) s += U[i * n + kk] * U[j * n + kk];
      if (i == j) {
        if (A[i * n + i] - s >= 0) {
          U[i * n + j] = std::sqrt(A[i * n + i] - s);
          L[j * n + i] = U[i * n + j];
        } else {
          return 1;
        }
      } else {
        U[i * n + j] = (T)(1.0 / (double)U[j * n + j] * (double)(A[i * n + j] - s));
        L[j * n + i] = U[i * n + j];
      }
    }
  return 0;
}

// Forward and backward substitution, CPUsplineLib.cpp:1392-1419 (and the
// identical 8-parameter copy at :15-41).
template <typename T>
void lu_evaluate(const T* L, const T* U, const T* b, int n, T* x) {
  T y[8] = {0};
  for (int i = 0; i < n; i++) {
    y[i] = b[i];
    for (int j = 0; j < i; j++) y[i] -= L[j * n + i] * y[j];
    y[i] /= L[i * n + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    x[i] = y[i];
    for (int j = i + 1; j < n; j++) x[i] -= U[j * n + i] * x[j];
    x[i] /= U[i * n + i];
  }
}

// Unpivoted LU inverse returning the diagonal, VC/CPUmleFit_LM/MatInvLib.h:17-77.
template <typename T>
void mat_inv_n(T* M, T* Minv, T* diag, int sz) {
  T tmp1 = 0;
  T yy[25];
  for (int jj = 0; jj < sz; jj++) {
    for (int ii = 0; ii <= jj; ii++)
      if (ii > 0) {
        for (int kk = 0; kk <= ii - 1; kk++) tmp1 += M[ii + kk * sz] * M[kk + jj * sz];
        M[ii + jj * sz] -= tmp1;
        tmp1 = 0;
      }
    for (int ii = jj + 1; ii < sz; ii++)
      if (jj > 0) {
        for (int kk = 0; kk <= jj - 1; kk++) tmp1 += M[ii + kk * sz] * M[kk + jj * sz];
        M[ii + jj * sz] = (1 / M[jj + jj * sz]) * (M[ii + jj * sz] - tmp1);
        tmp1 = 0;
      } else {
        M[ii + jj * sz] = (1 / M[jj + jj * sz]) * M[ii + jj * sz];
      }
  }
  tmp1 = 0;
  for (int num = 0; num < sz; num++) {
    yy[0] = (num == 0) ? 1 : 0;
    for (int ii = 1; ii < sz; ii++) {
      int b = (ii == num) ? 1 : 0;
      for (int jj = 0; jj <= ii - 1; jj++) tmp1 += M[ii + jj * sz] * yy[jj];
      yy[ii] = b - tmp1;
      tmp1 = 0;
    }
    Minv[sz - 1 + num * sz] = yy[sz - 1] / M[(sz - 1) + (sz - 1) * sz];
    for (int ii = sz - 2; ii >= 0; ii--) {
      for (int jj = ii + 1; jj < sz; jj++) tmp1 += M[ii + jj * sz] * Minv[jj + num * sz];
      Minv[ii + num * sz] = (1 / M[ii + ii * sz]) * (yy[ii] - tmp1);
      tmp1 = 0;
    }
  }
  if (diag)
    for (int ii = 0; ii < sz; ii++) diag[ii] = Minv[ii * sz + ii];
}

// Initial N and bg from the raw max/min: N0 = max(0, (max - bg) * 2 * PI *
// 1.5 * 1.5) in double through the 1.5 literals; bg0 = max(bg, 0.01)
// (VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2478-2481, :2839-2840, :3237-3238).
template <typename T>
void initial_guess(int sz, const T* s_data, T* theta) {
  T Nmax;
  center_of_mass<T>(sz, s_data, &theta[0], &theta[1]);
  max_min<T>(sz, s_data, &Nmax, &theta[3]);
  double n0 = (double)((T)((Nmax - theta[3]) * 2) * (T)kPI) * 1.5 * 1.5;
  theta[2] = (T)mmax(0.0, n0);
  theta[3] = (T)mmax((double)theta[3], 0.01);
}

// Accumulation of deviance, gradient and (upper-mirrored) Hessian for one pixel,
// VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2537-2560 (and the copies in every mode).
// pow_in_double selects `data / pow(model, 2)` (double pow, the usual form) vs
// `data / pow(model, 2.0f)` (float pow, mode 8's initial pass, :3320).
template <typename T>
void accumulate_pixel(T model, T data, const T* dudt, int NV, bool pow_in_double, T* err,
                      T* jac, T* hes) {
  if (data > 0) {
    *err = *err + 2 * ((model - data) - data * xlog(model / data));
  } else {
    *err = *err + 2 * model;
    data = 0;
  }
  T t1 = 1 - data / model;
  for (int l = 0; l < NV; l++) jac[l] += t1 * dudt[l];
  T t2;
  if (pow_in_double)
    t2 = (T)((double)data / std::pow((double)model, 2));
  else
    t2 = data / (T)std::pow(model, (T)2.0f);
  for (int l = 0; l < NV; l++)
    for (int m = l; m < NV; m++) {
      hes[l * NV + m] += t2 * dudt[l] * dudt[m];
      hes[m * NV + l] = hes[l * NV + m];
    }
}

// Fisher information and log-likelihood accumulation for one pixel,
// VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2730-2742.
template <typename T>
void accumulate_fisher(T model, T data, const T* dudt, int NV, T* M, T* Div) {
  for (int kk = 0; kk < NV; kk++)
    for (int ll = kk; ll < NV; ll++) {
      M[kk * NV + ll] += dudt[ll] * dudt[kk] / model;
      M[ll * NV + kk] = M[kk * NV + ll];
    }
  if (model > 0) {
    if (data > 0)
      *Div += data * xlog(model) - model - data * xlog(data) + data;
    else
      *Div += -model;
  }
}

// ---------------------------------------------------------------------------
// Mode-specific parts. A "Model" evaluates the pixel model and its derivative
// vector for the current theta over one ROI: prepare() computes the weights at
// the ROI-level fractional positions, pixel() evaluates one pixel. The LM loop
// (fit_roi below) is shared; the modes differ only in constants, bounds and the
// quirks listed at each place.

// Position of pixel (ii, jj): (xc + jj + off, yc + ii + off) in the reference's
// X/Y naming, where xc = (sz + 1) / 2 - theta[0] uses integer division
// (CPUmleFit_LM.cpp:2512-2518).
template <typename T>
struct RoiFrame {
  T xc, yc, off;
};

template <typename T>
struct Model3D {
  // CPUmleFit_LM.cpp:2411-2760
  static constexpr int NV = 5;
  const T* coeff;
  int n[3];  // Y, X, Z nData
  T wf[64], wdY[64], wdX[64], wdZ[64];
  T zc;
  RoiFrame<T> fr;
  void prepare(const T* theta, int sz) {
    fr.xc = (sz + 1) / 2 - theta[0];
    fr.yc = (sz + 1) / 2 - theta[1];
    zc = theta[4];
    T frac[3] = {fr.yc - std::floor(fr.yc), fr.xc - std::floor(fr.xc), zc - std::floor(zc)};
    T* wd[3] = {wdY, wdX, wdZ};
    compute_delta<T, 3>(frac, wf, wd);
  }
  void pixel(int ii, int jj, const T* theta, T* dudt, T* model) const {
    T pos[3] = {fr.yc + ii + fr.off, fr.xc + jj + fr.off, zc};
    T* wd[3] = {(T*)wdY, (T*)wdX, (T*)wdZ};
    derivative<T, 3>(pos, n, wf, wd, coeff, theta, dudt, model);
  }
};

template <typename T>
struct Model4D {
  // CPUmleFit_LM.cpp:2763-3158
  static constexpr int NV = 6;
  const T* coeff;
  int n[4];
  T wf[256], wdY[256], wdX[256], wdZ[256], wdW[256];
  T zc, wc;
  RoiFrame<T> fr;
  void prepare(const T* theta, int sz) {
    fr.xc = (sz + 1) / 2 - theta[0];
    fr.yc = (sz + 1) / 2 - theta[1];
    zc = theta[4];
    wc = theta[5];
    T frac[4] = {fr.yc - std::floor(fr.yc), fr.xc - std::floor(fr.xc), zc - std::floor(zc),
                 wc - std::floor(wc)};
    T* wd[4] = {wdY, wdX, wdZ, wdW};
    compute_delta<T, 4>(frac, wf, wd);
  }
  void pixel(int ii, int jj, const T* theta, T* dudt, T* model) const {
    T pos[4] = {fr.yc + ii + fr.off, fr.xc + jj + fr.off, zc, wc};
    T* wd[4] = {(T*)wdY, (T*)wdX, (T*)wdZ, (T*)wdW};
    derivative<T, 4>(pos, n, wf, wd, coeff, theta, dudt, model);
  }
};

template <typename T>
struct Model53D {
  // CPUmleFit_LM.cpp:3163-3620. Mixture (1 - g2) * S3D + g2 * S5D; the 3D
  // coefficients share the 5D array's X/Y/Z sizes.
  static constexpr int NV = 8;
  const T* coeff5;
  const T* coeff3;
  int n[5];
  T wf[1024], wdY[1024], wdX[1024], wdZ[1024], wdW[1024], wdU[1024];
  T wf3[64], wdY3[64], wdX3[64], wdZ3[64];
  T zc, wc, uc, g2;
  RoiFrame<T> fr;
  void prepare(const T* theta, int sz) {
    fr.xc = (sz + 1) / 2 - theta[0];
    fr.yc = (sz + 1) / 2 - theta[1];
    zc = theta[4];
    wc = theta[5];
    uc = theta[6];
    T frac[5] = {fr.yc - std::floor(fr.yc), fr.xc - std::floor(fr.xc), zc - std::floor(zc),
                 wc - std::floor(wc), uc - std::floor(uc)};
    g2 = theta[7];
    T* wd3[3] = {wdY3, wdX3, wdZ3};
    compute_delta<T, 3>(frac, wf3, wd3);
    T* wd[5] = {wdY, wdX, wdZ, wdW, wdU};
    compute_delta<T, 5>(frac, wf, wd);
  }
  void pixel(int ii, int jj, const T* theta, T* dudt, T* model) const {
    T pos[5] = {fr.yc + ii + fr.off, fr.xc + jj + fr.off, zc, wc, uc};
    T* wd[5] = {(T*)wdY, (T*)wdX, (T*)wdZ, (T*)wdW, (T*)wdU};
    T dudt3[5], model5, model3;
    derivative<T, 5>(pos, n, wf, wd, coeff5, theta, dudt, &model5);
    T* wd3[3] = {(T*)wdY3, (T*)wdX3, (T*)wdZ3};
    derivative<T, 3>(pos, n, wf3, wd3, coeff3, theta, dudt3, &model3);
    for (int l = 0; l < 5; l++) dudt[l] = dudt[l] * g2 + (1 - g2) * dudt3[l];
    *model = model3 * (1 - g2) + model5 * g2;
    dudt[NV - 1] = model5 - model3;
  }
};

enum Mode { MODE6 = 6, MODE7 = 7, MODE8 = 8 };

// One ROI evaluation at the current theta: deviance, gradient and Hessian.
// s_var (sCMOS, may be null): per-pixel variance / gain^2 added to both model
// and data, as the reference's sCMOS kernels do for the other fit types
// (VC/GPUmleFit_LM/GPUmleFit_LM_sCMOS.cu:1045-1046, :1206-1207).
template <typename T, typename MDL>
void eval_roi(MDL& mdl, int sz, const T* s_data, const T* theta, bool pow_double, bool dup_dudt45,
              T* err, T* jac, T* hes, const T* s_var = nullptr) {
  constexpr int NV = MDL::NV;
  *err = 0;
  std::memset(jac, 0, NV * sizeof(T));
  std::memset(hes, 0, NV * NV * sizeof(T));
  mdl.prepare(theta, sz);
  T dudt[NV];
  for (int ii = 0; ii < sz; ii++)
    for (int jj = 0; jj < sz; jj++) {
      T model;
      mdl.pixel(ii, jj, theta, dudt, &model);
      T data = s_data[sz * jj + ii];
      if (s_var) {
        model += s_var[sz * jj + ii];
        data += s_var[sz * jj + ii];
      }
      if (dup_dudt45) dudt[5] = dudt[4];
      accumulate_pixel<T>(model, data, dudt, NV, pow_double, err, jac, hes);
    }
}

// The shared LM loop. See the mode notes inline; line numbers are for
// VC/CPUmleFit_LM/CPUmleFit_LM.cpp.
// Decision trace of one LM iteration (test infrastructure): TRACE_REC doubles
// per iteration, see the field list at the write below.
constexpr int TRACE_REC = 32;

template <typename T, typename MDL, Mode MODE>
void fit_roi(MDL& mdl, int subregion, const T* d_data, int sz, int iterations, const T* initP,
             T* d_Parameters, T* d_CRLBs, T* d_LogLikelihood, int Nfits,
             double* trace = nullptr, int trace_max = 0, const T* d_var = nullptr) {
  constexpr int NV = MDL::NV;
  const int* n = mdl.n;
  const T* s_data = d_data + (long long)sz * sz * subregion;
  const T* s_var = d_var ? d_var + (long long)sz * sz * subregion : nullptr;

  T newTheta[NV + 1], oldTheta[NV + 1];
  T newLambda = 1.0, oldLambda = 1.0;
  T newSign[NV] = {0}, oldSign[NV] = {0};
  T newUpdate[NV] = {0};
  T newClamp[NV], oldClamp[NV];
  T fade[NV];
  T sumUpdate = 1e10;
  int turn = 1;
  if (MODE == MODE6) {
    // :2434
    const T c[5] = {2.0, 2.0, 10000, 20, 20};
    for (int i = 0; i < NV; i++) newClamp[i] = oldClamp[i] = c[i], fade[i] = 0;
  } else if (MODE == MODE7) {
    // :2786-2788
    const T c[6] = {1.0, 1.0, 10000, 20, 2, 0.00001};
    const T fd[6] = {0.5, 0.5, 0.4, 0.5, 0.7, 0.8};
    for (int i = 0; i < NV; i++) newClamp[i] = oldClamp[i] = c[i], fade[i] = fd[i];
  } else {
    // :3191-3193
    const T c[8] = {1.0, 1.0, 10000, 20, 2, 2, 2, 0.1};
    for (int i = 0; i < NV; i++) newClamp[i] = c[i], fade[i] = 0.5;
  }
  T newErr = 1e12, oldErr = 1e13;
  T jacobian[NV] = {0};
  T hessian[NV * NV] = {0};
  T L[NV * NV] = {0}, U[NV * NV] = {0};
  T M[NV * NV], Diag[NV], Minv[NV * NV];
  for (int ii = 0; ii < NV * NV; ii++) M[ii] = 0, Minv[ii] = 0;

  initial_guess<T>(sz, s_data, newTheta);
  if (MODE == MODE6) {
    newTheta[4] = T(n[2]) / 2.0f;  // :2482
  } else if (MODE == MODE7) {
    // :2841-2850: initP (z, w) shared by all ROIs; 0 selects mid-grid.
    if (*initP != 0) {
      newTheta[4] = initP[0];
      newTheta[5] = initP[1];
    } else {
      newTheta[4] = T(n[2]) / 2.0f;
      newTheta[5] = T(n[3]) / 2.0f;
    }
  } else {
    // :3246-3256: initP (z, w, u, g2) shared by all ROIs.
    if (initP) {
      for (int i = 4; i < NV; i++) newTheta[i] = initP[i - 4];
    } else {
      newTheta[4] = T(n[2]) / 2.0f;
      newTheta[5] = T(n[3]) / 2.0f;
      newTheta[6] = T(n[4]) / 2.0f;
    }
  }
  for (int ii = 0; ii < NV; ii++) {
    oldTheta[ii] = newTheta[ii];
    if (MODE == MODE8) oldClamp[ii] = newClamp[ii];
  }
  // off = (nDataX - sz) / 2.0f (:2519); float arithmetic.
  mdl.fr.off = (T)((float)(n[1] - sz) / 2.0f);

  // Initial evaluation. Mode 7 copies dudt[4] into dudt[5] here only (:2893);
  // mode 8 uses float pow here only (:3320).
  eval_roi<T>(mdl, sz, s_data, newTheta, MODE != MODE8, MODE == MODE7, &newErr, jacobian, hessian,
              s_var);

  int kk;
  for (kk = 0; kk < iterations; kk++) {
    double* rec = (trace && kk < trace_max) ? trace + (long long)kk * TRACE_REC : nullptr;
    int flags = 0;
    if (rec) {
      rec[0] = kk;
      rec[1] = std::fabs((double)((newErr - oldErr) / newErr));
      rec[2] = newErr;
      rec[3] = oldErr;
    }
    bool conv = std::fabs((newErr - oldErr) / newErr) < kTOL;
    if (MODE == MODE8) conv = conv || (sumUpdate < kTOL1);  // :3355
    if (conv) {
      if (rec) rec[4] = 1;
      break;
    }
    if ((double)newErr > 1.5 * (double)oldErr) flags |= 2;
    else if (newErr < oldErr) flags |= 4;
    if ((double)newErr > 1.5 * (double)oldErr) {
      for (int i = 0; i < NV; i++) {
        newSign[i] = oldSign[i];
        newClamp[i] = oldClamp[i];
        newTheta[i] = oldTheta[i];
      }
      newLambda = oldLambda;
      newErr = oldErr;
      newLambda = 10 * newLambda;
    } else if (newErr < oldErr) {
      if (newLambda > 1)
        newLambda = (T)((double)newLambda * 0.8);
      else if (newLambda < 1)
        newLambda = 1;
    }
    for (int i = 0; i < NV; i++) hessian[i * NV + i] = hessian[i * NV + i] * newLambda;
    std::memset(L, 0, NV * sizeof(T));
    std::memset(U, 0, NV * sizeof(T));
    int info = cholesky<T>(hessian, NV, L, U);
    if (rec) {
      double mp = 1e300;
      for (int i = 0; i < NV; ++i) mp = std::min(mp, (double)U[i * NV + i]);
      rec[22] = (info == 0) ? mp : -1.0;
    }
    if (info == 0) {
      lu_evaluate<T>(L, U, jacobian, NV, newUpdate);
      if (MODE != MODE6) {
        // :2943-2950 / :3383-3390: a NaN step counts as a Cholesky failure.
        bool bad = false;
        for (int ll = 0; ll < (MODE == MODE7 ? 6 : NV); ll++)
          if (std::isnan(newUpdate[ll])) bad = true;
        if (bad) info = 1;
      }
    }
    if (rec) {
      flags |= (info == 0) ? 8 : 0;
      for (int i = 0; i < NV; ++i) rec[6 + i] = newUpdate[i];
    }
    if (info == 0) {
      if (MODE == MODE7) newUpdate[5] = newUpdate[5] * 10;  // :2951
      for (int i = 0; i < NV; i++) {
        oldSign[i] = newSign[i];
        oldClamp[i] = newClamp[i];
        oldTheta[i] = newTheta[i];
      }
      oldLambda = newLambda;
      oldErr = newErr;
      if (MODE == MODE7) {
        // "let it go", :2966-2971
        if (rec) rec[23] = std::fabs((double)newUpdate[4]);
        if ((std::fabs((double)newUpdate[4]) < 0.005) && turn) {
          flags |= 32;
          newClamp[5] = T(n[3]) / 10;
          oldClamp[5] = T(n[3]) / 10;
          turn = 0;
          newClamp[4] = 2;
          oldClamp[4] = 2;
        }
      }
      if (MODE == MODE8) sumUpdate = 0;
      for (int ll = 0; ll < NV; ll++) {
        if (newSign[ll] != 0) {
          bool flip = (newSign[ll] == 1 && newUpdate[ll] < 0) ||
                      (newSign[ll] == -1 && newUpdate[ll] > 0);
          if (flip) {
            if (MODE == MODE6)
              newClamp[ll] = (T)((double)newClamp[ll] * 0.5);  // :2610
            else
              newClamp[ll] = newClamp[ll] * fade[ll];
          }
        }
        newSign[ll] = (newUpdate[ll] > 0) ? 1 : -1;
        if (MODE == MODE8) {
          // :3416-3418
          newUpdate[ll] = newUpdate[ll] / (1 + std::fabs(newUpdate[ll] / newClamp[ll]));
          newTheta[ll] = newTheta[ll] - newUpdate[ll];
          sumUpdate += std::fabs(newUpdate[ll]);
        } else {
          newTheta[ll] = newTheta[ll] - newUpdate[ll] / (1 + std::fabs(newUpdate[ll] / newClamp[ll]));
        }
      }
      if (MODE == MODE8) {
        // :3421-3445: x, y within (sz-1)/2 +- sz/4; periodic w; 1 <= u <= nu - 0.5.
        double lo = (double)((T(sz) - 1) / 2) - sz / 4.0;
        double hi = (double)((T(sz) - 1) / 2) + sz / 4.0;
        newTheta[0] = (T)mmax((double)newTheta[0], lo);
        newTheta[0] = (T)mmin((double)newTheta[0], hi);
        newTheta[1] = (T)mmax((double)newTheta[1], lo);
        newTheta[1] = (T)mmin((double)newTheta[1], hi);
      }
      newTheta[2] = (T)mmax((double)newTheta[2], 1.0);
      newTheta[3] = (T)mmax((double)newTheta[3], 0.01);
      newTheta[4] = (T)mmax((double)newTheta[4], 0.0);
      if (MODE == MODE6) {
        newTheta[4] = mmin(newTheta[4], T(n[2] - 4));  // :2634
      } else {
        newTheta[4] = (T)mmin((double)newTheta[4], (double)T(n[2]) - 0.5);
      }
      if (MODE == MODE7) {
        newTheta[5] = (T)mmax((double)newTheta[5], 0.0);
        newTheta[5] = (T)mmin((double)newTheta[5], (double)T(n[3]) - 0.5);
      }
      if (MODE == MODE8) {
        if (newTheta[5] <= 1)
          newTheta[5] = n[3] - 2 + newTheta[5];
        else if (newTheta[5] > (n[3] - 1))
          newTheta[5] = 2 + newTheta[5] - n[3];
        newTheta[6] = mmax(newTheta[6], (T)1);
        newTheta[6] = (T)mmin((double)newTheta[6], (double)T(n[4]) - 0.5);
        newTheta[7] = mmin(newTheta[7], (T)1);
        newTheta[7] = mmax(newTheta[7], (T)0);
      }
      eval_roi<T>(mdl, sz, s_data, newTheta, true, false, &newErr, jacobian, hessian, s_var);
    } else {
      newLambda = 10 * newLambda;
    }
    if (rec) {
      rec[4] = flags;
      rec[5] = newLambda;
      for (int i = 0; i < NV; ++i) rec[14 + i] = newTheta[i];
      int sg = 0;
      for (int i = 0; i < NV; ++i) sg |= (newSign[i] > 0 ? 1 : 0) << i;
      rec[24] = sg;
      for (int i = 0; i < NV && 25 + i < TRACE_REC; ++i) rec[25 + i] = newClamp[i];
    }
  }
  if (trace && kk < trace_max && !(kk < iterations)) {
    // cap reached: mark a terminal record
    double* rec = trace + (long long)kk * TRACE_REC;
    rec[0] = kk;
    rec[4] = 64;
  }

  // CRLB and log-likelihood (:2714-2755). Modes 6 and 7 re-evaluate at the
  // final theta; mode 8 reuses the weights, positions and g2 of its last
  // evaluation (:3568-3584), which differ from theta after a rejected step.
  if (MODE != MODE8) mdl.prepare(newTheta, sz);
  T Div = 0.0;
  T dudt[NV];
  for (int ii = 0; ii < sz; ii++)
    for (int jj = 0; jj < sz; jj++) {
      T model;
      mdl.pixel(ii, jj, newTheta, dudt, &model);
      T data = s_data[sz * jj + ii];
      if (s_var) {
        model += s_var[sz * jj + ii];
        data += s_var[sz * jj + ii];
      }
      accumulate_fisher<T>(model, data, dudt, NV, M, &Div);
    }
  mat_inv_n<T>(M, Minv, Diag, NV);
  for (int i = 0; i < NV; i++) d_Parameters[(long long)Nfits * i + subregion] = newTheta[i];
  d_Parameters[(long long)Nfits * NV + subregion] = (T)kk;
  for (int i = 0; i < NV; i++) d_CRLBs[(long long)Nfits * i + subregion] = Diag[i];
  d_LogLikelihood[subregion] = Div;
}

template <typename T>
void fit6(const T* data, const T* coeff, int cx, int cy, int cz, int sz, int iterations,
          int nfits, T* P, T* CRLB, T* LL, int threads, const T* var = nullptr) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
  for (int i = 0; i < nfits; i++) {
    Model3D<T> m;
    m.coeff = coeff;
    // The reference's nDatax is the first coefficient dimension minus 3; it is
    // the X clamp and the row length. nDatay (second dimension) is the Y clamp.
    m.n[0] = cy - 3;
    m.n[1] = cx - 3;
    m.n[2] = cz - 3;
    fit_roi<T, Model3D<T>, MODE6>(m, i, data, sz, iterations, nullptr, P, CRLB, LL, nfits, nullptr,
                                  0, var);
  }
}

template <typename T>
void fit7(const T* data, const T* coeff, int cx, int cy, int cz, int cw, int sz, int iterations,
          const T* initP, int nfits, T* P, T* CRLB, T* LL, int threads, const T* var = nullptr) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
  for (int i = 0; i < nfits; i++) {
    Model4D<T>* m = new Model4D<T>;
    m->coeff = coeff;
    m->n[0] = cy - 3;
    m->n[1] = cx - 3;
    m->n[2] = cz - 3;
    m->n[3] = cw - 3;
    fit_roi<T, Model4D<T>, MODE7>(*m, i, data, sz, iterations, initP, P, CRLB, LL, nfits, nullptr, 0,
                                  var);
    delete m;
  }
}

template <typename T>
void fit8(const T* data, const T* coeff5, const T* coeff3, int cx, int cy, int cz, int cw, int cu,
          int sz, int iterations, const T* initP, int nfits, T* P, T* CRLB, T* LL, int threads,
          const T* var = nullptr) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads > 0 ? threads : 1)
  for (int i = 0; i < nfits; i++) {
    Model53D<T>* m = new Model53D<T>;
    m->coeff5 = coeff5;
    m->coeff3 = coeff3;
    m->n[0] = cy - 3;
    m->n[1] = cx - 3;
    m->n[2] = cz - 3;
    m->n[3] = cw - 3;
    m->n[4] = cu - 3;
    fit_roi<T, Model53D<T>, MODE8>(*m, i, data, sz, iterations, initP, P, CRLB, LL, nfits, nullptr,
                                   0, var);
    delete m;
  }
}

}  // namespace

extern "C" {

// Fit entry points. cx..cu are the coefficient array sizes (nData + 3) in the
// reference's dimension order (Y fastest, then X, Z, W, U); P, CRLB and LL use
// the reference's column-major output layout. threads > 1 runs ROIs in
// parallel with OpenMP (every ROI is independent).
void oracle_fit6_f32(const float* data, const float* coeff, int cx, int cy, int cz, int sz,
                     int iterations, int nfits, float* P, float* CRLB, float* LL, int threads) {
  fit6<float>(data, coeff, cx, cy, cz, sz, iterations, nfits, P, CRLB, LL, threads);
}
void oracle_fit6_f64(const double* data, const double* coeff, int cx, int cy, int cz, int sz,
                     int iterations, int nfits, double* P, double* CRLB, double* LL, int threads) {
  fit6<double>(data, coeff, cx, cy, cz, sz, iterations, nfits, P, CRLB, LL, threads);
}
void oracle_fit7_f32(const float* data, const float* coeff, int cx, int cy, int cz, int cw,
                     int sz, int iterations, const float* initP, int nfits, float* P, float* CRLB,
                     float* LL, int threads) {
  fit7<float>(data, coeff, cx, cy, cz, cw, sz, iterations, initP, nfits, P, CRLB, LL, threads);
}
void oracle_fit7_f64(const double* data, const double* coeff, int cx, int cy, int cz, int cw,
                     int sz, int iterations, const double* initP, int nfits, double* P,
                     double* CRLB, double* LL, int threads) {
  fit7<double>(data, coeff, cx, cy, cz, cw, sz, iterations, initP, nfits, P, CRLB, LL, threads);
}
void oracle_fit8_f32(const float* data, const float* coeff5, const float* coeff3, int cx, int cy,
                     int cz, int cw, int cu, int sz, int iterations, const float* initP, int nfits,
                     float* P, float* CRLB, float* LL, int threads) {
  fit8<float>(data, coeff5, coeff3, cx, cy, cz, cw, cu, sz, iterations, initP, nfits, P, CRLB, LL,
              threads);
}
void oracle_fit8_f64(const double* data, const double* coeff5, const double* coeff3, int cx,
                     int cy, int cz, int cw, int cu, int sz, int iterations, const double* initP,
                     int nfits, double* P, double* CRLB, double* LL, int threads) {
  fit8<double>(data, coeff5, coeff3, cx, cy, cz, cw, cu, sz, iterations, initP, nfits, P, CRLB,
               LL, threads);
}

// Component entry points for unit tests.
float oracle_eval_bspline_f32(float xi, int deg) { return eval_bspline<float>(xi, deg); }
double oracle_eval_bspline_f64(double xi, int deg) { return eval_bspline<double>(xi, deg); }

void oracle_delta3d_f32(float xs, float ys, float zs, float* f, float* dY, float* dX, float* dZ) {
  // Reference argument order is (x_delta, y_delta, z_delta) with outputs
  // (f, d/dY, d/dX, d/dZ): delta_dxf holds the Y-axis derivative weights.
  float frac[3] = {ys, xs, zs};
  float* wd[3] = {dY, dX, dZ};
  compute_delta<float, 3>(frac, f, wd);
}

void oracle_derivative3d_f32(float xi, float yi, float zi, int nx, int ny, int nz, const float* f,
                             const float* dY, const float* dX, const float* dZ, const float* coeff,
                             const float* theta, float* dudt, float* model) {
  float pos[3] = {yi, xi, zi};
  int n[3] = {ny, nx, nz};
  float* wd[3] = {(float*)dY, (float*)dX, (float*)dZ};
  derivative<float, 3>(pos, n, f, wd, coeff, theta, dudt, model);
}

int oracle_cholesky_f32(const float* A, int n, float* L, float* U) {
  return cholesky<float>(A, n, L, U);
}

void oracle_lu_evaluate_f32(const float* L, const float* U, const float* b, int n, float* x) {
  lu_evaluate<float>(L, U, b, n, x);
}

void oracle_mat_inv_f64(double* M, double* Minv, double* diag, int n) {
  mat_inv_n<double>(M, Minv, diag, n);
}

}  // extern "C"

extern "C" {

void oracle_delta5d_f32(float xs, float ys, float zs, float ws, float us, float* f, float* dY,
                        float* dX, float* dZ, float* dW, float* dU) {
  float frac[5] = {ys, xs, zs, ws, us};
  float* wd[5] = {dY, dX, dZ, dW, dU};
  compute_delta<float, 5>(frac, f, wd);
}

void oracle_derivative5d_f32(float xi, float yi, float zi, float wi, float ui, int nx, int ny,
                             int nz, int nw, int nu, const float* f, const float* dY,
                             const float* dX, const float* dZ, const float* dW, const float* dU,
                             const float* coeff, const float* theta, float* dudt, float* model) {
  float pos[5] = {yi, xi, zi, wi, ui};
  int n[5] = {ny, nx, nz, nw, nu};
  float* wd[5] = {(float*)dY, (float*)dX, (float*)dZ, (float*)dW, (float*)dU};
  derivative<float, 5>(pos, n, f, wd, coeff, theta, dudt, model);
}

}  // extern "C"

namespace {
template <typename T, typename MDL>
void eval_entry(MDL& mdl, const T* rois, int sz, int nfits, const T* theta, int fisher, T* out) {
  constexpr int NV = MDL::NV;
  constexpr int NH = NV * (NV + 1) / 2;
  for (int r = 0; r < nfits; ++r) {
    const T* s_data = rois + (long long)sz * sz * r;
    T th[NV + 1];
    for (int i = 0; i < NV; ++i) th[i] = theta[(long long)i * nfits + r];
    mdl.fr.off = (T)((float)(mdl.n[1] - sz) / 2.0f);
    T* o = out + (long long)r * (1 + NV + NH);
    T err = 0, jac[NV], hes[NV * NV];
    if (!fisher) {
      eval_roi<T>(mdl, sz, s_data, th, true, false, &err, jac, hes);
    } else {
      T M[NV * NV];
      for (int i = 0; i < NV * NV; ++i) M[i] = 0;
      mdl.prepare(th, sz);
      T dudt[NV];
      for (int ii = 0; ii < sz; ii++)
        for (int jj = 0; jj < sz; jj++) {
          T model;
          mdl.pixel(ii, jj, th, dudt, &model);
          accumulate_fisher<T>(model, s_data[sz * jj + ii], dudt, NV, M, &err);
        }
      for (int i = 0; i < NV; ++i) jac[i] = 0;
      for (int i = 0; i < NV * NV; ++i) hes[i] = M[i];
    }
    o[0] = err;
    for (int i = 0; i < NV; ++i) o[1 + i] = jac[i];
    int k = 0;
    for (int l = 0; l < NV; ++l)
      for (int m = l; m < NV; ++m) o[1 + NV + k++] = hes[l * NV + m];
  }
}
}  // namespace

extern "C" {
// One evaluation per ROI at given theta (NV x nfits column-major); out as
// bsfit_eval_device: value, gradient, packed upper-triangle Hessian / Fisher.
void oracle_eval6_f64(const double* rois, const double* coeff, int cx, int cy, int cz, int sz,
                      int nfits, const double* theta, int fisher, double* out) {
  Model3D<double> m;
  m.coeff = coeff;
  m.n[0] = cy - 3;
  m.n[1] = cx - 3;
  m.n[2] = cz - 3;
  eval_entry<double, Model3D<double>>(m, rois, sz, nfits, theta, fisher, out);
}
void oracle_eval7_f64(const double* rois, const double* coeff, int cx, int cy, int cz, int cw,
                      int sz, int nfits, const double* theta, int fisher, double* out) {
  Model4D<double>* m = new Model4D<double>;
  m->coeff = coeff;
  m->n[0] = cy - 3;
  m->n[1] = cx - 3;
  m->n[2] = cz - 3;
  m->n[3] = cw - 3;
  eval_entry<double, Model4D<double>>(*m, rois, sz, nfits, theta, fisher, out);
  delete m;
}
}  // extern "C"

extern "C" {
// Decision trace of one ROI (test infrastructure): writes up to trace_max
// records of 32 doubles: [0] iteration, [1] |dErr/err|, [2] newErr, [3] oldErr,
// [4] flags (1 converged, 2 rejected, 4 improved, 8 Cholesky ok, 32 let-it-go,
// 64 cap), [5] lambda, [6..13] solve result, [14..21] theta after the step,
// [22] smallest Cholesky diagonal (-1 on failure), [23] |dz| (fit type 7),
// [24] sign bits, [25..31] clamps. Returns the output row as fit6/7 would.
void oracle_trace_f32(int fittype, const float* data, const float* coeff, const float* coeff3,
                      const int* dims, int sz, int iterations, const float* initP, int roi,
                      int nfits, float* P, float* CRLB, float* LL, double* trace, int trace_max) {
  if (fittype == 6) {
    Model3D<float> m; m.coeff = coeff; m.n[0] = dims[1] - 3; m.n[1] = dims[0] - 3; m.n[2] = dims[2] - 3;
    fit_roi<float, Model3D<float>, MODE6>(m, roi, data, sz, iterations, nullptr, P, CRLB, LL, nfits, trace, trace_max);
  } else if (fittype == 7) {
    Model4D<float>* m = new Model4D<float>; m->coeff = coeff; m->n[0] = dims[1] - 3; m->n[1] = dims[0] - 3; m->n[2] = dims[2] - 3; m->n[3] = dims[3] - 3;
    fit_roi<float, Model4D<float>, MODE7>(*m, roi, data, sz, iterations, initP, P, CRLB, LL, nfits, trace, trace_max);
    delete m;
  }
}
void oracle_trace_f64(int fittype, const double* data, const double* coeff, const double* coeff3,
                      const int* dims, int sz, int iterations, const double* initP, int roi,
                      int nfits, double* P, double* CRLB, double* LL, double* trace, int trace_max) {
  if (fittype == 6) {
    Model3D<double> m; m.coeff = coeff; m.n[0] = dims[1] - 3; m.n[1] = dims[0] - 3; m.n[2] = dims[2] - 3;
    fit_roi<double, Model3D<double>, MODE6>(m, roi, data, sz, iterations, nullptr, P, CRLB, LL, nfits, trace, trace_max);
  } else if (fittype == 7) {
    Model4D<double>* m = new Model4D<double>; m->coeff = coeff; m->n[0] = dims[1] - 3; m->n[1] = dims[0] - 3; m->n[2] = dims[2] - 3; m->n[3] = dims[3] - 3;
    fit_roi<double, Model4D<double>, MODE7>(*m, roi, data, sz, iterations, initP, P, CRLB, LL, nfits, trace, trace_max);
    delete m;
  }
}
}  // extern "C"

namespace {
// Fit type 8 evaluation at given theta (the mixture model of Model53D).
void eval8(const double* rois, const double* coeff5, const double* coeff3, const int* dims, int sz,
           int nfits, const double* theta, int fisher, double* out) {
  Model53D<double>* m = new Model53D<double>;
  m->coeff5 = coeff5;
  m->coeff3 = coeff3;
  m->n[0] = dims[1] - 3;
  m->n[1] = dims[0] - 3;
  m->n[2] = dims[2] - 3;
  m->n[3] = dims[3] - 3;
  m->n[4] = dims[4] - 3;
  eval_entry<double, Model53D<double>>(*m, rois, sz, nfits, theta, fisher, out);
  delete m;
}
}  // namespace

extern "C" {
void oracle_eval8_f64(const double* rois, const double* coeff5, const double* coeff3, int cx,
                      int cy, int cz, int cw, int cu, int sz, int nfits, const double* theta,
                      int fisher, double* out) {
  int dims[5] = {cx, cy, cz, cw, cu};
  eval8(rois, coeff5, coeff3, dims, sz, nfits, theta, fisher, out);
}
}  // extern "C"

// ---------------------------------------------------------------------------
// 4Pi fit (four interference channels, shared parameters).
//
// The reference ships this fitter only as a compiled binary; its source is not
// part of the reference. The method below is restated from what the reference
// does publish: the call (demo_4pi/bspline_based_4piloc_v4.m:196-214:
// imstack [s, s, N, 4], shared flags, 100 iterations, the 4D (x, y, z, phase)
// coefficients, per-ROI per-channel parameter offsets dT [NV, 4, N], initial z
// and phase per ROI, per-channel phase shifts, phase in knot units with the
// +1 knot convention, :216), the forward model of one channel
// (demo_4pi/store/simBSplinePSF.m:15-61: the 4D spline at the channel's
// position with the phase shifted by the channel's phase shift and wrapped to
// one period) and the LM machinery of the other B-spline fit types. The
// coefficient array is the caller's bsarray of the phase-resolved PSF
// (bspline_based_4piloc_v4.m:80-88: samples at phases 0 .. (nPhi) dphi with
// 2 pi at sample nPhi - 1), so one period spans P = nW - 1 knots (nW = the
// array's phase size - 3) and a phase position lives in [1, 1 + P).
// The choices that are this implementation's own: all six parameters shared
// (the demo's shared = [1 1 1 1 1 1]), channel c evaluated at theta + dT[c]
// with its phase shifted by shift[c]; clamps {1, 1, 1e4, 20, 2, 2} with fade
// 0.5; initial x, y, N, bg the mean over channels of the single-channel rule
// (x, y corrected by the channel's offset); bounds N >= 1, bg >= 0.01,
// 0 <= z <= nZ - 0.5; the phase parameter and each channel's shifted phase
// wrapped into [1, 1 + P) one period at a time.
// THIS DEFINES THE METHOD: parity for it is not pinned to a reference.

namespace {

// Wrap of a phase position into [1, 1 + P), P = nW - 1, by one period.
template <typename T>
inline T wrap_phase(T w, int nw) {
  const T P = (T)(nw - 1);
  if (w < (T)1) return w + P;
  if (w >= (T)nw) return w - P;
  return w;
}

template <typename T>
struct Model4Pi {
  static constexpr int NV = 6;
  static constexpr int C = 4;
  const T* coeff;
  int n[4];
  const T* dT;        // [C][NV] offsets of this ROI
  T shift[C];         // per-channel phase shifts (knot units)
  Model4D<T>* ch[C];  // per-channel 4D evaluators (weights per channel)
  void prepare(const T* theta, int sz) {
    for (int c = 0; c < C; ++c) {
      T tc[NV];
      for (int t = 0; t < NV; ++t) tc[t] = theta[t] + dT[c * NV + t];
      tc[5] = wrap_phase<T>(tc[5] + shift[c], n[3]);
      ch[c]->prepare(tc, sz);
    }
  }
  // model and dudt of channel c at pixel (ii, jj)
  void pixel(int c, int ii, int jj, const T* theta, T* dudt, T* model) const {
    T tc[NV];
    for (int t = 0; t < NV; ++t) tc[t] = theta[t] + dT[c * NV + t];
    ch[c]->pixel(ii, jj, tc, dudt, model);
  }
};

template <typename T>
void eval_4pi(Model4Pi<T>& mdl, int sz, const T* const* planes, const T* theta, bool fisher,
              T* err, T* jac, T* hes) {
  constexpr int NV = 6;
  *err = 0;
  for (int i = 0; i < NV; ++i) jac[i] = 0;
  for (int i = 0; i < NV * NV; ++i) hes[i] = 0;
  mdl.prepare(theta, sz);
  for (int c = 0; c < Model4Pi<T>::C; ++c)
    for (int ii = 0; ii < sz; ii++)
      for (int jj = 0; jj < sz; jj++) {
        T dudt[NV], model;
        mdl.pixel(c, ii, jj, theta, dudt, &model);
        const T data = planes[c][sz * jj + ii];
        if (!fisher)
          accumulate_pixel<T>(model, data, dudt, NV, true, err, jac, hes);
        else
          accumulate_fisher<T>(model, data, dudt, NV, hes, err);
      }
}

template <typename T>
void fit_4pi_roi(const T* coeff, const int* n, int sz, int nfits, int r, const T* imstack,
                 const T* dT, const T* initZ, const T* initPhi, const T* shift, int iterations,
                 T* P, T* CRLB, T* LL) {
  constexpr int NV = 6, C = 4;
  Model4D<T> chm[C];
  Model4Pi<T> mdl;
  mdl.coeff = coeff;
  for (int a = 0; a < 4; ++a) mdl.n[a] = n[a];
  mdl.dT = dT + (long long)r * C * NV;
  for (int c = 0; c < C; ++c) {
    mdl.shift[c] = shift[c];
    chm[c].coeff = coeff;
    for (int a = 0; a < 4; ++a) chm[c].n[a] = n[a];
    chm[c].fr.off = (T)((float)(n[1] - sz) / 2.0f);
    mdl.ch[c] = &chm[c];
  }
  const T* planes[C];
  for (int c = 0; c < C; ++c) planes[c] = imstack + ((long long)c * nfits + r) * sz * sz;
  // initial values: mean over the channels of the single-channel rule
  // (CPUgaussLib.cpp:172-225, CPUmleFit_LM.cpp:2477-2482)
  T th[NV], oth[NV];
  {
    T sx = 0, sy = 0, sn = 0, sb = 0;
    for (int c = 0; c < C; ++c) {
      T t4[4];
      initial_guess<T>(sz, planes[c], t4);
      sx += t4[0] - mdl.dT[c * NV + 0];
      sy += t4[1] - mdl.dT[c * NV + 1];
      sn += t4[2];
      sb += t4[3];
    }
    th[0] = sx / (T)C;
    th[1] = sy / (T)C;
    th[2] = sn / (T)C;
    th[3] = sb / (T)C;
  }
  th[4] = initZ[r];
  th[5] = wrap_phase<T>(initPhi[r], n[3]);
  const T clamp0[NV] = {1, 1, 10000, 20, 2, 2};
  T clampv[NV], oclamp[NV], sign[NV] = {0}, osign[NV] = {0}, upd[NV];
  for (int i = 0; i < NV; ++i) clampv[i] = oclamp[i] = clamp0[i], oth[i] = th[i];
  T lambda = 1, olambda = 1;
  T err = 1e12, oerr = 1e13;
  T jac[NV], hes[NV * NV], L[NV * NV], U[NV * NV];
  eval_4pi<T>(mdl, sz, planes, th, false, &err, jac, hes);
  int kk;
  for (kk = 0; kk < iterations; kk++) {
    if (std::fabs((err - oerr) / err) < kTOL) break;
    if ((double)err > 1.5 * (double)oerr) {
      for (int i = 0; i < NV; i++) sign[i] = osign[i], clampv[i] = oclamp[i], th[i] = oth[i];
      lambda = olambda;
      err = oerr;
      lambda = 10 * lambda;
    } else if (err < oerr) {
      if (lambda > 1) lambda = (T)((double)lambda * 0.8);
      else if (lambda < 1) lambda = 1;
    }
    for (int i = 0; i < NV; i++) hes[i * NV + i] *= lambda;
    int info = cholesky<T>(hes, NV, L, U);
    if (info == 0) {
      lu_evaluate<T>(L, U, jac, NV, upd);
      for (int i = 0; i < NV; ++i)
        if (std::isnan(upd[i])) info = 1;
    }
    if (info == 0) {
      for (int i = 0; i < NV; i++) osign[i] = sign[i], oclamp[i] = clampv[i], oth[i] = th[i];
      olambda = lambda;
      oerr = err;
      for (int l = 0; l < NV; l++) {
        if (sign[l] != 0 && ((sign[l] == 1 && upd[l] < 0) || (sign[l] == -1 && upd[l] > 0)))
          clampv[l] = clampv[l] * (T)0.5;
        sign[l] = (upd[l] > 0) ? 1 : -1;
        th[l] = th[l] - upd[l] / (1 + std::fabs(upd[l] / clampv[l]));
      }
      th[2] = (T)mmax((double)th[2], 1.0);
      th[3] = (T)mmax((double)th[3], 0.01);
      th[4] = (T)mmax((double)th[4], 0.0);
      th[4] = (T)mmin((double)th[4], (double)T(n[2]) - 0.5);
      th[5] = wrap_phase<T>(th[5], n[3]);
      eval_4pi<T>(mdl, sz, planes, th, false, &err, jac, hes);
    } else {
      lambda = 10 * lambda;
    }
  }
  T M[NV * NV], Minv[NV * NV], diag[NV], Div = 0;
  eval_4pi<T>(mdl, sz, planes, th, true, &Div, jac, M);
  mat_inv_n<T>(M, Minv, diag, NV);
  for (int i = 0; i < NV; i++) P[(long long)nfits * i + r] = th[i];
  P[(long long)nfits * NV + r] = (T)kk;
  for (int i = 0; i < NV; i++) CRLB[(long long)nfits * i + r] = diag[i];
  LL[r] = Div;
}

template <typename T>
void fit4pi(const T* imstack, const T* coeff, const int* cdims, int sz, int nfits, int iterations,
            const T* dT, const T* initZ, const T* initPhi, const T* shift, T* P, T* CRLB, T* LL,
            int threads) {
  int n[4] = {cdims[1] - 3, cdims[0] - 3, cdims[2] - 3, cdims[3] - 3};
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads > 0 ? threads : 1)
  for (int r = 0; r < nfits; ++r)
    fit_4pi_roi<T>(coeff, n, sz, nfits, r, imstack, dT, initZ, initPhi, shift, iterations, P, CRLB,
                   LL);
}

}  // namespace

extern "C" {
// 4Pi fit: imstack [C=4][N][s][s] (MATLAB [s, s, N, 4]); coeff (x, y, z, phase)
// with dims (Y, X, Z, W); dT [N][4][6] (MATLAB [6, 4, N]); initZ, initPhi [N];
// shift [4] (knot units). P [7][N], CRLB [6][N], LL [N].
void oracle_fit4pi_f32(const float* imstack, const float* coeff, const int* cdims, int sz, int nfits,
                       int iterations, const float* dT, const float* initZ, const float* initPhi,
                       const float* shift, float* P, float* CRLB, float* LL, int threads) {
  fit4pi<float>(imstack, coeff, cdims, sz, nfits, iterations, dT, initZ, initPhi, shift, P, CRLB,
                LL, threads);
}
void oracle_fit4pi_f64(const double* imstack, const double* coeff, const int* cdims, int sz,
                       int nfits, int iterations, const double* dT, const double* initZ,
                       const double* initPhi, const double* shift, double* P, double* CRLB,
                       double* LL, int threads) {
  fit4pi<double>(imstack, coeff, cdims, sz, nfits, iterations, dT, initZ, initPhi, shift, P, CRLB,
                 LL, threads);
}
}  // extern "C"

extern "C" {
// One 4Pi evaluation per ROI at given theta (6 x nfits column-major); out as
// bsfit_eval4pi_device: value, gradient, packed upper-triangle Hessian / Fisher.
void oracle_eval4pi_f64(const double* imstack, const double* coeff, const int* cdims, int sz,
                        int nfits, const double* dT, const double* shift, const double* theta,
                        int fisher, double* out) {
  constexpr int NV = 6, C = 4, NH = NV * (NV + 1) / 2;
  int n[4] = {cdims[1] - 3, cdims[0] - 3, cdims[2] - 3, cdims[3] - 3};
  Model4D<double>* chm = new Model4D<double>[C];
  for (int r = 0; r < nfits; ++r) {
    Model4Pi<double> mdl;
    mdl.coeff = coeff;
    for (int a = 0; a < 4; ++a) mdl.n[a] = n[a];
    mdl.dT = dT + (long long)r * C * NV;
    for (int c = 0; c < C; ++c) {
      mdl.shift[c] = shift[c];
      chm[c].coeff = coeff;
      for (int a = 0; a < 4; ++a) chm[c].n[a] = n[a];
      chm[c].fr.off = (double)((float)(n[1] - sz) / 2.0f);
      mdl.ch[c] = &chm[c];
    }
    const double* planes[C];
    for (int c = 0; c < C; ++c) planes[c] = imstack + ((long long)c * nfits + r) * sz * sz;
    double th[NV];
    for (int i = 0; i < NV; ++i) th[i] = theta[(long long)i * nfits + r];
    double err = 0, jac[NV], hes[NV * NV];
    eval_4pi<double>(mdl, sz, planes, th, fisher != 0, &err, jac, hes);
    double* o = out + (long long)r * (1 + NV + NH);
    o[0] = err;
    for (int i = 0; i < NV; ++i) o[1 + i] = fisher ? 0.0 : jac[i];
    int k = 0;
    for (int l = 0; l < NV; ++l)
      for (int m = l; m < NV; ++m) o[1 + NV + k++] = hes[l * NV + m];
  }
  delete[] chm;
}
}  // extern "C"

extern "C" {
// sCMOS variants: var holds the per-pixel variance / gain^2 in the ROI layout
// (restated from the reference's sCMOS kernels of the other fit types; the
// reference's B-spline fit types ignore the variance map).
void oracle_fit6_scmos_f64(const double* data, const double* var, const double* coeff, int cx,
                           int cy, int cz, int sz, int iterations, int nfits, double* P,
                           double* CRLB, double* LL, int threads) {
  fit6<double>(data, coeff, cx, cy, cz, sz, iterations, nfits, P, CRLB, LL, threads, var);
}
void oracle_fit6_scmos_f32(const float* data, const float* var, const float* coeff, int cx, int cy,
                           int cz, int sz, int iterations, int nfits, float* P, float* CRLB,
                           float* LL, int threads) {
  fit6<float>(data, coeff, cx, cy, cz, sz, iterations, nfits, P, CRLB, LL, threads, var);
}
void oracle_fit7_scmos_f64(const double* data, const double* var, const double* coeff, int cx,
                           int cy, int cz, int cw, int sz, int iterations, const double* initP,
                           int nfits, double* P, double* CRLB, double* LL, int threads) {
  fit7<double>(data, coeff, cx, cy, cz, cw, sz, iterations, initP, nfits, P, CRLB, LL, threads, var);
}
void oracle_fit7_scmos_f32(const float* data, const float* var, const float* coeff, int cx, int cy,
                           int cz, int cw, int sz, int iterations, const float* initP, int nfits,
                           float* P, float* CRLB, float* LL, int threads) {
  fit7<float>(data, coeff, cx, cy, cz, cw, sz, iterations, initP, nfits, P, CRLB, LL, threads, var);
}
void oracle_fit8_scmos_f64(const double* data, const double* var, const double* coeff5,
                           const double* coeff3, int cx, int cy, int cz, int cw, int cu, int sz,
                           int iterations, const double* initP, int nfits, double* P, double* CRLB,
                           double* LL, int threads) {
  fit8<double>(data, coeff5, coeff3, cx, cy, cz, cw, cu, sz, iterations, initP, nfits, P, CRLB, LL,
               threads, var);
}
void oracle_fit8_scmos_f32(const float* data, const float* var, const float* coeff5,
                           const float* coeff3, int cx, int cy, int cz, int cw, int cu, int sz,
                           int iterations, const float* initP, int nfits, float* P, float* CRLB,
                           float* LL, int threads) {
  fit8<float>(data, coeff5, coeff3, cx, cy, cz, cw, cu, sz, iterations, initP, nfits, P, CRLB, LL,
              threads, var);
}
}  // extern "C"
