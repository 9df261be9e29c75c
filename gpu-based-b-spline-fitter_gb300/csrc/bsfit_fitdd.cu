// Parity-grade fit: the reference method (VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2411-3620,
// VC = "MultiD_bspline/visual code") evaluated in double-float arithmetic on
// the FP32 pipe, for fit types 6, 7 and 8.
//
// Why: the reference method's LM trajectory has discrete decisions (the
// 1e-6 relative-deviance stop, accept / reject, the update-sign clamp fades,
// fit type 7's "let it go" switch) that react to rounding. With FP32
// evaluation the fits agree with the reference's FP64 results within the
// tolerances (x, y 1e-4 px, z 1e-2 nm, N and bg 1e-5 relative, extra
// dimensions 1e-4, CRLB 1e-4 relative) on a third of 4D ROIs; measured on the
// CPU, the deviance, gradient, Hessian and Fisher information all need about
// 1e-13 relative accuracy before the agreement reaches that of a second FP64
// build of the reference (one compiled with FMA contraction). A double-float
// value (hi + lo, two floats, about 48 significant bits) gives that on the
// FP32 pipe; GB300 issues FP64 at 1/57 of the FP32 rate.
//
// Structure: the separable three-stage evaluation of the FP32 kernels
// (bsfit_fit.cu) with every stage in double-float: (A) the non-lateral
// contraction at every lateral node of the ROI's knot window into
// shared-memory maps, (B) the Y contraction per (X node, pixel row), (C) the
// X contraction per pixel fused with the Poisson deviance, gradient and
// Hessian (or Fisher information and log-likelihood), then a reduce-scatter
// over the lanes. The LM state is double-float, lane l owning parameter l;
// the damped Hessian is factored by a lane-parallel double-float Cholesky.
// The CRLB inverts the Fisher matrix in FP64 (once per fit). Coefficients and
// pixels are the caller's floats, exact in double-float.
//
// Constants follow the reference's FP64 build: its float literals (2.0f/3.0f,
// 1.0f/6.0f, 4.0f/3.0f, TOLERANCE 1e-6f, ...) stay float values, its double
// literals (the fades 0.4, 0.7, 0.8, the clamps 1e-5 and 0.1, 0.8 in the
// damping, 0.01, 0.005) are carried as double-float pairs.
#include <cstdint>
#include <mutex>

#include "bsfit_device.cuh"
#include "bsfit_internal.h"

namespace bsfit {
namespace ddf {

// ---------------------------------------------------------------------------
// Double-float arithmetic (Dekker / Knuth error-free transformations; the
// "sloppy" sums of Hida, Li and Bailey's double-double library): value =
// hi + lo with |lo| <= ulp(hi) / 2 after normalisation. Sums and products are
// accurate to a few units of 2^-48 relative to the magnitudes involved.

struct dd {
  float hi, lo;
};

__device__ __forceinline__ dd mk(float h) { return dd{h, 0.0f}; }
__device__ __forceinline__ dd mk(float h, float l) { return dd{h, l}; }
__device__ __forceinline__ dd norm(float s, float e) {
  const float h = s + e;
  return dd{h, e - (h - s)};
}
__device__ __forceinline__ dd neg(dd a) { return dd{-a.hi, -a.lo}; }
__device__ __forceinline__ dd add(dd a, dd b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  return norm(s, e);
}
__device__ __forceinline__ dd sub(dd a, dd b) { return add(a, neg(b)); }
__device__ __forceinline__ dd add(dd a, float b) {
  float s, e;
  two_sum(a.hi, b, s, e);
  e += a.lo;
  return norm(s, e);
}
// exact difference of two floats
__device__ __forceinline__ dd diff(float a, float b) {
  float s, e;
  two_sum(a, -b, s, e);
  return dd{s, e};
}
__device__ __forceinline__ dd mul(dd a, dd b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return norm(p, e);
}
__device__ __forceinline__ dd mul(dd a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return norm(p, e);
}
// exact product of two floats
__device__ __forceinline__ dd prod(float a, float b) {
  const float p = a * b;
  return dd{p, fmaf(a, b, -p)};
}
// a / b
__device__ __forceinline__ dd div(dd a, dd b) {
  const float inv = __frcp_rn(b.hi);
  const float q1 = a.hi * inv;
  const float p = q1 * b.hi;
  const float pe = fmaf(q1, b.hi, -p);
  // a - q1 * b: a.hi - p is exact (the two are within a factor of two)
  const float r = (((a.hi - p) - pe) + a.lo) - q1 * b.lo;
  const float q2 = r * inv;
  return norm(q1, q2);
}
__device__ __forceinline__ dd div(float a, dd b) { return div(mk(a), b); }
__device__ __forceinline__ dd div(dd a, float b) { return div(a, mk(b)); }
__device__ __forceinline__ dd recip(dd b) { return div(mk(1.0f), b); }
__device__ __forceinline__ dd dsqrt(dd a) {
  if (!(a.hi > 0.0f)) return mk(sqrtf(a.hi));
  const float x = sqrtf(a.hi);
  const dd r = sub(a, prod(x, x));
  return norm(x, r.hi * (0.5f / x));
}
__device__ __forceinline__ dd dabs(dd a) { return (a.hi < 0.0f) ? neg(a) : a; }
__device__ __forceinline__ bool lt(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool gt(dd a, dd b) { return lt(b, a); }
__device__ __forceinline__ bool lt0(dd a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo < 0.0f); }
__device__ __forceinline__ bool gt0(dd a) { return a.hi > 0.0f || (a.hi == 0.0f && a.lo > 0.0f); }
__device__ __forceinline__ bool is_zero(dd a) { return a.hi == 0.0f && a.lo == 0.0f; }
__device__ __forceinline__ bool is_nan(dd a) { return a.hi != a.hi || a.lo != a.lo; }
__device__ __forceinline__ float to_f(dd a) { return a.hi + a.lo; }
__device__ __forceinline__ double to_d(dd a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dd dmax(dd a, dd b) { return gt(a, b) ? a : b; }
__device__ __forceinline__ dd dmin(dd a, dd b) { return lt(a, b) ? a : b; }

__device__ __forceinline__ dd shfl(dd v, int src) {
  return dd{__shfl_sync(kFull, v.hi, src), __shfl_sync(kFull, v.lo, src)};
}
__device__ __forceinline__ dd shfl_xor(dd v, int o) {
  return dd{__shfl_xor_sync(kFull, v.hi, o), __shfl_xor_sync(kFull, v.lo, o)};
}

// Accumulator: hi collects the rounded partial sums, lo every rounding error
// (normalised on read).
struct Acc {
  float hi, lo;
  __device__ __forceinline__ void zero() { hi = lo = 0.0f; }
  __device__ __forceinline__ void add(float p, float e) {
    float s, t;
    two_sum(hi, p, s, t);
    hi = s;
    lo += t + e;
  }
  __device__ __forceinline__ void add(dd v) { add(v.hi, v.lo); }
  __device__ __forceinline__ void mac(dd a, dd b) {  // += a * b
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    add(p, e);
  }
  __device__ __forceinline__ void mac(dd a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    add(p, e);
  }
  __device__ __forceinline__ dd get() const { return norm(hi, lo); }
};

// Double-float constants of the reference's double literals: the nearest
// float, then the nearest float to the remainder.
__device__ __forceinline__ dd c_0p4() { return dd{0.4000000059604645f, -5.9604645663569045e-09f}; }
__device__ __forceinline__ dd c_0p7() { return dd{0.699999988079071f, 1.1920929132713809e-08f}; }
__device__ __forceinline__ dd c_0p8() { return dd{0.800000011920929f, -1.1920929132713809e-08f}; }
__device__ __forceinline__ dd c_0p01() { return dd{0.009999999776482582f, 2.2351741291171123e-10f}; }
__device__ __forceinline__ dd c_1em5() { return dd{9.999999747378752e-06f, 2.526212474884132e-13f}; }
__device__ __forceinline__ dd c_0p1() { return dd{0.10000000149011612f, -1.4901161415892261e-09f}; }
__device__ __forceinline__ dd c_0p005() { return dd{0.004999999888241291f, 1.1175870645585562e-10f}; }

// ---------------------------------------------------------------------------
// Natural logarithm in double-float (table-driven, after P. T. P. Tang,
// "Table-driven implementation of the logarithm function in IEEE floating-point
// arithmetic", ACM TOMS 16(4), 1990): x = 2^k f, f in [1, 2); c = 1 + j/128
// nearest to f; log x = k log 2 + log c + log1p(r), r = (f - c) / c, |r| <=
// 2^-8, with log1p(r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5 - r^3/6 + r^4/7).
// kLogTab[j] = log(1 + j/128) as the nearest float and the nearest float to
// the remainder, computed with 60-digit decimal arithmetic; kLogTab[128] is
// log 2.
__device__ const float2 kLogTab[129] = {
    {0.e+00f, 0.e+00f}, {7.7821403e-03f, 1.6100356e-10f}, {1.5504187e-02f, -4.3701048e-10f},
    {2.3167059e-02f, 4.560415e-10f}, {3.0771658e-02f, 8.422374e-10f}, {3.8318865e-02f, -6.9906503e-10f},
    {4.5809537e-02f, -1.1410233e-09f}, {5.3244516e-02f, -1.7346591e-09f}, {6.062462e-02f, 7.905942e-12f},
    {6.795066e-02f, 3.4083132e-09f}, {7.522342e-02f, -2.3030047e-09f}, {8.244367e-02f, -2.2728754e-10f},
    {8.9612156e-02f, 2.536962e-09f}, {9.672963e-02f, -2.28319e-09f}, {1.03796795e-01f, -1.3289232e-09f},
    {1.1081436e-01f, 3.5759316e-09f}, {1.1778303e-01f, 3.2986907e-09f}, {1.2470348e-01f, -3.2924463e-09f},
    {1.3157636e-01f, -1.4832839e-09f}, {1.3840233e-01f, -5.0360454e-09f}, {1.4518201e-01f, -3.66716e-09f},
    {1.5191604e-01f, 5.5588985e-11f}, {1.5860502e-01f, 5.9580794e-09f}, {1.6524957e-01f, 1.6911217e-09f},
    {1.7185026e-01f, -7.145759e-09f}, {1.7840765e-01f, 3.3065968e-09f}, {1.8492234e-01f, 9.619685e-10f},
    {1.9139485e-01f, 2.3879427e-09f}, {1.9782574e-01f, -1.4181957e-09f}, {2.0421554e-01f, -5.328085e-11f},
    {2.1056476e-01f, 6.7534525e-09f}, {2.1687394e-01f, -5.5050804e-09f}, {2.2314355e-01f, 3.5408485e-09f},
    {2.293741e-01f, 5.267307e-09f}, {2.3556606e-01f, 6.5973813e-09f}, {2.4171993e-01f, 5.5230855e-09f},
    {2.4783616e-01f, 6.2250236e-09f}, {2.5391522e-01f, -1.0518075e-08f}, {2.5995752e-01f, 2.2830717e-09f},
    {2.6596355e-01f, -5.885186e-09f}, {2.719337e-01f, 1.0869003e-08f}, {2.7786845e-01f, 1.3154985e-09f},
    {2.8376818e-01f, -3.901826e-09f}, {2.896333e-01f, -1.1297649e-08f}, {2.9546422e-01f, -4.7689754e-09f},
    {3.0126134e-01f, -5.0331814e-09f}, {3.0702505e-01f, -9.861567e-09f}, {3.127557e-01f, 6.0778103e-09f},
    {3.1845373e-01f, 1.9658553e-09f}, {3.2411948e-01f, -9.809915e-09f}, {3.2975328e-01f, 6.686494e-09f},
    {3.3535555e-01f, -8.129597e-09f}, {3.409266e-01f, -6.1104133e-10f}, {3.4646678e-01f, -1.2362654e-08f},
    {3.5197642e-01f, -1.2984646e-09f}, {3.5745588e-01f, 9.471959e-09f}, {3.629055e-01f, -8.629968e-09f},
    {3.6832556e-01f, -1.2631127e-10f}, {3.737164e-01f, -4.181178e-09f}, {3.7907836e-01f, -5.4768194e-09f},
    {3.844117e-01f, 6.291008e-09f}, {3.8971674e-01f, 6.7171126e-09f}, {3.949938e-01f, -3.6049104e-09f},
    {4.0024316e-01f, 1.018187e-09f}, {4.054651e-01f, 1.1872889e-08f}, {4.1065994e-01f, -1.4065406e-08f},
    {4.158279e-01f, -5.027569e-09f}, {4.209693e-01f, -1.2778508e-08f}, {4.260844e-01f, -3.9124277e-09f},
    {4.3117347e-01f, -8.778201e-09f}, {4.3623677e-01f, -2.1860347e-09f}, {4.4127455e-01f, 7.2675066e-09f},
    {4.462871e-01f, 7.081697e-09f}, {4.5127463e-01f, 1.0731866e-08f}, {4.5623744e-01f, -1.8592937e-09f},
    {4.611757e-01f, 5.1593254e-09f}, {4.6608973e-01f, 4.4302144e-09f}, {4.7097972e-01f, -5.135289e-09f},
    {4.758459e-01f, 1.711776e-09f}, {4.8068854e-01f, -1.2781857e-08f}, {4.8550782e-01f, -2.945779e-10f},
    {4.90304e-01f, -5.1799036e-09f}, {4.9507725e-01f, 1.4409851e-08f}, {4.9982786e-01f, 7.770561e-09f},
    {5.04556e-01f, 1.0519699e-08f}, {5.092619e-01f, -4.357195e-09f}, {5.1394576e-01f, -7.2405086e-09f},
    {5.1860774e-01f, 2.8574195e-08f}, {5.2324814e-01f, 7.720999e-09f}, {5.278671e-01f, 1.0839714e-08f},
    {5.324648e-01f, -3.3956955e-09f}, {5.370415e-01f, -1.9412717e-08f}, {5.415973e-01f, -2.4295618e-08f},
    {5.4613245e-01f, -7.737253e-09f}, {5.5064714e-01f, -2.1596593e-08f}, {5.551415e-01f, -1.0387525e-09f},
    {5.596158e-01f, -2.908541e-09f}, {5.6407017e-01f, -2.6872515e-08f}, {5.6850475e-01f, -1.5375939e-08f},
    {5.729197e-01f, 2.7190021e-08f}, {5.773154e-01f, -2.5075192e-08f}, {5.8169174e-01f, -2.308737e-09f},
    {5.86049e-01f, 2.4713204e-08f}, {5.9038746e-01f, -1.6967464e-08f}, {5.9470713e-01f, -2.363911e-08f},
    {5.990082e-01f, -1.2906712e-08f}, {6.0329086e-01f, -4.4464676e-09f}, {6.0755527e-01f, -1.9970466e-08f},
    {6.1180156e-01f, -2.3587457e-08f}, {6.1602986e-01f, 1.8626341e-08f}, {6.202404e-01f, 1.9451107e-08f},
    {6.244333e-01f, 8.974418e-09f}, {6.2860864e-01f, 1.5413738e-08f}, {6.3276666e-01f, 5.54287e-09f},
    {6.3690746e-01f, 3.9317105e-09f}, {6.410312e-01f, -2.6233213e-08f}, {6.4513797e-01f, -4.305584e-09f},
    {6.492279e-01f, 2.9430744e-08f}, {6.533013e-01f, -2.6605571e-08f}, {6.5735805e-01f, 2.2361986e-08f},
    {6.613985e-01f, 1.1843601e-08f}, {6.654226e-01f, 1.4155961e-08f}, {6.694307e-01f, -1.9179776e-08f},
    {6.734227e-01f, -1.899407e-08f}, {6.773988e-01f, 2.2741892e-08f}, {6.8135923e-01f, -6.6641124e-09f},
    {6.85304e-01f, 1.7026379e-08f}, {6.892333e-01f, -2.1831259e-08f}, {6.931472e-01f, -1.9046542e-09f}};

__device__ __forceinline__ dd dlog(dd x) {
  if (!(x.hi > 0.0f)) return mk(x.hi == 0.0f ? __int_as_float(0xff800000) : __int_as_float(0x7fc00000));
  if (!(x.hi < 3.0e38f)) return mk(x.hi);  // +inf, or NaN
  // x = 2^k f with f in [1, 2); x.lo scaled by 2^-k alike
  const int bits = __float_as_int(x.hi);
  const int ex = (bits >> 23) & 0xff;
  if (ex < 2 || ex > 252) return mk(logf(x.hi));  // outside the fitter's range
  const int k = ex - 127;
  const float f = __int_as_float((bits & 0x007fffff) | 0x3f800000);
  const float flo = x.lo * __int_as_float((127 - k) << 23);
  const int j = __float2int_rn((f - 1.0f) * 128.0f);
  const float c = 1.0f + (float)j * (1.0f / 128.0f);
  // r = ((f - c) + flo) / c; f - c is exact
  const dd u = add(mk(f - c), flo);
  const dd r = div(u, mk(c));
  // log1p(r)
  const float rh = r.hi;
  const dd r2 = prod(rh, rh);  // r.hi^2 exactly
  const float r2l = r2.lo + 2.0f * rh * r.lo;
  const float p = fmaf(fmaf(fmaf(fmaf(rh, 1.0f / 7.0f, -1.0f / 6.0f), rh, 0.2f), rh, -0.25f), rh,
                       1.0f / 3.0f);
  const float t3 = (r2.hi * rh) * p;
  dd s = sub(r, dd{0.5f * r2.hi, 0.5f * r2l});
  s = add(s, t3);
  const float2 T = __ldg(&kLogTab[j]);
  const float2 L2 = __ldg(&kLogTab[128]);
  s = add(s, dd{T.x, T.y});
  // k log 2: k * ln2_hi exactly (two-product), plus k * ln2_lo
  const float kf = (float)k;
  dd kl = prod(kf, L2.x);
  kl = add(kl, kf * L2.y);
  return add(kl, s);
}

// ---------------------------------------------------------------------------
// Basis and weights (CPUsplineLib.cpp:1289-1326) in double-float, in the
// reference's polynomial forms with its float literals: for a = |x|,
// B3 = 2/3 - a^2 + a^3/2 (a < 1), 4/3 - 2a + a^2 - a^3/6 (1 <= a < 2);
// B2 = 3/4 - a^2 (a < 1/2), 9/8 - 3a/2 + a^2/2 (1/2 <= a < 3/2).

__device__ __forceinline__ dd bspline3(dd x) {
  // The reference's pieces are half-open in the signed argument: [-1, 1)
  // takes the inner form, [1, 2) and [-2, -1) the outer one. With its float
  // literals the two forms differ by about 4e-8 at |x| = 1, so the signed
  // bounds are kept (x = -1 is inner, x = 1 outer).
  const dd a = dabs(x);
  const bool ge_m1 = !lt(x, mk(-1.0f)), lt_p1 = lt(x, mk(1.0f));
  const bool ge_m2 = !lt(x, mk(-2.0f)), lt_p2 = lt(x, mk(2.0f));
  if (ge_m1 && lt_p1) {
    const dd a2 = mul(a, a);
    const dd a3 = mul(a2, a);
    return add(sub(mk(2.0f / 3.0f), a2), dd{0.5f * a3.hi, 0.5f * a3.lo});
  }
  if (ge_m2 && lt_p2) {
    const dd a2 = mul(a, a);
    const dd a3 = mul(a2, a);
    dd v = sub(mk(4.0f / 3.0f), dd{2.0f * a.hi, 2.0f * a.lo});
    v = add(v, a2);
    return sub(v, mul(a3, 1.0f / 6.0f));
  }
  return mk(0.0f);
}

__device__ __forceinline__ dd bspline2(dd x) {
  // [-1/2, 1/2) inner, [1/2, 3/2) and [-3/2, -1/2) outer; the two forms agree
  // exactly at |x| = 1/2 (their constants are exact).
  const dd a = dabs(x);
  const dd a2 = mul(a, a);
  if (!lt(x, mk(-0.5f)) && lt(x, mk(0.5f))) return sub(mk(0.75f), a2);
  if (!lt(x, mk(-1.5f)) && lt(x, mk(1.5f))) {
    dd v = sub(mk(1.125f), mul(a, 1.5f));
    return add(v, dd{0.5f * a2.hi, 0.5f * a2.lo});
  }
  return mk(0.0f);
}

// Weight j of an axis at fractional position t: j = 0..3 the value weight
// B3(t - o) of the node at offset o = j - 1; j = 4..6 the derivative weight
// B2(t - o - 1/2) of the node difference C[o + 1] - C[o], o = j - 5.
__device__ __forceinline__ dd axis_weight(dd t, int j) {
  const float off = (j < 4) ? (float)(j - 1) : (float)(j - 5) + 0.5f;
  const dd x = add(t, -off);
  return (j < 4) ? bspline3(x) : bspline2(x);
}

// floor of a double-float value as an int, with the x86 conversion rule of
// the reference build (NaN or out of range: INT_MIN).
__device__ __forceinline__ int dfloor_int(dd x) {
  float f = floorf(x.hi);
  if (f == x.hi && x.lo < 0.0f) f -= 1.0f;
  if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT_MIN;
  return __float2int_rz(f);
}
__device__ __forceinline__ dd dfrac(dd x) {
  float f = floorf(x.hi);
  if (f == x.hi && x.lo < 0.0f) f -= 1.0f;
  return add(x, -f);
}
// Knot index (CPUsplineLib.cpp:1204-1226): floor(pos) clamped to [1, n - 1],
// or n when pos equals n exactly.
__device__ __forceinline__ int knot_index(dd pos, int n) {
  int c = dfloor_int(pos);
  c = c > 1 ? c : 1;
  c = c < n - 1 ? c : n - 1;
  if (pos.hi == (float)n && pos.lo == 0.0f) c = n;
  return c;
}

// ---------------------------------------------------------------------------

template <int MODE>
struct Traits;
template <>
struct Traits<6> {
  static constexpr int D = 3, NV = 5, NA = 2, NG = 3;
};
template <>
struct Traits<7> {
  static constexpr int D = 4, NV = 6, NA = 3, NG = 4;
};
template <>
struct Traits<8> {
  static constexpr int D = 5, NV = 8, NA = 8, NG = 10;
};

// Per-warp shared memory, in floats: pixels (s^2, padded to 4), lateral knots
// (s each, padded to 4), the 1-D weights (5 axes x 8 double-floats), then the
// maps as double-float pairs: the stage-A maps by X column (NA maps x WP rows
// per column, column stride AS) and the stage-B maps by (X node, pixel row)
// item (NG maps per item, item stride GP). For fit type 8 the stage-B maps
// are written over stage-A columns already read (stage B walks the columns in
// order; G column c ends before A column c starts), as in the FP32 kernels.
struct Layout {
  int s, s2p, wp, na, ng;
  bool alias;
  __host__ __device__ constexpr int as() const { return na * wp + 1; }  // float2 units
  __host__ __device__ constexpr int gp() const { return ng | 1; }
  __host__ __device__ constexpr int gs() const { return s * gp(); }
  __host__ __device__ constexpr int off_kx() const { return s2p; }
  __host__ __device__ constexpr int off_ky() const { return off_kx() + ((s + 3) & ~3); }
  __host__ __device__ constexpr int off_w() const { return off_ky() + ((s + 3) & ~3); }  // even
  __host__ __device__ constexpr int off_maps() const { return off_w() + 5 * 8 * 2; }  // even
  // map offsets in float2 units from off_maps
  __host__ __device__ constexpr int a_rel() const {
    return alias ? gs() + (wp - 1) * (gs() > as() ? gs() - as() : 0) : wp * gs();
  }
  __host__ __device__ constexpr int maps2() const {
    return (a_rel() + wp * as() > wp * gs()) ? a_rel() + wp * as() : wp * gs();
  }
  __host__ __device__ constexpr int total() const { return off_maps() + 2 * maps2(); }  // floats
};

__host__ __device__ constexpr Layout make_layout(int mode, int s) {
  Layout L{};
  L.s = s;
  L.s2p = (s * s + 3) & ~3;
  L.wp = s + 4;
  L.na = mode == 6 ? 2 : mode == 7 ? 3 : 8;
  L.ng = mode == 6 ? 3 : mode == 7 ? 4 : 10;
  L.alias = mode == 8;
  return L;
}

constexpr bool layouts_ok() {
  const int modes[3] = {6, 7, 8};
  for (int mi = 0; mi < 3; ++mi)
    for (int s = 1; s <= 51; ++s) {
      const Layout L = make_layout(modes[mi], s);
      if (L.s2p < s * s || L.off_kx() + s > L.off_ky() || L.off_ky() + s > L.off_w() ||
          (L.off_w() & 1) || (L.off_maps() & 1) || L.off_w() + 80 > L.off_maps())
        return false;
      if (L.a_rel() + L.wp * L.as() > L.maps2() || L.wp * L.gs() > L.maps2()) return false;
      if (L.as() < L.na * L.wp || L.gp() < L.ng) return false;
      if (L.alias)
        for (int c = 0; c < L.wp; ++c)
          if ((c + 1) * L.gs() > L.a_rel() + c * L.as()) return false;
    }
  return true;
}
static_assert(layouts_ok(), "double-float per-warp shared-memory regions overlap");

// ---------------------------------------------------------------------------
// One ROI evaluation's per-lane partial sums.

template <int MODE>
__device__ __forceinline__ void channel_pass(const FitArgs& a, const Layout& L, float* ws, int lane,
                                             const dd* th, bool dup45, bool fisher, Acc& err,
                                             Acc (&acc)[Traits<MODE>::NV + Traits<MODE>::NV *
                                                                                (Traits<MODE>::NV + 1) / 2],
                                             bool maps_ready = false) {
  using TR = Traits<MODE>;
  constexpr int D = TR::D;
  constexpr int NV = TR::NV;
  const int s = L.s;
  const ModelDev& m = a.m;
  int* kxs = reinterpret_cast<int*>(ws + L.off_kx());
  int* kys = reinterpret_cast<int*>(ws + L.off_ky());
  float2* w = reinterpret_cast<float2*>(ws + L.off_w());  // [axis * 8 + j]
  float2* maps = reinterpret_cast<float2*>(ws + L.off_maps());
  float2* G = maps;                // G[(xr * s + py) * GP + map]
  float2* A = maps + L.a_rel();    // A[xr * AS + map * wp + yr]
  const int wp = L.wp, AS = L.as(), GP = L.gp(), GS = L.gs();
  __syncwarp();

  // Positions (CPUmleFit_LM.cpp:2512-2523): pixel jj at (xc + jj) + off along
  // X, pixel ii at (yc + ii) + off along Y.
  const float half = (float)((s + 1) / 2);
  const dd xc = sub(mk(half), th[0]);
  const dd yc = sub(mk(half), th[1]);
  const float off = (float)(m.n[1] - s) / 2.0f;
  const dd zc = th[4];
  const dd wc = (D >= 4) ? th[5] : mk(0.0f);
  const dd uc = (D >= 5) ? th[6] : mk(0.0f);
  for (int j = lane; j < s; j += 32) {
    kxs[j] = knot_index(add(xc, (float)j + off), m.n[1]);
    kys[j] = knot_index(add(yc, (float)j + off), m.n[0]);
  }
  {
    dd fr[5] = {dfrac(yc), dfrac(xc), dfrac(zc), dfrac(wc), dfrac(uc)};
    for (int k = lane; k < 7 * D; k += 32) {
      const int ax = k / 7;
      const dd v = axis_weight(fr[ax], k - ax * 7);
      w[ax * 8 + (k - ax * 7)] = make_float2(v.hi, v.lo);
    }
  }
  __syncwarp();
  int kxmin, kxmax, kymin, kymax;
  {
    int a0 = INT_MAX, a1 = INT_MIN, b0 = INT_MAX, b1 = INT_MIN;
    for (int j = lane; j < s; j += 32) {
      a0 = min(a0, kxs[j]);
      a1 = max(a1, kxs[j]);
      b0 = min(b0, kys[j]);
      b1 = max(b1, kys[j]);
    }
    kxmin = warp_min(a0);
    kxmax = warp_max(a1);
    kymin = warp_min(b0);
    kymax = warp_max(b1);
  }
  const int xb = kxmin - 1, wx = min(kxmax - kxmin + 4, wp);
  const int yb = kymin - 1, wy = min(kymax - kymin + 4, wp);
  const int kz = knot_index(zc, m.n[2]);
  const int kw = (D >= 4) ? knot_index(wc, m.n[3]) : 0;
  const int ku = (D >= 5) ? knot_index(uc, m.n[4]) : 0;
  auto W = [&](int ax, int j) {
    const float2 v = w[ax * 8 + j];
    return dd{v.x, v.y};
  };

  // (A) non-lateral contraction at every lateral node of the window; skipped
  // with maps_ready (the workspace holds the maps of the previous evaluation,
  // made at the same spatial parameters)
  if (!maps_ready) {
    dd bz[4], dz[3];
#pragma unroll
    for (int q = 0; q < 4; ++q) bz[q] = W(2, q);
#pragma unroll
    for (int q = 0; q < 3; ++q) dz[q] = W(2, 4 + q);
    const int64_t sz_ = m.st[2];
    const int nodes = wx * wy;
    // value and z-derivative contractions of one z column of 4 floats
    auto zcol = [&](const float* p, dd& v, dd& d) {
      const float c0 = __ldg(p), c1 = __ldg(p + sz_), c2 = __ldg(p + 2 * sz_), c3 = __ldg(p + 3 * sz_);
      Acc av, ad;
      av.zero();
      ad.zero();
      av.mac(bz[0], c0);
      av.mac(bz[1], c1);
      av.mac(bz[2], c2);
      av.mac(bz[3], c3);
      ad.mac(diff(c1, c0), dz[0]);
      ad.mac(diff(c2, c1), dz[1]);
      ad.mac(diff(c3, c2), dz[2]);
      v = av.get();
      d = ad.get();
    };
    if constexpr (D == 3) {
      const float* base = m.coeff + (int64_t)(kz - 1) * sz_;
      for (int t = lane; t < nodes; t += 32) {
        const int xr = t / wy, yr = t - xr * wy;
        dd v, d;
        zcol(base + (int64_t)(xb + xr) * m.st[1] + (yb + yr), v, d);
        A[xr * AS + yr] = make_float2(v.hi, v.lo);
        A[xr * AS + wp + yr] = make_float2(d.hi, d.lo);
      }
    } else if constexpr (D == 4) {
      dd bw[4], dw[3];
#pragma unroll
      for (int q = 0; q < 4; ++q) bw[q] = W(3, q);
#pragma unroll
      for (int q = 0; q < 3; ++q) dw[q] = W(3, 4 + q);
      const int64_t sw_ = m.st[3];
      const float* base = m.coeff + (int64_t)(kz - 1) * sz_ + (int64_t)(kw - 1) * sw_;
      for (int t = lane; t < nodes; t += 32) {
        const int xr = t / wy, yr = t - xr * wy;
        const float* p = base + (int64_t)(xb + xr) * m.st[1] + (yb + yr);
        dd vz[4], dzv[4];
#pragma unroll
        for (int iw = 0; iw < 4; ++iw) zcol(p + iw * sw_, vz[iw], dzv[iw]);
        Acc av, ad, aw;
        av.zero();
        ad.zero();
        aw.zero();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          av.mac(vz[q], bw[q]);
          ad.mac(dzv[q], bw[q]);
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) aw.mac(sub(vz[q + 1], vz[q]), dw[q]);
        const dd v = av.get(), d = ad.get(), dwv = aw.get();
        A[xr * AS + yr] = make_float2(v.hi, v.lo);
        A[xr * AS + wp + yr] = make_float2(d.hi, d.lo);
        A[xr * AS + 2 * wp + yr] = make_float2(dwv.hi, dwv.lo);
      }
    } else {
      // 5D (z, w, u) for the mixture's 5D part plus its 3D part (z only, on
      // coeff3 with the same lateral and z knots), with the reference's two
      // derivative index quirks as correction maps (see bsfit_fit.cu).
      dd bw[4], dw[3], bu[4], du[3];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        bw[q] = W(3, q);
        bu[q] = W(4, q);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        dw[q] = W(3, 4 + q);
        du[q] = W(4, 4 + q);
      }
      // Correction weights of the z-derivative term 27 (CPUsplineLib.cpp:313),
      // R[lvZ-1][lvW-1][lvU-1] = (weight read) - (weight intended).
      dd R[2][2][2];
#pragma unroll
      for (int lz = 1; lz <= 2; ++lz)
#pragma unroll
        for (int lw = 1; lw <= 2; ++lw)
#pragma unroll
          for (int lu = 1; lu <= 2; ++lu) {
            const int v = (lw - 1) + 2 * (lu - 1);
            const dd dBz1 = (lz == 1) ? dz[1] : dz[0];
            const dd dBz2 = (lz == 1) ? dz[2] : mk(0.0f);
            const dd Bz2 = (lz == 1) ? bz[2] : bz[3];
            dd rp;
            if (v < 3) {
              const int vp = v + 1, lwp = (vp & 1) + 1, lup = (vp >> 1) + 1;
              rp = mul(mul(dBz2, lwp == 1 ? bw[2] : bw[3]), lup == 1 ? bu[1] : bu[0]);
            } else {
              rp = mul(mul(Bz2, dw[2]), bu[1]);
            }
            R[lz - 1][lw - 1][lu - 1] =
                sub(rp, mul(mul(dBz1, lw == 1 ? bw[2] : bw[3]), lu == 1 ? bu[2] : bu[3]));
          }
      const int64_t sw_ = m.st[3], su_ = m.st[4];
      const float* base = m.coeff + (int64_t)(kz - 1) * sz_ + (int64_t)(kw - 1) * sw_ +
                          (int64_t)(ku - 1) * su_;
      const float* base3 = m.coeff3 + (int64_t)(kz - 1) * sz_;
      for (int t = lane; t < nodes; t += 32) {
        const int xr = t / wy, yr = t - xr * wy;
        const int64_t lat = (int64_t)(xb + xr) * m.st[1] + (yb + yr);
        const float* p = base + lat;
        dd vw[4], dzw[4], dww[4];
        Acc qz;
        qz.zero();
        dd sq[4][2];  // [u][w in {0,1}]: sum over z in {0,1} of Bz * C
#pragma unroll 1
        for (int iu = 0; iu < 4; ++iu) {
          dd vz[4], dzz[4];
#pragma unroll
          for (int iw = 0; iw < 4; ++iw) {
            const float* q = p + iu * su_ + iw * sw_;
            const float c0 = __ldg(q), c1 = __ldg(q + sz_), c2 = __ldg(q + 2 * sz_), c3 = __ldg(q + 3 * sz_);
            Acc av, ad;
            av.zero();
            ad.zero();
            av.mac(bz[0], c0);
            av.mac(bz[1], c1);
            av.mac(bz[2], c2);
            av.mac(bz[3], c3);
            const dd d10 = diff(c1, c0), d21 = diff(c2, c1), d32 = diff(c3, c2);
            ad.mac(d10, dz[0]);
            ad.mac(d21, dz[1]);
            ad.mac(d32, dz[2]);
            vz[iw] = av.get();
            dzz[iw] = ad.get();
            if (iu >= 2 && iw >= 2) {
              // lvW = iw - 1, lvU = iu - 1; z nodes 1..2 (lvZ 1), 0..1 (lvZ 2)
              qz.mac(d21, R[0][iw - 2][iu - 2]);
              qz.mac(d10, R[1][iw - 2][iu - 2]);
            }
            if (iw <= 1) {
              Acc sqa;
              sqa.zero();
              sqa.mac(bz[0], c0);
              sqa.mac(bz[1], c1);
              sq[iu][iw] = sqa.get();
            }
          }
          Acc a0, a1, a2;
          a0.zero();
          a1.zero();
          a2.zero();
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            a0.mac(vz[q], bw[q]);
            a1.mac(dzz[q], bw[q]);
          }
#pragma unroll
          for (int q = 0; q < 3; ++q) a2.mac(sub(vz[q + 1], vz[q]), dw[q]);
          vw[iu] = a0.get();
          dzw[iu] = a1.get();
          dww[iu] = a2.get();
        }
        Acc av, az, aw, au;
        av.zero();
        az.zero();
        aw.zero();
        au.zero();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          av.mac(vw[q], bu[q]);
          az.mac(dzw[q], bu[q]);
          aw.mac(dww[q], bu[q]);
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) au.mac(sub(vw[q + 1], vw[q]), du[q]);
        // u-term-16 correction (CPUsplineLib.cpp:420-421)
        Acc qu;
        qu.zero();
#pragma unroll
        for (int iw = 0; iw < 2; ++iw)
          qu.mac(sub(sub(sq[2][iw], sq[1][iw]), sub(sq[3][iw], sq[2][iw])), bw[iw]);
        const dd quv = mul(qu.get(), du[2]);
        const float* p3 = base3 + lat;
        dd v3, d3;
        zcol(p3, v3, d3);
        float2* o = A + xr * AS + yr;
        const dd vals[8] = {av.get(), az.get(), aw.get(), au.get(), qz.get(), quv, v3, d3};
#pragma unroll
        for (int c = 0; c < 8; ++c) o[c * wp] = make_float2(vals[c].hi, vals[c].lo);
      }
    }
  }
  __syncwarp();

  // (B) Y contraction for every (X node, pixel row)
  if (!maps_ready) {
    dd by[4], dy[3];
#pragma unroll
    for (int q = 0; q < 4; ++q) by[q] = W(0, q);
#pragma unroll
    for (int q = 0; q < 3; ++q) dy[q] = W(0, 4 + q);
    constexpr int NG = TR::NG;
    const int items = wx * s;
    for (int t0 = 0; t0 < items; t0 += 32) {
      const int t = t0 + lane;
      const bool act = t < items;
      const int xr = act ? t / s : 0, py = act ? t - xr * s : 0;
      dd gv[NG];
      if (act) {
        const int oy = min(max(kys[py] - 1 - yb, 0), wy - 4);
        const float2* a0 = A + xr * AS + oy;
        auto ld = [&](const float2* q, int k) {
          const float2 v = q[k];
          return dd{v.x, v.y};
        };
        auto yval = [&](const float2* q) {
          Acc r;
          r.zero();
#pragma unroll
          for (int k = 0; k < 4; ++k) r.mac(ld(q, k), by[k]);
          return r.get();
        };
        auto yder = [&](const float2* q) {
          const dd v0 = ld(q, 0), v1 = ld(q, 1), v2 = ld(q, 2), v3 = ld(q, 3);
          Acc r;
          r.zero();
          r.mac(sub(v1, v0), dy[0]);
          r.mac(sub(v2, v1), dy[1]);
          r.mac(sub(v3, v2), dy[2]);
          return r.get();
        };
        gv[0] = yval(a0);
        gv[1] = yder(a0);
        if constexpr (MODE != 8) {
#pragma unroll
          for (int c = 1; c < TR::NA; ++c) gv[c + 1] = yval(a0 + c * wp);
        } else {
#pragma unroll
          for (int c = 1; c <= 3; ++c) gv[c + 1] = yval(a0 + c * wp);
          {
            const float2* q = a0 + 4 * wp;  // lateral side 2: offsets +1, +2
            Acc r;
            r.zero();
            r.mac(ld(q, 2), by[2]);
            r.mac(ld(q, 3), by[3]);
            gv[5] = r.get();
          }
          {
            const float2* q = a0 + 5 * wp;  // lateral side 1: offsets -1, 0
            Acc r;
            r.zero();
            r.mac(ld(q, 0), by[0]);
            r.mac(ld(q, 1), by[1]);
            gv[6] = r.get();
          }
          gv[7] = yval(a0 + 6 * wp);
          gv[8] = yder(a0 + 6 * wp);
          gv[9] = yval(a0 + 7 * wp);
        }
      }
      if (L.alias) __syncwarp();  // G is written over A columns already read
      if (act) {
        float2* go = G + (xr * s + py) * GP;
#pragma unroll
        for (int c = 0; c < NG; ++c) go[c] = make_float2(gv[c].hi, gv[c].lo);
      }
    }
  }
  __syncwarp();

  // (C) X contraction per pixel, fused with the likelihood sums
  {
    dd bx[4], dx[3];
#pragma unroll
    for (int q = 0; q < 4; ++q) bx[q] = W(1, q);
#pragma unroll
    for (int q = 0; q < 3; ++q) dx[q] = W(1, 4 + q);
    const dd N = th[2], bg = th[3];
    const int s2 = s * s;
    for (int p = lane; p < s2; p += 32) {
      const int px = p / s, py = p - px * s;  // px = jj (X), py = ii (Y)
      const int ox = min(max(kxs[px] - 1 - xb, 0), wx - 4);
      const float2* g = G + (ox * s + py) * GP;  // X node k of map c at g[k * GS + c]
      auto ld = [&](int c, int k) {
        const float2 v = g[k * GS + c];
        return dd{v.x, v.y};
      };
      auto xval = [&](int c) {
        Acc r;
        r.zero();
#pragma unroll
        for (int k = 0; k < 4; ++k) r.mac(ld(c, k), bx[k]);
        return r.get();
      };
      auto xder = [&](int c) {
        const dd v0 = ld(c, 0), v1 = ld(c, 1), v2 = ld(c, 2), v3 = ld(c, 3);
        Acc r;
        r.zero();
        r.mac(sub(v1, v0), dx[0]);
        r.mac(sub(v2, v1), dx[1]);
        r.mac(sub(v3, v2), dx[2]);
        return r.get();
      };
      const dd f = xval(0);
      const dd dX = xder(0);
      const dd dY = xval(1);
      dd dudt[NV];
      dd model;
      if constexpr (MODE != 8) {
        dudt[0] = neg(mul(N, dX));
        dudt[1] = neg(mul(N, dY));
        dudt[2] = f;
        dudt[3] = mk(1.0f);
#pragma unroll
        for (int c = 1; c < TR::NA; ++c) dudt[3 + c] = mul(N, xval(c + 1));
        if (MODE == 7 && dup45) dudt[5] = dudt[4];
        model = add(bg, mul(N, f));
      } else {
        Acc az, au;
        az.zero();
        au.zero();
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          az.mac(ld(2, k), bx[k]);
          au.mac(ld(4, k), bx[k]);
        }
        az.mac(ld(5, 2), bx[2]);
        az.mac(ld(5, 3), bx[3]);
        au.mac(ld(6, 0), bx[0]);
        au.mac(ld(6, 1), bx[1]);
        const dd dZ = az.get(), dU = au.get(), dW = xval(3);
        const dd f3 = xval(7), dX3 = xder(7), dY3 = xval(8), dZ3 = xval(9);
        // mixture (CPUmleFit_LM.cpp:3311-3322)
        const dd g2 = th[7], h2m = sub(mk(1.0f), g2);
        const dd m5 = add(bg, mul(N, f)), m3 = add(bg, mul(N, f3));
        dudt[0] = add(mul(neg(mul(N, dX)), g2), mul(h2m, neg(mul(N, dX3))));
        dudt[1] = add(mul(neg(mul(N, dY)), g2), mul(h2m, neg(mul(N, dY3))));
        dudt[2] = add(mul(f, g2), mul(h2m, f3));
        dudt[3] = add(g2, h2m);
        dudt[4] = add(mul(mul(N, dZ), g2), mul(h2m, mul(N, dZ3)));
        dudt[5] = mul(N, dW);
        dudt[6] = mul(N, dU);
        dudt[7] = sub(m5, m3);
        model = add(mul(m3, h2m), mul(m5, g2));
      }
      float d = ws[p];
      if (!fisher) {
        // CPUmleFit_LM.cpp:2540-2559
        dd term, dm = mk(0.0f);
        if (d > 0.0f) {
          const dd lq = dlog(div(model, d));
          term = sub(add(model, -d), mul(lq, d));
          dm = div(d, model);
        } else {
          term = model;
          d = 0.0f;
        }
        err.add(2.0f * term.hi, 2.0f * term.lo);
        const dd t1 = sub(mk(1.0f), dm);
        const dd t2 = div(dm, model);
#pragma unroll
        for (int l = 0; l < NV; ++l) acc[l].mac(t1, dudt[l]);
        int k = NV;
#pragma unroll
        for (int l = 0; l < NV; ++l) {
          const dd tl = mul(t2, dudt[l]);
#pragma unroll
          for (int mm = l; mm < NV; ++mm, ++k) acc[k].mac(tl, dudt[mm]);
        }
      } else {
        // Fisher information and log-likelihood (CPUmleFit_LM.cpp:2730-2742);
        // the log-likelihood term d log m - m - d log d + d as d log(m/d) - (m - d)
        const dd im = recip(model);
        int k = NV;
#pragma unroll
        for (int l = 0; l < NV; ++l) {
          const dd tl = mul(dudt[l], im);
#pragma unroll
          for (int mm = l; mm < NV; ++mm, ++k) acc[k].mac(tl, dudt[mm]);
        }
        if (gt0(model)) {
          if (d > 0.0f) {
            const dd lq = dlog(div(model, d));
            err.add(sub(mul(lq, d), add(model, -d)));
          } else {
            err.add(neg(model));
          }
        }
      }
    }
  }
}

// Reduce-scatter of C double-float sums (the exchange rule of reduce_scatter
// in bsfit_device.cuh: every total is a butterfly sum tree over the 32 lanes).
template <int C, int O, int N>
__device__ __forceinline__ void reduce_scatter_dd(dd (&v)[N], int lane) {
  if constexpr (O > 0) {
    constexpr int P = C / 2;
    const bool up = (lane & O) != 0;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const dd send = up ? v[i] : v[i + P];
      const dd keep = up ? v[i + P] : v[i];
      v[i] = add(keep, shfl_xor(send, O));
    }
    if constexpr ((C & 1) != 0) v[P] = add(v[2 * P], shfl_xor(v[2 * P], O));
    reduce_scatter_dd<P + (C & 1), O / 2>(v, lane);
  }
}

template <int SLOTS, typename Code>
__device__ __forceinline__ dd rs_gather_dd(dd t0, dd t1, Code codes, int sh) {
  if constexpr (SLOTS > 1) {
    const int code = (int)((codes >> sh) & 63u);
    const dd a0 = shfl(t0, code >> 1);
    const dd a1 = shfl(t1, code >> 1);
    return (code & 1) ? a1 : a0;
  } else {
    return shfl(t0, (int)((codes >> sh) & 31u));
  }
}

__device__ __forceinline__ dd warp_sum_dd(dd v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = add(v, shfl_xor(v, o));
  return v;
}

// One evaluation: lane l < NV receives gradient entry l (gl) and Hessian (or
// Fisher) row l (hr); the deviance (or log-likelihood) is on every lane.
template <int MODE>
__device__ void evaluate(const FitArgs& a, const Layout& L, float* ws, int lane, const dd* th,
                         bool dup45, bool fisher, dd& err_out, dd& gl, dd (&hr)[Traits<MODE>::NV],
                         bool maps_ready = false) {
  constexpr int NV = Traits<MODE>::NV;
  constexpr int K = NV + NV * (NV + 1) / 2;
  Acc err;
  err.zero();
  Acc acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k].zero();
  channel_pass<MODE>(a, L, ws, lane, th, dup45, fisher, err, acc, maps_ready);
  dd v[K];
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = acc[k].get();
  reduce_scatter_dd<K, 16>(v, lane);
  constexpr GatherCodes<NV, K> GC{};
  const dd t0 = v[0];
  const dd t1 = (rs_slots(K) > 1) ? v[1 < K ? 1 : 0] : mk(0.0f);
  const int sh = GC.B * (lane < NV ? lane : NV - 1);
  gl = rs_gather_dd<rs_slots(K)>(t0, t1, GC.grad, sh);
#pragma unroll
  for (int k = 0; k < NV; ++k) hr[k] = rs_gather_dd<rs_slots(K)>(t0, t1, GC.row[k], sh);
  err_out = warp_sum_dd(err.get());
}

// ---------------------------------------------------------------------------
// LM (lane-parallel, double-float)

template <int MODE>
__device__ __forceinline__ void clamp_fade(int l, dd& c, dd& f) {
  if (MODE == 6) {
    c = mk((l < 2) ? 2.0f : (l == 2) ? 10000.0f : 20.0f);
    f = mk(0.5f);
  } else if (MODE == 7) {
    c = (l < 2) ? mk(1.0f) : (l == 2) ? mk(10000.0f) : (l == 3) ? mk(20.0f) : (l == 4) ? mk(2.0f) : c_1em5();
    f = (l < 2) ? mk(0.5f) : (l == 2) ? c_0p4() : (l == 3) ? mk(0.5f) : (l == 4) ? c_0p7() : c_0p8();
  } else {
    c = (l < 2) ? mk(1.0f) : (l == 2) ? mk(10000.0f) : (l == 3) ? mk(20.0f) : (l < 7) ? mk(2.0f) : c_0p1();
    f = mk(0.5f);
  }
}

// Lane-parallel solve of (L L^T) x = b: lane i holds b_i, row i of L (lr),
// column i below the diagonal (lc[k] = L[k][i]) and 1 / L_ii (invd).
template <int NV>
__device__ __forceinline__ dd lane_solve(int lane, const dd (&lr)[NV], const dd (&lc)[NV], dd invd, dd b) {
  dd y = b;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const dd yk = shfl(mul(y, invd), k);
    if (lane == k) y = yk;
    else if (lane > k) y = sub(y, mul(lr[k], yk));
  }
  dd x = y;
#pragma unroll
  for (int k = NV - 1; k >= 0; --k) {
    const dd xk = shfl(mul(x, invd), k);
    if (lane == k) x = xk;
    else if (lane < k) x = sub(x, mul(lc[k], xk));
  }
  return x;
}

// Initial x, y, N, bg (CPUgaussLib.cpp:172-225, CPUmleFit_LM.cpp:2477-2482) in
// double-float: the centroid sums are exact products summed in double-float.
__device__ __forceinline__ void initial_guess(const float* data, int s, int lane, dd (&g)[4]) {
  const int s2 = s * s;
  Acc tx, ty, ts;
  tx.zero();
  ty.zero();
  ts.zero();
  float mx = 0.0f, mn = 10e10f;
  bool nan_seen = false;
  for (int p = lane; p < s2; p += 32) {
    const float d = data[p];
    const int jj = p / s, ii = p - jj * s;
    const dd px = prod(d, (float)ii), py = prod(d, (float)jj);
    tx.add(px.hi, px.lo);
    ty.add(py.hi, py.lo);
    ts.add(d, 0.0f);
    nan_seen |= (d != d);
    mx = (mx > d) ? mx : d;
    mn = (mn < d) ? mn : d;
  }
  const dd sx = warp_sum_dd(tx.get()), sy = warp_sum_dd(ty.get()), st = warp_sum_dd(ts.get());
  if (__any_sync(kFull, nan_seen)) {
    mx = 0.0f;
    mn = 10e10f;
    for (int p0 = 0; p0 < s2; ++p0) {
      const float d = data[p0];
      mx = (mx > d) ? mx : d;
      mn = (mn < d) ? mn : d;
    }
  } else {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
      mn = fminf(mn, __shfl_xor_sync(kFull, mn, o));
    }
  }
  g[0] = div(sx, st);
  g[1] = div(sy, st);
  // N0 = max(0, ((max - min) * 2) * PI * 1.5 * 1.5), PI the float literal
  dd n0 = diff(mx, mn);
  n0 = dd{2.0f * n0.hi, 2.0f * n0.lo};
  n0 = mul(mul(mul(n0, 3.141592f), 1.5f), 1.5f);
  g[2] = lt0(n0) ? mk(0.0f) : n0;  // (0 > n0) ? 0 : n0, NaN kept
  g[3] = dmax(mk(mn), c_0p01());
}

struct Result {
  float par, crlb, ll;
  int kk;
};

__device__ __forceinline__ dd from_double(double v) {
  const float h = __double2float_rn(v);
  return dd{h, __double2float_rn(v - (double)h)};
}

template <int MODE>
__device__ Result fit_roi(const FitArgs& a, const Layout& L, float* ws, int lane, int64_t roi) {
  using TR = Traits<MODE>;
  constexpr int NV = TR::NV;
  const int s = L.s;
  dd par;
  {
    dd g[4];
    initial_guess(ws, s, lane, g);
    dd v = mk(0.0f);
    v = (lane == 0) ? g[0] : (lane == 1) ? g[1] : (lane == 2) ? g[2] : (lane == 3) ? g[3] : v;
    if (MODE == 6) {
      if (lane == 4) v = mk((float)a.m.n[2] / 2.0f);
    } else if (MODE == 7) {
      const float* ip = a.m.init_p;
      const bool use = a.m.init_p_len >= 2 && ip[0] != 0.0f;
      if (lane == 4) v = mk(use ? ip[0] : (float)a.m.n[2] / 2.0f);
      if (lane == 5) v = mk(use ? ip[1] : (float)a.m.n[3] / 2.0f);
    } else {
      if (lane >= 4 && lane < 8) v = mk(a.m.init_p[lane - 4]);
    }
    par = v;
  }
  dd opar = par, par_eval = par, cl, fd;
  float sg = 0.0f, osg = 0.0f;
  clamp_fade<MODE>(lane, cl, fd);
  dd ocl = cl;
  dd gl = mk(0.0f);
  dd hr[NV];
  dd lambda = mk(1.0f), olambda = mk(1.0f), sum_update = mk(1e10f);
  dd err = mk(1e12f), oerr = mk(1e13f);
  int turn = 1;
  int kk = 0;
  bool need_eval = true, first = true, fisher = false;
  if (a.handoff) {
    // Continue from the LM state of the FP64 reference-order kernel after its
    // first steps (see Handoff): the steps whose decisions rest on rounding
    // noise (fit type 7's initial Hessian is singular: its initial pass copies
    // dudt[4] into dudt[5]) were taken in the reference's own arithmetic.
    const double* r = a.handoff + roi * (int64_t)kHandoffStride;
    const int l = lane < NV ? lane : 0;
    par = from_double(r[Handoff::nt + l]);
    opar = from_double(r[Handoff::ot + l]);
    par_eval = from_double(r[Handoff::te + l]);
    sg = (float)r[Handoff::ns + l];
    osg = (float)r[Handoff::os + l];
    cl = from_double(r[Handoff::nc + l]);
    ocl = from_double(r[Handoff::oc + l]);
    lambda = from_double(r[Handoff::new_lambda]);
    olambda = from_double(r[Handoff::old_lambda]);
    err = from_double(r[Handoff::new_err]);
    oerr = from_double(r[Handoff::old_err]);
    sum_update = from_double(r[Handoff::sum_update]);
    turn = (int)r[Handoff::turn];
    kk = (int)r[Handoff::kk];
    const int state = (int)r[Handoff::state];
    first = false;
    if (state == Handoff::kCurrent) {
      need_eval = false;
      gl = from_double(r[Handoff::jac + l]);
#pragma unroll
      for (int k = 0; k < NV; ++k) hr[k] = from_double(r[Handoff::hes + l * NV + k]);
    } else if (state == Handoff::kConverged) {
      fisher = true;
    }
  }
  dd ll = mk(0.0f);
  bool evaluated = false;  // the workspace holds maps of this ROI's last evaluation
  for (;;) {
    if (need_eval) {
      // The CRLB pass at the position of this kernel's last evaluation reuses
      // its stage-A/B maps (they depend on the spatial parameters only). Not
      // for fit type 8, whose kernel the extra state pushes into more spills
      // (measured 3% slower).
      bool maps_ready = false;
      if (MODE != 8 && fisher && evaluated) {
        const bool spatial = lane < NV && lane != 2 && lane != 3;
        const bool same = !spatial || (__float_as_uint(par.hi) == __float_as_uint(par_eval.hi) &&
                                       __float_as_uint(par.lo) == __float_as_uint(par_eval.lo));
        maps_ready = __all_sync(kFull, same);
      }
      if (!fisher) par_eval = par;
      dd the[NV];
      // (a hand-off may enter here with fisher set: par_eval is then the
      // parameters of the FP64 kernel's last evaluation)
#pragma unroll
      for (int k = 0; k < NV; ++k)
        the[k] = shfl((MODE == 8 && fisher && k != 2 && k != 3) ? par_eval : par, k);
      dd e;
      evaluate<MODE>(a, L, ws, lane, the, first && MODE == 7, fisher, e, gl, hr, maps_ready);
      first = false;
      need_eval = false;
      evaluated = true;
      if (fisher) {
        ll = e;
        break;
      }
      err = e;
    }
    if (kk >= a.iterations) {
      fisher = true;
      need_eval = true;
      continue;
    }
    // |(newErr - oldErr) / newErr| < TOLERANCE (1e-6f), CPUmleFit_LM.cpp:2565
    {
      const dd rel = dabs(div(sub(err, oerr), err));
      const bool conv = rel.hi < 1e-6f || (rel.hi == 1e-6f && rel.lo < 0.0f);
      const bool conv5 = MODE == 8 && (sum_update.hi < 1e-5f || (sum_update.hi == 1e-5f && sum_update.lo < 0.0f));
      if (conv || conv5) {  // :3355
        fisher = true;
        need_eval = true;
        continue;
      }
    }
    if (gt0(sub(err, mul(oerr, 1.5f)))) {
      sg = osg;
      cl = ocl;
      par = opar;
      lambda = olambda;
      err = oerr;
      lambda = mul(lambda, 10.0f);
    } else if (lt(err, oerr)) {
      if (gt(lambda, mk(1.0f)))
        lambda = mul(lambda, c_0p8());
      else if (lt(lambda, mk(1.0f)))
        lambda = mk(1.0f);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (lane == k) hr[k] = mul(hr[k], lambda);
    // A parameter with an exactly zero Hessian row is held for this step (as
    // in the FP32 kernels).
    bool frz = false;
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (lane == k) frz = is_zero(hr[k]);
    const unsigned fmask = __ballot_sync(kFull, frz && lane < NV);
    dd am[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      am[k] = ((fmask >> k) & 1u) ? mk(0.0f) : hr[k];
      if (frz) am[k] = mk((k == lane) ? 1.0f : 0.0f);
    }
    const dd rhs = frz ? mk(0.0f) : gl;
    // right-looking Cholesky (CPUsplineLib.cpp:1363-1390 computes the same
    // factor; it fails on a negative pivot only)
    dd lr[NV], lc[NV], invd = mk(1.0f);
    bool ok = true;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      lr[j] = mk(0.0f);
      lc[j] = mk(0.0f);
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const dd ajj = shfl(am[j], j);
      if (lt0(ajj) || is_nan(ajj)) {
        ok = false;
        break;
      }
      const dd ljj = dsqrt(ajj);
      const dd inv = recip(ljj);
      const dd lij = (lane > j) ? mul(am[j], inv) : ((lane == j) ? ljj : mk(0.0f));
      lr[j] = lij;
      if (lane == j) invd = inv;
#pragma unroll
      for (int k = j + 1; k < NV; ++k) {
        const dd lkj = shfl(lij, k);
        if (lane == j) lc[k] = lkj;
        if (lane > j && k <= lane) am[k] = sub(am[k], mul(lij, lkj));
      }
    }
    dd upd = mk(0.0f);
    if (ok) {
      upd = lane_solve<NV>(lane, lr, lc, invd, rhs);
      if (MODE != 6) {
        // CPUmleFit_LM.cpp:2943-2950: a NaN step counts as a failed solve
        if (__any_sync(kFull, lane < NV && is_nan(upd))) ok = false;
      }
    }
    if (ok) {
      if (MODE == 7 && lane == 5) upd = mul(upd, 10.0f);  // :2951
      osg = sg;
      ocl = cl;
      opar = par;
      olambda = lambda;
      oerr = err;
      if (MODE == 7) {
        // "let it go" (:2966-2971)
        const dd dz = shfl(upd, 4);
        if (lt(dabs(dz), c_0p005()) && turn) {
          if (lane == 5) cl = ocl = div(mk((float)a.m.n[3]), mk(10.0f));
          if (lane == 4) cl = ocl = mk(2.0f);
          turn = 0;
        }
      }
      if (sg != 0.0f) {
        if ((sg == 1.0f && lt0(upd)) || (sg == -1.0f && gt0(upd))) cl = mul(cl, fd);
      }
      sg = gt0(upd) ? 1.0f : -1.0f;
      const dd step = div(upd, add(dabs(div(upd, cl)), 1.0f));
      par = sub(par, step);
      if (MODE == 8) sum_update = warp_sum_dd(lane < NV ? dabs(step) : mk(0.0f));
      // bounds (CPUmleFit_LM.cpp:2626-2634, :3003-3010, :3421-3447)
      if (MODE == 8 && lane < 2) {
        const float lo = (float)(s - 1) / 2.0f - (float)s / 4.0f;
        const float hi = (float)(s - 1) / 2.0f + (float)s / 4.0f;
        par = dmax(par, mk(lo));
        par = dmin(par, mk(hi));
      }
      if (lane == 2) par = dmax(par, mk(1.0f));
      if (lane == 3) par = dmax(par, c_0p01());
      if (lane == 4) {
        par = dmax(par, mk(0.0f));
        const float zmax = (MODE == 6) ? (float)(a.m.n[2] - 4) : (float)a.m.n[2] - 0.5f;
        par = dmin(par, mk(zmax));
      }
      if (MODE == 7 && lane == 5) {
        par = dmax(par, mk(0.0f));
        par = dmin(par, mk((float)a.m.n[3] - 0.5f));
      }
      if (MODE == 8) {
        if (lane == 5) {
          const int nw = a.m.n[3];
          if (!gt(par, mk(1.0f)))
            par = add(par, (float)(nw - 2));
          else if (gt(par, mk((float)(nw - 1))))
            par = add(par, (float)(2 - nw));
        }
        if (lane == 6) {
          par = dmax(par, mk(1.0f));
          par = dmin(par, mk((float)a.m.n[4] - 0.5f));
        }
        if (lane == 7) {
          par = dmin(par, mk(1.0f));
          par = dmax(par, mk(0.0f));
        }
      }
      need_eval = true;
    } else {
      lambda = mul(lambda, 10.0f);
    }
    ++kk;
  }

  // CRLB = diag(M^-1) (the reference: unpivoted LU in its precision,
  // VC/CPUmleFit_LM/MatInvLib.h:17-77), here in FP64 once per fit on the
  // Jacobi-scaled matrix S = D^-1 M D^-1: lane-parallel Cholesky S = L L^T,
  // diag(S^-1)_c = sum_k ((L^-1)_kc)^2, (M^-1)_cc = (S^-1)_cc / M_cc. A
  // parameter with an exactly zero Fisher row gets +inf.
  float crlb = 0.0f;
  {
    double mrow[NV], dk[NV];
    double mydiag = 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      mrow[k] = to_d(hr[k]);
      if (lane == k) mydiag = mrow[k];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) dk[k] = __shfl_sync(kFull, mydiag, k);
    const double sd = sqrt(mydiag);
    double mr[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double den = sd * sqrt(dk[k]);
      mr[k] = (lane == k) ? 1.0 : ((den > 0.0) ? mrow[k] / den : 0.0);
    }
    double lr[NV], invd = 1.0;
    bool okc = true;
#pragma unroll
    for (int j = 0; j < NV; ++j) lr[j] = 0.0;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const double ajj = __shfl_sync(kFull, mr[j], j);
      if (!(ajj > 0.0)) okc = false;
      const double ljj = sqrt(ajj);
      const double inv = 1.0 / ljj;
      const double lij = (lane > j) ? mr[j] * inv : ((lane == j) ? ljj : 0.0);
      lr[j] = lij;
      if (lane == j) invd = inv;
#pragma unroll
      for (int k = j + 1; k < NV; ++k) {
        const double lkj = __shfl_sync(kFull, lij, k);
        if (lane > j && k <= lane) mr[k] = fma(-lij, lkj, mr[k]);
      }
    }
    double acc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      double part = 0.0, z = 0.0;
#pragma unroll
      for (int k = c; k < NV; ++k) {
        const double zk = __shfl_sync(kFull, ((k == c ? 1.0 : 0.0) - part) * invd, k);
        if (lane == k) z = zk;
        else if (lane > k) part = fma(lr[k], zk, part);
      }
      acc[c] = (lane >= c && lane < NV) ? z * z : 0.0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int c = 0; c < NV; ++c) acc[c] += __shfl_xor_sync(kFull, acc[c], o);
#pragma unroll
    for (int c = 0; c < NV; ++c)
      if (lane == c) crlb = okc ? (float)(acc[c] / dk[c]) : __int_as_float(0x7fc00000);
#pragma unroll
    for (int c = 0; c < NV; ++c)
      if (lane == c && dk[c] == 0.0) crlb = __int_as_float(0x7f800000);
  }
  return Result{to_f(par), crlb, to_f(ll), kk};
}

// Minimum resident 4-warp blocks per SM: 3D fits in 128 registers (16 warps per
// SM, 4 bytes of spill); 4D and 5D keep their register need (167 and 255; a
// 128-register cap spills 0.5 and 1.5 KB per thread).
template <int MODE>
__global__ void __launch_bounds__(128, MODE == 6 ? 4 : 1) fitdd_kernel(FitArgs a) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  constexpr int NV = Traits<MODE>::NV;
  const Layout L = make_layout(MODE, a.s);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float* ws = smem + wib * L.total();
  const int64_t total_warps = (int64_t)gridDim.x * wpb;
  int64_t roi = (int64_t)blockIdx.x * wpb + wib;
  for (;;) {
    if (a.claim) {
      unsigned long long i = 0;
      if (lane == 0) i = atomicAdd(a.claim, 1ull);
      roi = (int64_t)__shfl_sync(kFull, i, 0);
    }
    if (roi >= a.nfits) break;
    const int s2 = a.s * a.s;
    const float* src = a.rois + roi * (int64_t)s2;
    for (int p = lane; p < s2; p += 32) ws[p] = __ldg(src + p);
    __syncwarp();
    const Result r = fit_roi<MODE>(a, L, ws, lane, roi);
    float thv[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) thv[k] = __shfl_sync(kFull, r.par, k);
    const int64_t n = a.out_n, o = a.out_offset + roi;
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < NV; ++i) a.P[i * n + o] = thv[i];
      a.P[NV * n + o] = (float)r.kk;
      a.LL[o] = r.ll;
    }
    if (lane < NV) a.CRLB[lane * n + o] = r.crlb;
    __syncwarp();
    if (!a.claim) roi += total_warps;
  }
}

// One double-float evaluation per ROI at caller-given (float) parameters:
// per ROI 1 + NV + NV(NV+1)/2 doubles: the deviance (or log-likelihood), the
// gradient (zeros with fisher), the packed upper-triangle Hessian (or Fisher
// matrix), row-major.
template <int MODE>
__global__ void __launch_bounds__(128) evaldd_kernel(FitArgs a, const float* theta, double* out,
                                                     int fisher) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  constexpr int NV = Traits<MODE>::NV;
  constexpr int NH = NV * (NV + 1) / 2;
  const Layout L = make_layout(MODE, a.s);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float* ws = smem + wib * L.total();
  const int64_t total_warps = (int64_t)gridDim.x * wpb;
  for (int64_t roi = (int64_t)blockIdx.x * wpb + wib; roi < a.nfits; roi += total_warps) {
    const int s2 = a.s * a.s;
    const float* src = a.rois + roi * (int64_t)s2;
    for (int p = lane; p < s2; p += 32) ws[p] = __ldg(src + p);
    __syncwarp();
    dd th[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) th[k] = mk(theta[k * a.nfits + roi]);
    dd e, gl, hr[NV];
    evaluate<MODE>(a, L, ws, lane, th, false, fisher != 0, e, gl, hr);
    double* o = out + roi * (1 + NV + NH);
    if (lane == 0) o[0] = to_d(e);
    if (lane < NV) {
      o[1 + lane] = fisher ? 0.0 : to_d(gl);
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (k >= lane) o[1 + NV + lane * NV - (lane * (lane - 1)) / 2 + (k - lane)] = to_d(hr[k]);
    }
    __syncwarp();
  }
}

}  // namespace ddf

int fitdd_smem_floats(int mode, int s) { return ddf::make_layout(mode, s).total(); }

cudaError_t launch_evaldd(const FitArgs& a, const float* theta, double* out, int fisher,
                          cudaStream_t stream) {
  if (a.nfits <= 0) return cudaSuccess;
  const int mode = a.m.fittype;
  void (*kern)(FitArgs, const float*, double*, int) = nullptr;
  if (mode == 6) kern = ddf::evaldd_kernel<6>;
  else if (mode == 7) kern = ddf::evaldd_kernel<7>;
  else if (mode == 8) kern = ddf::evaldd_kernel<8>;
  else return cudaErrorInvalidValue;
  const int per_warp = fitdd_smem_floats(mode, a.s) * 4;
  int wpb = 4, bps = 0, sms = 0;
  cudaError_t e = pick_launch((const void*)kern, per_warp, &wpb, &bps, &sms);
  if (e != cudaSuccess) return e;
  int64_t grid = (a.nfits + wpb - 1) / wpb;
  const int64_t cap = (int64_t)sms * bps;
  if (grid > cap) grid = cap;
  kern<<<(unsigned)grid, 32 * wpb, per_warp * wpb, stream>>>(a, theta, out, fisher);
  return cudaGetLastError();
}

cudaError_t launch_fitdd(const FitArgs& a, cudaStream_t stream) {
  if (a.nfits <= 0) return cudaSuccess;
  const int mode = a.m.fittype;
  void (*kern)(FitArgs) = nullptr;
  if (mode == 6) kern = ddf::fitdd_kernel<6>;
  else if (mode == 7) kern = ddf::fitdd_kernel<7>;
  else if (mode == 8) kern = ddf::fitdd_kernel<8>;
  else return cudaErrorInvalidValue;
  const int per_warp = fitdd_smem_floats(mode, a.s) * 4;
  int wpb = 4, bps = 0, sms = 0;
  cudaError_t e = pick_launch((const void*)kern, per_warp, &wpb, &bps, &sms);
  if (e != cudaSuccess) return e;
  const int smem = per_warp * wpb;
  int64_t need = (a.nfits + wpb - 1) / wpb;
  int64_t grid = (int64_t)sms * bps;
  if (need < grid) grid = need;
  // ROIs claimed one at a time from a pooled work counter when they outnumber
  // the resident warps (as launch_fit does); without it, a fixed share per warp.
  FitArgs b = a;
  b.claim = nullptr;
  unsigned long long* claim = nullptr;
  if (need > grid) {
    cudaError_t ea = cudaMallocAsync(reinterpret_cast<void**>(&claim), sizeof(*claim), stream);
    if (ea == cudaSuccess) {
      ea = cudaMemsetAsync(claim, 0, sizeof(*claim), stream);
      if (ea == cudaSuccess) {
        b.claim = claim;
      } else {
        cudaFreeAsync(claim, stream);
        claim = nullptr;
      }
    } else {
      claim = nullptr;
    }
    if (ea != cudaSuccess) (void)cudaGetLastError();
  }
  kern<<<(unsigned)grid, 32 * wpb, smem, stream>>>(b);
  e = cudaGetLastError();
  if (claim) cudaFreeAsync(claim, stream);
  return e;
}

}  // namespace bsfit
