// Device-side building blocks of the B-spline fitter: the cardinal B-spline
// basis, knot selection, warp reductions and error-free FP32 transformations.
// Paths in comments are relative to the reference project root; VC stands for
// "MultiD_bspline/visual code".
#pragma once

#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

namespace bsfit {

constexpr unsigned kFull = 0xffffffffu;

// int(floor(v)) with the x86 conversion rule of the reference build
// (cvttss2si): NaN and out-of-range values give INT_MIN. CUDA's float-to-int
// conversion saturates instead, so the rule is stated explicitly.
__device__ __forceinline__ int floor_to_int(float v) {
  float f = floorf(v);
  if (!(f >= -2147483648.0f && f < 2147483648.0f)) return INT_MIN;
  return __float2int_rz(f);
}

// Knot index along one axis: floor(pos) clamped to [1, n - 1], or n when pos
// equals n exactly (VC/CPUmleFit_LM/CPUsplineLib.cpp:1204-1226).
__device__ __forceinline__ int knot_index(float pos, int n) {
  int c = floor_to_int(pos);
  c = c > 1 ? c : 1;
  c = c < n - 1 ? c : n - 1;
  if (pos == (float)n) c = n;
  return c;
}

// Centred cubic B-spline with the reference's half-open intervals
// (CPUsplineLib.cpp:1311-1324).
__device__ __forceinline__ float bspline3(float x) {
  float x2 = x * x;
  float x3 = x2 * x;
  if (x >= 1.0f && x < 2.0f) return 4.0f / 3.0f - 2.0f * x + x2 - 1.0f / 6.0f * x3;
  if (x >= 0.0f && x < 1.0f) return 2.0f / 3.0f - x2 + 0.5f * x3;
  if (x >= -1.0f && x < 0.0f) return 2.0f / 3.0f - x2 - 0.5f * x3;
  if (x >= -2.0f && x < -1.0f) return 4.0f / 3.0f + 2.0f * x + x2 + 1.0f / 6.0f * x3;
  return 0.0f;
}

// Centred quadratic B-spline, the derivative basis (CPUsplineLib.cpp:1296-1309).
__device__ __forceinline__ float bspline2(float x) {
  float x2 = x * x;
  if (x >= 0.5f && x < 1.5f) return 1.125f - 1.5f * x + 0.5f * x2;
  if (x >= -0.5f && x < 0.5f) return 0.75f - x2;
  if (x >= -1.5f && x < -0.5f) return 1.125f + 1.5f * x + 0.5f * x2;
  return 0.0f;
}

// One of the seven 1-D weights of an axis, indexed j = 0..6:
//   j = 0..3: value weight of the node at offset j - 1 from the floor knot,
//   j = 4..6: derivative weight of the node difference C[o + 1] - C[o] at
//             offset o = j - 5.
// The argument expressions follow the reference's loop form
// (CPUsplineLib.cpp:1138-1158): side 1 uses B3(t + v - 1), B2(t - 1 + v - 1/2)
// for the nodes at offsets 1 - v; side 2 uses B3(t - v), B2(t - 1 - v + 1/2)
// for offsets v. The derivative weight of offset +2 is identically zero.
__device__ __forceinline__ float axis_weight(float t, int j) {
  float dt = t - 1.0f;
  switch (j) {
    case 0: return bspline3((t + 2.0f) - 1.0f);         // offset -1 (side 1, v = 2)
    case 1: return bspline3((t + 1.0f) - 1.0f);         // offset  0 (side 1, v = 1)
    case 2: return bspline3(t - 1.0f);                  // offset +1 (side 2, v = 1)
    case 3: return bspline3(t - 2.0f);                  // offset +2 (side 2, v = 2)
    case 4: return bspline2((dt + 2.0f) - 0.5f);        // offset -1
    case 5: return bspline2((dt + 1.0f) - 0.5f);        // offset  0
    default: return bspline2((dt - 1.0f) + 0.5f);       // offset +1
  }
}

// ---------------------------------------------------------------------------
// Warp reductions (butterfly: every lane ends with the total).

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ int warp_min(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

template <int K>
__device__ __forceinline__ void warp_sum_array(float (&v)[K]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += __shfl_xor_sync(kFull, v[k], o);
  }
}

// Error-free transformations (Knuth two-sum, FMA two-product).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

// Compensated accumulator: value = hi + lo.
struct FPair {
  float hi, lo;
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo += e;
  }
};

__device__ __forceinline__ FPair warp_sum_pair(FPair v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float h = __shfl_xor_sync(kFull, v.hi, o);
    float l = __shfl_xor_sync(kFull, v.lo, o);
    float s, e;
    two_sum(v.hi, h, s, e);
    v.hi = s;
    v.lo = v.lo + l + e;
  }
  // renormalise
  float s, e;
  two_sum(v.hi, v.lo, s, e);
  v.hi = s;
  v.lo = e;
  return v;
}

}  // namespace bsfit
