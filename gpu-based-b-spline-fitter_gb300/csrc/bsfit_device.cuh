// Device-side building blocks of the B-spline fitter: the cardinal B-spline
// basis, knot selection, warp reductions and error-free FP32 transformations.
// Paths in comments are relative to the reference project root; VC stands for
// "MultiD_bspline/visual code".
#pragma once

#include <climits>
#include <cstdint>
#include <type_traits>
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

// Branch-free forms of the two bases. With a = |x| the reference's half-open
// pieces are B3 = 2/3 - a^2 + a^3/2 (a < 1), (2 - a)^3 / 6 (1 <= a < 2), 0, and
// B2 = 3/4 - a^2 (a < 1/2), (3/2 - a)^2 / 2 (1/2 <= a < 3/2), 0; they agree
// with the reference's intervals at every boundary (both sides give the same
// value there).
__device__ __forceinline__ float bspline3_sym(float x) {
  const float a = fabsf(x);
  const float a2 = a * a;
  const float inner = fmaf(0.5f * a, a2, 2.0f / 3.0f - a2);
  const float b = 2.0f - a;
  const float outer = b * b * b * (1.0f / 6.0f);
  return (a < 1.0f) ? inner : ((a < 2.0f) ? outer : 0.0f);
}

__device__ __forceinline__ float bspline2_sym(float x) {
  const float a = fabsf(x);
  const float inner = 0.75f - a * a;
  const float b = 1.5f - a;
  const float outer = 0.5f * b * b;
  return (a < 0.5f) ? inner : ((a < 1.5f) ? outer : 0.0f);
}

// One of the seven 1-D weights of an axis at fractional position t, indexed
// j = 0..6:
//   j = 0..3: value weight B3(t - o) of the node at offset o = j - 1 from the
//             floor knot,
//   j = 4..6: derivative weight B2(t - o - 1/2) of the node difference
//             C[o + 1] - C[o] at offset o = j - 5.
// These are the reference's loop forms (CPUsplineLib.cpp:1138-1158: side 1
// B3(t + v - 1), B2(t - 1 + v - 1/2) at offsets 1 - v; side 2 B3(t - v),
// B2(t - 1 - v + 1/2) at offsets v) with the argument formed in one rounding.
// The derivative weight of offset +2 is identically zero.
__device__ __forceinline__ float axis_weight(float t, int j) {
  const float off = (j < 4) ? (float)(j - 1) : (float)(j - 5) + 0.5f;
  const float x = t - off;
  return (j < 4) ? bspline3_sym(x) : bspline2_sym(x);
}

// ---------------------------------------------------------------------------
// Four-node contractions in a fixed operation order: the value
// ((c0 b0 + c1 b1) + c2 b2) + c3 b3 and the difference form
// ((c1 - c0) d0 + (c2 - c1) d1) + (c3 - c2) d2, each a multiply and a chain of
// FMAs. The packed forms below evaluate two independent contractions with the
// same operations per half, so scalar and packed code give identical results.

__device__ __forceinline__ float contract4(float c0, float c1, float c2, float c3, float b0,
                                           float b1, float b2, float b3) {
  return fmaf(c3, b3, fmaf(c2, b2, fmaf(c1, b1, c0 * b0)));
}

__device__ __forceinline__ float dcontract4(float c0, float c1, float c2, float c3, float d0,
                                            float d1, float d2) {
  return fmaf(c3 - c2, d2, fmaf(c2 - c1, d1, (c1 - c0) * d0));
}

// Packed two-lane FP32 (the paired FMA of sm_100 and later): each half is the
// correctly rounded scalar operation.
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);  // a - b, one rounding
}
__device__ __forceinline__ float2 contract4x2(float2 c0, float2 c1, float2 c2, float2 c3,
                                              float2 b0, float2 b1, float2 b2, float2 b3) {
  return __ffma2_rn(c3, b3, __ffma2_rn(c2, b2, __ffma2_rn(c1, b1, __fmul2_rn(c0, b0))));
}
__device__ __forceinline__ float2 dcontract4x2(float2 c0, float2 c1, float2 c2, float2 c3,
                                               float2 d0, float2 d1, float2 d2) {
  return __ffma2_rn(sub2(c3, c2), d2,
                    __ffma2_rn(sub2(c2, c1), d1, __fmul2_rn(sub2(c1, c0), d0)));
}

// ---------------------------------------------------------------------------
// Warp reductions (butterfly: every lane ends with the total).

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ int warp_min(int v) { return __reduce_min_sync(kFull, v); }

__device__ __forceinline__ int warp_max(int v) { return __reduce_max_sync(kFull, v); }

template <int K>
__device__ __forceinline__ void warp_sum_array(float (&v)[K]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += __shfl_xor_sync(kFull, v[k], o);
  }
}

// Reduce-scatter of C values (C <= 64) over the warp, five exchange levels
// o = 16, 8, 4, 2, 1 between lanes l and l ^ o. Of the c values a lane still
// holds, the first floor(c/2) pair with the next floor(c/2): the lane with bit
// o set keeps the second of each pair, its partner the first, and an odd last
// value is kept (and summed) by both. Every value's total is the sum tree of
// warp_sum (halves differing in bit 16 first, then 8, ...), and floating-point
// addition is commutative, so every lane holding a value has the same total as
// a 32-wide butterfly over the value would give; the exchanges number
// one per value a lane keeps at each level (c -> ceil(c/2)) instead of 31 per
// 32 values (3D: 20 values, 10 + 5 + 3 + 2 + 1 = 21 exchanges instead of 31).
// Slot 0 (and slot 1 when C > 32) ends with the value RsSources records.
template <int C, int O, int N>
__device__ __forceinline__ void reduce_scatter(float (&v)[N], int lane) {
  static_assert(C <= N && C <= 64, "reduce_scatter: too many values");
  if constexpr (O > 0) {
    constexpr int P = C / 2;
    const bool up = (lane & O) != 0;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const float send = up ? v[i] : v[i + P];
      const float keep = up ? v[i + P] : v[i];
      v[i] = keep + __shfl_xor_sync(kFull, send, O);
    }
    if constexpr ((C & 1) != 0) v[P] = v[2 * P] + __shfl_xor_sync(kFull, v[2 * P], O);
    reduce_scatter<P + (C & 1), O / 2>(v, lane);
  }
}

// Slots a lane holds after reduce_scatter<C, 16> (1 for C <= 32, else 2).
__host__ __device__ constexpr int rs_slots(int c) {
  for (int o = 16; o > 0; o >>= 1) c = c / 2 + (c & 1);
  return c;
}

// Where each value ends after reduce_scatter<C, 16>: src[x] = 2 * lane + slot
// of the lowest lane holding value x (the exchange rule above, replayed).
template <int C>
struct RsSources {
  int src[C];
  __host__ __device__ constexpr RsSources() : src() {
    for (int x = 0; x < C; ++x) src[x] = -1;
    for (int lane = 0; lane < 32; ++lane) {
      int map[64] = {};
      for (int i = 0; i < C; ++i) map[i] = i;
      int c = C;
      for (int o = 16; o > 0; o >>= 1) {
        const int P = c / 2;
        const int sh = (lane & o) ? P : 0;
        for (int i = 0; i < P; ++i) map[i] = map[i + sh];
        if (c & 1) map[P] = map[2 * P];
        c = P + (c & 1);
      }
      for (int slot = 0; slot < c; ++slot)
        if (src[map[slot]] < 0) src[map[slot]] = 2 * lane + slot;
    }
  }
};

// Where lane l < NV finds gradient entry l (grad) and Hessian entry (l, k)
// (row[k]) after reduce_scatter of the K = NV + NV(NV+1)/2 sums: B bits per
// lane, the source lane (one slot per lane), or 2 * lane + slot (two slots).
template <int NV, int K>
struct GatherCodes {
  static constexpr int SLOTS = rs_slots(K);
  static constexpr int B = SLOTS > 1 ? 6 : 5;
  using Code = typename std::conditional<NV * B <= 32, unsigned, unsigned long long>::type;
  Code grad;
  Code row[NV];
  __host__ __device__ constexpr GatherCodes() : grad(0), row() {
    const RsSources<K> rs{};
    const int div = SLOTS > 1 ? 1 : 2;  // one slot: the lane alone
    for (int l = 0; l < NV; ++l) grad |= (Code)(rs.src[l] / div) << (B * l);
    for (int k = 0; k < NV; ++k)
      for (int l = 0; l < NV; ++l) {
        const int lo = l < k ? l : k, hi = l < k ? k : l;
        const int x = NV + lo * NV - (lo * (lo - 1)) / 2 + (hi - lo);
        row[k] |= (Code)(rs.src[x] / div) << (B * l);
      }
  }
};

// This lane's value (its field of codes, starting at bit sh) from the lane
// that holds it.
template <int SLOTS, typename Code>
__device__ __forceinline__ float rs_gather(float t0, float t1, Code codes, int sh) {
  if constexpr (SLOTS > 1) {
    const int code = (int)((codes >> sh) & 63u);
    const float a0 = __shfl_sync(kFull, t0, code >> 1);
    const float a1 = __shfl_sync(kFull, t1, code >> 1);
    return (code & 1) ? a1 : a0;
  } else {
    return __shfl_sync(kFull, t0, (int)((codes >> sh) & 31u));
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
