// Two 3D ROIs per warp in the two halves of paired FP32 operations: the
// "packed" form of the fit type 6 kernels.
//
// Every lane works for both ROIs of its warp: the evaluation runs the one-ROI
// form's node, item and pixel loops once, with each value a pair (ROI of slot
// 0, ROI of slot 1) and each multiply-add one paired FP32 instruction
// (f32x2), so the evaluation's arithmetic, its shared-memory traffic (the maps
// of both ROIs interleaved) and its loop and address work are shared by the
// two ROIs. The LM state, the claiming of ROIs, the initial guess and the CRLB
// are those of the half-warp pair form (bsfit_pair.cuh: slot h's state on the
// 16 lanes of half h).
//
// Results are bit-identical to the one-ROI form: lane l sums the pixels
// l, l + 32, ... of both ROIs as lane l of the one-ROI form does; each half of
// a paired operation is the one-ROI form's scalar operation (the four-node
// contractions in the order the compiler gives the one-ROI form's expression,
// csum4x2 / dsum4x2); the reduce-scatter, the gathers and the compensated
// deviance sum follow the one-ROI form's trees; where the two ROIs' windows
// put a row or a column at different offsets, each ROI's maps are read at its
// own offset.
#pragma once

#include "bsfit_pair.cuh"

namespace bsfit {

namespace pk {

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// c0 b0 + c1 b1 + c2 b2 + c3 b3 as the compiler contracts the one-ROI form's
// expression: fma(c3, b3, fma(c2, b2, fma(c0, b0, c1 b1))).
__device__ __forceinline__ float2 csum4x2(float2 c0, float2 c1, float2 c2, float2 c3, float2 b0,
                                          float2 b1, float2 b2, float2 b3) {
  return fma2(c3, b3, fma2(c2, b2, fma2(c0, b0, mul2(c1, b1))));
}
// (c1 - c0) d0 + (c2 - c1) d1 + (c3 - c2) d2 likewise:
// fma(c3 - c2, d2, fma(c1 - c0, d0, (c2 - c1) d1)).
__device__ __forceinline__ float2 dsum4x2(float2 c0, float2 c1, float2 c2, float2 c3, float2 d0,
                                          float2 d1, float2 d2) {
  return fma2(sub2(c3, c2), d2, fma2(sub2(c1, c0), d0, mul2(sub2(c2, c1), d1)));
}

// Compensated pair of paired sums (FPair per half).
struct FPair2 {
  float2 hi, lo;
  __device__ __forceinline__ void add(float2 x) {
    const float2 s = add2(hi, x);
    const float2 bb = sub2(s, hi);
    const float2 e = add2(sub2(hi, sub2(s, bb)), sub2(x, bb));
    hi = s;
    lo = add2(lo, e);
  }
};

__device__ __forceinline__ float2 shfl_xor2(float2 v, int o) {
  return f2(__shfl_xor_sync(kFull, v.x, o), __shfl_xor_sync(kFull, v.y, o));
}

// warp_sum_pair of each half.
__device__ __forceinline__ FPair2 warp_sum_pair2(FPair2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float2 h = shfl_xor2(v.hi, o);
    const float2 l = shfl_xor2(v.lo, o);
    const float2 s = add2(v.hi, h);
    const float2 bb = sub2(s, v.hi);
    const float2 e = add2(sub2(v.hi, sub2(s, bb)), sub2(h, bb));
    v.hi = s;
    v.lo = add2(add2(v.lo, l), e);
  }
  const float2 s = add2(v.hi, v.lo);
  const float2 bb = sub2(s, v.hi);
  const float2 e = add2(sub2(v.hi, sub2(s, bb)), sub2(v.lo, bb));
  v.hi = s;
  v.lo = e;
  return v;
}

// reduce_scatter of each half (the same exchanges, two shuffles each).
template <int C, int O, int N>
__device__ __forceinline__ void reduce_scatter2(float2 (&v)[N], int lane) {
  static_assert(C <= N && C <= 64, "reduce_scatter2: too many values");
  if constexpr (O > 0) {
    constexpr int P = C / 2;
    const bool up = (lane & O) != 0;
#pragma unroll
    for (int i = 0; i < P; ++i) {
      const float2 send = up ? v[i] : v[i + P];
      const float2 keep = up ? v[i + P] : v[i];
      v[i] = add2(keep, shfl_xor2(send, O));
    }
    if constexpr ((C & 1) != 0) v[P] = add2(v[2 * P], shfl_xor2(v[2 * P], O));
    reduce_scatter2<P + (C & 1), O / 2>(v, lane);
  }
}

}  // namespace pk

// Per-warp shared-memory layout of the packed form (floats): the two slots'
// pixels, their per-row and per-column window offsets, their 1-D weights
// interleaved by slot, and the maps. Stage-A maps: one pair per (lateral node,
// map) (value, d/dz), stored by X column, AS2 pairs per column with AS2 = s
// (mod 16) so a pass's lanes stay on distinct banks across columns. Stage-B
// items per (X node, pixel row): a 16-byte (value, d/dY) pair of pairs and an
// 8-byte d/dz pair, a column being s of the first then s of the second (GS
// floats, a multiple of 4). As in the one-ROI form's 3D layout, G column c is
// written over A columns already consumed: with A at a_rel,
// (c + 1) GS <= a_rel + c AS for every column.
struct PackLayout {
  int s, s2p, wp;
  __host__ __device__ constexpr int s4() const { return (s + 3) & ~3; }
  __host__ __device__ constexpr int as2() const {
    return 2 * wp + ((s - 2 * wp) % 16 + 16) % 16;
  }
  __host__ __device__ constexpr int as() const { return 2 * as2(); }
  __host__ __device__ constexpr int gs() const { return (6 * s + 3) & ~3; }
  __host__ __device__ constexpr int off_k() const { return 2 * s2p; }
  __host__ __device__ constexpr int off_w() const { return off_k() + 4 * s4(); }
  __host__ __device__ constexpr int off_maps() const { return off_w() + 48; }
  __host__ __device__ constexpr int a_rel() const {
    return (gs() + (wp - 1) * (gs() > as() ? gs() - as() : 0) + 3) & ~3;
  }
  __host__ __device__ constexpr int maps_size() const {
    return (a_rel() + wp * as() > wp * gs()) ? a_rel() + wp * as() : wp * gs();
  }
  __host__ __device__ constexpr int total() const { return (off_maps() + maps_size() + 3) & ~3; }
};

__host__ __device__ constexpr PackLayout make_pack_layout(int s) {
  PackLayout L{};
  L.s = s;
  L.s2p = (s * s + 3) & ~3;
  L.wp = s + 4;
  return L;
}

// Regions disjoint, 16-byte alignment of the vector accesses, and the
// aliasing rule, for every ROI size.
constexpr bool pack_layouts_ok() {
  for (int s = 1; s <= 51; ++s) {
    const PackLayout L = make_pack_layout(s);
    if (2 * s * s > L.off_k() || L.off_k() % 4 || L.off_w() % 4 || L.off_maps() % 4 ||
        L.a_rel() % 4 || L.gs() % 4 || L.as2() < 2 * L.wp || (L.as2() - s) % 16 ||
        L.gs() < 6 * s || L.off_maps() + L.maps_size() > L.total())
      return false;
    for (int c = 0; c < L.wp; ++c)
      if ((c + 1) * L.gs() > L.a_rel() + c * L.as()) return false;
  }
  return true;
}
static_assert(pack_layouts_ok(), "packed per-warp shared-memory layout");

// One evaluation of both slots' ROIs. par: this lane's half's parameter
// (lane l of half h holds parameter l of slot h's ROI), fisher: the half's
// mode. Outputs as evaluate() for one ROI, on each half for its own ROI.
__device__ __forceinline__ void evaluate_packed(const FitArgs& a, const PackLayout& L, float* ws,
                                                int lane, float par, bool fisher, FPair& err_out,
                                                float& gl, float (&hr)[5]) {
  using namespace pk;
  constexpr int NV = 5;
  constexpr int NH = NV * (NV + 1) / 2;
  constexpr int K = NV + NH;
  const int s = L.s, wp = L.wp, AS2 = L.as2(), GS = L.gs();
  const ModelDev& m = a.m;
  const int hl = lane & 15, hb = lane & 16;
  float tA[NV], tB[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    tA[k] = __shfl_sync(kFull, par, k);
    tB[k] = __shfl_sync(kFull, par, 16 + k);
  }
  const bool fA = __shfl_sync(kFull, (int)fisher, 0) != 0;
  const bool fB = __shfl_sync(kFull, (int)fisher, 16) != 0;
  int* kx0 = reinterpret_cast<int*>(ws + L.off_k());
  int* ky0 = kx0 + L.s4();
  int* kx1 = ky0 + L.s4();
  int* ky1 = kx1 + L.s4();
  float* W = ws + L.off_w();  // W[(axis * 8 + j) * 2 + slot]
  float* G = ws + L.off_maps();
  float2* A2 = reinterpret_cast<float2*>(ws + L.off_maps() + L.a_rel());
  __syncwarp();  // the previous evaluation's readers are done

  // Positions and knots of both slots (channel_pass).
  const float half = (float)((s + 1) / 2);
  const float off = (float)(m.n[1] - s) / 2.0f;
  const float xcA = half - tA[0], ycA = half - tA[1];
  const float xcB = half - tB[0], ycB = half - tB[1];
  for (int j = lane; j < s; j += 32) {
    kx0[j] = knot_index((xcA + (float)j) + off, m.n[1]);
    ky0[j] = knot_index((ycA + (float)j) + off, m.n[0]);
    kx1[j] = knot_index((xcB + (float)j) + off, m.n[1]);
    ky1[j] = knot_index((ycB + (float)j) + off, m.n[0]);
  }
  {
    const float frA[3] = {ycA - floorf(ycA), xcA - floorf(xcA), tA[4] - floorf(tA[4])};
    const float frB[3] = {ycB - floorf(ycB), xcB - floorf(xcB), tB[4] - floorf(tB[4])};
    for (int k = lane; k < 42; k += 32) {
      const int slot = k >= 21;
      const int kk = k - 21 * slot;
      const int ax = kk / 7, j = kk - 7 * ax;
      W[(ax * 8 + j) * 2 + slot] = axis_weight(slot ? frB[ax] : frA[ax], j);
    }
  }
  __syncwarp();
  int xbA, wxA, ybA, wyA, xbB, wxB, ybB, wyB;
  {
    int a0 = INT_MAX, a1 = INT_MIN, b0 = INT_MAX, b1 = INT_MIN;
    int c0 = INT_MAX, c1 = INT_MIN, d0 = INT_MAX, d1 = INT_MIN;
    for (int j = lane; j < s; j += 32) {
      a0 = min(a0, kx0[j]);
      a1 = max(a1, kx0[j]);
      b0 = min(b0, ky0[j]);
      b1 = max(b1, ky0[j]);
      c0 = min(c0, kx1[j]);
      c1 = max(c1, kx1[j]);
      d0 = min(d0, ky1[j]);
      d1 = max(d1, ky1[j]);
    }
    const int kxminA = __reduce_min_sync(kFull, a0), kxmaxA = __reduce_max_sync(kFull, a1);
    const int kyminA = __reduce_min_sync(kFull, b0), kymaxA = __reduce_max_sync(kFull, b1);
    const int kxminB = __reduce_min_sync(kFull, c0), kxmaxB = __reduce_max_sync(kFull, c1);
    const int kyminB = __reduce_min_sync(kFull, d0), kymaxB = __reduce_max_sync(kFull, d1);
    xbA = kxminA - 1;
    wxA = min(kxmaxA - kxminA + 4, wp);
    ybA = kyminA - 1;
    wyA = min(kymaxA - kyminA + 4, wp);
    xbB = kxminB - 1;
    wxB = min(kxmaxB - kxminB + 4, wp);
    ybB = kyminB - 1;
    wyB = min(kymaxB - kyminB + 4, wp);
  }
  for (int j = lane; j < s; j += 32) {
    kx0[j] = min(max(kx0[j] - 1 - xbA, 0), wxA - 4) * GS;
    ky0[j] = min(max(ky0[j] - 1 - ybA, 0), wyA - 4);
    kx1[j] = min(max(kx1[j] - 1 - xbB, 0), wxB - 4) * GS;
    ky1[j] = min(max(ky1[j] - 1 - ybB, 0), wyB - 4);
  }
  const int kzA = knot_index(tA[4], m.n[2]), kzB = knot_index(tB[4], m.n[2]);
  auto WP = [&](int ax, int j) { return f2(W[(ax * 8 + j) * 2], W[(ax * 8 + j) * 2 + 1]); };

  // (A) z contraction at every lateral node of the common window; a slot
  // whose window is smaller reads its last node again for the extra ones
  // (their maps are never read for it).
  const int wx = max(wxA, wxB), wy = max(wyA, wyB);
  {
    const float2 BZ0 = WP(2, 0), BZ1 = WP(2, 1), BZ2 = WP(2, 2), BZ3 = WP(2, 3);
    const float2 DZ0 = WP(2, 4), DZ1 = WP(2, 5), DZ2 = WP(2, 6);
    const int64_t sz_ = m.st[2];
    const int st1 = (int)m.st[1], sz32 = (int)sz_;
    const float* bA = m.coeff + (int64_t)(kzA - 1) * sz_;
    const float* bB = m.coeff + (int64_t)(kzB - 1) * sz_;
    const int nodes = wx * wy;
    Stride2D ix(lane, wy);
    for (int t = lane; t < nodes; t += 32, ix.next()) {
      const int xr = ix.r, yr = ix.c;
      const int la = (xbA + min(xr, wxA - 1)) * st1 + (ybA + min(yr, wyA - 1));
      const int lb = (xbB + min(xr, wxB - 1)) * st1 + (ybB + min(yr, wyB - 1));
      const float2 c0 = f2(__ldg(bA + la), __ldg(bB + lb));
      const float2 c1 = f2(__ldg(bA + sz32 + la), __ldg(bB + sz32 + lb));
      const float2 c2 = f2(__ldg(bA + 2 * sz32 + la), __ldg(bB + 2 * sz32 + lb));
      const float2 c3 = f2(__ldg(bA + 3 * sz32 + la), __ldg(bB + 3 * sz32 + lb));
      A2[xr * AS2 + yr] = csum4x2(c0, c1, c2, c3, BZ0, BZ1, BZ2, BZ3);
      A2[xr * AS2 + wp + yr] = dsum4x2(c0, c1, c2, c3, DZ0, DZ1, DZ2);
    }
  }
  __syncwarp();

  // (B) Y contraction for every (X node, pixel row); G is written over the A
  // columns already read (every pass reads, synchronises, then writes).
  {
    const float2 BY0 = WP(0, 0), BY1 = WP(0, 1), BY2 = WP(0, 2), BY3 = WP(0, 3);
    const float2 DY0 = WP(0, 4), DY1 = WP(0, 5), DY2 = WP(0, 6);
    const int items = wx * s;
    Stride2D ix(lane, s);
    for (int t0 = 0; t0 < items; t0 += 32, ix.next()) {
      const bool act = t0 + lane < items;
      const int xr = ix.r, py = ix.c;
      float2 g0, g1, g2;
      if (act) {
        const float2* col = A2 + xr * AS2;
        const int oa = ky0[py], ob = ky1[py];
        float2 v[4], z[4];
        if (oa == ob) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            v[i] = col[oa + i];
            z[i] = col[wp + oa + i];
          }
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            v[i] = f2(col[oa + i].x, col[ob + i].y);
            z[i] = f2(col[wp + oa + i].x, col[wp + ob + i].y);
          }
        }
        g0 = csum4x2(v[0], v[1], v[2], v[3], BY0, BY1, BY2, BY3);
        g1 = dsum4x2(v[0], v[1], v[2], v[3], DY0, DY1, DY2);
        g2 = csum4x2(z[0], z[1], z[2], z[3], BY0, BY1, BY2, BY3);
      }
      __syncwarp();
      if (act) {
        float* gc = G + xr * GS;
        *reinterpret_cast<float4*>(gc + 4 * py) = make_float4(g0.x, g0.y, g1.x, g1.y);
        *reinterpret_cast<float2*>(gc + 4 * s + 2 * py) = g2;
      }
    }
  }
  __syncwarp();

  // (C) X contraction per pixel fused with the likelihood sums of both slots.
  float2 acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = f2(0.0f, 0.0f);
  FPair2 er{f2(0.0f, 0.0f), f2(0.0f, 0.0f)};
  {
    const float2 BX0 = WP(1, 0), BX1 = WP(1, 1), BX2 = WP(1, 2), BX3 = WP(1, 3);
    const float2 DX0 = WP(1, 4), DX1 = WP(1, 5), DX2 = WP(1, 6);
    const float2 N2 = f2(tA[2], tB[2]), NN2 = f2(-tA[2], -tB[2]), BG2 = f2(tA[3], tB[3]);
    const float2 ONE = f2(1.0f, 1.0f), TWO = f2(2.0f, 2.0f);
    const float* dA = ws;
    const float* dB = ws + L.s2p;
    const int s2 = s * s;
    Stride2D ix(lane, s);
    for (int p = lane; p < s2; p += 32, ix.next()) {
      const int px = ix.r, py = ix.c;
      const int oa = kx0[px], ob = kx1[px];
      float4 q[4];
      float2 r[4];
      if (oa == ob) {
        const float* g = G + oa;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          q[k] = *reinterpret_cast<const float4*>(g + k * GS + 4 * py);
          r[k] = *reinterpret_cast<const float2*>(g + k * GS + 4 * s + 2 * py);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float4 qa = *reinterpret_cast<const float4*>(G + oa + k * GS + 4 * py);
          const float4 qb = *reinterpret_cast<const float4*>(G + ob + k * GS + 4 * py);
          const float2 ra = *reinterpret_cast<const float2*>(G + oa + k * GS + 4 * s + 2 * py);
          const float2 rb = *reinterpret_cast<const float2*>(G + ob + k * GS + 4 * s + 2 * py);
          q[k] = make_float4(qa.x, qb.y, qa.z, qb.w);
          r[k] = f2(ra.x, rb.y);
        }
      }
      const float2 v0 = f2(q[0].x, q[0].y), v1 = f2(q[1].x, q[1].y);
      const float2 v2 = f2(q[2].x, q[2].y), v3 = f2(q[3].x, q[3].y);
      const float2 f = csum4x2(v0, v1, v2, v3, BX0, BX1, BX2, BX3);
      const float2 dX = dsum4x2(v0, v1, v2, v3, DX0, DX1, DX2);
      const float2 dY = csum4x2(f2(q[0].z, q[0].w), f2(q[1].z, q[1].w), f2(q[2].z, q[2].w),
                                f2(q[3].z, q[3].w), BX0, BX1, BX2, BX3);
      const float2 dc = csum4x2(r[0], r[1], r[2], r[3], BX0, BX1, BX2, BX3);
      float2 du[NV];
      du[0] = mul2(NN2, dX);
      du[1] = mul2(NN2, dY);
      du[2] = f;
      du[3] = ONE;
      du[4] = mul2(N2, dc);
      const float2 model = fma2(N2, f, BG2);
      const float2 d = f2(dA[p], dB[p]);
      const float2 inv = f2(__frcp_rn(model.x), __frcp_rn(model.y));
      // Deviance, gradient and Hessian (CPUmleFit_LM.cpp:2540-2559), or in a
      // slot whose Fisher pass this is, Fisher information and log-likelihood
      // (:2730-2742), each half exactly the one-ROI form's operations for its
      // mode: one log per pixel (of d / m, or of m), the second (of d) only
      // when a slot is in its Fisher pass; a slot in its Fisher pass takes the
      // gradient weight 0 and the Hessian weight 1 / m.
      const float2 dm0 = mul2(d, inv);
      const bool pa = d.x > 0.0f, pb = d.y > 0.0f;
      const float2 L1 = f2(logf(fA ? model.x : dm0.x), logf(fB ? model.y : dm0.y));
      const float2 tp = mul2(TWO, fma2(d, L1, sub2(model, d)));
      const float2 tn = mul2(TWO, model);
      float2 term = f2(pa ? tp.x : tn.x, pb ? tp.y : tn.y);
      if (fA || fB) {
        const float l2a = logf(d.x), l2b = logf(d.y);
        const float lla = pa ? (d.x * L1.x - model.x - d.x * l2a + d.x) : -model.x;
        const float llb = pb ? (d.y * L1.y - model.y - d.y * l2b + d.y) : -model.y;
        if (fA) term.x = (model.x > 0.0f) ? lla : 0.0f;
        if (fB) term.y = (model.y > 0.0f) ? llb : 0.0f;
      }
      er.add(term);
      const float2 dm = f2(pa ? dm0.x : 0.0f, pb ? dm0.y : 0.0f);
      const float2 t1 = sub2(ONE, dm);
      const float2 t2 = mul2(dm, inv);
      const float2 w1 = f2(fA ? 0.0f : t1.x, fB ? 0.0f : t1.y);
      const float2 w2 = f2(fA ? inv.x : t2.x, fB ? inv.y : t2.y);
#pragma unroll
      for (int l = 0; l < NV; ++l) acc[l] = fma2(w1, du[l], acc[l]);
      int k = NV;
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        const float2 tl = mul2(w2, du[l]);
#pragma unroll
        for (int mm = l; mm < NV; ++mm, ++k) acc[k] = fma2(tl, du[mm], acc[k]);
      }
    }
  }

  // Reduce-scatter of the K sums of each slot, then gradient entry l and
  // Hessian row l of slot h gathered onto lane l of half h.
  reduce_scatter2<K, 16>(acc, lane);
  constexpr GatherCodes<NV, K> GC{};
  static_assert(rs_slots(K) == 1, "3D sums fit one slot per lane");
  const int sh = GC.B * (hl < NV ? hl : NV - 1);
  {
    const float ga = rs_gather<1>(acc[0].x, 0.0f, GC.grad, sh);
    const float gb = rs_gather<1>(acc[0].y, 0.0f, GC.grad, sh);
    gl = hb ? gb : ga;
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const float ha = rs_gather<1>(acc[0].x, 0.0f, GC.row[k], sh);
    const float hbv = rs_gather<1>(acc[0].y, 0.0f, GC.row[k], sh);
    hr[k] = hb ? hbv : ha;
  }
  const FPair2 tot = warp_sum_pair2(er);
  err_out = hb ? FPair{tot.hi.y, tot.lo.y} : FPair{tot.hi.x, tot.lo.x};
}

// Plain form: FitArgs as fit_kernel<6>; each warp holds one packed workspace.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) fit_pack_kernel(FitArgs a) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const PackLayout L = make_pack_layout(a.s);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int half = lane >> 4;
  float* ws = smem + wib * L.total();
  PairClaim c;
  c.counter = a.claim;
  c.next = ((int64_t)blockIdx.x * wpb + wib) * 2 + half;
  c.step = (int64_t)gridDim.x * wpb * 2;
  fit_pair_loop(a, a.s, ws + half * L.s2p, lane, c, nullptr,
                [&](float par, bool fisher, FPair& e, float& gn, float (&hn)[5]) {
                  evaluate_packed(a, L, ws, lane, par, fisher, e, gn, hn);
                });
}

// Batched form: BatchArgs as batch_kernel<6>; both slots work in the same
// segment and move to the next one together once neither finds a ROI left.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) batch_pack_kernel(const __grid_constant__ BatchArgs a) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int half = lane >> 4;
  float* ws = smem + wib * make_pack_layout(a.s_max).total();
  for (int seg = 0; seg < a.nseg; ++seg) {
    const BatchSeg& g = a.seg[seg];
    FitArgs fa;
    fa.m = g.m;
    fa.rois = g.rois;
    fa.s = g.s;
    fa.nfits = g.n;
    fa.iterations = g.iterations;
    fa.P = g.P;
    fa.CRLB = g.CRLB;
    fa.LL = g.LL;
    fa.out_n = g.n;
    fa.out_offset = 0;
    fa.trace = nullptr;
    fa.trace_max = 0;
    fa.flags = a.flags;
    fa.dT = nullptr;
    fa.z0 = nullptr;
    fa.w0 = nullptr;
    fa.n_starts = 0;
    fa.strict = 0;
    fa.var = nullptr;
    fa.claim = nullptr;
    fa.handoff = nullptr;
    PairClaim c;
    c.counter = &a.next[g.slot];
    c.next = 0;
    c.step = 0;
    const PackLayout L = make_pack_layout(g.s);
    fit_pair_loop(fa, g.s, ws + half * L.s2p, lane, c, &a.done[g.slot],
                  [&](float par, bool fisher, FPair& e, float& gn, float (&hn)[5]) {
                    evaluate_packed(fa, L, ws, lane, par, fisher, e, gn, hn);
                  });
  }
}

}  // namespace bsfit
