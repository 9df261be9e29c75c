// Per-ROI Levenberg-Marquardt Poisson-MLE fit of a cubic B-spline PSF,
// one warp per ROI, for fit types 6 (3D), 7 (4D colour) and 8 (5D + 3D), and
// the four-channel 4Pi fit (model tag kFit4Pi: one 4D (x, y, z, phase) spline
// seen by four interference channels at shifted phases, shared parameters).
//
// Method: the reference CPU fitter, VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2411-3620
// (VC = "MultiD_bspline/visual code"), with the same initial guesses, damping
// schedule, clamps, bounds, quirks and iteration cap. The arithmetic is
// reorganised for the GPU:
//
//  * Model evaluation is separable. For one ROI evaluation all pixels share the
//    non-lateral knot (z, w, u) and the fractional positions, and pixel (ii, jj)
//    only moves the lateral knots. The warp therefore (A) contracts the
//    non-lateral axes at every lateral node of the ROI's knot window into
//    shared-memory maps (value and one map per non-lateral derivative), (B)
//    contracts the Y axis for every (X node, pixel row), and (C) contracts the
//    X axis per pixel, fused with the Poisson deviance, gradient and Hessian.
//    This is the tensor-product sum of CPUsplineLib.cpp:1199-1288 (3D),
//    :761-970 (4D), :43-475 (5D) in a different summation order.
//  * Derivatives keep the reference's "difference of neighbouring
//    coefficients times the quadratic basis" form along every axis.
//  * Reductions are warp butterflies; the deviance is accumulated as a
//    compensated FP32 pair, since it drives the convergence test.
//  * The LM step is an FP32 Cholesky solve (CPUsplineLib.cpp:1363-1419) plus
//    one refinement step whose residual is computed with error-free FP32
//    products (float-float), instead of FP64: GB300 issues FP64 at 1/57 of the
//    FP32 rate and a one-lane FP64 instruction costs as much as a full warp.
//  * The CRLB is the diagonal of the inverse Fisher matrix, computed in FP32
//    lane-parallel on the Jacobi-scaled matrix D^-1 M D^-1 (unit diagonal) by
//    Cholesky and the squared columns of L^-1; the reference inverts M itself
//    in FP32 with an unpivoted LU (VC/CPUmleFit_LM/MatInvLib.h:17-77). The
//    double-float kernels (bsfit_fitdd.cu) invert it in FP64.
//
// Every global read of the coefficient arrays stays inside the array: the
// knots are clamped exactly as in the reference, and the one coefficient the
// reference reads past its knot window (the zero-weight fifth node of a
// derivative difference) is never read.
#pragma once

#include <cstdint>
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "bsfit_device.cuh"
#include "bsfit_internal.h"

// Minimum resident blocks of 4 warps per SM requested per model: trades
// registers for occupancy (measured: 6 blocks for 3D at 85 registers, 4 for
// the 4D and 4Pi models at 128, 3 for the 5D model at 168 without spills).
#ifndef BSFIT_MINBLOCKS6
#define BSFIT_MINBLOCKS6 6
#endif
#define BSFIT_MINBLOCKS(MODE) ((MODE) == 6 ? BSFIT_MINBLOCKS6 : (MODE) == 8 ? 3 : 4)

namespace bsfit {

// Optional phase timing (diagnostic builds with -DBSFIT_PHASE_TIMING): lane 0
// of every warp adds the clock64() cycles spent in each phase of the fit.
#ifdef BSFIT_PHASE_TIMING
static __device__ unsigned long long g_phase_cycles[16];
#define PHASE_DECL() long long _ph_t0 = clock64()
#define PHASE_RESET() _ph_t0 = clock64()
#define PHASE_MARK(k)                                                       \
  do {                                                                      \
    long long _ph_t1 = clock64();                                           \
    if ((threadIdx.x & 31) == 0)                                            \
      atomicAdd(&g_phase_cycles[k], (unsigned long long)(_ph_t1 - _ph_t0)); \
    _ph_t0 = _ph_t1;                                                        \
  } while (0)
#else
#define PHASE_DECL() \
  do {               \
  } while (0)
#define PHASE_RESET() \
  do {                \
  } while (0)
#define PHASE_MARK(k) \
  do {                \
  } while (0)
#endif

// Asynchronous 4-byte global -> shared copy (cp.async, cached in L1), its
// group commit and the waits for all but the most recent group / for all.
__device__ __forceinline__ void cp_async4(float* dst_smem, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int MODE>
struct ModeTraits;

template <>
struct ModeTraits<6> {
  static constexpr int D = 3;    // spline dimensions
  static constexpr int NV = 5;   // fitted parameters
  static constexpr int NA = 2;   // non-lateral maps: value, d/dz
  static constexpr int NG = 3;   // after the Y pass: value, d/dY, d/dz
  static constexpr int NCH = 1;  // image channels per ROI
  // stage-B maps written over consumed stage-A columns (see WarpLayout): on
  // where it lets more warps fit per SM
  static constexpr bool ALIAS = true;
  // sums reduced over the lanes with the trimmed reduce-scatter (reduce_scatter
  // of the K sums) rather than padded to 32 per exchange tree: a per-model
  // choice by measurement (3D +5%, 4D +1.4%; 5D and 4Pi 1-3% slower)
  static constexpr bool TRIM_RS = true;
};
template <>
struct ModeTraits<7> {
  static constexpr int D = 4;
  static constexpr int NV = 6;
  static constexpr int NA = 3;  // value, d/dz, d/dw
  static constexpr int NG = 4;  // value, d/dY, d/dz, d/dw
  static constexpr int NCH = 1;
  static constexpr bool ALIAS = false;
  static constexpr bool TRIM_RS = true;
};
// 4Pi: the 4D evaluation of fit type 7 once per channel.
template <>
struct ModeTraits<kFit4Pi> {
  static constexpr int D = 4;
  static constexpr int NV = 6;  // x, y, N, bg, z, phase
  static constexpr int NA = 3;
  static constexpr int NG = 4;
  static constexpr int NCH = k4PiChannels;
  static constexpr bool ALIAS = false;
  static constexpr bool TRIM_RS = false;
};

template <>
struct ModeTraits<8> {
  static constexpr int D = 5;
  static constexpr int NV = 8;
  // value, d/dz, d/dw, d/du of the 5D spline, the two correction maps of the
  // reference's 5D derivative (z term 27, u term 16), value and d/dz of the 3D
  // spline
  static constexpr int NA = 8;
  // value, d/dY, d/dz, d/dw, d/du, z correction, u correction (5D); value,
  // d/dY, d/dz (3D)
  static constexpr int NG = 10;
  static constexpr int NCH = 1;
  static constexpr bool ALIAS = true;
  static constexpr bool TRIM_RS = false;
};

// Per-warp shared-memory layout (floats): the ROI's pixels (one plane per
// channel), the per-pixel knots, the 1-D weights, the 4Pi channel offsets, and
// the maps. WP = s + 4 bounds the knot window along each lateral axis.
//
// The stage-A maps (NA per lateral node) and the stage-B maps (NG per X node
// and pixel row) are both stored by X node ("column"): A column xr holds
// NA x WP floats, G column xr holds NG x s. For the models whose maps would
// otherwise bound the warps per SM by shared memory (3D, 5D), the two share
// one region: stage B reads only A column xr to write G column xr and walks the
// columns in order, so G is written over A columns already consumed. With G
// at the start of the region and A at offset a_rel with
// (xr + 1) * GS <= a_rel + xr * AS for every column, a G column never reaches
// an A column that is still to be read (the reads and writes of one pass of
// the warp are separated by __syncwarp). The other models keep the two map
// sets apart (a_rel = WP * GS) and write G without that synchronisation,
// which would cost them registers.
//
// Bank-conflict-free access: stage B reads A, and stage C reads G, with s
// lanes per column in each pass of the warp at the same offsets in every
// column. A's column stride is padded to the next value congruent to s modulo
// 32, which puts those 32 lanes on 32 consecutive banks. G stores the maps of
// one (X node, pixel row) item together, GP floats per item, written and read
// as 16-byte vectors where the item has 3 or 4 maps (GP = 4: a quarter-warp's
// eight consecutive items cover the 32 banks), as 8-byte pairs for the 5D
// model's 10 maps (GP = 10: a half-warp's sixteen consecutive items sit 10
// banks apart, 2 banks each, all distinct), and otherwise with GP odd (the
// consecutive items of a pass an odd stride apart: 32 distinct banks).
struct WarpLayout {
  int s, s2p, wp, na, ng, nch, nvar;  // nvar: sCMOS variance planes (0 or nch)
  bool alias;
  int stage;  // floats of the 5D gather staging buffers (0: gathers go to registers)
  __host__ __device__ static constexpr int bank_pad(int x, int s) {
    return x + ((s - x) % 32 + 32) % 32;
  }
  __host__ __device__ constexpr int as() const { return bank_pad(na * wp, s); }  // A column stride
  // G item stride (see above): 4 for three or four maps (16-byte vectors), 10
  // for ten (8-byte pairs), else odd (scalar accesses)
  __host__ __device__ constexpr int gp() const {
    return (ng == 3 || ng == 4) ? 4 : ng == 10 ? 10 : (ng | 1);
  }
  __host__ __device__ constexpr int gs() const { return s * gp(); }             // G column stride
  __host__ __device__ constexpr int off_kx() const { return (nch + nvar) * s2p; }
  __host__ __device__ constexpr int off_ky() const { return off_kx() + ((s + 3) & ~3); }
  __host__ __device__ constexpr int off_w() const { return off_ky() + ((s + 3) & ~3); }
  __host__ __device__ constexpr int off_dt() const { return off_w() + 40; }
  __host__ __device__ constexpr int off_maps() const { return off_dt() + (nch > 1 ? nch * 6 : 0); }
  __host__ __device__ constexpr int a_rel() const {
    return alias ? gs() + (wp - 1) * (gs() > as() ? gs() - as() : 0) : wp * gs();
  }
  __host__ __device__ constexpr int off_g() const { return off_maps(); }
  __host__ __device__ constexpr int off_a() const { return off_maps() + a_rel(); }
  __host__ __device__ constexpr int maps_size() const {
    return (a_rel() + wp * as() > wp * gs()) ? a_rel() + wp * as() : wp * gs();
  }
  __host__ __device__ constexpr int off_stage() const { return off_maps() + maps_size(); }
  __host__ __device__ constexpr int total() const { return (off_stage() + stage + 3) & ~3; }
};

// Staged 5D gathers: two buffers of kStageQ coefficients (the 4 x 4 x 4 (u, w,
// z) block of the 5D table and the 4 z values of the 3D table) for 32 nodes,
// lane-major (coefficient q of the node of lane l at q * 32 + l).
constexpr int kStageQ = 68;
constexpr int kStageFloats = 2 * kStageQ * 32;

__host__ __device__ constexpr WarpLayout make_layout(int mode, int s, bool var = false,
                                                     int stg = 0) {
  WarpLayout L{};
  L.s = s;
  L.s2p = (s * s + 3) & ~3;
  L.wp = s + 4;
  L.na = mode == 6 ? 2 : (mode == 7 || mode == kFit4Pi) ? 3 : 8;
  L.ng = mode == 6 ? 3 : (mode == 7 || mode == kFit4Pi) ? 4 : 10;
  L.nch = mode == kFit4Pi ? k4PiChannels : 1;
  L.nvar = var ? L.nch : 0;
  L.alias = mode == 6 || mode == 8;
  L.stage = (stg && mode == 8) ? kStageFloats : 0;
  return L;
}

// Every region starts after the previous one ends (pixels nch * s^2, knots s
// each, weights 5 axes x 8, offsets nch x 6, maps), both map sets fit in the
// maps region, and the aliasing rule above holds for every column, for every
// model and ROI size.
constexpr bool layouts_disjoint() {
  const int modes[4] = {6, 7, 8, kFit4Pi};
  for (int mi = 0; mi < 4; ++mi)
    for (int s = 1; s <= 51; ++s)
      for (int var = 0; var < 2; ++var) {
        const WarpLayout L = make_layout(modes[mi], s, var != 0);
        if ((L.nch + L.nvar) * s * s > L.off_kx() || L.off_kx() + s > L.off_ky() ||
            L.off_ky() + s > L.off_w() || L.off_w() + 5 * 8 > L.off_dt() ||
            L.off_dt() + (L.nch > 1 ? L.nch * 6 : 0) > L.off_maps() ||
            L.off_a() + L.wp * L.as() > L.total() || L.off_g() + L.wp * L.gs() > L.total())
          return false;
        for (int c = 0; c < L.wp; ++c)
          if ((c + 1) * L.gs() > L.a_rel() + c * L.as()) return false;
        if (L.as() < L.na * L.wp || L.gp() < L.ng || (L.as() - s) % 32 != 0 ||
            (L.gp() % 2 == 0 && L.gp() != 4 && L.gp() != 10) || L.total() % 4 != 0 ||
            L.off_g() % 4 != 0)
          return false;
      }
  return true;
}
static_assert(layouts_disjoint(), "per-warp shared-memory regions overlap");
static_assert(make_layout(6, 13).alias == ModeTraits<6>::ALIAS &&
                  make_layout(7, 13).alias == ModeTraits<7>::ALIAS &&
                  make_layout(8, 13).alias == ModeTraits<8>::ALIAS &&
                  make_layout(kFit4Pi, 13).alias == ModeTraits<kFit4Pi>::ALIAS,
              "layout aliasing and stage-B synchronisation must agree");


// ---------------------------------------------------------------------------
// One ROI evaluation: deviance, gradient and Hessian (or Fisher information and
// log-likelihood when FISHER is set) at theta.

template <int MODE>
struct Eval {
  using T = ModeTraits<MODE>;
  static constexpr int D = T::D;
  static constexpr int NV = T::NV;
  static constexpr int NH = NV * (NV + 1) / 2;
};

// index of (l, m), l <= m, in the packed upper triangle of an NV x NV matrix
template <int NV>
__device__ __forceinline__ int hidx(int l, int m) {
  // index of (l, m), l <= m, in the packed upper triangle
  return l * NV - (l * (l - 1)) / 2 + (m - l);
}

// floor(a / b) for 0 <= a <= 64 and 1 <= b <= 64 without an integer division:
// q = trunc(a * r + 2^-10) with r the approximate reciprocal of b (relative
// error at most 2^-21). When a / b is an integer k <= 64, a * r >= k - 2^-15
// and the 2^-10 lifts it above k; otherwise a / b <= k + 1 - 1/b with
// 1/b >= 2^-6, so a * r + 2^-10 < k + 1 - 2^-6 + 2^-15 + 2^-10 < k + 1. The
// window and ROI widths (at most 55) and lane counts stay in that domain.
__device__ __forceinline__ int small_div(int a, int b) {
  const float r = __fdividef(1.0f, (float)b);
  return __float2int_rz(fmaf((float)a, r, 0.0009765625f));
}

// Row/column of item t of a row-major (rows x w) grid for a lane that starts at
// t = lane and advances by `step` (32, or 16 for a half-warp's lanes): avoids a
// runtime integer division per item.
struct Stride2D {
  int r, c, dr, dc, w;
  __device__ __forceinline__ Stride2D(int lane, int w_, int step = 32) : w(w_) {
    r = small_div(lane, w);
    c = lane - r * w;
    dr = small_div(step, w);
    dc = step - dr * w;
  }
  __device__ __forceinline__ void next() {
    r += dr;
    c += dc;
    if (c >= w) {
      c -= w;
      ++r;
    }
  }
};

// Phase position of a 4Pi channel wrapped into [1, 1 + P) by one period,
// P = nW - 1: the phase axis of the coefficients holds one period of phase
// samples plus one (the caller's bsarray of the phase-resolved PSF).
__device__ __forceinline__ float wrap_phase(float w, int nw) {
  const float P = (float)(nw - 1);
  if (w < 1.0f) return w + P;
  if (w >= (float)nw) return w - P;
  return w;
}

// One image channel of one ROI evaluation: model and derivatives at th for
// every pixel of `data`, accumulated into this lane's partial sums (err, and
// acc = gradient 0 .. NV-1, packed Hessian or Fisher upper triangle NV ..).
//
// LW lanes work on the ROI: the whole warp (LW = 32, lane = 0..31, gm = the
// full mask), or one half of it (LW = 16, lane = 0..15 within the half, gm =
// the half's mask; the two halves evaluate two ROIs in their own workspaces).
// Every node, item and pixel is computed by the same operations either way.
// The per-pixel sums keep the whole warp's order in both forms: with LW = 32
// lane l sums pixels l, l + 32, l + 64, ... into (err, acc); with LW = 16 lane
// l sums those pixels into (err, acc) and pixels l + 16, l + 48, ... (the
// sequence of warp lane l + 16) into (err2, acc2), so the reductions that
// follow can form the same sums as the whole warp's.
template <int MODE, int KP, bool VAR, int STG = 0, int LW = 32>
__device__ __forceinline__ void channel_pass(const FitArgs& a, const WarpLayout& L, float* ws,
                                             const float* data, int lane, const float* th,
                                             bool dup45, bool FISHER, FPair& err,
                                             float (&acc)[KP], FPair& err2, float (&acc2)[KP],
                                             unsigned gm = kFull, bool maps_ready = false) {
  static_assert(LW == 32 || (LW == 16 && MODE == 6 && !VAR && STG == 0),
                "half-warp ROIs: the 3D EMCCD model only");
  using TR = ModeTraits<MODE>;
  constexpr int D = TR::D;
  constexpr int NV = TR::NV;
  const int s = L.s;
  const ModelDev& m = a.m;
  int* kxs = reinterpret_cast<int*>(ws + L.off_kx());
  int* kys = reinterpret_cast<int*>(ws + L.off_ky());
  float* w = ws + L.off_w();
  float* A = ws + L.off_a();  // A[xr * AS + map * wp + yr]
  float* G = ws + L.off_g();  // G[(xr * s + py) * GP + map]
  const int wp = L.wp;
  const int AS = L.as(), GS = L.gs(), GP = L.gp();
  __syncwarp();  // the previous evaluation's readers of kxs / w / G are done
  PHASE_DECL();

  // Positions (CPUmleFit_LM.cpp:2512-2523): pixel jj sits at
  // (xc + jj) + off along X, pixel ii at (yc + ii) + off along Y.
  const float xc = (float)((s + 1) / 2) - th[0];
  const float yc = (float)((s + 1) / 2) - th[1];
  const float off = (float)(m.n[1] - s) / 2.0f;
  const float zc = th[4];
  const float wc = (D >= 4) ? th[5] : 0.0f;
  const float uc = (D >= 5) ? th[6] : 0.0f;

  for (int j = lane; j < s; j += LW) {
    kxs[j] = knot_index((xc + (float)j) + off, m.n[1]);
    kys[j] = knot_index((yc + (float)j) + off, m.n[0]);
  }
  // Fractional parts (Y, X, Z, W) and the 1-D weights, one per lane.
  {
    float fr[5];
    fr[0] = yc - floorf(yc);
    fr[1] = xc - floorf(xc);
    fr[2] = zc - floorf(zc);
    fr[3] = wc - floorf(wc);
    fr[4] = uc - floorf(uc);
    // 7 weights per axis: 35 for the 5D model, more than one per lane.
    for (int k = lane; k < 7 * D; k += LW) {
      const int ax = k / 7;
      w[ax * 8 + (k - ax * 7)] = axis_weight(fr[ax], k - ax * 7);
    }
  }
  __syncwarp();
  int kxmin, kxmax, kymin, kymax;
  {
    int a0 = INT_MAX, a1 = INT_MIN, b0 = INT_MAX, b1 = INT_MIN;
    for (int j = lane; j < s; j += LW) {
      a0 = min(a0, kxs[j]);
      a1 = max(a1, kxs[j]);
      b0 = min(b0, kys[j]);
      b1 = max(b1, kys[j]);
    }
    kxmin = __reduce_min_sync(gm, a0);
    kxmax = __reduce_max_sync(gm, a1);
    kymin = __reduce_min_sync(gm, b0);
    kymax = __reduce_max_sync(gm, b1);
  }
  // Window of lateral nodes [k - 1, k + 2] over all pixels. Its extent is at
  // most s + 4 (the per-pixel knots grow by one per pixel, plus one for
  // rounding); the caps keep every shared-memory access inside the warp's maps.
  const int xb = kxmin - 1, wx = min(kxmax - kxmin + 4, wp);
  const int yb = kymin - 1, wy = min(kymax - kymin + 4, wp);
  // Per pixel row: the window offset of its first Y node (clamped so the four
  // reads stay in the window); per pixel column: that of its first X node,
  // times the G column stride. Written over the knots by the lane that read
  // them; stages B and C read them after the synchronisation that ends stage A.
  for (int j = lane; j < s; j += LW) {
    kxs[j] = min(max(kxs[j] - 1 - xb, 0), wx - 4) * GS;
    kys[j] = min(max(kys[j] - 1 - yb, 0), wy - 4);
  }
  const int kz = knot_index(zc, m.n[2]);
  const int kw = (D >= 4) ? knot_index(wc, m.n[3]) : 0;
  const int ku = (D >= 5) ? knot_index(uc, m.n[4]) : 0;
  PHASE_MARK(0);

  // (A) Non-lateral contraction at every lateral node of the window. Skipped
  // with maps_ready: the caller guarantees that the maps in the workspace were
  // made by the previous evaluation at the same spatial parameters, so they
  // hold exactly the values these two stages would write.
  if (!maps_ready) {
    const float* wz = w + 2 * 8;
    const float bz0 = wz[0], bz1 = wz[1], bz2 = wz[2], bz3 = wz[3];
    const float dz0 = wz[4], dz1 = wz[5], dz2 = wz[6];
    const int64_t sz_ = m.st[2];
    const int nodes = wx * wy;
    if constexpr (D == 3) {
      // one base pointer per z plane and 32-bit lateral offsets (lateral
      // planes hold fewer than 2^29 elements); a 16-byte gather table as for
      // the 4D models measured no faster here (its lower L1 hit rate)
      const float* b0 = m.coeff + (int64_t)(kz - 1) * sz_;
      const float* b1 = b0 + sz_;
      const float* b2 = b1 + sz_;
      const float* b3 = b2 + sz_;
      const int st1 = (int)m.st[1];
      Stride2D ix(lane, wy, LW);
      for (int t = lane; t < nodes; t += LW, ix.next()) {
        const int xr = ix.r, yr = ix.c;
        const int lat = (xb + xr) * st1 + (yb + yr);
        float c0 = __ldg(b0 + lat), c1 = __ldg(b1 + lat), c2 = __ldg(b2 + lat), c3 = __ldg(b3 + lat);
        float v = c0 * bz0 + c1 * bz1 + c2 * bz2 + c3 * bz3;
        float dz = (c1 - c0) * dz0 + (c2 - c1) * dz1 + (c3 - c2) * dz2;
        A[xr * AS + yr] = v;
        A[xr * AS + wp + yr] = dz;
      }
    } else if constexpr (D == 4) {
      const float* ww = w + 3 * 8;
      const float bw[4] = {ww[0], ww[1], ww[2], ww[3]};
      const float dw[3] = {ww[4], ww[5], ww[6]};
      // Gathers from the gather table: per node, 16-byte entries at 32-bit
      // lateral offsets from one base per entry set (lateral planes hold fewer
      // than 2^29 elements).
      const int st1 = (int)m.st[1];
      Stride2D ix(lane, wy);
      const float2 BZ0 = bc2(bz0), BZ1 = bc2(bz1), BZ2 = bc2(bz2), BZ3 = bc2(bz3);
      const float2 DZ0 = bc2(dz0), DZ1 = bc2(dz1), DZ2 = bc2(dz2);
      // 4Pi: the four z planes of layer kw - 1 + iw at q4 + iw * zq_w; fit
      // type 7: layers (kw - 1, kw) at qp[0], (kw + 1, kw + 2) at qp[1], planes
      // 0, 1 in the entry at the node's offset and 2, 3 one plane further.
      const float4* q4 = m.zq + (int64_t)(kw - 1) * m.zq_w + (int64_t)(kz - 1) * m.zq_kz;
      const float4* qp[2] = {q4, q4 + 2 * m.zq_w};
      const int plane = (int)m.st[2];
      for (int t = lane; t < nodes; t += 32, ix.next()) {
        const int xr = ix.r, yr = ix.c;
        const int o0 = (xb + xr) * st1 + (yb + yr);
        // z contraction of the four w layers: two layers per packed operation
        // (fit type 7), or one at a time where the packed operands would push
        // the kernel past its register budget (4Pi, four channels); both
        // orders of operations are the same.
        float vz[4], dzv[4];
        if constexpr (MODE == kFit4Pi) {
          const float4* p = q4 + o0;
#pragma unroll
          for (int iw = 0; iw < 4; ++iw) {
            const float4 cq = __ldg(p + iw * m.zq_w);
            vz[iw] = contract4(cq.x, cq.y, cq.z, cq.w, bz0, bz1, bz2, bz3);
            dzv[iw] = dcontract4(cq.x, cq.y, cq.z, cq.w, dz0, dz1, dz2);
          }
        } else {
#pragma unroll
          for (int ip = 0; ip < 2; ++ip) {
            const float4 e01 = __ldg(qp[ip] + o0), e23 = __ldg(qp[ip] + plane + o0);
            const float2 c0 = make_float2(e01.x, e01.y), c1 = make_float2(e01.z, e01.w);
            const float2 c2 = make_float2(e23.x, e23.y), c3 = make_float2(e23.z, e23.w);
            const float2 v2 = contract4x2(c0, c1, c2, c3, BZ0, BZ1, BZ2, BZ3);
            const float2 d2 = dcontract4x2(c0, c1, c2, c3, DZ0, DZ1, DZ2);
            vz[2 * ip] = v2.x;
            vz[2 * ip + 1] = v2.y;
            dzv[2 * ip] = d2.x;
            dzv[2 * ip + 1] = d2.y;
          }
        }
        const float v = contract4(vz[0], vz[1], vz[2], vz[3], bw[0], bw[1], bw[2], bw[3]);
        const float dz = contract4(dzv[0], dzv[1], dzv[2], dzv[3], bw[0], bw[1], bw[2], bw[3]);
        const float dwv = dcontract4(vz[0], vz[1], vz[2], vz[3], dw[0], dw[1], dw[2]);
        A[xr * AS + yr] = v;
        A[xr * AS + wp + yr] = dz;
        A[xr * AS + 2 * wp + yr] = dwv;
      }
    } else {
      // 5D (z, w, u) for the mixture's 5D part, plus its 3D part (z only, on
      // coeff3 with the same lateral and z knots).
      const float* ww = w + 3 * 8;
      const float* wu = w + 4 * 8;
      const float bw[4] = {ww[0], ww[1], ww[2], ww[3]};
      const float dw[3] = {ww[4], ww[5], ww[6]};
      const float bu[4] = {wu[0], wu[1], wu[2], wu[3]};
      const float du[3] = {wu[4], wu[5], wu[6]};
      // Correction weights of the reference's z-derivative term 27 (reads
      // delta_dfz[32 n + 271], CPUsplineLib.cpp:313): per (lvZ, lvW, lvU) the
      // non-lateral factor R' of the weight actually read minus the factor R of
      // the intended weight dBz1(lvZ) Bw2(lvW) Bu2(lvU). For v = (lvW-1) +
      // 2 (lvU-1) < 3 the read weight is delta_dfz of block n + 8, i.e.
      // dBz2(lvZ) Bw2(lvW') Bu1(lvU') with v' = v + 1; for v = 3 it is the
      // W-derivative weight of block n - 24: Bz2(lvZ) dBw2(1) Bu1(1). The
      // lateral factor By2 Bx2 is the same in both.
      // Local node index per axis: offset + 1 (offsets -1..+2).
      // side 1, lv -> offset 1 - lv; side 2, lv -> offset lv.
      float R[2][2][2];  // [lvZ-1][lvW-1][lvU-1]
#pragma unroll
      for (int lz = 1; lz <= 2; ++lz)
#pragma unroll
        for (int lw = 1; lw <= 2; ++lw)
#pragma unroll
          for (int lu = 1; lu <= 2; ++lu) {
            const int v = (lw - 1) + 2 * (lu - 1);
            const float dBz1 = (lz == 1) ? dz1 : dz0;   // side 1 derivative, offsets 0 / -1
            const float dBz2 = (lz == 1) ? dz2 : 0.0f;  // side 2 derivative, offsets +1 / +2
            const float Bz2 = (lz == 1) ? bz2 : bz3;
            float rp;
            if (v < 3) {
              const int vp = v + 1, lwp = (vp & 1) + 1, lup = (vp >> 1) + 1;
              rp = dBz2 * (lwp == 1 ? bw[2] : bw[3]) * (lup == 1 ? bu[1] : bu[0]);
            } else {
              rp = Bz2 * dw[2] * bu[1];
            }
            R[lz - 1][lw - 1][lu - 1] = rp - dBz1 * (lw == 1 ? bw[2] : bw[3]) * (lu == 1 ? bu[2] : bu[3]);
          }
      const int64_t sw_ = m.st[3], su_ = m.st[4];
      const float* base = m.coeff + (int64_t)(kz - 1) * sz_ + (int64_t)(kw - 1) * sw_ +
                          (int64_t)(ku - 1) * su_;
      const float* base3 = m.coeff3 + (int64_t)(kz - 1) * sz_;
      // Packed operands: the z and w weights broadcast to both halves, the
      // correction weights R of u = 2, 3 side by side.
      const float2 BZ0 = bc2(bz0), BZ1 = bc2(bz1), BZ2 = bc2(bz2), BZ3 = bc2(bz3);
      const float2 DZ0 = bc2(dz0), DZ1 = bc2(dz1), DZ2 = bc2(dz2);
      const float2 BW0 = bc2(bw[0]), BW1 = bc2(bw[1]), BW2 = bc2(bw[2]), BW3 = bc2(bw[3]);
      const float2 DW0 = bc2(dw[0]), DW1 = bc2(dw[1]), DW2 = bc2(dw[2]);
      float2 RP[2][2];  // [lvZ-1][lvW-1] = (R(lvU = 1), R(lvU = 2))
#pragma unroll
      for (int lz = 0; lz < 2; ++lz)
#pragma unroll
        for (int lw = 0; lw < 2; ++lw) RP[lz][lw] = make_float2(R[lz][lw][0], R[lz][lw][1]);
      if constexpr (STG != 0) {
      // Staged gathers: the 68 coefficients of the next round of 32 nodes are
      // copied global -> shared with asynchronous copies (cp.async) while the
      // current round is contracted from shared memory, so each lane has a
      // round of gathers in flight instead of a few loads; the arithmetic is
      // that of the unstaged loop, in the same order.
      float* stg = ws + L.off_stage();
      const int rounds = (nodes + 31) / 32;
      auto issue = [&](int r) {
        const int t = r * 32 + lane;
        if (t < nodes) {
          const int xr = t / wy, yr = t - xr * wy;
          const int64_t lat = (int64_t)(xb + xr) * m.st[1] + (yb + yr);
          const float* p = base + lat;
          float* d = stg + (r & 1) * (kStageQ * 32) + lane;
#pragma unroll
          for (int iu = 0; iu < 4; ++iu)
#pragma unroll
            for (int iw = 0; iw < 4; ++iw)
#pragma unroll
              for (int iz = 0; iz < 4; ++iz)
                cp_async4(d + (((iw * 4 + iu) * 4) + iz) * 32, p + iu * su_ + iw * sw_ + iz * sz_);
          const float* p3 = base3 + lat;
#pragma unroll
          for (int iz = 0; iz < 4; ++iz) cp_async4(d + (64 + iz) * 32, p3 + iz * sz_);
        }
        cp_async_commit();
      };
      issue(0);
      for (int r = 0; r < rounds; ++r) {
        __syncwarp();  // this round's buffer was last read two rounds ago
        if (r + 1 < rounds) issue(r + 1);
        else cp_async_commit();
        cp_async_wait_one();  // this lane's copies of round r have landed
        const int t = r * 32 + lane;
        if (t >= nodes) continue;
        const int xr = t / wy, yr = t - xr * wy;
        const float* sb = stg + (r & 1) * (kStageQ * 32) + lane;
        auto S = [&](int iu, int iw, int iz) { return sb[(((iw * 4 + iu) * 4) + iz) * 32]; };
        // z contraction of the 16 (u, w) columns, u = 2k and 2k + 1 side by
        // side in one packed operation.
        float2 vz2[2][4], dzz2[2][4];  // [u pair][w]
        float2 qz2 = make_float2(0.0f, 0.0f);  // z-term-27 correction, u = 2 | u = 3
        float2 sq2[2][2];  // [u pair][w in {0,1}]: sum over z in {0,1} of Bz * C
#pragma unroll
        for (int iw = 0; iw < 4; ++iw)
#pragma unroll
          for (int up = 0; up < 2; ++up) {
            const float2 c0 = make_float2(S(2 * up, iw, 0), S(2 * up + 1, iw, 0));
            const float2 c1 = make_float2(S(2 * up, iw, 1), S(2 * up + 1, iw, 1));
            const float2 c2 = make_float2(S(2 * up, iw, 2), S(2 * up + 1, iw, 2));
            const float2 c3 = make_float2(S(2 * up, iw, 3), S(2 * up + 1, iw, 3));
            vz2[up][iw] = contract4x2(c0, c1, c2, c3, BZ0, BZ1, BZ2, BZ3);
            dzz2[up][iw] = dcontract4x2(c0, c1, c2, c3, DZ0, DZ1, DZ2);
            if (up == 1 && iw >= 2) {
              // lvW = iw - 1, lvU = u - 1; Z nodes 1 - lvZ: local 1 (lvZ 1), 0 (lvZ 2)
              qz2 = __fadd2_rn(qz2, __ffma2_rn(sub2(c2, c1), RP[0][iw - 2],
                                               __fmul2_rn(sub2(c1, c0), RP[1][iw - 2])));
            }
            if (iw <= 1) sq2[up][iw] = __ffma2_rn(c1, BZ1, __fmul2_rn(c0, BZ0));
          }
        float vw[4], dzw[4], dww[4];
#pragma unroll
        for (int up = 0; up < 2; ++up) {
          const float2 a = contract4x2(vz2[up][0], vz2[up][1], vz2[up][2], vz2[up][3], BW0, BW1, BW2, BW3);
          const float2 b = contract4x2(dzz2[up][0], dzz2[up][1], dzz2[up][2], dzz2[up][3], BW0, BW1, BW2, BW3);
          const float2 c = dcontract4x2(vz2[up][0], vz2[up][1], vz2[up][2], vz2[up][3], DW0, DW1, DW2);
          vw[2 * up] = a.x;
          vw[2 * up + 1] = a.y;
          dzw[2 * up] = b.x;
          dzw[2 * up + 1] = b.y;
          dww[2 * up] = c.x;
          dww[2 * up + 1] = c.y;
        }
        const float v = contract4(vw[0], vw[1], vw[2], vw[3], bu[0], bu[1], bu[2], bu[3]);
        const float dzv = contract4(dzw[0], dzw[1], dzw[2], dzw[3], bu[0], bu[1], bu[2], bu[3]);
        const float dwv = contract4(dww[0], dww[1], dww[2], dww[3], bu[0], bu[1], bu[2], bu[3]);
        const float duv = dcontract4(vw[0], vw[1], vw[2], vw[3], du[0], du[1], du[2]);
        const float qz = qz2.x + qz2.y;
        float sq[4][2];
#pragma unroll
        for (int iw = 0; iw < 2; ++iw) {
          sq[0][iw] = sq2[0][iw].x;
          sq[1][iw] = sq2[0][iw].y;
          sq[2][iw] = sq2[1][iw].x;
          sq[3][iw] = sq2[1][iw].y;
        }
        // u-term-16 correction (CPUsplineLib.cpp:420-421): the term differences
        // the U node at offset 0 instead of +1 with weight
        // By1 Bx1 Bz1 Bw1 dBu2(1); lateral side 1 and z, w at offsets -1 / 0.
        float qu = 0.0f;
#pragma unroll
        for (int iw = 0; iw < 2; ++iw)
          qu += bw[iw] * ((sq[2][iw] - sq[1][iw]) - (sq[3][iw] - sq[2][iw]));
        qu *= du[2];
        float e0 = sb[64 * 32], e1 = sb[65 * 32], e2 = sb[66 * 32], e3 = sb[67 * 32];
        float* o = A + xr * AS + yr;
        o[0] = v;
        o[wp] = dzv;
        o[2 * wp] = dwv;
        o[3 * wp] = duv;
        o[4 * wp] = qz;
        o[5 * wp] = qu;
        o[6 * wp] = contract4(e0, e1, e2, e3, bz0, bz1, bz2, bz3);
        o[7 * wp] = dcontract4(e0, e1, e2, e3, dz0, dz1, dz2);
      }
      cp_async_wait_all();
      } else {
      // the 5D block by 64-bit node pointer and layer strides (uniform base
      // pointers per (u, w) layer with 32-bit offsets, as the 3D and 4D stage A
      // do, measured 3% slower here: they push the kernel into spills); the 3D
      // part's four z planes from the gather table (32-bit lateral offsets)
      const int st1 = (int)m.st[1];
      const float4* q3 = m.zq + (int64_t)(kz - 1) * m.zq_kz;
      Stride2D ix(lane, wy);
      for (int t = lane; t < nodes; t += 32, ix.next()) {
        const int xr = ix.r, yr = ix.c;
        const int o0 = (xb + xr) * st1 + (yb + yr);
        const float* p = base + o0;
        // z contraction of the 16 (u, w) columns, u = 2k and 2k + 1 side by
        // side in one packed operation.
        float2 vz2[2][4], dzz2[2][4];  // [u pair][w]
        float2 qz2 = make_float2(0.0f, 0.0f);  // z-term-27 correction, u = 2 | u = 3
        float2 sq2[2][2];  // [u pair][w in {0,1}]: sum over z in {0,1} of Bz * C
#pragma unroll
        for (int iw = 0; iw < 4; ++iw)
#pragma unroll
          for (int up = 0; up < 2; ++up) {
            const float* q0 = p + (2 * up) * su_ + iw * sw_;
            const float* q1 = q0 + su_;
            const float2 c0 = make_float2(__ldg(q0), __ldg(q1));
            const float2 c1 = make_float2(__ldg(q0 + sz_), __ldg(q1 + sz_));
            const float2 c2 = make_float2(__ldg(q0 + 2 * sz_), __ldg(q1 + 2 * sz_));
            const float2 c3 = make_float2(__ldg(q0 + 3 * sz_), __ldg(q1 + 3 * sz_));
            vz2[up][iw] = contract4x2(c0, c1, c2, c3, BZ0, BZ1, BZ2, BZ3);
            dzz2[up][iw] = dcontract4x2(c0, c1, c2, c3, DZ0, DZ1, DZ2);
            if (up == 1 && iw >= 2) {
              // lvW = iw - 1, lvU = u - 1; Z nodes 1 - lvZ: local 1 (lvZ 1), 0 (lvZ 2)
              qz2 = __fadd2_rn(qz2, __ffma2_rn(sub2(c2, c1), RP[0][iw - 2],
                                               __fmul2_rn(sub2(c1, c0), RP[1][iw - 2])));
            }
            if (iw <= 1) sq2[up][iw] = __ffma2_rn(c1, BZ1, __fmul2_rn(c0, BZ0));
          }
        float vw[4], dzw[4], dww[4];
#pragma unroll
        for (int up = 0; up < 2; ++up) {
          const float2 a = contract4x2(vz2[up][0], vz2[up][1], vz2[up][2], vz2[up][3], BW0, BW1, BW2, BW3);
          const float2 b = contract4x2(dzz2[up][0], dzz2[up][1], dzz2[up][2], dzz2[up][3], BW0, BW1, BW2, BW3);
          const float2 c = dcontract4x2(vz2[up][0], vz2[up][1], vz2[up][2], vz2[up][3], DW0, DW1, DW2);
          vw[2 * up] = a.x;
          vw[2 * up + 1] = a.y;
          dzw[2 * up] = b.x;
          dzw[2 * up + 1] = b.y;
          dww[2 * up] = c.x;
          dww[2 * up + 1] = c.y;
        }
        const float v = contract4(vw[0], vw[1], vw[2], vw[3], bu[0], bu[1], bu[2], bu[3]);
        const float dzv = contract4(dzw[0], dzw[1], dzw[2], dzw[3], bu[0], bu[1], bu[2], bu[3]);
        const float dwv = contract4(dww[0], dww[1], dww[2], dww[3], bu[0], bu[1], bu[2], bu[3]);
        const float duv = dcontract4(vw[0], vw[1], vw[2], vw[3], du[0], du[1], du[2]);
        const float qz = qz2.x + qz2.y;
        float sq[4][2];
#pragma unroll
        for (int iw = 0; iw < 2; ++iw) {
          sq[0][iw] = sq2[0][iw].x;
          sq[1][iw] = sq2[0][iw].y;
          sq[2][iw] = sq2[1][iw].x;
          sq[3][iw] = sq2[1][iw].y;
        }
        // u-term-16 correction (CPUsplineLib.cpp:420-421): the term differences
        // the U node at offset 0 instead of +1 with weight
        // By1 Bx1 Bz1 Bw1 dBu2(1); lateral side 1 and z, w at offsets -1 / 0.
        float qu = 0.0f;
#pragma unroll
        for (int iw = 0; iw < 2; ++iw)
          qu += bw[iw] * ((sq[2][iw] - sq[1][iw]) - (sq[3][iw] - sq[2][iw]));
        qu *= du[2];
        const float4 e = __ldg(q3 + o0);
        const float e0 = e.x, e1 = e.y, e2 = e.z, e3 = e.w;
        float* o = A + xr * AS + yr;
        o[0] = v;
        o[wp] = dzv;
        o[2 * wp] = dwv;
        o[3 * wp] = duv;
        o[4 * wp] = qz;
        o[5 * wp] = qu;
        o[6 * wp] = contract4(e0, e1, e2, e3, bz0, bz1, bz2, bz3);
        o[7 * wp] = dcontract4(e0, e1, e2, e3, dz0, dz1, dz2);
      }
      }
    }
  }
  __syncwarp();
  PHASE_MARK(1);

  // (B) Y contraction for every (X node, pixel row ii), column by column. Where
  // G is written over the A columns already read (the layout's aliasing rule),
  // every pass of the warp reads its A values, synchronises, then writes.
  if (!maps_ready) {
    const float by0 = w[0], by1 = w[1], by2 = w[2], by3 = w[3];
    const float dy0 = w[4], dy1 = w[5], dy2 = w[6];
    constexpr int NG = TR::NG;
    const int items = wx * s;
    // the two halves' item counts differ with their windows: both run the
    // larger count, so the synchronisation below is reached by the whole warp
    const int items_u = (LW == 32) ? items : max(items, __shfl_xor_sync(kFull, items, 16));
    Stride2D ix(lane, s, LW);
    for (int t0 = 0; t0 < items_u; t0 += LW, ix.next()) {
      const bool act = t0 + lane < items;
      const int xr = ix.r, py = ix.c;
      float gv[NG];
      if (act) {
        const int oy = kys[py];
        const float* a0 = A + xr * AS + oy;
        const float v0 = a0[0], v1 = a0[1], v2 = a0[2], v3 = a0[3];
        gv[0] = v0 * by0 + v1 * by1 + v2 * by2 + v3 * by3;
        gv[1] = (v1 - v0) * dy0 + (v2 - v1) * dy1 + (v3 - v2) * dy2;
        if constexpr (MODE != 8) {
#pragma unroll
          for (int c = 1; c < TR::NA; ++c) {
            const float* ac = a0 + c * wp;
            gv[c + 1] = ac[0] * by0 + ac[1] * by1 + ac[2] * by2 + ac[3] * by3;
          }
        } else {
#pragma unroll
          for (int c = 1; c <= 3; ++c) {  // d/dz, d/dw, d/du of the 5D spline
            const float* ac = a0 + c * wp;
            gv[c + 1] = ac[0] * by0 + ac[1] * by1 + ac[2] * by2 + ac[3] * by3;
          }
          const float* qz = a0 + 4 * wp;  // lateral side 2: offsets +1, +2
          gv[5] = qz[2] * by2 + qz[3] * by3;
          const float* qu = a0 + 5 * wp;  // lateral side 1: offsets -1, 0
          gv[6] = qu[0] * by0 + qu[1] * by1;
          const float* b3 = a0 + 6 * wp;  // 3D spline value
          const float u0 = b3[0], u1 = b3[1], u2 = b3[2], u3 = b3[3];
          gv[7] = u0 * by0 + u1 * by1 + u2 * by2 + u3 * by3;
          gv[8] = (u1 - u0) * dy0 + (u2 - u1) * dy1 + (u3 - u2) * dy2;
          const float* z3 = a0 + 7 * wp;
          gv[9] = z3[0] * by0 + z3[1] * by1 + z3[2] * by2 + z3[3] * by3;
        }
      }
      if constexpr (TR::ALIAS) __syncwarp();  // G aliases A (see WarpLayout)
      if (act) {
        float* go = G + (xr * s + py) * GP;
        if constexpr (MODE == 6) {
          *reinterpret_cast<float4*>(go) = make_float4(gv[0], gv[1], gv[2], 0.0f);
        } else if constexpr (NG == 4) {
          *reinterpret_cast<float4*>(go) = make_float4(gv[0], gv[1], gv[2], gv[3]);
        } else {
          static_assert(NG == 10, "5D items are stored as map pairs");
#pragma unroll
          for (int c = 0; c < NG; c += 2)
            *reinterpret_cast<float2*>(go + c) = make_float2(gv[c], gv[c + 1]);
        }
      }
    }
  }
  __syncwarp();
  PHASE_MARK(2);

  // (C) X contraction per pixel, fused with the likelihood sums.
  {
    const float bx0 = w[8], bx1 = w[9], bx2 = w[10], bx3 = w[11];
    const float dx0 = w[12], dx1 = w[13], dx2 = w[14];
    const float N = th[2], bg = th[3];
    const int s2 = s * s;
    // pixel p = px * s + py, px = jj (X), py = ii (Y), into the chain (er, ac)
    auto pixel = [&](int p, int px, int py, FPair& er, float (&ac)[KP]) {
      const float* g = G + (kxs[px] + py * GP);  // X node k of map c at g[k * GS + c]
      float dudt[NV];
      float model;
      if constexpr (MODE == 6) {
        // the item's three maps as one vector per X node (value, d/dY, d/dz)
        const float4* g4 = reinterpret_cast<const float4*>(g);
        const float4 q0 = g4[0], q1 = g4[s], q2 = g4[2 * s], q3 = g4[3 * s];
        float f = q0.x * bx0 + q1.x * bx1 + q2.x * bx2 + q3.x * bx3;
        float dX = (q1.x - q0.x) * dx0 + (q2.x - q1.x) * dx1 + (q3.x - q2.x) * dx2;
        float dY = q0.y * bx0 + q1.y * bx1 + q2.y * bx2 + q3.y * bx3;
        float dc = q0.z * bx0 + q1.z * bx1 + q2.z * bx2 + q3.z * bx3;
        dudt[0] = -N * dX;
        dudt[1] = -N * dY;
        dudt[2] = f;
        dudt[3] = 1.0f;
        dudt[4] = N * dc;
        model = bg + N * f;
      } else if constexpr (MODE != 8) {
        // the item's four maps as one vector per X node (value, d/dY, d/dz,
        // d/dw)
        const float4* g4 = reinterpret_cast<const float4*>(g);
        const float4 q0 = g4[0], q1 = g4[s], q2 = g4[2 * s], q3 = g4[3 * s];
        float f = q0.x * bx0 + q1.x * bx1 + q2.x * bx2 + q3.x * bx3;
        float dX = (q1.x - q0.x) * dx0 + (q2.x - q1.x) * dx1 + (q3.x - q2.x) * dx2;
        float dY = q0.y * bx0 + q1.y * bx1 + q2.y * bx2 + q3.y * bx3;
        float dz = q0.z * bx0 + q1.z * bx1 + q2.z * bx2 + q3.z * bx3;
        float dw = q0.w * bx0 + q1.w * bx1 + q2.w * bx2 + q3.w * bx3;
        dudt[0] = -N * dX;
        dudt[1] = -N * dY;
        dudt[2] = f;
        dudt[3] = 1.0f;
        dudt[4] = N * dz;
        dudt[5] = N * dw;
        if (MODE == 7 && dup45) dudt[5] = dudt[4];
        model = bg + N * f;
      } else {
        // 5D: the item's ten maps as five pairs per X node: (value, d/dY),
        // (d/dz, d/dw), (d/du, z correction), (u correction, 3D value),
        // (3D d/dY, 3D d/dz)
        float2 q[4][5];
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
          for (int c = 0; c < 5; ++c) q[k][c] = reinterpret_cast<const float2*>(g + k * GS)[c];
        float f = q[0][0].x * bx0 + q[1][0].x * bx1 + q[2][0].x * bx2 + q[3][0].x * bx3;
        float dX = (q[1][0].x - q[0][0].x) * dx0 + (q[2][0].x - q[1][0].x) * dx1 +
                   (q[3][0].x - q[2][0].x) * dx2;
        float dY = q[0][0].y * bx0 + q[1][0].y * bx1 + q[2][0].y * bx2 + q[3][0].y * bx3;
        dudt[0] = -N * dX;
        dudt[1] = -N * dY;
        // 5D derivatives with the reference's two term corrections
        float dZ = q[0][1].x * bx0 + q[1][1].x * bx1 + q[2][1].x * bx2 + q[3][1].x * bx3 +
                   (q[2][2].y * bx2 + q[3][2].y * bx3);
        float dW = q[0][1].y * bx0 + q[1][1].y * bx1 + q[2][1].y * bx2 + q[3][1].y * bx3;
        float dU = q[0][2].x * bx0 + q[1][2].x * bx1 + q[2][2].x * bx2 + q[3][2].x * bx3 +
                   (q[0][3].x * bx0 + q[1][3].x * bx1);
        // 3D spline
        float h0 = q[0][3].y, h1 = q[1][3].y, h2 = q[2][3].y, h3 = q[3][3].y;
        float f3 = h0 * bx0 + h1 * bx1 + h2 * bx2 + h3 * bx3;
        float dX3 = (h1 - h0) * dx0 + (h2 - h1) * dx1 + (h3 - h2) * dx2;
        float dY3 = q[0][4].x * bx0 + q[1][4].x * bx1 + q[2][4].x * bx2 + q[3][4].x * bx3;
        float dZ3 = q[0][4].y * bx0 + q[1][4].y * bx1 + q[2][4].y * bx2 + q[3][4].y * bx3;
        // mixture (CPUmleFit_LM.cpp:3311-3322)
        const float g2 = th[7], h2m = 1.0f - g2;
        const float m5 = bg + N * f, m3 = bg + N * f3;
        dudt[0] = dudt[0] * g2 + h2m * (-N * dX3);
        dudt[1] = dudt[1] * g2 + h2m * (-N * dY3);
        dudt[2] = f * g2 + h2m * f3;
        dudt[3] = g2 + h2m;
        dudt[4] = (N * dZ) * g2 + h2m * (N * dZ3);
        dudt[5] = N * dW;
        dudt[6] = N * dU;
        // m5 - m3 = N (f5 - f3): formed without the background, which cancels
        dudt[NV - 1] = N * (f - f3);
        model = m3 * h2m + m5 * g2;
      }
      float d = data[p];
      if constexpr (VAR) {
        // sCMOS: variance / gain^2 added to model and data
        // (VC/GPUmleFit_LM/GPUmleFit_LM_sCMOS.cu:1045-1046)
        const float v = data[L.nch * L.s2p + p];
        model += v;
        d += v;
      }
      const float inv = __frcp_rn(model);
      if (!FISHER) {
        // CPUmleFit_LM.cpp:2540-2559, with one reciprocal: d / m = d * (1 / m)
        // and log(m / d) = -log(d / m).
        float term;
        float dm = 0.0f;
        if (d > 0.0f) {
          dm = d * inv;
          term = 2.0f * ((model - d) + d * logf(dm));
        } else {
          term = 2.0f * model;
        }
        er.add(term);
        const float t1 = 1.0f - dm;
        const float t2 = dm * inv;
#pragma unroll
        for (int l = 0; l < NV; ++l) ac[l] = fmaf(t1, dudt[l], ac[l]);
        int k = NV;
#pragma unroll
        for (int l = 0; l < NV; ++l) {
          const float tl = t2 * dudt[l];
#pragma unroll
          for (int mm = l; mm < NV; ++mm, ++k) ac[k] = fmaf(tl, dudt[mm], ac[k]);
        }
      } else {
        // Fisher information and log-likelihood (CPUmleFit_LM.cpp:2730-2742).
        const float im = inv;
        int k = NV;
#pragma unroll
        for (int l = 0; l < NV; ++l) {
          const float tl = dudt[l] * im;
#pragma unroll
          for (int mm = l; mm < NV; ++mm, ++k) ac[k] = fmaf(tl, dudt[mm], ac[k]);
        }
        if (model > 0.0f) {
          float ll = (d > 0.0f) ? (d * logf(model) - model - d * logf(d) + d) : -model;
          er.add(ll);
        }
      }
    };
    if constexpr (LW == 32) {
      Stride2D ix(lane, s);
      for (int p = lane; p < s2; p += 32, ix.next()) pixel(p, ix.r, ix.c, err, acc);
    } else {
      Stride2D ia(lane, s), ib(lane + 16, s);
      for (int p = lane; p < s2; p += 32, ia.next(), ib.next()) {
        pixel(p, ia.r, ia.c, err, acc);
        if (p + 16 < s2) pixel(p + 16, ib.r, ib.c, err2, acc2);
      }
    }
  }
  PHASE_MARK(3);
}

// Outputs are distributed over the lanes: lane l < NV receives gradient entry
// l (gl) and Hessian row l (hr), or Fisher row l; err_out is on every lane.
// maps_ready (single-channel models): the workspace still holds the maps of the
// previous evaluation, made at the same spatial parameters (see channel_pass).
template <int MODE, bool VAR = false, int STG = 0>
__device__ void evaluate(const FitArgs& a, const WarpLayout& L, float* ws, int lane,
                         const float* th, bool dup45, bool FISHER, FPair& err_out, float& gl,
                         float (&hr)[ModeTraits<MODE>::NV], bool maps_ready = false) {
  using TR = ModeTraits<MODE>;
  constexpr int NV = TR::NV;
  constexpr int NH = NV * (NV + 1) / 2;
  constexpr int K = NV + NH;
  constexpr int KP = (K + 31) / 32 * 32;
  FPair err{0.0f, 0.0f};
  float acc[KP];
#pragma unroll
  for (int k = 0; k < KP; ++k) acc[k] = 0.0f;
  if constexpr (TR::NCH == 1) {
    channel_pass<MODE, KP, VAR, STG>(a, L, ws, ws, lane, th, dup45, FISHER, err, acc, err, acc,
                                     kFull, maps_ready);
  } else {
    // 4Pi: channel c sees the shared parameters plus its offsets dT[c], with
    // its phase shifted by shift[c] and wrapped; the sums run over all
    // channels' pixels.
    const float* dts = ws + L.off_dt();
    for (int ch = 0; ch < TR::NCH; ++ch) {
      float thc[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) thc[k] = th[k] + dts[ch * NV + k];
      thc[5] = wrap_phase(thc[5] + a.m.shift[ch], a.m.n[3]);
      channel_pass<MODE, KP, VAR>(a, L, ws, ws + ch * L.s2p, lane, thc, false, FISHER, err, acc, err,
                                  acc);
    }
  }
  PHASE_DECL();
  if constexpr (TR::TRIM_RS) {
    // Reduce-scatter of the K sums, then gradient entry l and Hessian row l
    // gathered onto lane l from the lanes that hold them.
    reduce_scatter<K, 16>(acc, lane);
    constexpr GatherCodes<NV, K> GC{};
    const float t0 = acc[0];
    const float t1 = (rs_slots(K) > 1) ? acc[1] : 0.0f;
    const int sh = GC.B * (lane < NV ? lane : NV - 1);
    gl = rs_gather<rs_slots(K)>(t0, t1, GC.grad, sh);
#pragma unroll
    for (int k = 0; k < NV; ++k) hr[k] = rs_gather<rs_slots(K)>(t0, t1, GC.row[k], sh);
  } else {
    // Padded form: one 32-value reduce-scatter per 32 sums (zeros past K);
    // lane t gets the total of value t (and t + 32).
    float t0, t1 = 0.0f;
    {
      float v[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] = acc[k];
      reduce_scatter<32, 16>(v, lane);
      t0 = v[0];
    }
    if constexpr (KP > 32) {
      float v[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) v[k] = acc[32 + (k % (KP - 32))];
#pragma unroll
      for (int k = KP - 32; k < 32; ++k) v[k] = 0.0f;
      reduce_scatter<32, 16>(v, lane);
      t1 = v[0];
    }
    gl = t0;  // value index l = gradient entry l on lane l
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const int lo = lane < k ? lane : k, hi = lane < k ? k : lane;
      const int idx = (lane < NV) ? NV + hidx<NV>(lo, hi) : 0;
      const float a0 = __shfl_sync(kFull, t0, idx & 31);
      const float a1 = (KP > 32) ? __shfl_sync(kFull, t1, idx & 31) : 0.0f;
      hr[k] = (idx < 32) ? a0 : a1;
    }
  }
  err_out = warp_sum_pair(err);
  PHASE_MARK(4);
}

// ---------------------------------------------------------------------------
// LM helpers (warp-uniform register state).


// Unpivoted Cholesky of the full matrix a (row-major NV x NV), lower factor in
// u (u[i*NV + j], j <= i). Fails on a negative pivot only
// (CPUsplineLib.cpp:1363-1390).
template <int NV>
__device__ __forceinline__ bool cholesky(const float (&a)[NV * NV], float (&u)[NV * NV]) {
#pragma unroll
  for (int i = 0; i < NV; i++) {
#pragma unroll
    for (int j = 0; j <= i; j++) {
      float s = 0.0f;
#pragma unroll
      for (int k = 0; k < j; k++) s = fmaf(u[i * NV + k], u[j * NV + k], s);
      if (i == j) {
        float piv = a[i * NV + i] - s;
        if (!(piv >= 0.0f)) return false;
        u[i * NV + j] = sqrtf(piv);
      } else {
        u[i * NV + j] = (a[i * NV + j] - s) / u[j * NV + j];
      }
    }
  }
  return true;
}

template <int NV>
__device__ __forceinline__ void chol_solve(const float (&u)[NV * NV], const float (&b)[NV],
                                           float (&x)[NV]) {
  float y[NV];
#pragma unroll
  for (int i = 0; i < NV; i++) {
    float t = b[i];
#pragma unroll
    for (int j = 0; j < i; j++) t -= u[i * NV + j] * y[j];
    y[i] = t / u[i * NV + i];
  }
#pragma unroll
  for (int i = NV - 1; i >= 0; i--) {
    float t = y[i];
#pragma unroll
    for (int j = i + 1; j < NV; j++) t -= u[j * NV + i] * x[j];
    x[i] = t / u[i * NV + i];
  }
}

// ---------------------------------------------------------------------------
// One ROI, one warp. The LM state is distributed over the lanes: lane l < NV
// owns parameter l (value, previous value, sign, clamp), gradient entry l and
// Hessian row l, so the small dense algebra of each step runs lane-parallel
// with shuffles (a right-looking Cholesky, two triangular solves, one
// refinement), and every per-parameter rule is one lane's instruction stream.
// The decisions (convergence, accept / reject, damping) are warp-uniform.

__device__ __forceinline__ float bcast(float v, int k) { return __shfl_sync(kFull, v, k); }

// Initial clamp and fade of parameter l (CPUmleFit_LM.cpp:2434, :2786-2788,
// :3191-3193).
template <int MODE>
__device__ __forceinline__ void clamp_fade(int l, float& c, float& f) {
  if (MODE == 6) {
    c = (l < 2) ? 2.0f : (l == 2) ? 10000.0f : 20.0f;
    f = 0.5f;
  } else if (MODE == 7) {
    c = (l < 2) ? 1.0f : (l == 2) ? 10000.0f : (l == 3) ? 20.0f : (l == 4) ? 2.0f : 0.00001f;
    f = (l < 2) ? 0.5f : (l == 2) ? 0.4f : (l == 3) ? 0.5f : (l == 4) ? 0.7f : 0.8f;
  } else if (MODE == kFit4Pi) {
    c = (l < 2) ? 1.0f : (l == 2) ? 10000.0f : (l == 3) ? 20.0f : 2.0f;
    f = 0.5f;
  } else {
    c = (l < 2) ? 1.0f : (l == 2) ? 10000.0f : (l == 3) ? 20.0f : (l < 7) ? 2.0f : 0.1f;
    f = 0.5f;
  }
}

// Lane-parallel solve of (L L^T) x = b: lane i holds b_i, row i of L (lr),
// column i of L below the diagonal (lc[k] = L[k][i]) and 1 / L_ii.
template <int NV>
__device__ __forceinline__ float lane_solve(int lane, const float (&lr)[NV], const float (&lc)[NV],
                                            float invd, float b) {
  float y = b;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const float yk = bcast(y * invd, k);
    if (lane == k) y = yk;
    else if (lane > k) y = fmaf(-lr[k], yk, y);
  }
  float x = y;
#pragma unroll
  for (int k = NV - 1; k >= 0; --k) {
    const float xk = bcast(x * invd, k);
    if (lane == k) x = xk;
    else if (lane < k) x = fmaf(-lc[k], xk, x);
  }
  return x;
}

// Stage one ROI in the warp's shared memory: its pixels (4Pi: the four
// channel planes, rois laid out [channel][roi][s][s]) and the 4Pi channel
// offsets dT [roi][channel][6].
template <int MODE, bool VAR = false>
__device__ __forceinline__ void load_roi(const FitArgs& a, const WarpLayout& L, float* ws,
                                         int lane, int64_t roi) {
  const int s2 = L.s * L.s;
  const int nch = ModeTraits<MODE>::NCH;
  for (int ch = 0; ch < nch; ++ch) {
    const float* src = a.rois + ((int64_t)ch * a.nfits + roi) * (int64_t)s2;
    float* dst = ws + ch * L.s2p;
    for (int p = lane; p < s2; p += 32) dst[p] = __ldg(src + p);
    if constexpr (VAR) {
      const float* vsrc = a.var + ((int64_t)ch * a.nfits + roi) * (int64_t)s2;
      float* vdst = ws + (nch + ch) * L.s2p;
      for (int p = lane; p < s2; p += 32) vdst[p] = __ldg(vsrc + p);
    }
  }
  if constexpr (ModeTraits<MODE>::NCH > 1) {
    constexpr int ND = ModeTraits<MODE>::NCH * ModeTraits<MODE>::NV;
    if (lane < ND) ws[L.off_dt() + lane] = a.dT ? __ldg(a.dT + roi * ND + lane) : 0.0f;
  }
  __syncwarp();
}

// Initial x, y, N, bg of one image (CPUgaussLib.cpp:172-225 centroid and
// max / min, CPUmleFit_LM.cpp:2477-2482), warp-uniform in g.
__device__ __forceinline__ void initial_guess(const float* data, int s, int lane, float (&g)[4]) {
  const int s2 = s * s;
  FPair tx{0.f, 0.f}, ty{0.f, 0.f}, ts{0.f, 0.f};
  float mx = 0.0f, mn = 10e10f;
  bool nan_seen = false;
  Stride2D ix(lane, s);
  for (int p = lane; p < s2; p += 32, ix.next()) {
    float d = data[p];
    const int jj = ix.r, ii = ix.c;
    tx.add(d * (float)ii);
    ty.add(d * (float)jj);
    ts.add(d);
    nan_seen |= (d != d);
    mx = (mx > d) ? mx : d;
    mn = (mn < d) ? mn : d;
  }
  tx = warp_sum_pair(tx);
  ty = warp_sum_pair(ty);
  ts = warp_sum_pair(ts);
  const float tsum = ts.hi + ts.lo;
  if (__any_sync(kFull, nan_seen)) {
    // The reference's max/min fold is order dependent with NaN pixels:
    // replay it sequentially.
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
  // N0 = max(0, (max - min) * 2 * pi * 1.5 * 1.5), bg0 = max(min, 0.01),
  // evaluated in double as in the reference's expression.
  const double n0 = ((double)mx - (double)mn) * 2.0 * (double)3.141592f * 1.5 * 1.5;
  g[0] = (tx.hi + tx.lo) / tsum;
  g[1] = (ty.hi + ty.lo) / tsum;
  g[2] = (float)((0.0 > n0) ? 0.0 : n0);
  g[3] = (mn > 0.01f) ? mn : 0.01f;
}

// Result of one fit, distributed like the LM state: lane l < NV holds
// parameter l and its variance; the log-likelihood and the iteration count are
// on every lane.
struct RoiResult {
  float par, crlb, ll;
  int kk;
};

// Fit of the ROI staged in ws (load_roi) from start `start` (0 unless
// multi-start).
template <int MODE, bool VAR = false, int STG = 0>
__device__ RoiResult fit_roi(const FitArgs& a, const WarpLayout& L, float* ws, int lane, int64_t roi,
                             int start) {
  using TR = ModeTraits<MODE>;
  constexpr int NV = TR::NV;
  const int s = L.s;

  PHASE_DECL();
  // Initial guesses (CPUgaussLib.cpp:172-225, CPUmleFit_LM.cpp:2477-2482),
  // then lane l keeps parameter l.
  float par;
  {
    float v = 0.0f;
    if constexpr (TR::NCH == 1) {
      float g[4];
      initial_guess(ws, s, lane, g);
      if (lane < 4) v = g[lane];
    } else {
      // 4Pi: the mean over the channels of the single-channel rule, the
      // centroid taken back by the channel's offset.
      const float* dts = ws + L.off_dt();
      float sum[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int ch = 0; ch < TR::NCH; ++ch) {
        float g[4];
        initial_guess(ws + ch * L.s2p, s, lane, g);
        sum[0] += g[0] - dts[ch * NV + 0];
        sum[1] += g[1] - dts[ch * NV + 1];
        sum[2] += g[2];
        sum[3] += g[3];
      }
      if (lane < 4) v = sum[lane] / (float)TR::NCH;
    }
    if (MODE == 6) {
      if (lane == 4) v = (float)a.m.n[2] / 2.0f;
    } else if (MODE == 7) {
      const float* ip = (a.n_starts > 0) ? a.starts[start] : a.m.init_p;
      const bool use = (a.n_starts > 0 || a.m.init_p_len >= 2) && ip[0] != 0.0f;
      if (lane == 4) v = use ? ip[0] : (float)a.m.n[2] / 2.0f;
      if (lane == 5) v = use ? ip[1] : (float)a.m.n[3] / 2.0f;
    } else if (MODE == 8) {
      // (z, w, u, g2) from initP, shared by all ROIs (CPUmleFit_LM.cpp:3246-3256)
      const float* ip = (a.n_starts > 0) ? a.starts[start] : a.m.init_p;
      if (lane >= 4 && lane < 8) v = ip[lane - 4];
    } else {
      // 4Pi: per-ROI initial z and phase, one array per start
      const int64_t i0 = (int64_t)start * a.nfits + roi;
      if (lane == 4) v = a.z0[i0];
      if (lane == 5) v = wrap_phase(a.w0[i0], a.m.n[3]);
    }
    par = v;
  }

  // Per-lane LM state (CPUmleFit_LM.cpp:2425-2450): lane l < NV owns
  // parameter l.
  float opar = par, sg = 0.0f, osg = 0.0f, cl, fd, par_eval = par;
  clamp_fade<MODE>(lane, cl, fd);
  float ocl = cl;
  float gl = 0.0f;   // gradient entry
  float hr[NV];      // Hessian row (damped in place), or the Fisher row
  // Warp-uniform state.
  float lambda = 1.0f, olambda = 1.0f, sum_update = 1e10f;
  FPair err{1e12f, 0.0f}, oerr{1e13f, 0.0f};
  int turn = 1;

  // One evaluation call site for the initial pass, every accepted step and the
  // final CRLB pass (keeps the kernel's instruction footprint small).
  int kk = 0;
  bool need_eval = true, first = true, fisher = false;
  FPair ll{0.0f, 0.0f};
  PHASE_MARK(5);
  for (;;) {
    if (need_eval) {
      FPair e;
      // Parameters of the evaluation, broadcast to every lane. Fit type 8's
      // CRLB pass keeps the positions and g2 of the last evaluation
      // (CPUmleFit_LM.cpp:3568-3584) with the current N and bg.
      // The maps of stages A and B depend on the spatial parameters only (not
      // on N, bg or g2). The CRLB pass usually evaluates at the position of
      // the last evaluation (after the stop test, or at the iteration cap after
      // an accepted step; fit type 8 by construction): it then reuses that
      // evaluation's maps, which are still in the workspace, and runs stage C
      // alone. After a rejected step the position differs and the pass is
      // complete. Bitwise equality, so the results are those of a full pass.
      bool maps_ready = false;
      if (fisher && TR::NCH == 1) {
        const bool spatial = lane < NV && lane != 2 && lane != 3 && !(MODE == 8 && lane == 7);
        const bool same = (MODE == 8) || !spatial || __float_as_uint(par) == __float_as_uint(par_eval);
        maps_ready = __all_sync(kFull, same);
      }
      if (!fisher) par_eval = par;
      float the[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k)
        the[k] = bcast((MODE == 8 && fisher && k != 2 && k != 3) ? par_eval : par, k);
      evaluate<MODE, VAR, STG>(a, L, ws, lane, the, first && MODE == 7, fisher, e, gl, hr,
                               maps_ready);
      first = false;
      need_eval = false;
      if (fisher) {
        ll = e;
        break;
      }
      err = e;
      PHASE_RESET();
    }
    if (kk >= a.iterations) {
      fisher = true;
      need_eval = true;
      continue;
    }
    float* rec = (a.trace && start == 0 && kk < a.trace_max && lane == 0)
                     ? a.trace + (roi * (int64_t)a.trace_max + kk) * TRACE_REC
                     : nullptr;
    // |(newErr - oldErr) / newErr| < 1e-6 (CPUmleFit_LM.cpp:2565)
    {
      const float dhi = err.hi - oerr.hi;
      const float dlo = err.lo - oerr.lo;
      const float rel = fabsf((dhi + dlo) / (err.hi + err.lo));
      if (rec) {
        rec[0] = (float)kk;
        rec[1] = rel;
        rec[2] = err.hi + err.lo;
        rec[3] = oerr.hi + oerr.lo;
        rec[4] = 0.0f;
      }
      if (rel < 1e-6f || (MODE == 8 && sum_update < 1e-5f)) {  // :3355
        if (rec) rec[4] = 1.0f;
        fisher = true;
        need_eval = true;
        continue;
      }
    }
    const float e_new = err.hi + err.lo, e_old = oerr.hi + oerr.lo;
    // newErr > 1.5 * oldErr, evaluated in double by the reference: the FMA
    // forms 1.5 * oldErr - newErr with one rounding, which keeps its sign.
    if (fmaf(1.5f, e_old, -e_new) < 0.0f) {
      sg = osg;
      cl = ocl;
      par = opar;
      lambda = olambda;
      err = oerr;
      lambda = 10.0f * lambda;
    } else if (e_new < e_old) {
      if (lambda > 1.0f)
        lambda = (float)((double)lambda * 0.8);
      else if (lambda < 1.0f)
        lambda = 1.0f;
    }
    // H_ll *= lambda, in place (cumulative across failed solves, as in the
    // reference).
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (lane == k) hr[k] *= lambda;
    // A parameter whose derivative is exactly zero at every pixel (z on the
    // mirror-padded boundary knot) has an exactly zero Hessian row. The
    // reference only survives that case through rounding noise of its double
    // derivative sums (a ~1e-29 pivot and a huge step of noise-determined
    // sign, cut to +-clamp); an exact zero would give NaN. Such a parameter is
    // held for this step instead: its row becomes the identity and its
    // gradient zero.
    bool frz = false;
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (lane == k) frz = (hr[k] == 0.0f);
    const unsigned fmask = __ballot_sync(kFull, frz && lane < NV);
    float am[NV], ar[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      am[k] = ((fmask >> k) & 1u) ? 0.0f : hr[k];
      if (frz) am[k] = (k == lane) ? 1.0f : 0.0f;
      ar[k] = am[k];
    }
    const float rhs = frz ? 0.0f : gl;
    // Right-looking Cholesky (CPUsplineLib.cpp:1363-1390 computes the same
    // factor; it fails on a negative pivot only).
    float lr[NV], lc[NV], invd = 1.0f;
    bool ok = true;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      lr[j] = 0.0f;
      lc[j] = 0.0f;
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const float ajj = bcast(am[j], j);
      if (!(ajj >= 0.0f)) {
        ok = false;
        break;
      }
      // 1/sqrt by the hardware reciprocal square root: the refinement step
      // below absorbs its rounding (the refined steps are unchanged on 3D).
      const float inv = rsqrtf(ajj);
      const float ljj = ajj * inv;
      const float lij = (lane > j) ? am[j] * inv : ((lane == j) ? ljj : 0.0f);
      lr[j] = lij;
      if (lane == j) invd = inv;
#pragma unroll
      for (int k = j + 1; k < NV; ++k) {
        const float lkj = bcast(lij, k);
        if (lane == j) lc[k] = lkj;
        if (lane > j && k <= lane) am[k] = fmaf(-lij, lkj, am[k]);
      }
    }
    float upd = 0.0f;
    if (ok) {
      upd = lane_solve<NV>(lane, lr, lc, invd, rhs);
      if (!(a.flags & FLAG_NO_REFINE)) {
        // One refinement step: r = b - A upd with error-free products.
        float sh = rhs, sl = 0.0f;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const float xk = bcast(upd, k);
          float p_, pe_, t_, te_;
          two_prod(ar[k], xk, p_, pe_);
          two_sum(sh, -p_, t_, te_);
          sh = t_;
          sl += te_ - pe_;
        }
        upd += lane_solve<NV>(lane, lr, lc, invd, sh + sl);
      }
      if (MODE != 6) {
        // CPUmleFit_LM.cpp:2943-2950: a NaN step counts as a failed solve
        if (__any_sync(kFull, lane < NV && upd != upd)) ok = false;
      }
    }
    if (ok) {
      if (MODE == 7 && lane == 5) upd = upd * 10.0f;  // :2951
      osg = sg;
      ocl = cl;
      opar = par;
      olambda = lambda;
      oerr = err;
      if (MODE == 7) {
        // "let it go" (:2966-2971)
        const float dz = bcast(upd, 4);
        if (fabsf(dz) < 0.005f && turn) {
          if (lane == 5) cl = ocl = (float)a.m.n[3] / 10.0f;
          if (lane == 4) cl = ocl = 2.0f;
          turn = 0;
        }
      }
      if (sg != 0.0f) {
        if ((sg == 1.0f && upd < 0.0f) || (sg == -1.0f && upd > 0.0f)) cl = cl * fd;
      }
      sg = (upd > 0.0f) ? 1.0f : -1.0f;
      const float step = upd / (1.0f + fabsf(upd / cl));
      par = par - step;
      if (MODE == 8) sum_update = warp_sum(lane < NV ? fabsf(step) : 0.0f);
      // Bounds (CPUmleFit_LM.cpp:2626-2634, :3003-3010, :3421-3447).
      if (MODE == 8 && lane < 2) {
        const float lo = (float)(s - 1) / 2.0f - (float)s / 4.0f;  // exact for s <= 51
        const float hi = (float)(s - 1) / 2.0f + (float)s / 4.0f;
        par = (par > lo) ? par : lo;
        par = (par < hi) ? par : hi;
      }
      if (lane == 2) par = (par > 1.0f) ? par : 1.0f;
      // max(bg, 0.01) in double: no float lies strictly between 0.01f and
      // 0.01, so the float comparison selects the same branch.
      if (lane == 3) par = (par > 0.01f) ? par : 0.01f;
      if (lane == 4) {
        par = (par > 0.0f) ? par : 0.0f;
        const float zmax = (MODE == 6) ? (float)(a.m.n[2] - 4) : (float)a.m.n[2] - 0.5f;
        par = (par < zmax) ? par : zmax;
      }
      if (MODE == 7 && lane == 5) {
        par = (par > 0.0f) ? par : 0.0f;
        const float wmax = (float)a.m.n[3] - 0.5f;
        par = (par < wmax) ? par : wmax;
      }
      if (MODE == kFit4Pi && lane == 5) par = wrap_phase(par, a.m.n[3]);
      if (MODE == 8) {
        if (lane == 5) {
          // periodic azimuth (:3436-3443): period nW - 2
          const int nw = a.m.n[3];
          if (par <= 1.0f)
            par = (float)(nw - 2) + par;
          else if (par > (float)(nw - 1))
            par = (2.0f + par) - (float)nw;
        }
        if (lane == 6) {
          par = (par > 1.0f) ? par : 1.0f;
          const float umax = (float)a.m.n[4] - 0.5f;
          par = (par < umax) ? par : umax;
        }
        if (lane == 7) {
          par = (par < 1.0f) ? par : 1.0f;
          par = (par > 0.0f) ? par : 0.0f;
        }
      }
      need_eval = true;
    } else {
      lambda = 10.0f * lambda;
    }
    if (a.trace) {
      // decision record (diagnostics): gathered from the parameter lanes
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        const float uk = bcast(ok ? upd : 0.0f, k);
        const float pk = bcast(par, k);
        if (rec) {
          rec[6 + k] = uk;
          rec[14 + k] = pk;
        }
      }
      if (rec) {
        rec[4] = (e_new > 1.5f * e_old ? 2.0f : 0.0f) + (e_new < e_old ? 4.0f : 0.0f) + (ok ? 8.0f : 0.0f);
        rec[5] = lambda;
        rec[22] = 0.0f;
      }
    }
    ++kk;
    PHASE_MARK(6);
  }

  // CRLB = diag(M^-1) of the Fisher matrix M (the reference inverts it with an
  // unpivoted LU, VC/CPUmleFit_LM/MatInvLib.h:17-77). Here, lane-parallel in
  // FP32 on the Jacobi-scaled matrix S = D^-1 M D^-1 (unit diagonal, so its
  // condition number is that of the parameters' correlations, not of their
  // units): Cholesky S = L L^T, then diag(S^-1)_c = sum_k ((L^-1)_kc)^2 with the
  // columns of L^-1 by forward substitution, and (M^-1)_cc = (S^-1)_cc / M_cc.
  // A parameter with an exactly zero Fisher row (zero derivative everywhere)
  // is decoupled: its variance is +inf, the others are unaffected.
  PHASE_RESET();
  float crlb = 0.0f;  // lane c: variance of parameter c
  {
    float mr[NV], dk[NV];
    float mydiag = 0.0f;
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (lane == k) mydiag = hr[k];
#pragma unroll
    for (int k = 0; k < NV; ++k) dk[k] = bcast(mydiag, k);
    const float sd = sqrtf(mydiag);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const float den = sd * sqrtf(dk[k]);
      mr[k] = (lane == k) ? 1.0f : ((den > 0.0f) ? hr[k] / den : 0.0f);
    }
    float lr[NV], invd = 1.0f;
    bool okc = true;
#pragma unroll
    for (int j = 0; j < NV; ++j) lr[j] = 0.0f;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const float ajj = bcast(mr[j], j);
      if (!(ajj > 0.0f)) okc = false;
      const float inv = rsqrtf(ajj);
      const float ljj = ajj * inv;
      const float lij = (lane > j) ? mr[j] * inv : ((lane == j) ? ljj : 0.0f);
      lr[j] = lij;
      if (lane == j) invd = inv;
#pragma unroll
      for (int k = j + 1; k < NV; ++k) {
        const float lkj = bcast(lij, k);
        if (lane > j && k <= lane) mr[k] = fmaf(-lij, lkj, mr[k]);
      }
    }
    // columns of L^-1: z = L^-1 e_c, lane i holds z_i; accumulate z_i^2 per c
    float acc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
      float part = 0.0f, z = 0.0f;
#pragma unroll
      for (int k = c; k < NV; ++k) {
        const float zk = bcast(((k == c ? 1.0f : 0.0f) - part) * invd, k);
        if (lane == k) z = zk;
        else if (lane > k) part = fmaf(lr[k], zk, part);
      }
      acc[c] = (lane >= c && lane < NV) ? z * z : 0.0f;
    }
    warp_sum_array<NV>(acc);
#pragma unroll
    for (int c = 0; c < NV; ++c)
      if (lane == c) crlb = okc ? acc[c] / dk[c] : __int_as_float(0x7fc00000);
    // decoupled zero rows
#pragma unroll
    for (int c = 0; c < NV; ++c)
      if (lane == c && dk[c] == 0.0f) crlb = __int_as_float(0x7f800000);
  }
  PHASE_MARK(7);
  return RoiResult{par, crlb, ll.hi + ll.lo, kk};
}

template <int MODE>
__device__ __forceinline__ void store_result(const FitArgs& a, int lane, int64_t roi,
                                             const RoiResult& r) {
  constexpr int NV = ModeTraits<MODE>::NV;
  float thv[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) thv[k] = bcast(r.par, k);
  if (lane == 0) {
    const int64_t n = a.out_n;
    const int64_t o = a.out_offset + roi;
#pragma unroll
    for (int i = 0; i < NV; ++i) a.P[i * n + o] = thv[i];
    a.P[NV * n + o] = (float)r.kk;
    a.LL[o] = r.ll;
  }
  if (lane < NV) a.CRLB[lane * a.out_n + a.out_offset + roi] = r.crlb;
  __syncwarp();
}

// Fit one ROI from every start and store the kept result. The ROI is staged
// once; a later start replaces the kept result when its log-likelihood is
// higher by more than 1e-4 (strict) or by at least 1e-4, the rule of the
// reference's multi-start callers (MultiD_fitter/simplefitter_cspline.m:480-490,
// demo_orientation/store/fitb5n3.m:36-45, demo_4pi/bspline_based_4piloc_v4.m:201-214).
// MULTI selects the multi-start kernels; the single-start ones carry no start
// loop (it would cost them registers).
template <int MODE, bool MULTI, bool VAR = false, int STG = 0>
__device__ __forceinline__ void fit_and_store(const FitArgs& a, const WarpLayout& L, float* ws,
                                              int lane, int64_t roi) {
  load_roi<MODE, VAR>(a, L, ws, lane, roi);
  if constexpr (MULTI) {
    // one call site for all starts (a second inlined copy of the fit would
    // double the kernel's instruction footprint)
    RoiResult best{0.0f, 0.0f, 0.0f, 0};
    const int ns = a.n_starts > 0 ? a.n_starts : 1;  // 0: the model's initP alone
    for (int k = 0; k < ns; ++k) {
      const RoiResult r = fit_roi<MODE>(a, L, ws, lane, roi, k);
      const float d = r.ll - best.ll;
      if (k == 0 || (a.strict ? (d > 1e-4f) : (d >= 1e-4f))) best = r;
    }
    store_result<MODE>(a, lane, roi, best);
  } else {
    store_result<MODE>(a, lane, roi, fit_roi<MODE, VAR, STG>(a, L, ws, lane, roi, 0));
  }
}

// MINB: minimum resident blocks of 4 warps per SM requested from the
// compiler (its register budget); the default is the measured choice per
// model, other values are the autotuner's variants (bsfit_tune.cu).
template <int MODE, bool MULTI, bool VAR = false, int MINB = BSFIT_MINBLOCKS(MODE), int STG = 0>
__global__ void __launch_bounds__(128, MINB) fit_kernel(FitArgs a) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const WarpLayout L = make_layout(MODE, a.s, VAR, STG);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float* ws = smem + wib * L.total();
  if (a.claim) {
    for (;;) {
      unsigned long long i = 0;
      if (lane == 0) i = atomicAdd(a.claim, 1ull);
      i = __shfl_sync(kFull, i, 0);
      if ((int64_t)i >= a.nfits) break;
      fit_and_store<MODE, MULTI, VAR, STG>(a, L, ws, lane, (int64_t)i);
    }
    return;
  }
  const int64_t total_warps = (int64_t)gridDim.x * wpb;
  for (int64_t roi = (int64_t)blockIdx.x * wpb + wib; roi < a.nfits; roi += total_warps)
    fit_and_store<MODE, MULTI, VAR, STG>(a, L, ws, lane, roi);
}

// Persistent batched fit: every warp claims ROIs one at a time from the
// segments' work counters (in segment order: the host sorts segments by
// decreasing cost, so the largest ROIs start first and the tail is short),
// fits them, and counts them done. The warp's shared memory is laid out for
// the largest ROI of the batch. MULTI: every ROI is fitted from its segment's
// starts and the best log-likelihood kept (fit_and_store), in a separate
// instantiation so the single-start kernel carries no start loop. CAP: the
// serving loop's capped form, where a warp stops after a.warp_rois ROIs (the
// grid then covers every ROI, and blocks retire as they finish); a separate
// instantiation, so the persistent kernels carry no counter.
template <int MODE, bool MULTI = false, int MINB = BSFIT_MINBLOCKS(MODE), int STG = 0,
          bool CAP = false>
__global__ void __launch_bounds__(128, MINB) batch_kernel(const __grid_constant__ BatchArgs a) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  float* ws = smem + wib * make_layout(MODE, a.s_max, false, STG).total();
  int seg = 0;
  int fitted = 0;  // ROIs this warp has fitted (CAP)
  while (seg < a.nseg && (!CAP || fitted < a.warp_rois)) {
    const BatchSeg& g = a.seg[seg];
    unsigned long long i = 0;
    if (lane == 0) i = atomicAdd(&a.next[g.slot], 1ull);
    i = __shfl_sync(kFull, i, 0);
    if ((int64_t)i >= g.n) {
      ++seg;
      continue;
    }
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
    if constexpr (MULTI) {
      fa.n_starts = g.n_starts;
      fa.strict = g.strict;
#pragma unroll 1
      for (int k = 0; k < g.n_starts; ++k)
#pragma unroll
        for (int j = 0; j < 4; ++j) fa.starts[k][j] = g.starts[k][j];
    }
    fit_and_store<MODE, MULTI, false, STG>(fa, make_layout(MODE, g.s, false, STG), ws, lane, (int64_t)i);
    if (lane == 0) atomicAdd(&a.done[g.slot], 1ull);
    if constexpr (CAP) ++fitted;
  }
}

}  // namespace bsfit
