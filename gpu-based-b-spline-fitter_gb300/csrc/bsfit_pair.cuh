// Two 3D ROIs per warp: the "pair" form of the fit type 6 kernels.
//
// Each half of the warp (16 lanes) fits its own ROI in its own shared-memory
// workspace, with its own LM state, and takes a new ROI as soon as its current
// one is stored; the halves share every instruction of the evaluation, the LM
// step and the CRLB. The per-evaluation work that does not grow with the ROI
// (knots and weights, the reduce-scatter of the sums, the LM step's Cholesky
// and solves, all executed by the whole warp for one ROI in the one-ROI form)
// then serves two ROIs, and the per-pixel rounds of 16 lanes waste fewer lanes
// on the last, partial round.
//
// Results are bit-identical to the one-ROI form (fit_roi): every node, item
// and pixel term is the same operation sequence; each lane sums its pixels
// into two chains that reproduce warp lanes l and l + 16 of the one-ROI form
// (channel_pass with LW = 16); the two chains are added first, which is the
// one-ROI form's first exchange level (lanes l and l ^ 16), and the other
// levels (8, 4, 2, 1) run within the half in the same order; floating-point
// addition is commutative and the two-sum of the compensated deviance is exact
// in either operand order, so every total is the same. The LM step and the
// CRLB are the same per-lane operations with the broadcasts taken from the
// half's lanes; their warp sums over lanes holding zeros beyond the parameters
// are unchanged by leaving the zeros out.
#pragma once

#include "bsfit_fit_kernels.cuh"

namespace bsfit {

// Half-warp reduce-scatter bookkeeping: after the two chains are added, the K
// sums go through reduce_scatter<K, 8> (levels 8, 4, 2, 1 within the half).
__host__ __device__ constexpr int half_rs_slots(int c) {
  for (int o = 8; o > 0; o >>= 1) c = c / 2 + (c & 1);
  return c;
}

// src[x] = 2 * lane + slot of the lowest half-lane holding value x after
// reduce_scatter<C, 8>.
template <int C>
struct HalfRsSources {
  int src[C];
  __host__ __device__ constexpr HalfRsSources() : src() {
    for (int x = 0; x < C; ++x) src[x] = -1;
    for (int lane = 0; lane < 16; ++lane) {
      int map[64] = {};
      for (int i = 0; i < C; ++i) map[i] = i;
      int c = C;
      for (int o = 8; o > 0; o >>= 1) {
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

// Where half-lane l < NV finds gradient entry l and Hessian entry (l, k): 5-bit
// codes 2 * lane + slot, one field per lane.
template <int NV, int K>
struct HalfGatherCodes {
  static constexpr int SLOTS = half_rs_slots(K);
  static_assert(SLOTS <= 2 && NV * 5 <= 32, "half-warp gather codes");
  unsigned grad;
  unsigned row[NV];
  __host__ __device__ constexpr HalfGatherCodes() : grad(0), row() {
    const HalfRsSources<K> rs{};
    for (int l = 0; l < NV; ++l) grad |= (unsigned)rs.src[l] << (5 * l);
    for (int k = 0; k < NV; ++k)
      for (int l = 0; l < NV; ++l) {
        const int lo = l < k ? l : k, hi = l < k ? k : l;
        const int x = NV + lo * NV - (lo * (lo - 1)) / 2 + (hi - lo);
        row[k] |= (unsigned)rs.src[x] << (5 * l);
      }
  }
};

template <int SLOTS>
__device__ __forceinline__ float half_gather(float t0, float t1, unsigned codes, int sh, int hb) {
  const int code = (int)((codes >> sh) & 31u);
  const float a0 = __shfl_sync(kFull, t0, hb + (code >> 1));
  if constexpr (SLOTS > 1) {
    const float a1 = __shfl_sync(kFull, t1, hb + (code >> 1));
    return (code & 1) ? a1 : a0;
  } else {
    return a0;
  }
}

// Value of lane k of this lane's half (hb = 0 or 16).
__device__ __forceinline__ float hbcast(float v, int hb, int k) {
  return __shfl_sync(kFull, v, hb + k);
}

// Compensated pair sum over the half: chain a (warp lane l's sequence) and
// chain b (warp lane l + 16's) added as warp_sum_pair's first level, then its
// levels 8, 4, 2, 1 and the final renormalisation.
__device__ __forceinline__ FPair half_sum_pair(FPair a, FPair b) {
  FPair v;
  {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    v.hi = s;
    v.lo = a.lo + b.lo + e;
  }
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    float h = __shfl_xor_sync(kFull, v.hi, o);
    float l = __shfl_xor_sync(kFull, v.lo, o);
    float s, e;
    two_sum(v.hi, h, s, e);
    v.hi = s;
    v.lo = v.lo + l + e;
  }
  float s, e;
  two_sum(v.hi, v.lo, s, e);
  v.hi = s;
  v.lo = e;
  return v;
}

// One 3D evaluation of each half's ROI (evaluate() of the one-ROI form).
__device__ __forceinline__ void evaluate_pair(const FitArgs& a, const WarpLayout& L, float* ws,
                                              int hl, int hb, unsigned hm, const float* th,
                                              bool FISHER, FPair& err_out, float& gl,
                                              float (&hr)[5]) {
  constexpr int NV = 5;
  constexpr int NH = NV * (NV + 1) / 2;
  constexpr int K = NV + NH;
  constexpr int KP = (K + 31) / 32 * 32;
  FPair ea{0.0f, 0.0f}, eb{0.0f, 0.0f};
  float aa[KP], ab[KP];
#pragma unroll
  for (int k = 0; k < KP; ++k) {
    aa[k] = 0.0f;
    ab[k] = 0.0f;
  }
  channel_pass<6, KP, false, 0, 16>(a, L, ws, ws, hl, th, false, FISHER, ea, aa, eb, ab, hm);
  float v[K];
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = aa[k] + ab[k];
  reduce_scatter<K, 8>(v, hl);
  constexpr HalfGatherCodes<NV, K> GC{};
  constexpr int SL = half_rs_slots(K);
  const float t0 = v[0];
  const float t1 = (SL > 1) ? v[1] : 0.0f;
  const int sh = 5 * (hl < NV ? hl : NV - 1);
  gl = half_gather<SL>(t0, t1, GC.grad, sh, hb);
#pragma unroll
  for (int k = 0; k < NV; ++k) hr[k] = half_gather<SL>(t0, t1, GC.row[k], sh, hb);
  err_out = half_sum_pair(ea, eb);
}

// initial_guess() of the one-ROI form for each half's ROI.
__device__ __forceinline__ void initial_guess_pair(const float* data, int s, int hl,
                                                   unsigned hm, float (&g)[4]) {
  const int s2 = s * s;
  FPair txa{0.f, 0.f}, tya{0.f, 0.f}, tsa{0.f, 0.f};
  FPair txb{0.f, 0.f}, tyb{0.f, 0.f}, tsb{0.f, 0.f};
  float mxa = 0.0f, mna = 10e10f, mxb = 0.0f, mnb = 10e10f;
  bool nan_seen = false;
  Stride2D ia(hl, s), ib(hl + 16, s);
  for (int p = hl; p < s2; p += 32, ia.next(), ib.next()) {
    {
      const float d = data[p];
      txa.add(d * (float)ia.c);
      tya.add(d * (float)ia.r);
      tsa.add(d);
      nan_seen |= (d != d);
      mxa = (mxa > d) ? mxa : d;
      mna = (mna < d) ? mna : d;
    }
    if (p + 16 < s2) {
      const float d = data[p + 16];
      txb.add(d * (float)ib.c);
      tyb.add(d * (float)ib.r);
      tsb.add(d);
      nan_seen |= (d != d);
      mxb = (mxb > d) ? mxb : d;
      mnb = (mnb < d) ? mnb : d;
    }
  }
  const FPair tx = half_sum_pair(txa, txb);
  const FPair ty = half_sum_pair(tya, tyb);
  const FPair ts = half_sum_pair(tsa, tsb);
  const float tsum = ts.hi + ts.lo;
  float mx = fmaxf(mxa, mxb), mn = fminf(mna, mnb);
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    mn = fminf(mn, __shfl_xor_sync(kFull, mn, o));
  }
  if ((__ballot_sync(kFull, nan_seen) & hm) != 0u) {
    // the reference's order-dependent max / min fold with NaN pixels
    mx = 0.0f;
    mn = 10e10f;
    for (int p0 = 0; p0 < s2; ++p0) {
      const float d = data[p0];
      mx = (mx > d) ? mx : d;
      mn = (mn < d) ? mn : d;
    }
  }
  const double n0 = ((double)mx - (double)mn) * 2.0 * (double)3.141592f * 1.5 * 1.5;
  g[0] = (tx.hi + tx.lo) / tsum;
  g[1] = (ty.hi + ty.lo) / tsum;
  g[2] = (float)((0.0 > n0) ? 0.0 : n0);
  g[3] = (mn > 0.01f) ? mn : 0.01f;
}

// lane_solve() with the broadcasts taken within the half.
__device__ __forceinline__ float lane_solve_half(int hl, int hb, const float (&lr)[5],
                                                 const float (&lc)[5], float invd, float b) {
  constexpr int NV = 5;
  float y = b;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const float yk = hbcast(y * invd, hb, k);
    if (hl == k) y = yk;
    else if (hl > k) y = fmaf(-lr[k], yk, y);
  }
  float x = y;
#pragma unroll
  for (int k = NV - 1; k >= 0; --k) {
    const float xk = hbcast(x * invd, hb, k);
    if (hl == k) x = xk;
    else if (hl < k) x = fmaf(-lc[k], xk, x);
  }
  return x;
}

// ROI source of one half: a shared work counter (dynamic claiming), or a fixed
// stride (first, first + step, ...).
struct PairClaim {
  unsigned long long* counter;  // null: fixed stride
  int64_t next, step;
  __device__ __forceinline__ int64_t take() {
    if (counter) return (int64_t)atomicAdd(counter, 1ull);
    const int64_t r = next;
    next += step;
    return r;
  }
};

// Fit every ROI the two halves claim, until both find none left. Each half
// stages its ROI's pixels at pix (its own) and keeps its LM state on its 16
// lanes; eval(par, fisher, err, gl, hr) evaluates both halves' ROIs at once
// (lane l of a half holds its ROI's parameter l and mode) and returns each
// half's deviance (or log-likelihood), gradient entry and Hessian (or Fisher)
// row on its lanes, as evaluate() does for one ROI. done: optional counter of
// finished ROIs (the batched form's).
template <class Eval>
__device__ __forceinline__ void fit_pair_loop(const FitArgs& a, int s, float* pix, int lane,
                                              PairClaim& claim, unsigned long long* done_ctr,
                                              Eval&& eval) {
  constexpr int MODE = 6;
  constexpr int NV = 5;
  constexpr int kNew = 0, kRun = 1, kOut = 2;
  const int hl = lane & 15;
  const int hb = lane & 16;
  const unsigned hm = hb ? 0xffff0000u : 0x0000ffffu;
  const int s2 = s * s;

  int st = kNew;
  int64_t roi = 0;
  float par = 0.0f, opar = 0.0f, sg = 0.0f, osg = 0.0f, cl = 1.0f, ocl = 1.0f, fd = 0.5f;
  float gl = 0.0f;
  float hr[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) hr[k] = 0.0f;
  float lambda = 1.0f, olambda = 1.0f;
  FPair err{1e12f, 0.0f}, oerr{1e13f, 0.0f}, ll{0.0f, 0.0f};
  int kk = 0;
  bool need_eval = false, fisher = false;

  for (;;) {
    // (1) halves without a ROI claim one, stage it and take its initial guess
    const bool want = (st == kNew);
    if (__any_sync(kFull, want)) {
      long long r = 0;
      if (want && hl == 0) r = (long long)claim.take();
      r = __shfl_sync(kFull, r, hb);
      bool ld = false;
      if (want) {
        roi = (int64_t)r;
        ld = roi < a.nfits;
        if (!ld) st = kOut;
      }
      if (ld) {
        const float* src = a.rois + roi * (int64_t)s2;
        for (int p = hl; p < s2; p += 16) pix[p] = __ldg(src + p);
      }
      __syncwarp();
      float g[4];
      initial_guess_pair(pix, s, hl, hm, g);
      if (ld) {
        // CPUmleFit_LM.cpp:2425-2450, 2477-2482: lane l keeps parameter l
        float v = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (hl == k) v = g[k];
        if (hl == 4) v = (float)a.m.n[2] / 2.0f;
        par = v;
        opar = par;
        sg = 0.0f;
        osg = 0.0f;
        clamp_fade<MODE>(hl, cl, fd);
        ocl = cl;
        lambda = 1.0f;
        olambda = 1.0f;
        err = FPair{1e12f, 0.0f};
        oerr = FPair{1e13f, 0.0f};
        kk = 0;
        need_eval = true;
        fisher = false;
        st = kRun;
      }
    }
    if (!__any_sync(kFull, st == kRun)) break;

    // (2) one evaluation of both halves; a half that needs none (a failed
    // solve, or no ROI) ignores its result
    {
      FPair e;
      float gn, hn[NV];
      eval(par, fisher, e, gn, hn);
      if (st == kRun && need_eval) {
        gl = gn;
#pragma unroll
        for (int k = 0; k < NV; ++k) hr[k] = hn[k];
        need_eval = false;
        if (fisher) ll = e;
        else err = e;
      }
    }

    // (3) halves whose Fisher pass just ran: CRLB, store, next ROI
    const bool fin = (st == kRun) && fisher && !need_eval;
    if (__any_sync(kFull, fin)) {
      // CRLB = diag(M^-1) from the Jacobi-scaled Fisher matrix (fit_roi)
      float crlb = 0.0f;
      {
        float mr[NV], dk[NV];
        float mydiag = 0.0f;
#pragma unroll
        for (int k = 0; k < NV; ++k)
          if (hl == k) mydiag = hr[k];
#pragma unroll
        for (int k = 0; k < NV; ++k) dk[k] = hbcast(mydiag, hb, k);
        const float sd = sqrtf(mydiag);
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const float den = sd * sqrtf(dk[k]);
          mr[k] = (hl == k) ? 1.0f : ((den > 0.0f) ? hr[k] / den : 0.0f);
        }
        float lr[NV], invd = 1.0f;
        bool okc = true;
#pragma unroll
        for (int j = 0; j < NV; ++j) lr[j] = 0.0f;
#pragma unroll
        for (int j = 0; j < NV; ++j) {
          const float ajj = hbcast(mr[j], hb, j);
          if (!(ajj > 0.0f)) okc = false;
          const float inv = rsqrtf(ajj);
          const float ljj = ajj * inv;
          const float lij = (hl > j) ? mr[j] * inv : ((hl == j) ? ljj : 0.0f);
          lr[j] = lij;
          if (hl == j) invd = inv;
#pragma unroll
          for (int k = j + 1; k < NV; ++k) {
            const float lkj = hbcast(lij, hb, k);
            if (hl > j && k <= hl) mr[k] = fmaf(-lij, lkj, mr[k]);
          }
        }
        float acc[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
          float part = 0.0f, z = 0.0f;
#pragma unroll
          for (int k = c; k < NV; ++k) {
            const float zk = hbcast(((k == c ? 1.0f : 0.0f) - part) * invd, hb, k);
            if (hl == k) z = zk;
            else if (hl > k) part = fmaf(lr[k], zk, part);
          }
          acc[c] = (hl >= c && hl < NV) ? z * z : 0.0f;
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
#pragma unroll
          for (int c = 0; c < NV; ++c) acc[c] += __shfl_xor_sync(kFull, acc[c], o);
        }
#pragma unroll
        for (int c = 0; c < NV; ++c)
          if (hl == c) crlb = okc ? acc[c] / dk[c] : __int_as_float(0x7fc00000);
#pragma unroll
        for (int c = 0; c < NV; ++c)
          if (hl == c && dk[c] == 0.0f) crlb = __int_as_float(0x7f800000);
      }
      float thv[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) thv[k] = hbcast(par, hb, k);
      if (fin) {
        const int64_t n = a.out_n;
        const int64_t o = a.out_offset + roi;
        if (hl == 0) {
#pragma unroll
          for (int i = 0; i < NV; ++i) a.P[i * n + o] = thv[i];
          a.P[NV * n + o] = (float)kk;
          a.LL[o] = ll.hi + ll.lo;
          if (done_ctr) atomicAdd(done_ctr, 1ull);
        }
        if (hl < NV) a.CRLB[hl * n + o] = crlb;
        st = kNew;
      }
    }

    // (4) the running halves' LM step (fit_roi), or the switch to the Fisher
    // pass at the iteration cap or on convergence
    bool step = false;
    if (st == kRun && !fisher && !need_eval) {
      if (kk >= a.iterations) {
        fisher = true;
        need_eval = true;
      } else {
        // |(newErr - oldErr) / newErr| < 1e-6 (CPUmleFit_LM.cpp:2565)
        const float dhi = err.hi - oerr.hi;
        const float dlo = err.lo - oerr.lo;
        const float rel = fabsf((dhi + dlo) / (err.hi + err.lo));
        if (rel < 1e-6f) {
          fisher = true;
          need_eval = true;
        } else {
          step = true;
        }
      }
    }
    if (__any_sync(kFull, step)) {
      if (step) {
        const float e_new = err.hi + err.lo, e_old = oerr.hi + oerr.lo;
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
#pragma unroll
        for (int k = 0; k < NV; ++k)
          if (hl == k) hr[k] *= lambda;
      }
      // Halves not stepping run the same instructions on values they do not
      // keep (their Hessian rows are re-evaluated or no longer needed).
      bool frz = false;
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (hl == k) frz = (hr[k] == 0.0f);
      const unsigned fmask = (__ballot_sync(kFull, frz && hl < NV) >> hb) & 0xffffu;
      float am[NV], ar[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        am[k] = ((fmask >> k) & 1u) ? 0.0f : hr[k];
        if (frz) am[k] = (k == hl) ? 1.0f : 0.0f;
        ar[k] = am[k];
      }
      const float rhs = frz ? 0.0f : gl;
      float lr[NV], lc[NV], invd = 1.0f;
      bool ok = true;
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        lr[j] = 0.0f;
        lc[j] = 0.0f;
      }
#pragma unroll
      for (int j = 0; j < NV; ++j) {
        const float ajj = hbcast(am[j], hb, j);
        // a negative pivot fails the solve (fit_roi stops the factorisation
        // there; the columns after it are not used)
        if (!(ajj >= 0.0f)) ok = false;
        const float inv = rsqrtf(ajj);
        const float ljj = ajj * inv;
        const float lij = (hl > j) ? am[j] * inv : ((hl == j) ? ljj : 0.0f);
        lr[j] = lij;
        if (hl == j) invd = inv;
#pragma unroll
        for (int k = j + 1; k < NV; ++k) {
          const float lkj = hbcast(lij, hb, k);
          if (hl == j) lc[k] = lkj;
          if (hl > j && k <= hl) am[k] = fmaf(-lij, lkj, am[k]);
        }
      }
      float upd = lane_solve_half(hl, hb, lr, lc, invd, rhs);
      if (!(a.flags & FLAG_NO_REFINE)) {
        float sh = rhs, sl = 0.0f;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
          const float xk = hbcast(upd, hb, k);
          float p_, pe_, t_, te_;
          two_prod(ar[k], xk, p_, pe_);
          two_sum(sh, -p_, t_, te_);
          sh = t_;
          sl += te_ - pe_;
        }
        upd += lane_solve_half(hl, hb, lr, lc, invd, sh + sl);
      }
      if (step) {
        if (ok) {
          osg = sg;
          ocl = cl;
          opar = par;
          olambda = lambda;
          oerr = err;
          if (sg != 0.0f) {
            if ((sg == 1.0f && upd < 0.0f) || (sg == -1.0f && upd > 0.0f)) cl = cl * fd;
          }
          sg = (upd > 0.0f) ? 1.0f : -1.0f;
          const float stp = upd / (1.0f + fabsf(upd / cl));
          par = par - stp;
          // bounds (CPUmleFit_LM.cpp:2626-2634)
          if (hl == 2) par = (par > 1.0f) ? par : 1.0f;
          if (hl == 3) par = (par > 0.01f) ? par : 0.01f;
          if (hl == 4) {
            par = (par > 0.0f) ? par : 0.0f;
            const float zmax = (float)(a.m.n[2] - 4);
            par = (par < zmax) ? par : zmax;
          }
          need_eval = true;
        } else {
          lambda = 10.0f * lambda;
        }
        ++kk;
      }
    }
  }
}

// The half-warp pair form: each half evaluates its own ROI in its own
// workspace with 16 lanes (evaluate_pair).
__device__ __forceinline__ void fit_pair(const FitArgs& a, const WarpLayout& L, float* ws,
                                         int lane, PairClaim& claim, unsigned long long* done_ctr) {
  const int hl = lane & 15;
  const int hb = lane & 16;
  const unsigned hm = hb ? 0xffff0000u : 0x0000ffffu;
  fit_pair_loop(a, L.s, ws, lane, claim, done_ctr,
                [&](float par, bool fisher, FPair& e, float& gn, float (&hn)[5]) {
                  float the[5];
#pragma unroll
                  for (int k = 0; k < 5; ++k) the[k] = hbcast(par, hb, k);
                  evaluate_pair(a, L, ws, hl, hb, hm, the, fisher, e, gn, hn);
                });
}

// Plain form: FitArgs as fit_kernel<6>; each warp holds two workspaces.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) fit_pair_kernel(FitArgs a) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const WarpLayout L = make_layout(6, a.s);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int half = lane >> 4;
  float* ws = smem + (wib * 2 + half) * L.total();
  PairClaim c;
  c.counter = a.claim;
  c.next = ((int64_t)blockIdx.x * wpb + wib) * 2 + half;
  c.step = (int64_t)gridDim.x * wpb * 2;
  fit_pair(a, L, ws, lane, c, nullptr);
}

// Batched form: BatchArgs as batch_kernel<6>. Both halves work in the same
// segment and move to the next one together once neither finds a ROI left.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) batch_pair_kernel(const __grid_constant__ BatchArgs a) {
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int half = lane >> 4;
  float* ws = smem + (wib * 2 + half) * make_layout(6, a.s_max).total();
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
    fit_pair(fa, make_layout(6, g.s), ws, lane, c, &a.done[g.slot]);
  }
}

}  // namespace bsfit
