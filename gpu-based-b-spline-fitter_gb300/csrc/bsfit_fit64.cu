// FP64 reference-precision fitter for fit types 6, 7 and 8.
//
// The FP32 kernels (bsfit_fit.cu) contract the spline separably and reorder
// every sum; the reference's LM then takes some discrete decisions (the 1e-6
// relative-deviance stop, update-sign clamp halving, accept / reject, the 4D
// "let it go" switch) differently from the reference run in double, as the
// reference's own float build does. This kernel instead computes what the
// reference computes with float promoted to double, in the reference's order
// of operations, so that its results follow the double-precision trajectory:
//   - per pixel, the 4^D-term tensor-product sums of VC/CPUmleFit_LM/
//     CPUsplineLib.cpp:1199-1288 (3D), :761-970 (4D), :43-475 (5D), with the
//     weights of :1129-1197 / :972-1126 / :477-758 and the basis of
//     :1289-1326 (float literals kept as float values), the two 5D index
//     quirks included (:313 and :420-421);
//   - the deviance, gradient and Hessian sums in pixel order (ii outer, jj
//     inner), VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2537-2560;
//   - the LM control, unpivoted Cholesky and substitution
//     (CPUsplineLib.cpp:1363-1419), bounds and clamps of
//     CPUmleFit_LM.cpp:2411-2760 (type 6), :2763-3158 (type 7), :3163-3620
//     (type 8); the Fisher sums and the LU inverse of MatInvLib.h:17-77.
// The file is compiled without floating-point contraction (-fmad=false), as
// the double build it follows. The only other source of difference is the
// last bit of log().
//
// Layout: one warp per ROI. Lanes evaluate pixels 32 at a time and publish
// each pixel's terms in a shared row (its deviance term, t1 * dudt[l], and
// (t2 * dudt[l]) * dudt[m], the products the reference adds); the sums are
// owned one or two entries per lane and accumulated over the rows in pixel
// order, so every sum has the reference's order. Lane 0 runs the LM control
// and the small dense solves on shared state. Coefficients are a double copy
// of the model's table followed by one table per axis of the neighbour
// differences (-c[i]) + c[i + stride] the derivative terms use (computed once
// per model, the same double operation). Throughput is bounded by the FP64
// pipe; this is the parity mode, the FP32 kernels are the production path.
#include <climits>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "bsfit_internal.h"

namespace bsfit {
namespace {

template <int MODE>
struct F64Traits;
template <>
struct F64Traits<6> {
  static constexpr int D = 3, NV = 5, WPB = 4, NCH = 1;
};
template <>
struct F64Traits<7> {
  static constexpr int D = 4, NV = 6, WPB = 1, NCH = 1;
};
template <>
struct F64Traits<8> {
  static constexpr int D = 5, NV = 8, WPB = 1, NCH = 1;
};
// 4Pi (the restatement in the oracle, oracle/bsfit_oracle.cpp fit_4pi_roi):
// four channels of the 4D model at theta + dT[c], phase shifted by the
// channel's shift and wrapped, summed into one likelihood.
template <>
struct F64Traits<kFit4Pi> {
  static constexpr int D = 4, NV = 6, WPB = 1, NCH = k4PiChannels;
};

// Float literals of the reference (VC/CPUmleFit_LM/definitions.h:15, :23-24).
constexpr float kPIf = 3.141592f;
constexpr float kTOLf = 1e-6f;
constexpr float kTOL1f = 1e-5f;

// LM state of one warp, written by lane 0 only (the owners of the sums write
// err / jac / hes / M / div between two warp barriers).
struct LMState {
  double nt[8], ot[8], ns[8], os[8], nc[8], oc[8], fade[8], upd[8], jac[8], diag[8];
  double hes[64], U[64], M[64], Minv[64];
  double newErr, oldErr, newLambda, oldLambda, sumUpdate, div;
  double frame[8];  // yc, xc, off, zc, wc, uc, g2 of the last preparation
  int turn, action, pad[2];
};
static_assert(sizeof(LMState) % 16 == 0, "LMState keeps the tables 16-byte aligned");
constexpr int kLMDoubles = (int)(sizeof(LMState) / sizeof(double));

template <int MODE>
struct F64Layout {
  using TR = F64Traits<MODE>;
  static constexpr int D = TR::D, NV = TR::NV;
  static constexpr int B = 1 << D, BB = B * B;
  static constexpr int WT = (D + 1) * BB;             // wf, then wd[0..D-1]
  static constexpr int WT3 = (MODE == 8) ? 4 * 64 : 0;  // fit type 8: the 3D tables
  static constexpr int AX = 40;                       // 1-D weights, 4 kinds x 5 axes x 2
  static constexpr int NE = 1 + NV + NV * (NV + 1) / 2;  // sums: deviance, gradient, Hessian
  static constexpr int RW = NE;                       // row: one term per sum
  static constexpr int ROWS = 32 * RW;
  static constexpr int off_wt = kLMDoubles;
  static constexpr int off_wt3 = off_wt + WT;
  static constexpr int off_ax = off_wt3 + WT3;
  static constexpr int off_rows = off_ax + AX;
  static constexpr int per_warp = off_rows + ROWS + (ROWS & 1);
};

// Phase position wrapped into [1, 1 + P), P = nw - 1, by one period.
__device__ __forceinline__ double wrap_phase64(double w, int nw) {
  const double P = (double)(nw - 1);
  if (w < 1.0) return w + P;
  if (w >= (double)nw) return w - P;
  return w;
}

__device__ __forceinline__ int floor_to_int64(double v) {
  const double f = floor(v);
  if (!(f >= -2147483648.0 && f < 2147483648.0)) return INT_MIN;
  return (int)f;
}

// Cardinal cubic and quadratic B-splines with the reference's float literals
// (CPUsplineLib.cpp:1289-1326), evaluated in double.
__device__ __forceinline__ double bspline3(double x) {
  constexpr float c43 = 4.0f / 3.0f, c16 = 1.0f / 6.0f, c23 = 2.0f / 3.0f;
  const double x2 = x * x, x3 = x2 * x;
  if (x >= 1.0 && x < 2.0) return (((double)c43 - 2.0 * x) + x2) - (double)c16 * x3;
  if (x >= 0.0 && x < 1.0) return ((double)c23 - x2) + 0.5 * x3;
  if (x >= -1.0 && x < 0.0) return ((double)c23 - x2) - 0.5 * x3;
  if (x >= -2.0 && x < -1.0) return (((double)c43 + 2.0 * x) + x2) + (double)c16 * x3;
  return 0.0;
}

__device__ __forceinline__ double bspline2(double x) {
  const double x2 = x * x;
  if (x >= 0.5 && x < 1.5) return (1.125 - 1.5 * x) + 0.5 * x2;
  if (x >= -0.5 && x < 0.5) return 0.75 - x2;
  if (x >= -1.5 && x < -0.5) return (1.125 + 1.5 * x) + 0.5 * x2;
  return 0.0;
}

// A model table: values c[0, total) followed by D difference tables,
// diff(d, i) = (-c[i]) + c[i + stride_d] (0 for a neighbour past the end: only
// the +1 neighbour of a position exactly on the last knot, whose weight is 0).
struct Coef {
  const double* c;
  int64_t total;
  __device__ __forceinline__ double val(int64_t i) const { return __ldg(c + i); }
  __device__ __forceinline__ double diff(int d, int64_t i) const {
    return __ldg(c + (int64_t)(d + 1) * total + i);
  }
};

// The 1-D weights of one axis (CPUsplineLib.cpp:1129-1197): kind 0 = B3(t+v-1),
// 1 = B3(t-v), 2 = B2(t-1+v-1/2), 3 = B2(t-1-v+1/2), v = 1, 2; stored at
// ax[(kind * 5 + axis) * 2 + v - 1].
__device__ __forceinline__ double axis_weight(double frac, int kind, int v) {
  const double dfrac = frac - 1.0;
  switch (kind) {
    case 0: return bspline3((frac + (double)v) - 1.0);
    case 1: return bspline3(frac - (double)v);
    case 2: return bspline2((dfrac + (double)v) - 0.5);
    default: return bspline2((dfrac - (double)v) + 0.5);
  }
}

// Tensor-product tables of D axes from ax[]: entry B*n + b, n the loop index
// (axis a at v = bit a of n, plus 1), b the side bits; the products run over
// the axes left to right.
template <int D>
__device__ __forceinline__ void build_tables(const double* ax, double* W, int lane) {
  constexpr int B = 1 << D, BB = B * B;
  for (int e = lane; e < BB; e += 32) {
    const int n = e >> D, b = e & (B - 1);
    double val[D], der[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const int v = (n >> a) & 1;
      const bool side2 = (b >> a) & 1;
      val[a] = ax[((side2 ? 1 : 0) * 5 + a) * 2 + v];
      der[a] = ax[((side2 ? 3 : 2) * 5 + a) * 2 + v];
    }
    double p = val[0];
#pragma unroll
    for (int a = 1; a < D; ++a) p = p * val[a];
    W[e] = p;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double q = (d == 0) ? der[0] : val[0];
#pragma unroll
      for (int a = 1; a < D; ++a) q = q * (a == d ? der[a] : val[a]);
      W[(1 + d) * BB + e] = q;
    }
  }
}

// Model value and derivatives at one pixel (CPUsplineLib.cpp:1199-1288 and
// the 4D / 5D copies). pos[a]: the pixel's position along axis a (Y, X, Z, W,
// U). Q5 adds the 5D model's two index quirks.
template <int D, bool Q5>
__device__ __forceinline__ void pixel_model(const Coef& c, const int* n, const int64_t* st,
                                            const double* pos, const double* W, double N, double bg,
                                            double* dudt, double* model) {
  constexpr int B = 1 << D, BB = B * B;
  int k[D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    int kc = floor_to_int64(pos[a]);
    kc = (kc > 1) ? kc : 1;
    kc = (kc < n[a] - 1) ? kc : n[a] - 1;
    if (pos[a] == (double)n[a]) kc = n[a];
    k[a] = kc + 1;
  }
  double f = 0.0;
  double dacc[D];
#pragma unroll
  for (int a = 0; a < D; ++a) dacc[a] = 0.0;
#pragma unroll 1
  for (int ni = 0; ni < B; ++ni) {
    int64_t lo[D], hi[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      const int lv = ((ni >> a) & 1) + 1;
      lo[a] = (int64_t)(k[a] - lv) * st[a];
      hi[a] = (int64_t)(k[a] + lv - 1) * st[a];
    }
    const double* wf = W + B * ni;
    double s = 0.0, sd[D];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      int64_t node = 0;
#pragma unroll
      for (int a = 0; a < D; ++a) node += ((b >> a) & 1) ? hi[a] : lo[a];
      const double t = c.val(node) * wf[b];
      s = (b == 0) ? t : s + t;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        double w = W[(1 + d) * BB + B * ni + b];
        int64_t nd = node;
        if constexpr (Q5) {
          if (d == 2 && b == 27) {
            // CPUsplineLib.cpp:313 reads delta_dfz[32 * nIndex + 271]; past
            // the end of that array it reads the next one of the frame, the
            // W-derivative weights, which follow the Z table here as well.
            w = W[3 * BB + B * ni + 271];
          }
          if (d == 4 && b == 16) {
            // CPUsplineLib.cpp:420-421: the side-1 U node is differenced.
            nd = node - hi[4] + lo[4];
          }
        }
        const double term = c.diff(d, nd) * w;  // (-c[nd] + c[nd + stride]) * w
        sd[d] = (b == 0) ? term : sd[d] + term;
      }
    }
    f = f + s;
#pragma unroll
    for (int d = 0; d < D; ++d) dacc[d] = dacc[d] + sd[d];
  }
  dudt[0] = -N * dacc[1];
  dudt[1] = -N * dacc[0];
#pragma unroll
  for (int a = 2; a < D; ++a) dudt[a + 2] = N * dacc[a];
  dudt[2] = f;
  dudt[3] = 1.0;
  *model = bg + N * f;
}

struct Fit64Ctx {
  const Fit64Args* a;
  Coef c, c3;
  const float* data;  // channel 0's pixels; channel c at data + c * nfits * s * s
  const float* var;
  const float* dT;    // 4Pi: this ROI's [4][6] channel offsets
  int s, lane;
};

template <int MODE>
struct Warp64 {
  using L = F64Layout<MODE>;
  static constexpr int D = L::D, NV = L::NV, RW = L::RW;
  LMState& st;
  double* wt;
  double* wt3;
  double* ax;
  double* rows;
  // Sum entries owned by this lane (entry t = lane + 32 h, also its index in a
  // row): kind 0 = deviance / log-likelihood, 1 = gradient l, 2 = Hessian /
  // Fisher (l, m), m >= l; -1 = none.
  int kind[2], el[2], em[2];

  __device__ Warp64(double* base, int lane)
      : st(*reinterpret_cast<LMState*>(base)),
        wt(base + L::off_wt),
        wt3(base + L::off_wt3),
        ax(base + L::off_ax),
        rows(base + L::off_rows) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int t = lane + 32 * h;
      kind[h] = -1;
      el[h] = em[h] = 0;
      if (t == 0) {
        kind[h] = 0;
      } else if (t <= NV) {
        kind[h] = 1;
        el[h] = t - 1;
      } else {
        int p = t - 1 - NV;
        for (int l = 0; l < NV; ++l) {
          if (p < NV - l) {
            kind[h] = 2;
            el[h] = l;
            em[h] = l + p;
            break;
          }
          p -= NV - l;
        }
      }
    }
  }

  // Frame and weight tables at theta (the models' prepare(),
  // CPUmleFit_LM.cpp:2512-2523 and the 4D / 5D copies).
  __device__ void prepare(const Fit64Ctx& cx, const double* th) {
    const int lane = cx.lane;
    const double half = (double)((cx.s + 1) / 2);
    const double xc = half - th[0], yc = half - th[1];
    const double zc = th[4];
    const double wc = (D >= 4) ? th[5] : 0.0;
    const double uc = (D >= 5) ? th[6] : 0.0;
    double fr[5] = {yc - floor(yc), xc - floor(xc), zc - floor(zc), wc - floor(wc), uc - floor(uc)};
    for (int t = lane; t < 8 * D; t += 32) {
      const int kind = t / (2 * D), r = t - kind * 2 * D, axis = r >> 1, v = (r & 1) + 1;
      double f = fr[0];
#pragma unroll
      for (int q = 1; q < 5; ++q)
        if (axis == q) f = fr[q];
      ax[(kind * 5 + axis) * 2 + v - 1] = axis_weight(f, kind, v);
    }
    if (lane == 0) {
      st.frame[0] = yc;
      st.frame[1] = xc;
      st.frame[3] = zc;
      st.frame[4] = wc;
      st.frame[5] = uc;
      st.frame[6] = (MODE == 8) ? th[7] : 0.0;
    }
    __syncwarp();
    build_tables<D>(ax, wt, lane);
    if constexpr (MODE == 8) build_tables<3>(ax, wt3, lane);
    __syncwarp();
  }

  // Value and derivative vector of pixel (ii, jj) with the prepared frame.
  __device__ void pixel(const Fit64Ctx& cx, int ii, int jj, double N, double bg, double* dudt,
                        double* model) const {
    const ModelDev& m = cx.a->m;
    double pos[5];
    pos[0] = (st.frame[0] + (double)ii) + st.frame[2];
    pos[1] = (st.frame[1] + (double)jj) + st.frame[2];
    pos[2] = st.frame[3];
    pos[3] = st.frame[4];
    pos[4] = st.frame[5];
    if constexpr (MODE == 8) {
      // Mixture (1 - g2) S3D + g2 S5D (CPUmleFit_LM.cpp:3280-3300).
      const double g2 = st.frame[6];
      double d3[5], m5, m3;
      pixel_model<5, true>(cx.c, m.n, m.st, pos, wt, N, bg, dudt, &m5);
      pixel_model<3, false>(cx.c3, m.n, m.st, pos, wt3, N, bg, d3, &m3);
#pragma unroll
      for (int l = 0; l < 5; ++l) dudt[l] = dudt[l] * g2 + (1.0 - g2) * d3[l];
      *model = m3 * (1.0 - g2) + m5 * g2;
      dudt[NV - 1] = m5 - m3;
    } else {
      pixel_model<D, false>(cx.c, m.n, m.st, pos, wt, N, bg, dudt, model);
    }
  }

  // The pixels of one plane, in the reference's order (ii outer, jj inner), 32
  // at a time: each lane publishes its pixel's terms in a row (the deviance
  // term, t1 * dudt[l] and (t2 * dudt[l]) * dudt[m]; or the log-likelihood term,
  // its use flag and (dudt[m] * dudt[l]) / model), then every owner adds its
  // entry of the rows in pixel order to acc.
  template <bool FISHER>
  __device__ void accumulate_plane(const Fit64Ctx& cx, const float* data, double N, double bg,
                                   bool dup45, double (&acc)[2]) {
    const int s = cx.s, s2 = s * s, lane = cx.lane;
    for (int r0 = 0; r0 < s2; r0 += 32) {
      const int q = r0 + lane;
      if (q < s2) {
        const int ii = q / s, jj = q - ii * s;
        double dudt[NV], model;
        pixel(cx, ii, jj, N, bg, dudt, &model);
        const int di = s * jj + ii;
        double dval = (double)data[di];
        if (cx.var) {
          const double v = (double)cx.var[di];
          model += v;
          dval += v;
        }
        double* row = rows + lane * RW;
        int k = 1 + NV;
        if constexpr (FISHER) {
          // CPUmleFit_LM.cpp:2730-2742
          double term = 0.0, use = 0.0;
          if (model > 0) {
            use = 1.0;
            term = (dval > 0) ? ((dval * log(model) - model) - dval * log(dval)) + dval : -model;
          }
          row[0] = term;
          row[1] = use;
#pragma unroll
          for (int l = 0; l < NV; ++l)
#pragma unroll
            for (int mm = l; mm < NV; ++mm, ++k) row[k] = (dudt[mm] * dudt[l]) / model;
        } else {
          // CPUmleFit_LM.cpp:2537-2560
          if (dup45) dudt[5] = dudt[4];
          double term;
          if (dval > 0) {
            term = 2.0 * ((model - dval) - dval * log(model / dval));
          } else {
            term = 2.0 * model;
            dval = 0.0;
          }
          const double t1 = 1.0 - dval / model;
          const double t2 = dval / (model * model);
          row[0] = term;
#pragma unroll
          for (int l = 0; l < NV; ++l) row[1 + l] = t1 * dudt[l];
#pragma unroll
          for (int l = 0; l < NV; ++l) {
            const double tl = t2 * dudt[l];
#pragma unroll
            for (int mm = l; mm < NV; ++mm, ++k) row[k] = tl * dudt[mm];
          }
        }
      }
      __syncwarp();
      const int cnt = (s2 - r0 < 32) ? s2 - r0 : 32;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int kd = kind[h];
        if (kd < 0 || (FISHER && kd == 1)) continue;
        const int e = lane + 32 * h;
        double a = acc[h];
        if (FISHER && kd == 0) {
          for (int j = 0; j < cnt; ++j)
            if (rows[j * RW + 1] != 0.0) a = a + rows[j * RW];
        } else {
          for (int j = 0; j < cnt; ++j) a = a + rows[j * RW + e];
        }
        acc[h] = a;
      }
      __syncwarp();
    }
  }

  // One pass over the ROI. FISHER = false: deviance, gradient and Hessian at
  // st.nt (CPUmleFit_LM.cpp:2530-2560) with the frame the caller prepared;
  // dup45 copies dudt[4] into dudt[5] (fit type 7's initial pass). FISHER =
  // true: Fisher matrix and log-likelihood at st.nt with the current frame
  // (:2714-2742). 4Pi: every channel at theta + dT[c], its phase shifted by the
  // channel's shift and wrapped, prepared here (Model4Pi of the restatement),
  // channel outer and pixel inner into the same sums.
  template <bool FISHER>
  __device__ void pass(const Fit64Ctx& cx, bool dup45) {
    constexpr int NCH = F64Traits<MODE>::NCH;
    double acc[2] = {0.0, 0.0};
    if constexpr (NCH == 1) {
      accumulate_plane<FISHER>(cx, cx.data, st.nt[2], st.nt[3], dup45, acc);
    } else {
      const int64_t plane = (int64_t)cx.a->nfits * cx.s * cx.s;
#pragma unroll 1
      for (int ch = 0; ch < NCH; ++ch) {
        double tc[NV];
#pragma unroll
        for (int t = 0; t < NV; ++t) tc[t] = st.nt[t] + (double)cx.dT[ch * NV + t];
        tc[5] = wrap_phase64(tc[5] + (double)cx.a->m.shift[ch], cx.a->m.n[3]);
        prepare(cx, tc);
        accumulate_plane<FISHER>(cx, cx.data + ch * plane, tc[2], tc[3], dup45, acc);
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int kd = kind[h], l = el[h], mm = em[h];
      if (kd == 0) {
        if (FISHER) st.div = acc[h];
        else st.newErr = acc[h];
      } else if (kd == 1) {
        if (!FISHER) st.jac[l] = acc[h];
      } else if (kd == 2) {
        double* Mx = FISHER ? st.M : st.hes;
        Mx[l * NV + mm] = acc[h];
        Mx[mm * NV + l] = acc[h];
      }
    }
    __syncwarp();
  }
};

// Unpivoted Cholesky (CPUsplineLib.cpp:1363-1390), lower factor in U[i*n+j],
// j <= i; the off-diagonal update multiplies by the reciprocal, as written.
template <int NV>
__device__ int cholesky64(const double* A, double* U) {
  for (int i = 0; i < NV; i++)
    for (int j = 0; j <= i; j++) {
      double s = 0.0;
      for (int k = 0; k < j; k++) s = s + U[i * NV + k] * U[j * NV + k];
      if (i == j) {
        if (A[i * NV + i] - s >= 0) U[i * NV + i] = sqrt(A[i * NV + i] - s);
        else return 1;
      } else {
        U[i * NV + j] = (1.0 / U[j * NV + j]) * (A[i * NV + j] - s);
      }
    }
  return 0;
}

// Forward and backward substitution (CPUsplineLib.cpp:1392-1419).
template <int NV>
__device__ void substitute64(const double* U, const double* b, double* x) {
  double y[NV];
  for (int i = 0; i < NV; i++) {
    y[i] = b[i];
    for (int j = 0; j < i; j++) y[i] = y[i] - U[i * NV + j] * y[j];
    y[i] = y[i] / U[i * NV + i];
  }
  for (int i = NV - 1; i >= 0; i--) {
    x[i] = y[i];
    for (int j = i + 1; j < NV; j++) x[i] = x[i] - U[j * NV + i] * x[j];
    x[i] = x[i] / U[i * NV + i];
  }
}

// LU inverse returning the diagonal (MatInvLib.h:17-77), column-major.
template <int SZ>
__device__ void mat_inv64(double* M, double* Minv, double* diag) {
  double tmp1 = 0.0;
  double yy[SZ];
  for (int jj = 0; jj < SZ; jj++) {
    for (int ii = 0; ii <= jj; ii++)
      if (ii > 0) {
        for (int kk = 0; kk <= ii - 1; kk++) tmp1 = tmp1 + M[ii + kk * SZ] * M[kk + jj * SZ];
        M[ii + jj * SZ] = M[ii + jj * SZ] - tmp1;
        tmp1 = 0.0;
      }
    for (int ii = jj + 1; ii < SZ; ii++)
      if (jj > 0) {
        for (int kk = 0; kk <= jj - 1; kk++) tmp1 = tmp1 + M[ii + kk * SZ] * M[kk + jj * SZ];
        M[ii + jj * SZ] = (1.0 / M[jj + jj * SZ]) * (M[ii + jj * SZ] - tmp1);
        tmp1 = 0.0;
      } else {
        M[ii + jj * SZ] = (1.0 / M[jj + jj * SZ]) * M[ii + jj * SZ];
      }
  }
  tmp1 = 0.0;
  for (int num = 0; num < SZ; num++) {
    yy[0] = (num == 0) ? 1.0 : 0.0;
    for (int ii = 1; ii < SZ; ii++) {
      const double b = (ii == num) ? 1.0 : 0.0;
      for (int jj = 0; jj <= ii - 1; jj++) tmp1 = tmp1 + M[ii + jj * SZ] * yy[jj];
      yy[ii] = b - tmp1;
      tmp1 = 0.0;
    }
    Minv[SZ - 1 + num * SZ] = yy[SZ - 1] / M[(SZ - 1) + (SZ - 1) * SZ];
    for (int ii = SZ - 2; ii >= 0; ii--) {
      for (int jj = ii + 1; jj < SZ; jj++) tmp1 = tmp1 + M[ii + jj * SZ] * Minv[jj + num * SZ];
      Minv[ii + num * SZ] = (1.0 / M[ii + ii * SZ]) * (yy[ii] - tmp1);
      tmp1 = 0.0;
    }
  }
  for (int ii = 0; ii < SZ; ii++) diag[ii] = Minv[ii * SZ + ii];
}

// Initial guesses (CPUgaussLib.cpp:172-225, CPUmleFit_LM.cpp:2478-2482,
// :2839-2850, :3237-3256), lane 0.
// The single-channel rule on one plane: x, y, N, bg into t[0..3].
__device__ void guess_plane(const float* d, int s, double* t) {
  double tx = 0.0, ty = 0.0, ts = 0.0;
  for (int ii = 0; ii < s; ii++)
    for (int jj = 0; jj < s; jj++) {
      const double v = (double)d[s * jj + ii];
      tx = tx + v * (double)ii;
      ty = ty + v * (double)jj;
      ts = ts + v;
    }
  t[0] = tx / ts;
  t[1] = ty / ts;
  double maxn = 0.0, minbg = (double)10e10f;
  for (int kk = 0; kk < s; kk++)
    for (int ll = 0; ll < s; ll++) {
      const double v = (double)d[kk * s + ll];
      maxn = (maxn > v) ? maxn : v;
      minbg = (minbg < v) ? minbg : v;
    }
  const double n0 = ((((maxn - minbg) * 2.0) * (double)kPIf) * 1.5) * 1.5;
  t[2] = (0.0 > n0) ? 0.0 : n0;
  t[3] = (minbg > 0.01) ? minbg : 0.01;
}

template <int MODE>
__device__ void initial_theta(const Fit64Ctx& cx, LMState& st, int64_t roi) {
  constexpr int NV = F64Traits<MODE>::NV;
  const int s = cx.s;
  if constexpr (MODE == kFit4Pi) {
    // mean over the channels of the single-channel rule, lateral offsets
    // removed; z and phase per ROI (fit_4pi_roi of the restatement)
    double sx = 0.0, sy = 0.0, sn = 0.0, sb = 0.0;
    for (int c = 0; c < k4PiChannels; ++c) {
      double t4[4];
      guess_plane(cx.data + (int64_t)c * cx.a->nfits * s * s, s, t4);
      sx = sx + (t4[0] - (double)cx.dT[c * NV + 0]);
      sy = sy + (t4[1] - (double)cx.dT[c * NV + 1]);
      sn = sn + t4[2];
      sb = sb + t4[3];
    }
    st.nt[0] = sx / 4.0;
    st.nt[1] = sy / 4.0;
    st.nt[2] = sn / 4.0;
    st.nt[3] = sb / 4.0;
    st.nt[4] = (double)cx.a->z0[roi];
    st.nt[5] = wrap_phase64((double)cx.a->w0[roi], cx.a->m.n[3]);
    return;
  }
  const float* d = cx.data;
  double tx = 0.0, ty = 0.0, ts = 0.0;
  for (int ii = 0; ii < s; ii++)
    for (int jj = 0; jj < s; jj++) {
      const double v = (double)d[s * jj + ii];
      tx = tx + v * (double)ii;
      ty = ty + v * (double)jj;
      ts = ts + v;
    }
  st.nt[0] = tx / ts;
  st.nt[1] = ty / ts;
  double maxn = 0.0, minbg = (double)10e10f;
  for (int kk = 0; kk < s; kk++)
    for (int ll = 0; ll < s; ll++) {
      const double v = (double)d[kk * s + ll];
      maxn = (maxn > v) ? maxn : v;
      minbg = (minbg < v) ? minbg : v;
    }
  const double n0 = ((((maxn - minbg) * 2.0) * (double)kPIf) * 1.5) * 1.5;
  st.nt[2] = (0.0 > n0) ? 0.0 : n0;
  st.nt[3] = (minbg > 0.01) ? minbg : 0.01;
  const ModelDev& m = cx.a->m;
  if (MODE == 6) {
    st.nt[4] = (double)m.n[2] / 2.0;
  } else if (MODE == 7) {
    const bool use = m.init_p_len >= 2 && m.init_p[0] != 0.0f;
    st.nt[4] = use ? (double)m.init_p[0] : (double)m.n[2] / 2.0;
    st.nt[5] = use ? (double)m.init_p[1] : (double)m.n[3] / 2.0;
  } else {
    for (int i = 4; i < NV; i++) st.nt[i] = (double)m.init_p[i - 4];
  }
}

__device__ __forceinline__ double dmax(double a, double b) { return (a > b) ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return (a < b) ? a : b; }

enum { kStop = 0, kEval = 1, kNoEval = 2 };

// One LM iteration up to the evaluation (CPUmleFit_LM.cpp:2569-2640 and the
// type 7 / 8 copies), lane 0. Returns kStop on convergence, kEval with the new
// theta in st.nt, or kNoEval after a failed factorization.
template <int MODE>
__device__ int lm_control(LMState& st, const ModelDev& m, int s) {
  constexpr int NV = F64Traits<MODE>::NV;
  bool conv = fabs((st.newErr - st.oldErr) / st.newErr) < (double)kTOLf;
  if (MODE == 8) conv = conv || (st.sumUpdate < (double)kTOL1f);
  if (conv) return kStop;
  if (st.newErr > 1.5 * st.oldErr) {
    for (int i = 0; i < NV; i++) {
      st.ns[i] = st.os[i];
      st.nc[i] = st.oc[i];
      st.nt[i] = st.ot[i];
    }
    st.newLambda = st.oldLambda;
    st.newErr = st.oldErr;
    st.newLambda = 10.0 * st.newLambda;
  } else if (st.newErr < st.oldErr) {
    if (st.newLambda > 1) st.newLambda = st.newLambda * 0.8;
    else if (st.newLambda < 1) st.newLambda = 1.0;
  }
  for (int i = 0; i < NV; i++) st.hes[i * NV + i] = st.hes[i * NV + i] * st.newLambda;
  int info = cholesky64<NV>(st.hes, st.U);
  if (info == 0) {
    substitute64<NV>(st.U, st.jac, st.upd);
    if (MODE != 6) {
      // CPUmleFit_LM.cpp:2943-2950 / :3383-3390
      for (int l = 0; l < NV; l++)
        if (isnan(st.upd[l])) info = 1;
    }
  }
  if (info != 0) {
    st.newLambda = 10.0 * st.newLambda;
    return kNoEval;
  }
  if (MODE == 7) st.upd[5] = st.upd[5] * 10.0;  // :2951
  for (int i = 0; i < NV; i++) {
    st.os[i] = st.ns[i];
    st.oc[i] = st.nc[i];
    st.ot[i] = st.nt[i];
  }
  st.oldLambda = st.newLambda;
  st.oldErr = st.newErr;
  if (MODE == 7) {
    // "let it go", :2966-2971
    if (fabs(st.upd[4]) < 0.005 && st.turn) {
      st.nc[5] = (double)m.n[3] / 10.0;
      st.oc[5] = st.nc[5];
      st.turn = 0;
      st.nc[4] = 2.0;
      st.oc[4] = 2.0;
    }
  }
  if (MODE == 8) st.sumUpdate = 0.0;
  for (int ll = 0; ll < NV; ll++) {
    const double u = st.upd[ll];
    if (st.ns[ll] != 0) {
      const bool flip = (st.ns[ll] == 1 && u < 0) || (st.ns[ll] == -1 && u > 0);
      if (flip) st.nc[ll] = (MODE == 6) ? st.nc[ll] * 0.5 : st.nc[ll] * st.fade[ll];
    }
    st.ns[ll] = (u > 0) ? 1.0 : -1.0;
    if (MODE == 8) {
      const double v = u / (1.0 + fabs(u / st.nc[ll]));
      st.upd[ll] = v;
      st.nt[ll] = st.nt[ll] - v;
      st.sumUpdate = st.sumUpdate + fabs(v);
    } else {
      st.nt[ll] = st.nt[ll] - u / (1.0 + fabs(u / st.nc[ll]));
    }
  }
  if (MODE == 8) {
    // :3421-3445
    const double lo = ((double)s - 1.0) / 2.0 - (double)s / 4.0;
    const double hi = ((double)s - 1.0) / 2.0 + (double)s / 4.0;
    st.nt[0] = dmin(dmax(st.nt[0], lo), hi);
    st.nt[1] = dmin(dmax(st.nt[1], lo), hi);
  }
  st.nt[2] = dmax(st.nt[2], 1.0);
  st.nt[3] = dmax(st.nt[3], 0.01);
  st.nt[4] = dmax(st.nt[4], 0.0);
  if (MODE == 6) st.nt[4] = dmin(st.nt[4], (double)(m.n[2] - 4));
  else st.nt[4] = dmin(st.nt[4], (double)m.n[2] - 0.5);
  if (MODE == 7) {
    st.nt[5] = dmax(st.nt[5], 0.0);
    st.nt[5] = dmin(st.nt[5], (double)m.n[3] - 0.5);
  }
  if (MODE == kFit4Pi) st.nt[5] = wrap_phase64(st.nt[5], m.n[3]);
  if (MODE == 8) {
    if (st.nt[5] <= 1) st.nt[5] = (double)(m.n[3] - 2) + st.nt[5];
    else if (st.nt[5] > (double)(m.n[3] - 1)) st.nt[5] = (2.0 + st.nt[5]) - (double)m.n[3];
    st.nt[6] = dmax(st.nt[6], 1.0);
    st.nt[6] = dmin(st.nt[6], (double)m.n[4] - 0.5);
    st.nt[7] = dmin(st.nt[7], 1.0);
    st.nt[7] = dmax(st.nt[7], 0.0);
  }
  return kEval;
}

template <int MODE>
__device__ void init_state(LMState& st) {
  constexpr int NV = F64Traits<MODE>::NV;
  st.newLambda = st.oldLambda = 1.0;
  st.sumUpdate = 1e10;
  st.turn = 1;
  st.newErr = 1e12;
  st.oldErr = 1e13;
  for (int i = 0; i < 8; i++) {
    st.ns[i] = st.os[i] = 0.0;
    st.upd[i] = 0.0;
    st.jac[i] = 0.0;
  }
  for (int i = 0; i < 64; i++) st.hes[i] = st.M[i] = st.Minv[i] = st.U[i] = 0.0;
  if (MODE == 6) {
    // :2434
    const double c[5] = {2.0, 2.0, 10000, 20, 20};
    for (int i = 0; i < NV; i++) st.nc[i] = st.oc[i] = c[i], st.fade[i] = 0.0;
  } else if (MODE == kFit4Pi) {
    const double c[6] = {1, 1, 10000, 20, 2, 2};
    for (int i = 0; i < NV; i++) st.nc[i] = st.oc[i] = c[i], st.fade[i] = 0.5;
  } else if (MODE == 7) {
    // :2786-2788
    const double c[6] = {1.0, 1.0, 10000, 20, 2, 0.00001};
    const double fd[6] = {0.5, 0.5, 0.4, 0.5, 0.7, 0.8};
    for (int i = 0; i < NV; i++) st.nc[i] = st.oc[i] = c[i], st.fade[i] = fd[i];
  } else {
    // :3191-3193
    const double c[8] = {1.0, 1.0, 10000, 20, 2, 2, 2, 0.1};
    for (int i = 0; i < NV; i++) st.nc[i] = c[i], st.fade[i] = 0.5;
  }
}

template <int MODE>
__global__ void __launch_bounds__(32 * F64Traits<MODE>::WPB, 1) fit64_kernel(
    const __grid_constant__ Fit64Args a) {
  using L = F64Layout<MODE>;
  constexpr int NV = L::NV, WPB = F64Traits<MODE>::WPB;
  extern __shared__ double smem64[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  Warp64<MODE> w(smem64 + (int64_t)warp * L::per_warp, lane);
  LMState& st = w.st;
  Fit64Ctx cx;
  cx.a = &a;
  cx.c = Coef{a.c, a.total};
  cx.c3 = Coef{a.c3, a.total3};
  cx.s = a.s;
  cx.lane = lane;
  const int64_t s2 = (int64_t)a.s * a.s;
  const int64_t nw = (int64_t)gridDim.x * WPB;
  for (int64_t roi = (int64_t)blockIdx.x * WPB + warp; roi < a.nfits; roi += nw) {
    cx.data = a.rois + roi * s2;
    cx.var = a.var ? a.var + roi * s2 : nullptr;
    cx.dT = (MODE == kFit4Pi) ? a.dT + roi * (int64_t)(k4PiChannels * NV) : nullptr;
    if (lane == 0) {
      init_state<MODE>(st);
      initial_theta<MODE>(cx, st, roi);
      for (int i = 0; i < NV; i++) {
        st.ot[i] = st.nt[i];
        if (MODE == 8) st.oc[i] = st.nc[i];
      }
      st.frame[2] = (double)((float)(a.m.n[1] - a.s) / 2.0f);  // :2519, float arithmetic
    }
    __syncwarp();
    // Initial evaluation; fit type 7 copies dudt[4] into dudt[5] here only.
    // (4Pi prepares per channel inside the pass.)
    if (MODE != kFit4Pi) w.prepare(cx, st.nt);
    w.template pass<false>(cx, MODE == 7);
    if (MODE != kFit4Pi && a.handoff) {
      // Hand-off: the first LM steps in the reference's double arithmetic and
      // order, then the LM state for the double-float kernels. The step left
      // pending is the last one whose evaluation the double-float kernel makes.
      double te[8];
      if (lane == 0)
        for (int i = 0; i < 8; i++) te[i] = st.nt[i];
      int kk = 0, state = Handoff::kCurrent;
      const int K = a.handoff_iters < a.iterations ? a.handoff_iters : a.iterations;
      while (kk < K) {
        if (lane == 0) st.action = lm_control<MODE>(st, a.m, a.s);
        __syncwarp();
        const int act = st.action;
        __syncwarp();
        if (act == kStop) {
          state = Handoff::kConverged;
          break;
        }
        ++kk;
        state = Handoff::kCurrent;
        if (act == kEval) {
          if (kk == K) {
            state = Handoff::kEvalPending;
            break;
          }
          w.prepare(cx, st.nt);
          w.template pass<false>(cx, false);
          if (lane == 0)
            for (int i = 0; i < 8; i++) te[i] = st.nt[i];
        }
      }
      if (lane == 0) {
        double* r = a.handoff + roi * (int64_t)kHandoffStride;
        for (int i = 0; i < 8; i++) {
          const bool in = i < NV;
          r[Handoff::nt + i] = in ? st.nt[i] : 0.0;
          r[Handoff::ot + i] = in ? st.ot[i] : 0.0;
          r[Handoff::ns + i] = in ? st.ns[i] : 0.0;
          r[Handoff::os + i] = in ? st.os[i] : 0.0;
          r[Handoff::nc + i] = in ? st.nc[i] : 0.0;
          r[Handoff::oc + i] = in ? st.oc[i] : 0.0;
          r[Handoff::te + i] = in ? te[i] : 0.0;
          r[Handoff::jac + i] = in ? st.jac[i] : 0.0;
        }
        for (int i = 0; i < NV * NV; i++) r[Handoff::hes + i] = st.hes[i];
        r[Handoff::new_lambda] = st.newLambda;
        r[Handoff::old_lambda] = st.oldLambda;
        r[Handoff::new_err] = st.newErr;
        r[Handoff::old_err] = st.oldErr;
        r[Handoff::sum_update] = st.sumUpdate;
        r[Handoff::turn] = (double)st.turn;
        r[Handoff::kk] = (double)kk;
        r[Handoff::state] = (double)state;
      }
      __syncwarp();
      continue;
    }
    int kk = 0;
    for (; kk < a.iterations; kk++) {
      if (lane == 0) st.action = lm_control<MODE>(st, a.m, a.s);
      __syncwarp();
      const int act = st.action;
      __syncwarp();
      if (act == kStop) break;
      if (act == kEval) {
        if (MODE != kFit4Pi) w.prepare(cx, st.nt);
        w.template pass<false>(cx, false);
      }
    }
    // CRLB and log-likelihood: types 6 and 7 re-prepare at the final theta;
    // type 8 keeps the frame, weights and g2 of its last evaluation
    // (CPUmleFit_LM.cpp:3568-3584).
    if (MODE != 8 && MODE != kFit4Pi) w.prepare(cx, st.nt);
    w.template pass<true>(cx, false);
    if (lane == 0) {
      mat_inv64<NV>(st.M, st.Minv, st.diag);
      const int64_t n = a.nfits;
      for (int i = 0; i < NV; i++) {
        a.P[n * i + roi] = st.nt[i];
        a.CRLB[n * i + roi] = st.diag[i];
      }
      a.P[n * NV + roi] = (double)kk;
      a.LL[roi] = st.div;
    }
    __syncwarp();
  }
}

// dst = [c | diff_0 | ... | diff_{D-1}], each `total` long (see Coef).
struct Strides5 {
  int64_t st[5];
};

__global__ void widen_kernel(const float* __restrict__ src, double* __restrict__ dst,
                             int64_t total, int D, Strides5 st) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double c0 = (double)src[i];
    dst[i] = c0;
    for (int d = 0; d < D; ++d) {
      const int64_t j = i + st.st[d];
      const double c1 = (j < total) ? (double)src[j] : 0.0;
      dst[(int64_t)(d + 1) * total + i] = -c0 + c1;
    }
  }
}

// Blocks per SM and SM count of fit64_kernel<MODE> on a device, computed once
// (the kernel's shared-memory limit is set then), so later launches, including
// ones captured into a CUDA graph, make no attribute or occupancy calls.
struct Launch64 {
  int dev = -1, per_sm = 0, sms = 0;
};
std::mutex g_launch64_mu;

template <int MODE>
cudaError_t launch64(const Fit64Args& a, cudaStream_t stream) {
  using L = F64Layout<MODE>;
  constexpr int WPB = F64Traits<MODE>::WPB;
  const size_t smem = (size_t)L::per_warp * WPB * sizeof(double);
  static Launch64 cache[8];  // per device
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 8) return cudaErrorInvalidDevice;
  int per_sm = 0, sms = 0;
  {
    std::lock_guard<std::mutex> lk(g_launch64_mu);
    Launch64& c = cache[dev];
    if (c.dev != dev) {
      e = cudaFuncSetAttribute(fit64_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c.per_sm, fit64_kernel<MODE>, 32 * WPB,
                                                          smem);
      if (e != cudaSuccess) return e;
      c.dev = dev;
    }
    per_sm = c.per_sm;
    sms = c.sms;
  }
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int64_t need = (a.nfits + WPB - 1) / WPB;
  const int64_t cap = (int64_t)sms * per_sm;
  const int grid = (int)(need < cap ? need : cap);
  fit64_kernel<MODE><<<grid, 32 * WPB, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace

int fit64_smem_bytes(int mode) {
  switch (mode) {
    case 6: return F64Layout<6>::per_warp * F64Traits<6>::WPB * 8;
    case 7: return F64Layout<7>::per_warp * F64Traits<7>::WPB * 8;
    case 8: return F64Layout<8>::per_warp * F64Traits<8>::WPB * 8;
    case kFit4Pi: return F64Layout<kFit4Pi>::per_warp * F64Traits<kFit4Pi>::WPB * 8;
    default: return 0;
  }
}

cudaError_t widen_to_f64(const float* src, double* dst, int64_t total, int naxes,
                         const int64_t* strides, cudaStream_t stream) {
  if (total <= 0) return cudaSuccess;
  if (naxes < 0 || naxes > 5) return cudaErrorInvalidValue;
  Strides5 st{};
  for (int d = 0; d < naxes; ++d) st.st[d] = strides[d];
  const int64_t blocks = (total + 255) / 256;
  widen_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, stream>>>(src, dst, total,
                                                                              naxes, st);
  return cudaGetLastError();
}

cudaError_t launch_fit64(const Fit64Args& a, cudaStream_t stream) {
  if (a.nfits <= 0) return cudaSuccess;
  switch (a.m.fittype) {
    case 6: return launch64<6>(a, stream);
    case 7: return launch64<7>(a, stream);
    case 8: return launch64<8>(a, stream);
    case kFit4Pi: return launch64<kFit4Pi>(a, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bsfit
