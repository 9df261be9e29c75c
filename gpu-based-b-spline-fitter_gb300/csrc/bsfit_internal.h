// Internal types shared by the host library and the kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bsfit {

// Model tag of the four-channel 4Pi fit (the reference's separate
// GPUmleFit_LM_4Pi_bspline entry, which has no fit-type number).
constexpr int kFit4Pi = 9;
constexpr int k4PiChannels = 4;

// A PSF model resident on the device.
struct ModelDev {
  int fittype;           // 6, 7, 8, or kFit4Pi
  const float* coeff;    // device
  const float* coeff3;   // device (fit type 8)
  int cd[5];             // coefficient sizes, MATLAB order (Y, X, Z, W, U)
  int64_t st[5];         // element strides of those axes
  // nData per axis as the reference uses it: n[0] clamps Y (size(coeff,2) - 3),
  // n[1] clamps X and sets the lateral offset (size(coeff,1) - 3), n[2..] Z, W, U.
  int n[5];
  float init_p[4];
  int init_p_len;
  float shift[4];        // 4Pi models: per-channel phase shifts (knot units)
  // Stage-A gather table of the FP32 kernels (build_zq), device; null for fit
  // type 6. Per lateral node, the four z planes of one z knot as one 16-byte
  // entry (4Pi: one per w layer; fit type 8: of its 3D table), or for fit
  // type 7 two adjacent w
  // layers of them interleaved in two entries (planes 0, 1 and 2, 3 of both
  // layers), so that a node's gathers are 16-byte loads. Entry strides, with
  // the lateral node innermost as in the coefficient table: zq_kz between
  // consecutive z knots, zq_w between consecutive (first) w layers.
  const float4* zq;
  int64_t zq_kz, zq_w;
};

// Number of float4 entries of a model's stage-A gather table (0: none), and
// its construction from the model's device coefficients on a stream.
int64_t zq_entries(const ModelDev& m);
cudaError_t build_zq(const ModelDev& m, float4* zq, cudaStream_t stream);
// Sets m.zq and its strides for a table at zq (null clears them).
void set_zq(ModelDev& m, float4* zq);

struct FitArgs {
  ModelDev m;
  const float* rois;     // device, nfits * s * s
  int s;
  int64_t nfits;
  int iterations;
  float* P;              // device outputs, column-major with leading dim out_n
  float* CRLB;
  float* LL;
  int64_t out_n;
  int64_t out_offset;
  // Diagnostics: optional per-ROI decision trace (TRACE_REC floats per
  // iteration, trace_max iterations per ROI) and option bits.
  float* trace;
  int trace_max;
  int flags;
  // 4Pi only: per-ROI channel offsets dT [nfits][4][6], initial z and phase
  // [n_starts or 1][nfits]; rois holds [4][nfits][s][s].
  const float* dT;
  const float* z0;
  const float* w0;
  // Multi-start: n_starts > 1 fits every ROI from each start and keeps the
  // best log-likelihood (a later start replaces the kept result when its LL is
  // higher by more than 1e-4, or by at least 1e-4 unless strict). Fit types 7
  // and 8 take the starts' initP vectors from starts[]; 4Pi from z0 / w0.
  int n_starts;
  int strict;
  float starts[8][4];
  // sCMOS: per-pixel variance / gain^2 in the ROI layout, added to model and
  // data in the likelihood (null: EMCCD)
  const float* var;
  // Work counter (zeroed device word): warps claim ROIs one at a time, so the
  // launch ends within one ROI's time of its average warp; null: each warp
  // takes every (grid warps)-th ROI. Set by launch_fit.
  unsigned long long* claim;
  // Double-float kernels only: per-ROI LM state after the first LM steps of
  // the FP64 reference-order kernel (kHandoffStride doubles per ROI, see
  // Handoff), or null to start from the initial guess.
  const double* handoff;
};

// LM state handed from the FP64 reference-order kernel to the double-float
// kernels after the first LM steps: per ROI, kHandoffStride doubles at these
// offsets (parameter arrays of 8).
struct Handoff {
  static constexpr int nt = 0, ot = 8, ns = 16, os = 24, nc = 32, oc = 40, te = 48;
  static constexpr int new_lambda = 56, old_lambda = 57, new_err = 58, old_err = 59,
                       sum_update = 60, turn = 61, kk = 62, state = 63;
  static constexpr int jac = 64, hes = 72;  // gradient (8), damped Hessian (8 x 8, row-major NV)
  // state: 0 an evaluation at nt is pending (the last step was accepted);
  // 1 the gradient and Hessian of the last evaluation (at te) are current;
  // 2 converged: the CRLB pass follows.
  enum { kEvalPending = 0, kCurrent = 1, kConverged = 2 };
};
constexpr int kHandoffStride = 136;

constexpr int kMaxStarts = 8;

constexpr int TRACE_REC = 32;
constexpr int FLAG_NO_REFINE = 1;  // skip the refinement step of the LM solve
constexpr int FLAG_PARITY = 2;     // double-float parity kernels (bsfit_fitdd.cu)

// Batched form: ROI segments of one fit type fitted by one persistent launch.
constexpr int kMaxBatchSegs = 48;

struct BatchSeg {
  ModelDev m;
  const float* rois;
  float* P;
  float* CRLB;
  float* LL;
  int64_t n;
  int s;
  int iterations;
  int slot;  // index of this segment's counters in next[] / done[]
  // multi-start (fit types 7, 8; the multi-start batched kernel only): the
  // starts' initP vectors and the keep rule, as FitArgs
  int n_starts;
  int strict;
  float starts[kMaxStarts][4];
};

struct BatchArgs {
  int nseg;
  int s_max;
  int flags;
  // ROIs a warp fits before it ends (0: until the queue is empty; > 0: the
  // capped form of the default kernel). With a cap the grid covers every ROI
  // and blocks retire as they finish, so the work of a launch on a
  // higher-priority stream starts as soon as a block's resources free up
  // instead of after the whole launch.
  int warp_rois;
  // Work queue in caller-provided device scratch: next[i] is the next
  // unclaimed ROI of segment i, done[i] counts its finished ROIs.
  unsigned long long* next;
  unsigned long long* done;
  BatchSeg seg[kMaxBatchSegs];
};

// FP64 reference-precision fit (fit types 6, 7, 8): double copies of the
// coefficient tables, float ROIs, double outputs in the column-major layout.
struct Fit64Args {
  ModelDev m;
  // device: the model's table widened to double, followed by one table per
  // axis of neighbour differences (-c[i]) + c[i + stride] (widen_to_f64)
  const double* c;
  const double* c3;      // the same for fit type 8's 3D table (3 axes)
  int64_t total;         // elements of c
  int64_t total3;        // elements of c3
  const float* rois;     // device, nfits * s * s
  const float* var;      // sCMOS variance / gain^2 in the ROI layout, or null
  int s;
  int64_t nfits;
  int iterations;
  double* P;
  double* CRLB;
  double* LL;
  // 4Pi: rois [4][nfits][s][s], channel offsets dT [nfits][4][6], initial z
  // and phase [nfits]
  const float* dT;
  const float* z0;
  const float* w0;
  // Hand-off mode (fit types 6, 7, 8): run the initial evaluation and at most
  // handoff_iters LM steps per ROI, then write the LM state to handoff
  // (kHandoffStride doubles per ROI) instead of outputs.
  double* handoff;
  int handoff_iters;
};

cudaError_t launch_fit64(const Fit64Args& a, cudaStream_t stream);
// dst: (1 + naxes) * total doubles, the values then the difference tables.
cudaError_t widen_to_f64(const float* src, double* dst, int64_t total, int naxes,
                         const int64_t* strides, cudaStream_t stream);
int fit64_smem_bytes(int mode);

int warp_smem_floats(int mode, int s, bool var = false, int stg = 0);
cudaError_t launch_batch(const BatchArgs& a, int mode, bool multi, cudaStream_t stream);
cudaError_t launch_fit(const FitArgs& a, cudaStream_t stream);
// Double-float parity-grade fit of fit types 6, 7, 8 (plain ROIs, one start).
cudaError_t launch_fitdd(const FitArgs& a, cudaStream_t stream);
int fitdd_smem_floats(int mode, int s);
// One double-float evaluation per ROI (double outputs, layout of launch_eval).
cudaError_t launch_evaldd(const FitArgs& a, const float* theta, double* out, int fisher,
                          cudaStream_t stream);
// Launch shape of a fitter kernel (warps per block among 4, 2, 1 keeping the
// most warps resident; blocks per SM; SM count), cached per kernel, size and
// device.
cudaError_t pick_launch(const void* kern, int per_warp, int* wpb, int* bps, int* sms);
// The same with the warps per block forced (force_wpb 1, 2 or 4; 0 chooses).
cudaError_t pick_launch_wpb(const void* kern, int per_warp, int force_wpb, int* wpb, int* bps,
                            int* sms);

// Autotuner (bsfit_tune.cu): the launch configuration of the single-start FP32
// fit kernels (plain and batched) per fit type, ROI size and device. variant 0
// is the default kernel; wpb 0 lets the occupancy choice stand.
struct TuneConfig {
  int variant;
  int wpb;
};
using FitKern = void (*)(FitArgs);
using BatchKern = void (*)(const BatchArgs);
int tune_num_variants(int mode);
int tune_min_blocks(int mode, int variant);
// 1 when the variant stages the 5D gathers through shared memory (its
// per-warp shared memory includes the staging buffers)
int tune_staged(int mode, int variant);
// ROIs fitted per warp by a variant (2: the pair and packed forms of fit type 6)
int tune_rois_per_warp(int mode, int variant);
// Shared-memory floats per warp of a variant at ROI size s
int tune_warp_floats(int mode, int variant, int s, bool var);
FitKern fit_variant(int mode, int variant);     // variant >= 1
BatchKern batch_variant(int mode, int variant);  // variant >= 1
bool tune_lookup(int mode, int s, int dev, TuneConfig* out);
bool tune_store(int mode, int s, int dev, TuneConfig c);
void tune_clear(int mode, int s, int dev);
cudaError_t measure_fp32_peak(double* tflops);
// FP32 FMA throughput of scalar and of paired (FFMA2) FMA chains, TFLOP/s.
cudaError_t measure_fp32_peak2(double* scalar, double* paired);
cudaError_t launch_eval(const FitArgs& a, const float* theta, float* out, int fisher,
                        cudaStream_t stream);

}  // namespace bsfit
