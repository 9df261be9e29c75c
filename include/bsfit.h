/*
 * bsfit: GB300-native multi-dimensional cubic B-spline PSF maximum-likelihood
 * fitter. C ABI of the shared library libbsfit.so.
 *
 * The entry points replace the reference's drop-in boundary for the B-spline
 * fit types (6 = 3D, 7 = 4D colour, 8 = 5D + 3D mixture) of
 * GPUmleFit_LM_multiD / CPUmleFit_LM (Li-Lab-SUSTech/GPU-based-B-spline-Fitter).
 * Paths cited below are relative to the reference project root; VC stands for
 * "MultiD_bspline/visual code".
 *
 * Array conventions (identical to the reference mex):
 *  - ROI stack: float, MATLAB column-major [s, s, N]; pixel (ii, jj) of ROI n
 *    at imstack[n*s*s + s*jj + ii].
 *  - Coefficients: float, column-major with dims[0] fastest (MATLAB
 *    size(coeff)), i.e. (Y, X, Z[, W[, U]]) as produced by bsarray.
 *  - Outputs: P [N x (NV+1)] column-major (P[k*N + i]; the last column is the
 *    iteration count), CRLB [N x NV] (variances), LL [N]. NV = 5, 6, 8 for fit
 *    types 6, 7, 8. Parameter order: x, y, photons, background, z[, w[, u, g2]].
 *
 * Every call returns a status code; no call resets a device.
 */
#ifndef BSFIT_H
#define BSFIT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bsfit_status {
  BSFIT_OK = 0,
  /* GPUmleFit_LM:WrongNoArgs (VC/GPUmleFit_LM/mexFunction.cpp:247-248) */
  BSFIT_E_WRONG_NO_ARGS = 1,
  /* GPUmleFit_LM:WrongDataType: a required array is missing (mex :251-252) */
  BSFIT_E_WRONG_DATA_TYPE = 2,
  /* GPUmleFit_LM:SubregionSize: s > 51 (mex :259-260) */
  BSFIT_E_SUBREGION_SIZE = 3,
  /* GPUmleFit_LM:SubregionShape: non-square ROI (mex :261-262) */
  BSFIT_E_SUBREGION_SHAPE = 4,
  /* fit types 1-5 (Gaussian / cubic spline) are not part of this library */
  BSFIT_E_UNSUPPORTED_FITTYPE = 5,
  /* GPUmleFit_LM:NotEnoughMemory (mex :409-456) */
  BSFIT_E_NOT_ENOUGH_MEMORY = 6,
  /* GPUmleFit_LM:cudaFail (mex :140-176), without the device reset */
  BSFIT_E_CUDA = 7,
  /* GPUmleFit_LM:NoDevice / nodevices (mex :186-203) */
  BSFIT_E_NO_DEVICE = 8,
  /* coefficient array too small (< 5 along an axis) or too large (> 2^20
   * along an axis, 2^29 or more elements per lateral plane), wrong rank, or
   * lateral sizes unequal (the reference indexes past the array there) */
  BSFIT_E_COEFF_SIZE = 9,
  /* initP missing or too short for fit types 7 and 8 (the reference
   * dereferences it, or leaves g2 uninitialised) */
  BSFIT_E_INIT_P = 10,
  /* invalid handle or argument of the device-level API */
  BSFIT_E_INVALID = 11,
  /* a bounded device-side wait ran out (batched / serving forms) */
  BSFIT_E_TIMEOUT = 12,
  /* more segments than the allocation-free entry point's fixed scratch holds */
  BSFIT_E_STATIC_LIMIT = 13,
  /* 4Pi fit with unshared parameters, or a channel count other than 4 */
  BSFIT_E_UNSHARED = 14
} bsfit_status;

/* Human-readable text of a status code (replaces mexErrMsgIdAndTxt texts). */
const char* bsfit_status_str(int status);

/* Library version string. */
const char* bsfit_version(void);

/*
 * Synchronous drop-in call with host buffers. Replaces the B-spline branch of
 * mexFunction in VC/GPUmleFit_LM/mexFunction.cpp:208-762 (argument parsing
 * :247-385, device buffers :466-518, launch :598-674, copies back :685-734):
 *
 *   [P, CRLB, LL] = GPUmleFit_LM_multiD(imstack, fittype, iterations, coeff,
 *                                        varmap, silent, initP, coeff3)
 *
 * imstack: [roi_size, roi_size2, nfits]; roi_size2 must equal roi_size and
 *   roi_size must be <= 51.
 * coeff / coeff_dims / coeff_ndim: 3, 4 or 5 dims for fit types 6, 7, 8.
 * varmap: accepted and ignored for fit types 6-8, as in the reference
 *   (mex :661-674 pass no variance map to the B-spline kernels).
 * silent: 0 prints the reference's summary lines to stdout.
 * init_p: fit type 7: (z, w), both taken from init_p when init_p[0] != 0,
 *   else mid-grid (CPUmleFit_LM.cpp:2841-2850); fit type 8: (z, w, u, g2),
 *   required (without it the reference leaves g2 uninitialised,
 *   CPUmleFit_LM.cpp:3246-3256); ignored for 6.
 * coeff3: fit type 8 only, the 3D coefficients (same Y, X, Z sizes).
 * P, CRLB, LL: caller-allocated host outputs.
 */
int bsfit_GPUmleFit_LM_multiD(const float* imstack, int64_t roi_size, int64_t roi_size2,
                              int64_t nfits, int32_t fittype, int32_t iterations,
                              const float* coeff, int32_t coeff_ndim, const int64_t* coeff_dims,
                              const float* varmap, int64_t varmap_numel, int32_t silent,
                              const float* init_p, int64_t init_p_numel, const float* coeff3,
                              int32_t coeff3_ndim, const int64_t* coeff3_dims, float* P,
                              float* CRLB, float* LL);

/* Number of fitted parameters for a fit type (5, 6, 8), or 0 if unsupported. */
int bsfit_num_params(int32_t fittype);

/* Measured FP32 FMA throughput of the current device in TFLOP/s (2 FLOP per
 * FMA), the roofline denominator of the fitter kernels. No reference
 * counterpart: a measurement utility. */
int bsfit_measure_fp32_peak(double* tflops);
/* The same probe with scalar FMA chains and with paired FP32 FMAs (FFMA2, two
 * FMAs per instruction), TFLOP/s each. */
int bsfit_measure_fp32_peaks(double* scalar_tflops, double* paired_tflops);

/*
 * Device-resident model: the coefficient tables of one PSF model uploaded once
 * and reused across calls (the reference uploads them on every call,
 * mex :484-518). Copies from host memory; coeff3 only for fit type 8. Beside
 * the tables the model holds a gather table for the FP32 kernels (the z planes
 * of each lateral node packed in 16-byte entries): 8x the coefficient table for
 * fit type 7, 4x for 4Pi, 4x coeff3 for fit type 8, none for fit type 6. The
 * call returns after the tables are built.
 */
typedef struct bsfit_model_s* bsfit_model;

int bsfit_model_create(int32_t fittype, const float* coeff, int32_t coeff_ndim,
                       const int64_t* coeff_dims, const float* coeff3, int32_t coeff3_ndim,
                       const int64_t* coeff3_dims, const float* init_p, int64_t init_p_numel,
                       bsfit_model* out);
int bsfit_model_release(bsfit_model model);

/* Fit type of a model (6, 7, 8; BSFIT_FITTYPE_4PI for 4Pi models), 0 for NULL. */
int32_t bsfit_model_fittype(bsfit_model model);

/*
 * Asynchronous fit on a CUDA stream with device pointers (replaces the launch
 * wrappers VC/GPUmleFit_LM/wrapper.cu:256-279 and their kernels
 * VC/GPUmleFit_LM/GPUmleFit_LM_EMCCD.cu:1208-2405). d_rois: nfits ROIs of
 * roi_size^2 floats; d_P / d_CRLB / d_LL: device outputs in the layout above.
 * stream: a cudaStream_t (NULL = legacy default stream). When the ROIs
 * outnumber the warps resident on the device, the warps claim ROIs from an
 * 8-byte work counter taken from the stream-ordered pool (cudaMallocAsync /
 * cudaFreeAsync on `stream`); otherwise it uses no device memory beyond its
 * arguments. bsfit_batch_fit_device_static allocates nothing at all.
 */
int bsfit_fit_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                     int32_t iterations, float* d_P, float* d_CRLB, float* d_LL, void* stream);

/*
 * Parity-grade fit (fit types 6, 7, 8): the same method, call and output
 * layout as bsfit_fit_device, evaluated in double-float arithmetic (two
 * floats per value, about 48 significant bits) on the FP32 pipe, with the
 * Fisher matrix inverted in FP64. It follows the trajectory of the
 * reference's FP64 build (VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2411-3620 with
 * float promoted to double) as closely as a second FP64 build of the
 * reference does (one compiled with FMA contraction): the LM's discrete
 * decisions react to rounding, and the FP32 kernels agree with the FP64
 * results within the stated tolerances on fewer ROIs (a third of 4D ROIs).
 * Plain EMCCD ROIs, one start; several times slower than bsfit_fit_device.
 * Fit type 7's first LM step is taken by the FP64 reference-order kernel of
 * bsfit_fit_f64_device (its initial Hessian is exactly singular: the
 * reference's initial pass copies dudt[4] into dudt[5],
 * CPUmleFit_LM.cpp:2893, so that step is set by the rounding of the
 * reference's double sums); the model's double tables are made on first use
 * as for bsfit_fit_f64_device, and the LM state passes through a buffer of
 * 1088 bytes per ROI from the stream-ordered pool (cudaMallocAsync /
 * cudaFreeAsync on `stream`). Same work counter as bsfit_fit_device.
 */
int bsfit_fit_parity_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                            int64_t nfits, int32_t iterations, float* d_P, float* d_CRLB,
                            float* d_LL, void* stream);

/* bsfit_fit_parity_device with an explicit number of leading LM steps taken
 * by the FP64 reference-order kernel (0: none; -1: the default per fit type,
 * 1 for fit type 7, 0 otherwise). More steps follow the FP64 trajectory
 * further at the FP64 kernel's speed. */
int bsfit_fit_parity_steps_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                                  int64_t nfits, int32_t iterations, int32_t exact_steps,
                                  float* d_P, float* d_CRLB, float* d_LL, void* stream);

/* Host drop-in call of the parity-grade fit: the arguments, checks and
 * outputs of bsfit_GPUmleFit_LM_multiD (VC/GPUmleFit_LM/mexFunction.cpp:208-762),
 * fitted by the kernels of bsfit_fit_parity_device. */
int bsfit_GPUmleFit_LM_multiD_parity(const float* imstack, int64_t roi_size, int64_t roi_size2,
                                     int64_t nfits, int32_t fittype, int32_t iterations,
                                     const float* coeff, int32_t coeff_ndim,
                                     const int64_t* coeff_dims, const float* varmap,
                                     int64_t varmap_numel, int32_t silent, const float* init_p,
                                     int64_t init_p_numel, const float* coeff3,
                                     int32_t coeff3_ndim, const int64_t* coeff3_dims, float* P,
                                     float* CRLB, float* LL);

/*
 * One model evaluation per ROI at given parameters, without the LM loop: the
 * Poisson deviance, its gradient and the Hessian approximation the reference
 * accumulates (VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2537-2560), or with fisher != 0
 * the log-likelihood and the Fisher information of the CRLB pass (:2725-2742).
 * d_theta: NV x nfits column-major parameters; d_out: per ROI 1 + NV + NV(NV+1)/2
 * floats: value, gradient (zeros for fisher), packed upper triangle row-major.
 */
int bsfit_eval_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                      const float* d_theta, int32_t fisher, float* d_out, void* stream);

/*
 * bsfit_eval_device in double-float (the evaluation of bsfit_fit_parity_device),
 * with double outputs in the same per-ROI layout: the deviance (or
 * log-likelihood), gradient and packed Hessian (or Fisher information) of
 * VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2537-2560 / :2725-2742 at d_theta.
 */
int bsfit_eval_parity_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                             int64_t nfits, const float* d_theta, int32_t fisher, double* d_out,
                             void* stream);

/*
 * Diagnostic form of bsfit_fit_device (no counterpart in the reference): also
 * writes, per ROI and LM iteration, a 32-float decision record to d_trace
 * (trace_max records per ROI: iteration, |dErr/err|, new and old deviance,
 * decision bits 1 converged / 2 rejected / 4 improved / 8 solve accepted,
 * lambda, the step (8), theta after the step (8), deviance after the step).
 * flags bit 0 skips the refinement step of the LM solve.
 */
int bsfit_trace_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                       int32_t iterations, int32_t flags, float* d_P, float* d_CRLB, float* d_LL,
                       float* d_trace, int32_t trace_max, void* stream);

/*
 * Batched form (no counterpart in the reference, whose callers loop over blocks
 * of 20,000 / 5,000 ROIs and call the mex once per block and start,
 * MultiD_fitter/simplefitter_cspline.m:309-313,463-524): segments of ROIs,
 * each with its own model, ROI size, iteration cap and output buffers, fitted
 * by one persistent launch per fit type with a device work queue. Segments may
 * mix ROI sizes and models; fit types are launched one after the other on the
 * stream. At most BSFIT_MAX_SEGMENTS segments per call.
 */
#define BSFIT_MAX_SEGMENTS 48

typedef struct bsfit_segment {
  bsfit_model model;
  const float* d_rois;   /* device, nfits * roi_size^2 floats */
  int64_t roi_size;
  int64_t nfits;
  int32_t iterations;
  float* d_P;            /* device outputs, column-major, leading dimension nfits */
  float* d_CRLB;
  float* d_LL;
} bsfit_segment;

/* Bytes of device scratch bsfit_batch_fit_device needs for nseg segments
 * (two 64-bit counters per segment, 256-byte aligned). */
int64_t bsfit_batch_scratch_bytes(int32_t nseg);

/* Asynchronous batched fit on a stream. d_scratch: caller-provided device
 * memory of at least bsfit_batch_scratch_bytes(nseg) bytes, zeroed by the
 * call itself (stream-ordered); after completion it holds, per segment, the
 * number of claimed and of finished ROIs. Allocates nothing. */
int bsfit_batch_fit_device(const bsfit_segment* segs, int32_t nseg, void* d_scratch,
                           int64_t scratch_bytes, void* stream);

/* Multi-start of the batched fit (fit types 7 and 8): starts[i] gives segment
 * i's initP vectors (n_starts <= BSFIT_MAX_STARTS; z, w for fit type 7; z, w,
 * u, g2 for 8) and keep rule; every ROI is fitted from each start inside the
 * persistent launch and the best log-likelihood kept (a later start replaces
 * the kept result when its LL is higher by at least 1e-4, or by more than
 * 1e-4 with strict != 0), bit for bit the results of
 * bsfit_fit_multistart_device on each segment. n_starts = 0 fits the segment
 * once from its model's initP (the results of bsfit_batch_fit_device). Fit
 * type 6 has no initP: its segments take n_starts <= 1 and are fitted once;
 * more starts return BSFIT_E_UNSUPPORTED_FITTYPE. */
typedef struct bsfit_starts {
  int32_t n_starts;
  int32_t strict;
  float initp[8][4];  /* BSFIT_MAX_STARTS x 4, unused entries ignored */
} bsfit_starts;

int bsfit_batch_fit_multistart_device(const bsfit_segment* segs, const bsfit_starts* starts,
                                      int32_t nseg, void* d_scratch, int64_t scratch_bytes,
                                      void* stream);

/*
 * Serving form (no counterpart in the reference, whose GUI fits one block at a
 * time, MultiD_fitter/simplefitter_cspline.m:309-313): a continuous-batching
 * request loop. Each request is a list of segments with HOST buffers (use
 * page-locked memory for asynchronous copies); requests that arrive while
 * others run are admitted as slots (max_inflight CUDA streams) and arena memory
 * (arena_bytes of device memory, reserved once at creation: the HBM budget)
 * free up, in submission order, and run concurrently on the GPU. A request
 * completes independently of the others: poll returns the ids of finished
 * requests (their outputs are filled), wait blocks up to a timeout. Progress
 * is driven by these calls; no device-side wait exists. Latency = submission to
 * completion (a host callback at the end of the request's stream).
 */
typedef struct bsfit_host_segment {
  bsfit_model model;
  const float* rois;     /* host, nfits * roi_size^2 floats */
  int64_t roi_size;
  int64_t nfits;
  int32_t iterations;
  float* P;              /* host outputs, layout as bsfit_GPUmleFit_LM_multiD */
  float* CRLB;
  float* LL;
} bsfit_host_segment;

typedef struct bsfit_server_s* bsfit_server;

int bsfit_server_create(int32_t max_inflight, int64_t arena_bytes, bsfit_server* out);
int bsfit_server_destroy(bsfit_server server);
/* Requests fitted by one launch: a free slot takes the oldest queued request
 * and up to max_requests_per_launch - 1 more queued single-start requests
 * that fit the arena (at most BSFIT_MAX_SEGMENTS segments in all), fitted by one
 * persistent batched launch; each request is still copied back and completed
 * on its own. 1 (the default) launches every request alone. Results do not
 * depend on the setting. */
int bsfit_server_set_merge(bsfit_server server, int32_t max_requests_per_launch);
/* Priority launches (no counterpart in the reference): with enable set, each
 * launch goes to one of three streams of its slot by its estimated device time
 * (short ones, like a 3D frame, at the device's highest stream priority), and
 * its warps end after a few ROIs each so that its blocks retire while it runs:
 * a short request submitted while a long one (a 5D frame) runs starts on the
 * SMs its blocks free instead of after the long launch. Off by default.
 * Results do not depend on the setting. */
int bsfit_server_set_priority(bsfit_server server, int32_t enable);
/* As bsfit_server_submit, with per-segment starts (bsfit_starts, see
 * bsfit_batch_fit_multistart_device): the request's fits run the callers'
 * multi-start inside the batched launch. */
int bsfit_server_submit_multistart(bsfit_server server, const bsfit_host_segment* segs,
                                   const bsfit_starts* starts, int32_t nseg,
                                   int64_t* request_id);
/* Non-blocking: admits the request or queues it; BSFIT_E_NOT_ENOUGH_MEMORY if it
 * can never fit the arena. */
int bsfit_server_submit(bsfit_server server, const bsfit_host_segment* segs, int32_t nseg,
                        int64_t* request_id);
/* Retires finished requests, admits queued ones, returns up to max_ids ids of
 * finished requests (each id is returned once). */
int bsfit_server_poll(bsfit_server server, int64_t* done_ids, int32_t max_ids, int32_t* n_done);
/* Blocks until the request finished (its status) or timeout_s passed
 * (BSFIT_E_TIMEOUT). */
int bsfit_server_wait(bsfit_server server, int64_t request_id, double timeout_s);
/* Latency quantiles over completed requests, fits/s from the first submission
 * to the last completion, and the request counts. Any pointer may be NULL. */
int bsfit_server_stats(bsfit_server server, double* p50_ms, double* p99_ms, double* fits_per_s,
                       int64_t* completed, int64_t* in_flight, int64_t* queued);
int bsfit_server_reset_stats(bsfit_server server);
/* Per-request latencies (submission to completion, ms) recorded since the last
 * reset, in completion order: up to max_n (request id, latency) pairs. */
int bsfit_server_latencies(bsfit_server server, int64_t* ids, double* ms, int32_t max_n,
                           int32_t* n);

/*
 * Allocation-free batched fit (no counterpart in the reference). For callers
 * that cannot allocate device memory when they fit - a fixed-rate acquisition
 * loop, where cudaMalloc may synchronise the device, or an application that
 * reserved the GPU's memory for its own pool - this variant of
 * bsfit_batch_fit_device keeps the work-queue counters in a fixed device array
 * inside the library instead of caller scratch, and allocates nothing.
 * Limit: BSFIT_STATIC_MAX_SEGMENTS segments per call (BSFIT_E_STATIC_LIMIT
 * beyond). The array is shared by all calls on a device: each call zeroes the
 * counters it uses before its launch, and calls that overlap on the GPU race
 * on them, so serialise such calls. The first call on each device looks the
 * array's address up (cudaGetSymbolAddress); make it before any stream capture.
 * The address is kept per device and CUDA context: after a device reset the
 * next call looks it up again (make that call, too, before any capture).
 */
#define BSFIT_STATIC_MAX_SEGMENTS 48
int bsfit_batch_fit_device_static(const bsfit_segment* segs, int32_t nseg, void* stream);

/*
 * Autotuner (no counterpart in the reference, which launches every fit with
 * fixed 64-thread blocks, one thread per ROI: VC/GPUmleFit_LM/mexFunction.cpp:407).
 * The FP32 fit kernels of fit types 6, 7, 8 (single start, EMCCD; plain and
 * batched) have a launch configuration per fit type, ROI size and device: the
 * kernel variant (its minimum resident 4-warp blocks per SM, which sets the
 * register budget: bsfit_tune_min_blocks; for fit type 6 also the ROIs per
 * warp, one or two: bsfit_tune_rois_per_warp) and the warps per block (4, 2 or
 * 1; 0 keeps the occupancy choice). Variant 0 with 0 warps per block is the
 * default. Every configuration gives bit-identical results. The batched form
 * uses the configuration of its largest ROI size.
 */
int bsfit_tune_num_variants(int32_t fittype);                  /* 0 if none */
int bsfit_tune_min_blocks(int32_t fittype, int32_t variant);   /* 0 if out of range */
int bsfit_tune_rois_per_warp(int32_t fittype, int32_t variant); /* 0 if out of range */
/* Sets the configuration for (fittype, roi_size) on the current device;
 * variant -1 restores the default. */
int bsfit_tune_set(int32_t fittype, int64_t roi_size, int32_t variant, int32_t warps_per_block);
/* The configuration in force: variant -1 when the default applies. */
int bsfit_tune_get(int32_t fittype, int64_t roi_size, int32_t* variant, int32_t* warps_per_block);
/* Times every configuration on the caller's ROIs (a sample of the workload:
 * one untimed and `reps` timed bsfit_fit_device calls each, CUDA events on
 * `stream`), sets the fastest for (fit type, roi_size) on the current device
 * and returns it. all_ms (optional, 3 * bsfit_tune_num_variants doubles):
 * mean ms per call of (variant v, warps per block 4 / 2 / 1) at
 * [v * 3 + {0, 1, 2}], -1 where the configuration cannot launch. The outputs
 * hold the last timed call's results. Synchronises the stream. */
int bsfit_autotune_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                          int32_t iterations, float* d_P, float* d_CRLB, float* d_LL, int32_t reps,
                          int32_t* best_variant, int32_t* best_wpb, double* best_ms,
                          double* all_ms, void* stream);

/*
 * 4Pi fit: four interference channels of one emitter fitted with shared
 * parameters (x, y, N, bg, z, phase; NV = 6) against one 4D (x, y, z, phase)
 * B-spline. Replaces GPUmleFit_LM_4Pi_bspline, which the reference ships only
 * as a compiled mex; its interface is taken from the caller,
 * demo_4pi/bspline_based_4piloc_v4.m:196-216:
 *
 *   [P, CRLB, LL] = GPUmleFit_LM_4Pi_bspline(imstack, shared, iterations,
 *                        coeff, dT, initZ, initPhi, phase_shift)
 *
 * imstack: [s, s, N, 4] (channel slowest). shared: 6 flags, all 1 (the only
 *   setting any reference caller uses; others give BSFIT_E_UNSHARED).
 * coeff: the bsarray of the phase-resolved PSF, dims (Y, X, Z, W) with the
 *   phase samples covering one period plus one (the period is W - 4 knots,
 *   bspline_based_4piloc_v4.m:80-88).
 * dT: [6, 4, N] per-ROI per-channel parameter offsets (channel c is evaluated
 *   at theta + dT[:, c, n]). initZ, initPhi: [N] initial z and phase, in knot
 *   units. phase_shift: [4] per-channel phase shifts in knot units.
 * P: [N x 7] (last column = iterations; the phase column is in knots,
 *   [1, 1 + period)), CRLB: [N x 6], LL: [N].
 * The method (the LM machinery of fit type 7 without its quirks, all channels'
 * pixels in one likelihood) is this library's restatement; with the source of
 * the reference's 4Pi fitter absent, parity with it is not pinned.
 */
#define BSFIT_FITTYPE_4PI 9  /* model tag of 4Pi models (not a reference fit type) */
#define BSFIT_4PI_CHANNELS 4
int bsfit_GPUmleFit_LM_4Pi_bspline(const float* imstack, int64_t roi_size, int64_t roi_size2,
                                   int64_t nfits, int64_t n_channels, const uint32_t* shared,
                                   int64_t shared_numel, int32_t iterations, const float* coeff,
                                   int32_t coeff_ndim, const int64_t* coeff_dims, const float* dT,
                                   int64_t dT_numel, const float* initZ, int64_t initZ_numel,
                                   const float* initPhi, int64_t initPhi_numel,
                                   const float* phase_shift, int64_t phase_shift_numel,
                                   int32_t silent, float* P, float* CRLB, float* LL);

/* Device-resident 4Pi model: 4D coefficients and the channels' phase shifts. */
int bsfit_model_create_4pi(const float* coeff, int32_t coeff_ndim, const int64_t* coeff_dims,
                           const float* phase_shift, int32_t n_channels, bsfit_model* out);

/* Asynchronous 4Pi fit with device pointers: d_rois [4][nfits][s][s],
 * d_dT [nfits][4][6] (NULL = no offsets), d_initZ / d_initPhi [nfits]; outputs
 * as for bsfit_fit_device with NV = 6. */
int bsfit_fit4pi_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                        int32_t iterations, const float* d_dT, const float* d_initZ,
                        const float* d_initPhi, float* d_P, float* d_CRLB, float* d_LL,
                        void* stream);

/* One 4Pi likelihood evaluation per ROI at given parameters (d_theta [6][nfits]);
 * d_out as for bsfit_eval_device with NV = 6. */
int bsfit_eval4pi_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                         const float* d_dT, const float* d_theta, int32_t fisher, float* d_out,
                         void* stream);

/*
 * Multi-start, fused into one launch (no reference counterpart as one call:
 * the reference's callers loop over starts, re-uploading and refitting the
 * whole stack each time, MultiD_fitter/simplefitter_cspline.m:463-490,
 * demo_orientation/store/fitb5n3.m:15-46, demo_4pi/bspline_based_4piloc_v4.m:193-215).
 * Each ROI is staged once and fitted from every start; the result of a later
 * start replaces the kept one when its log-likelihood is higher by at least
 * 1e-4 (strict != 0: by more than 1e-4), the callers' rule, so the outputs
 * equal those loops over single-start calls.
 * Fit types 7 and 8: init_p_starts is a host array of n_starts x start_len
 * initP vectors (start_len >= 2 for 7, >= 4 for 8), n_starts <= 8. Fit type 6
 * has no initP and returns BSFIT_E_UNSUPPORTED_FITTYPE.
 * 4Pi: d_initZ and d_initPhi hold n_starts x nfits values (start-major).
 */
#define BSFIT_MAX_STARTS 8
int bsfit_fit_multistart_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                                int64_t nfits, int32_t iterations, const float* init_p_starts,
                                int32_t start_len, int32_t n_starts, int32_t strict, float* d_P,
                                float* d_CRLB, float* d_LL, void* stream);
int bsfit_fit4pi_multistart_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                                   int64_t nfits, int32_t iterations, const float* d_dT,
                                   const float* d_initZ, const float* d_initPhi, int32_t n_starts,
                                   int32_t strict, float* d_P, float* d_CRLB, float* d_LL,
                                   void* stream);

/*
 * Cubic B-spline coefficients of a sampled PSF stack on the device: the
 * reference's coefficient builder bsarray for degree 3 without smoothing (the
 * mirror-boundary cubic prefilter along every axis, then a one-sample mirror
 * pad; MultiD_bspline/bsarray/directFilter.m:200-298, symExpFilt.m:27-44,
 * getBSplineFiltCoeffs.m:45-50), in double as the MATLAB builder computes.
 * d_samples: double, ndim <= 5 axes with dims[0] fastest (MATLAB order);
 * d_work: double scratch of the samples' size; outputs: d_coeff (float, the
 * fitter's coefficient input) and/or d_coeff64 (double), prod(dims[i] + 2)
 * elements each. Either output may be NULL, not both.
 */
int bsfit_bsarray_coeffs_device(const double* d_samples, int32_t ndim, const int64_t* dims,
                                double* d_work, float* d_coeff, double* d_coeff64,
                                void* stream);
/* The same with host buffers, synchronous: float coefficients out. */
int bsfit_bsarray_coeffs(const double* samples, int32_t ndim, const int64_t* dims, float* coeff);

/*
 * sCMOS likelihood for fit types 6, 7, 8 (no reference counterpart: the
 * reference's B-spline branch ignores its variance map; its sCMOS kernels of
 * the Gaussian and cubic-spline fit types add the per-pixel variance / gain^2
 * to both model and data, VC/GPUmleFit_LM/GPUmleFit_LM_sCMOS.cu:1045-1046, and
 * this applies the same to the B-spline likelihood). d_var: variance / gain^2
 * in the ROI layout ([nfits][s][s]); outputs as bsfit_fit_device. The drop-in
 * call bsfit_GPUmleFit_LM_multiD keeps ignoring varmap, as the reference does.
 */
int bsfit_fit_scmos_device(bsfit_model model, const float* d_rois, const float* d_var,
                           int64_t roi_size, int64_t nfits, int32_t iterations, float* d_P,
                           float* d_CRLB, float* d_LL, void* stream);

/*
 * FP64 reference-precision fit (fit types 6, 7, 8): the reference's CPU method
 * (VC/CPUmleFit_LM/CPUmleFit_LM.cpp:2411-3620 with CPUsplineLib.cpp and
 * MatInvLib.h) evaluated in double in its own order of operations, so that the
 * LM takes the decisions of the reference built with float promoted to double.
 * float ROIs ([nfits][s][s]) and optional sCMOS variance (d_var, same layout,
 * or NULL); double outputs in bsfit_fit_device's column-major layout. The
 * model's coefficient table is widened to double on the first call (one
 * synchronisation of `stream`). Bounded by the device's FP64 rate: a
 * precision mode next to the FP32 production path, not a replacement.
 */
int bsfit_fit_f64_device(bsfit_model model, const float* d_rois, const float* d_var,
                         int64_t roi_size, int64_t nfits, int32_t iterations, double* d_P,
                         double* d_CRLB, double* d_LL, void* stream);

/*
 * The synchronous drop-in call (bsfit_GPUmleFit_LM_multiD: same arguments,
 * checks and status codes, varmap likewise ignored) with double outputs from
 * the FP64 reference-precision kernel: the reference's results as its CPU
 * method computes them in double.
 */
int bsfit_GPUmleFit_LM_multiD_f64(const float* imstack, int64_t roi_size, int64_t roi_size2,
                                  int64_t nfits, int32_t fittype, int32_t iterations,
                                  const float* coeff, int32_t coeff_ndim,
                                  const int64_t* coeff_dims, const float* varmap,
                                  int64_t varmap_numel, int32_t silent, const float* init_p,
                                  int64_t init_p_numel, const float* coeff3, int32_t coeff3_ndim,
                                  const int64_t* coeff3_dims, double* P, double* CRLB,
                                  double* LL);

/* The 4Pi fit in double (the FP64 reference-precision kernel's 4Pi form):
 * arguments as bsfit_fit4pi_device (d_dT required), double outputs P [7][nfits],
 * CRLB [6][nfits], LL [nfits]; results bit-identical to this project's double
 * restatement of the 4Pi fit (the reference ships only a compiled 4Pi mex). */
int bsfit_fit4pi_f64_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                            int64_t nfits, int32_t iterations, const float* d_dT,
                            const float* d_initZ, const float* d_initPhi, double* d_P,
                            double* d_CRLB, double* d_LL, void* stream);

/*
 * Frame -> ROI front end (the step before the fit in the reference's
 * acquisition loop, MultiD_fitter/simplefitter_cspline.m:197-319, with the peak
 * finder MultiD_fitter/shared/maximumfind2.c): photon conversion, filtering,
 * strict 3x3 non-maximum suppression, the cutoff and border filter, and the ROI
 * cut-out, on a stack of frames in device memory.
 */
typedef struct bsfit_frontend {
  float offset;      /* imphot = (frame - offset) * conversion (single precision) */
  float conversion;
  const float* kernel;  /* host, ksize x ksize filter kernel h(u, v) at kernel[u + ksize v] */
  int32_t ksize;        /* 1 .. 31 */
  int32_t subtract_first_column_min;  /* 1: filter imphot - min(imphot(:, 1)) (difference of Gaussians) */
  double cutoff;        /* keep maxima whose filtered value exceeds it */
  int32_t roi_size;     /* odd, <= 51 */
  int32_t mirror;       /* cut ROIs with x reversed */
} bsfit_frontend;

/* The reference's peak-finding kernels (simplefitter_cspline.m:197-211): mode 0
 * fspecial('gaussian', max(3, ceil(3 sigma + 1)), sigma); mode 1 the difference
 * of Gaussians of size max(ceil(6 sigma + 1), 3) with widths sigma and
 * max(1, 2.5 sigma). kernel holds at least 31 x 31 floats. Host only. */
int bsfit_peak_kernel(int32_t mode, double sigma, float* kernel, int32_t* ksize);

/* Scratch bytes for bsfit_find_rois_device. */
int64_t bsfit_find_rois_scratch_bytes(int64_t nframes, int64_t height, int64_t width);

/* d_frames: float [nframes][width][height] (MATLAB [height, width, nframes]),
 * nframes <= 65535. Writes, in the reference's order (frames, then columns,
 * then rows), up to `capacity` ROIs to d_rois ([capacity][s][s], the fitter's
 * layout) and their coordinates to d_coords (column-major [capacity x 3]: x, y
 * 1-based, frame number from 1). *n_found is the number of ROIs found, which
 * may exceed capacity (only the first `capacity` are written). d_filtered, if
 * not NULL, receives the filtered frames. Synchronises `stream` before
 * returning (for n_found). */
int bsfit_find_rois_device(const float* d_frames, int64_t nframes, int64_t height, int64_t width,
                           const bsfit_frontend* fe, float* d_rois, float* d_coords,
                           int64_t capacity, int64_t* n_found, float* d_filtered, void* d_scratch,
                           int64_t scratch_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BSFIT_H */
