// Host library behind the C ABI declared in include/bsfit.h.
//
// It replaces the reference's mex boundary for the B-spline fit types
// (VC/GPUmleFit_LM/mexFunction.cpp:208-762, VC = "MultiD_bspline/visual code"):
// the same argument checks and error classes, returned as status codes; no
// device is ever reset. Device buffers of the plain call come from the
// stream-ordered allocator, so repeated calls reuse pooled memory instead of
// allocating and freeing per call as the reference does.
#include <algorithm>
#include <initializer_list>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/bsfit.h"
#include "bsfit_internal.h"

using bsfit::FitArgs;
using bsfit::ModelDev;

struct bsfit_model_s {
  ModelDev dev;
  float* d_coeff = nullptr;
  float* d_coeff3 = nullptr;
  float4* d_zq = nullptr;  // stage-A gather table of the FP32 kernels (fit types 7, 8, 4Pi)
  // Double copies for the FP64 reference-precision fit, made on first use.
  double* d_coeff64 = nullptr;
  double* d_coeff3_64 = nullptr;
  std::mutex f64_mu;
};

namespace {

constexpr int kMaxRoi = 51;  // IMSZBIG (VC/GPUmleFit_LM/definitions.h:13)

int num_params(int fittype) {
  switch (fittype) {
    case 6: return 5;
    case 7: return 6;
    case 8: return 8;
    default: return 0;
  }
}

int coeff_rank(int fittype) { return fittype == 6 ? 3 : fittype == 7 ? 4 : 5; }

int check_coeff(int fittype, int ndim, const int64_t* dims) {
  if (!dims) return BSFIT_E_WRONG_DATA_TYPE;
  if (ndim != coeff_rank(fittype)) return BSFIT_E_COEFF_SIZE;
  for (int i = 0; i < ndim; ++i)
    if (dims[i] < 5 || dims[i] > (1 << 20)) return BSFIT_E_COEFF_SIZE;
  // The reference indexes X rows with size(coeff, 1) and clamps Y with
  // size(coeff, 2); unequal lateral sizes read outside the array there.
  if (dims[0] != dims[1]) return BSFIT_E_COEFF_SIZE;
  // offsets spanning a lateral node and up to three z planes are 32-bit in the
  // kernels
  if (dims[0] * dims[1] >= (int64_t(1) << 29)) return BSFIT_E_COEFF_SIZE;
  return BSFIT_OK;
}

void fill_model(ModelDev& m, int fittype, const int64_t* dims, const float* init_p,
                int64_t init_p_numel) {
  std::memset(&m, 0, sizeof(m));
  m.fittype = fittype;
  int r = coeff_rank(fittype);
  int64_t st = 1;
  for (int i = 0; i < 5; ++i) {
    m.cd[i] = i < r ? (int)dims[i] : 1;
    m.st[i] = st;
    st *= m.cd[i];
  }
  m.n[0] = m.cd[1] - 3;
  m.n[1] = m.cd[0] - 3;
  for (int i = 2; i < r; ++i) m.n[i] = m.cd[i] - 3;
  m.init_p_len = 0;
  if (init_p) {
    int k = (int)(init_p_numel < 4 ? init_p_numel : 4);
    for (int i = 0; i < k; ++i) m.init_p[i] = init_p[i];
    m.init_p_len = k;
  }
}

int64_t numel(int ndim, const int64_t* dims) {
  int64_t n = 1;
  for (int i = 0; i < ndim; ++i) n *= dims[i];
  return n;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return BSFIT_OK;
  if (e == cudaErrorMemoryAllocation) return BSFIT_E_NOT_ENOUGH_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return BSFIT_E_NO_DEVICE;
  return BSFIT_E_CUDA;
}

// The stage-A gather table of a model whose coefficients are on the device:
// allocated, built on the legacy default stream and waited for, so that fits
// on any stream see it.
cudaError_t make_zq(bsfit_model_s* m) {
  const int64_t n = bsfit::zq_entries(m->dev);
  if (n <= 0) return cudaSuccess;
  cudaError_t e = cudaMalloc(&m->d_zq, (size_t)n * sizeof(float4));
  if (e == cudaSuccess) e = bsfit::build_zq(m->dev, m->d_zq, nullptr);
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
  if (e == cudaSuccess) bsfit::set_zq(m->dev, m->d_zq);
  return e;
}

// Argument checks of a model (shared by bsfit_model_create and the drop-in
// call, which builds its model on a stream instead).
int check_model_args(int fittype, const float* coeff, int ndim, const int64_t* dims,
                     const float* coeff3, int ndim3, const int64_t* dims3, const float* init_p,
                     int64_t init_p_numel) {
  if (num_params(fittype) == 0) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (!coeff) return BSFIT_E_WRONG_DATA_TYPE;
  int st = check_coeff(fittype, ndim, dims);
  if (st) return st;
  if (fittype == 7 && (!init_p || init_p_numel < 2)) return BSFIT_E_INIT_P;
  if (fittype == 8) {
    // The reference leaves g2 uninitialised without initP (CPUmleFit_LM.cpp:3246-3256).
    if (!init_p || init_p_numel < 4) return BSFIT_E_INIT_P;
    if (!coeff3 || !dims3 || ndim3 != 3) return BSFIT_E_WRONG_DATA_TYPE;
    for (int i = 0; i < 3; ++i)
      if (dims3[i] != dims[i]) return BSFIT_E_COEFF_SIZE;
  }
  return BSFIT_OK;
}

// Streams and events of the synchronous drop-in call, created once per host
// thread and device (the call is synchronous, so a thread never has two in
// flight).
struct CallStreams {
  static constexpr int kEvents = 8;
  int device = -1;
  cudaStream_t copy = nullptr, comp[2] = {nullptr, nullptr};
  cudaEvent_t ev[kEvents] = {}, join = nullptr;
  ~CallStreams() { release(); }
  void release() {
    if (device < 0) return;
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return;  // runtime already gone
    for (auto* st : {&copy, &comp[0], &comp[1]})
      if (*st) cudaStreamDestroy(*st);
    for (auto& x : ev)
      if (x) cudaEventDestroy(x);
    if (join) cudaEventDestroy(join);
    device = -1;
  }
};

CallStreams* call_streams() {
  static thread_local CallStreams cs;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  if (cs.device == dev) return &cs;
  cs.release();
  bool ok = cudaStreamCreateWithFlags(&cs.copy, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&cs.comp[0], cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&cs.comp[1], cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&cs.join, cudaEventDisableTiming) == cudaSuccess;
  for (auto& x : cs.ev) ok = ok && cudaEventCreateWithFlags(&x, cudaEventDisableTiming) == cudaSuccess;
  // Keep freed blocks of this process's default pool cached instead of
  // returning them at every synchronisation, so repeated calls reuse them.
  cudaMemPool_t pool = nullptr;
  if (ok && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cs.device = dev;
  if (!ok) {
    cs.release();
    return nullptr;
  }
  return &cs;
}

// Argument checks of the synchronous drop-in calls, in the reference's order
// (mex :247-263), then the device count.
int call_checks(const float* imstack, int64_t roi_size, int64_t roi_size2, int64_t nfits,
                int fittype, bool outputs) {
  if (!imstack) return BSFIT_E_WRONG_DATA_TYPE;
  if (roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (roi_size2 != roi_size) return BSFIT_E_SUBREGION_SHAPE;
  if (roi_size < 1 || nfits < 0) return BSFIT_E_INVALID;
  if (num_params(fittype) == 0) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (!outputs) return BSFIT_E_INVALID;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count < 1) return BSFIT_E_NO_DEVICE;
  return BSFIT_OK;
}

}  // namespace

extern "C" {

const char* bsfit_status_str(int status) {
  switch (status) {
    case BSFIT_OK: return "ok";
    case BSFIT_E_WRONG_NO_ARGS:
      return "Inputs must include: GPUmleFit_LM(data,fittype,iterations,startparameter,var,silent)";
    case BSFIT_E_WRONG_DATA_TYPE: return "Data must be comprised of single floats (missing array)";
    case BSFIT_E_SUBREGION_SIZE: return "X,Y dimension of data must be smaller than 51";
    case BSFIT_E_SUBREGION_SHAPE: return "Fit Box must be square";
    case BSFIT_E_UNSUPPORTED_FITTYPE: return "fit type not supported (B-spline fit types are 6, 7, 8)";
    case BSFIT_E_NOT_ENOUGH_MEMORY: return "Not enough memory on the GPU";
    case BSFIT_E_CUDA: return "CUDA call failed";
    case BSFIT_E_NO_DEVICE: return "No CUDA capable devices were detected";
    case BSFIT_E_COEFF_SIZE: return "coefficient array has the wrong rank or size";
    case BSFIT_E_INIT_P: return "initP missing or too short for this fit type";
    case BSFIT_E_INVALID: return "invalid argument";
    case BSFIT_E_TIMEOUT: return "bounded device wait timed out";
    case BSFIT_E_STATIC_LIMIT:
      return "too many segments for the allocation-free entry point (its fixed scratch holds 48)";
    case BSFIT_E_UNSHARED:
      return "4Pi fit: only four channels with all six parameters shared are supported";
    default: return "unknown status";
  }
}

const char* bsfit_version(void) { return "bsfit-gb300 0.1 (sm_103a)"; }

int bsfit_num_params(int32_t fittype) { return num_params(fittype); }

int bsfit_measure_fp32_peak(double* tflops) {
  if (!tflops) return BSFIT_E_INVALID;
  return cuda_status(bsfit::measure_fp32_peak(tflops));
}

int bsfit_measure_fp32_peaks(double* scalar_tflops, double* paired_tflops) {
  if (!scalar_tflops || !paired_tflops) return BSFIT_E_INVALID;
  return cuda_status(bsfit::measure_fp32_peak2(scalar_tflops, paired_tflops));
}

int bsfit_model_create(int32_t fittype, const float* coeff, int32_t coeff_ndim,
                       const int64_t* coeff_dims, const float* coeff3, int32_t coeff3_ndim,
                       const int64_t* coeff3_dims, const float* init_p, int64_t init_p_numel,
                       bsfit_model* out) {
  if (!out) return BSFIT_E_INVALID;
  *out = nullptr;
  int st = check_model_args(fittype, coeff, coeff_ndim, coeff_dims, coeff3, coeff3_ndim,
                            coeff3_dims, init_p, init_p_numel);
  if (st) return st;
  bsfit_model_s* m = new (std::nothrow) bsfit_model_s;
  if (!m) return BSFIT_E_NOT_ENOUGH_MEMORY;
  fill_model(m->dev, fittype, coeff_dims, init_p, init_p_numel);
  size_t bytes = (size_t)numel(coeff_ndim, coeff_dims) * sizeof(float);
  cudaError_t e = cudaMalloc(&m->d_coeff, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_coeff, coeff, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && fittype == 8) {
    size_t b3 = (size_t)numel(3, coeff3_dims) * sizeof(float);
    e = cudaMalloc(&m->d_coeff3, b3);
    if (e == cudaSuccess) e = cudaMemcpy(m->d_coeff3, coeff3, b3, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    cudaFree(m->d_coeff);
    cudaFree(m->d_coeff3);
    delete m;
    return cuda_status(e);
  }
  m->dev.coeff = m->d_coeff;
  m->dev.coeff3 = m->d_coeff3;
  e = make_zq(m);
  if (e != cudaSuccess) {
    cudaFree(m->d_coeff);
    cudaFree(m->d_coeff3);
    cudaFree(m->d_zq);
    delete m;
    return cuda_status(e);
  }
  *out = m;
  return BSFIT_OK;
}

int32_t bsfit_model_fittype(bsfit_model model) { return model ? model->dev.fittype : 0; }

int bsfit_model_release(bsfit_model model) {
  if (!model) return BSFIT_E_INVALID;
  cudaFree(model->d_coeff);
  cudaFree(model->d_coeff3);
  cudaFree(model->d_zq);
  cudaFree(model->d_coeff64);
  cudaFree(model->d_coeff3_64);
  delete model;
  return BSFIT_OK;
}

int bsfit_fit_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                     int32_t iterations, float* d_P, float* d_CRLB, float* d_LL, void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype == bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.out_n = nfits;
  a.out_offset = 0;
  a.trace = nullptr;
  a.trace_max = 0;
  a.flags = 0;
  return cuda_status(bsfit::launch_fit(a, (cudaStream_t)stream));
}

int bsfit_trace_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                       int32_t iterations, int32_t flags, float* d_P, float* d_CRLB, float* d_LL,
                       float* d_trace, int32_t trace_max, void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype == bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0 || trace_max < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_P || !d_CRLB || !d_LL || (trace_max > 0 && !d_trace)) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.out_n = nfits;
  a.trace = d_trace;
  a.trace_max = trace_max;
  a.flags = flags;
  return cuda_status(bsfit::launch_fit(a, (cudaStream_t)stream));
}

int bsfit_eval_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                      const float* d_theta, int32_t fisher, float* d_out, void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype == bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_theta || !d_out) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  return cuda_status(bsfit::launch_eval(a, d_theta, d_out, fisher, (cudaStream_t)stream));
}

int bsfit_eval_parity_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                             int64_t nfits, const float* d_theta, int32_t fisher, double* d_out,
                             void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype == bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_theta || !d_out) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  return cuda_status(bsfit::launch_evaldd(a, d_theta, d_out, fisher, (cudaStream_t)stream));
}

int64_t bsfit_batch_scratch_bytes(int32_t nseg) {
  if (nseg < 0) return 0;
  return (((int64_t)nseg * 2 * 8) + 255) / 256 * 256;
}

}  // extern "C"

namespace {

// The batched fit behind bsfit_batch_fit_device (starts null) and
// bsfit_batch_fit_multistart_device (starts[i] for segment i). warp_rois: the
// ROIs a warp fits before it ends (BatchArgs::warp_rois; 0: persistent; -1:
// the per-fit-type caps of batch_fit_capped).
int batch_fit(const bsfit_segment* segs, const bsfit_starts* starts, int32_t nseg,
              void* d_scratch, int64_t scratch_bytes, void* stream, int warp_rois = 0) {
  if (nseg < 0 || nseg > BSFIT_MAX_SEGMENTS) return BSFIT_E_INVALID;
  if (nseg == 0) return BSFIT_OK;
  if (!segs || !d_scratch || scratch_bytes < bsfit_batch_scratch_bytes(nseg)) return BSFIT_E_INVALID;
  for (int i = 0; i < nseg; ++i) {
    const bsfit_segment& g = segs[i];
    if (!g.model) return BSFIT_E_INVALID;
    if (g.model->dev.fittype == bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
    if (g.roi_size < 1 || g.roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
    if (g.nfits < 0) return BSFIT_E_INVALID;
    if (g.nfits > 0 && (!g.d_rois || !g.d_P || !g.d_CRLB || !g.d_LL)) return BSFIT_E_INVALID;
    if (starts) {
      const bsfit_starts& q = starts[i];
      if (q.n_starts < 0 || q.n_starts > BSFIT_MAX_STARTS) return BSFIT_E_INVALID;
      // fit type 6 has no initP: one start, fitted by the single-start kernel
      if (g.model->dev.fittype == 6 && q.n_starts > 1) return BSFIT_E_UNSUPPORTED_FITTYPE;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* next = (unsigned long long*)d_scratch;
  unsigned long long* done = next + nseg;
  cudaError_t e = cudaMemsetAsync(d_scratch, 0, (size_t)nseg * 2 * 8, st);
  if (e != cudaSuccess) return cuda_status(e);
  // One persistent launch per fit type; within it, segments by decreasing
  // cost (pixels x iteration cap) so the longest fits start first.
  for (int mode = 6; mode <= 8; ++mode) {
    bsfit::BatchArgs a;
    std::memset(&a, 0, sizeof(a));
    int order[BSFIT_MAX_SEGMENTS];
    int k = 0;
    for (int i = 0; i < nseg; ++i)
      if (segs[i].model->dev.fittype == mode && segs[i].nfits > 0) order[k++] = i;
    if (k == 0) continue;
    for (int x = 1; x < k; ++x)
      for (int y = x; y > 0; --y) {
        const bsfit_segment& p0 = segs[order[y - 1]];
        const bsfit_segment& p1 = segs[order[y]];
        if (p0.roi_size * p0.roi_size * (int64_t)p0.iterations <
            p1.roi_size * p1.roi_size * (int64_t)p1.iterations) {
          int t = order[y - 1];
          order[y - 1] = order[y];
          order[y] = t;
        }
      }
    a.nseg = k;
    a.next = next;
    a.done = done;
    a.flags = 0;
    a.warp_rois = warp_rois >= 0 ? warp_rois : (mode == 6 ? 4 : mode == 7 ? 2 : 1);
    for (int j = 0; j < k; ++j) {
      const bsfit_segment& g = segs[order[j]];
      bsfit::BatchSeg& b = a.seg[j];
      b.m = g.model->dev;
      b.rois = g.d_rois;
      b.P = g.d_P;
      b.CRLB = g.d_CRLB;
      b.LL = g.d_LL;
      b.n = g.nfits;
      b.s = (int)g.roi_size;
      b.iterations = g.iterations;
      b.slot = order[j];  // counters stay in the caller's segment order
      if (starts) {
        const bsfit_starts& q = starts[order[j]];
        b.n_starts = q.n_starts;
        b.strict = q.strict ? 1 : 0;
        for (int k = 0; k < q.n_starts; ++k)
          for (int c = 0; c < 4; ++c) b.starts[k][c] = q.initp[k][c];
      }
      if (b.s > a.s_max) a.s_max = b.s;
    }
    e = bsfit::launch_batch(a, mode, starts != nullptr && mode != 6, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return BSFIT_OK;
}

}  // namespace

namespace bsfit {
// The serving loop's batched fit: capped, the warps of each fit type's launch
// end after a few ROIs (3D 4, 4D 2, 5D 1: about 0.1 to 1.5 ms of a warp), so
// the blocks of a long launch retire while it runs.
int batch_fit_capped(const bsfit_segment* segs, const bsfit_starts* starts, int32_t nseg,
                     void* d_scratch, int64_t scratch_bytes, void* stream, bool capped) {
  return batch_fit(segs, starts, nseg, d_scratch, scratch_bytes, stream, capped ? -1 : 0);
}
}  // namespace bsfit

extern "C" {

int bsfit_batch_fit_device(const bsfit_segment* segs, int32_t nseg, void* d_scratch,
                           int64_t scratch_bytes, void* stream) {
  return batch_fit(segs, nullptr, nseg, d_scratch, scratch_bytes, stream);
}

int bsfit_batch_fit_multistart_device(const bsfit_segment* segs, const bsfit_starts* starts,
                                      int32_t nseg, void* d_scratch, int64_t scratch_bytes,
                                      void* stream) {
  if (!starts) return BSFIT_E_INIT_P;
  return batch_fit(segs, starts, nseg, d_scratch, scratch_bytes, stream);
}

}  // extern "C"

namespace {

// The synchronous drop-in call of the FP32 kernels (bsfit_GPUmleFit_LM_multiD).
int multid_call(const float* imstack, int64_t roi_size, int64_t roi_size2, int64_t nfits,
                int32_t fittype, int32_t iterations, const float* coeff, int32_t coeff_ndim,
                const int64_t* coeff_dims, int32_t silent, const float* init_p,
                int64_t init_p_numel, const float* coeff3, int32_t coeff3_ndim,
                const int64_t* coeff3_dims, float* P, float* CRLB, float* LL) {
  int st = call_checks(imstack, roi_size, roi_size2, nfits, fittype, P && CRLB && LL);
  if (st) return st;
  const int nv = num_params(fittype);
  if (!silent) {
    std::printf("subregion size: %lld fittype: %d\n", (long long)roi_size, fittype);
    std::printf("Number of fits: %lld no padding\n", (long long)nfits);
  }
  st = check_model_args(fittype, coeff, coeff_ndim, coeff_dims, coeff3, coeff3_ndim,
                        coeff3_dims, init_p, init_p_numel);
  if (st) return st;
  if (nfits == 0) return BSFIT_OK;
  // Memory check (mex :409-456): refuse work above 95% of free memory.
  const size_t s2 = (size_t)roi_size * roi_size;
  const size_t in_bytes = (size_t)nfits * s2 * sizeof(float);
  const size_t out_bytes = (size_t)nfits * (2 * nv + 2) * sizeof(float);
  const size_t c_bytes = (size_t)numel(coeff_ndim, coeff_dims) * sizeof(float);
  const size_t c3_bytes = fittype == 8 ? (size_t)numel(3, coeff3_dims) * sizeof(float) : 0;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
      (double)(in_bytes + out_bytes + c_bytes + c3_bytes) > 0.95 * (double)free_b)
    return BSFIT_E_NOT_ENOUGH_MEMORY;
  // Pipeline: a copy stream uploads the coefficients and the ROIs chunk by
  // chunk; two compute streams fit the chunks alternately as their uploads
  // land, so chunk i + 1 uploads while chunk i fits and the tail of one fit
  // launch overlaps the start of the next. The first chunk is small, so the
  // first fit starts after a short upload, and the chunks double from there
  // (uploads run several times faster than fits, so they stay ahead). Each
  // chunk's results go back to the host as soon as its fit ends, one strided
  // copy per output (the outputs are column-major over all ROIs), so only the
  // last chunk's copy remains after the last fit. Device buffers come from the
  // stream-ordered pool, so repeated calls allocate nothing.
  CallStreams* cs = call_streams();
  if (!cs) return BSFIT_E_CUDA;
  cudaStream_t cp = cs->copy, c0 = cs->comp[0], c1 = cs->comp[1];
  int64_t cb[CallStreams::kEvents + 1];
  int nchunk = 0;
  {
    const int64_t first_chunk = 16384;
    int64_t b = 0, c = first_chunk;
    while (b < nfits && nchunk < CallStreams::kEvents) {
      cb[nchunk++] = b;
      b += c;
      c *= 2;
    }
    cb[nchunk] = nfits;
  }
  float *d_rois = nullptr, *d_out = nullptr, *d_c = nullptr, *d_c3 = nullptr;
  float4* d_zq = nullptr;
  cudaError_t e = cudaMallocAsync(&d_rois, in_bytes, cp);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_out, out_bytes, cp);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_c, c_bytes, cp);
  if (e == cudaSuccess && c3_bytes) e = cudaMallocAsync(&d_c3, c3_bytes, cp);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_c, coeff, c_bytes, cudaMemcpyHostToDevice, cp);
  if (e == cudaSuccess && c3_bytes)
    e = cudaMemcpyAsync(d_c3, coeff3, c3_bytes, cudaMemcpyHostToDevice, cp);
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  fill_model(a.m, fittype, coeff_dims, init_p, init_p_numel);
  a.m.coeff = d_c;
  a.m.coeff3 = d_c3;
  // the stage-A gather table, built on the copy stream after the upload (every
  // chunk's fit waits for an event recorded on that stream after it)
  const int64_t zq_n = bsfit::zq_entries(a.m);
  if (e == cudaSuccess && zq_n > 0) e = cudaMallocAsync(&d_zq, (size_t)zq_n * sizeof(float4), cp);
  if (e == cudaSuccess && zq_n > 0) e = bsfit::build_zq(a.m, d_zq, cp);
  bsfit::set_zq(a.m, d_zq);
  a.s = (int)roi_size;
  a.iterations = iterations;
  a.P = d_out;
  a.CRLB = d_out + (size_t)nfits * (nv + 1);
  a.LL = a.CRLB + (size_t)nfits * nv;
  a.out_n = nfits;
  for (int i = 0; i < nchunk && e == cudaSuccess; ++i) {
    const int64_t b = cb[i], n = cb[i + 1] - b;
    e = cudaMemcpyAsync(d_rois + (size_t)b * s2, imstack + (size_t)b * s2, (size_t)n * s2 * 4,
                        cudaMemcpyHostToDevice, cp);
    if (e == cudaSuccess) e = cudaEventRecord(cs->ev[i], cp);
    cudaStream_t cs_i = (i & 1) ? c1 : c0;
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cs_i, cs->ev[i], 0);
    if (e == cudaSuccess) {
      a.rois = d_rois + (size_t)b * s2;
      a.nfits = n;
      a.out_offset = b;
      e = bsfit::launch_fit(a, cs_i);
    }
  }
  // Results of each chunk, on the stream that fitted it (enqueued after every
  // launch: a copy into pageable host memory returns only when it is done).
  const size_t ld = (size_t)nfits * sizeof(float);
  for (int i = 0; i < nchunk && e == cudaSuccess; ++i) {
    const int64_t b = cb[i], n = cb[i + 1] - b;
    cudaStream_t cs_i = (i & 1) ? c1 : c0;
    e = cudaMemcpy2DAsync(P + b, ld, a.P + b, ld, (size_t)n * sizeof(float), nv + 1,
                          cudaMemcpyDeviceToHost, cs_i);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(CRLB + b, ld, a.CRLB + b, ld, (size_t)n * sizeof(float), nv,
                            cudaMemcpyDeviceToHost, cs_i);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(LL + b, a.LL + b, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, cs_i);
  }
  // Join before the buffers are freed on c0, on the error path too: c0 waits
  // for c1 (its last copies, or the kernels of chunks already launched there
  // when a later step failed) and for the copy stream, which allocated the
  // buffers. Where the join itself cannot be enqueued, the host waits for that
  // stream instead, so no freed block is still in use by a kernel or copy.
  for (cudaStream_t other : {c1, cp}) {
    if (cudaEventRecord(cs->join, other) != cudaSuccess ||
        cudaStreamWaitEvent(c0, cs->join, 0) != cudaSuccess) {
      const cudaError_t es = cudaStreamSynchronize(other);
      if (e == cudaSuccess) e = es;
    }
  }
  if (d_rois) cudaFreeAsync(d_rois, c0);
  if (d_out) cudaFreeAsync(d_out, c0);
  if (d_c) cudaFreeAsync(d_c, c0);
  if (d_c3) cudaFreeAsync(d_c3, c0);
  if (d_zq) cudaFreeAsync(d_zq, c0);
  cudaError_t e2 = cudaStreamSynchronize(c0);
  if (e == cudaSuccess) e = e2;
  return cuda_status(e);
}

}  // namespace

extern "C" {

int bsfit_GPUmleFit_LM_multiD(const float* imstack, int64_t roi_size, int64_t roi_size2,
                              int64_t nfits, int32_t fittype, int32_t iterations,
                              const float* coeff, int32_t coeff_ndim, const int64_t* coeff_dims,
                              const float* varmap, int64_t varmap_numel, int32_t silent,
                              const float* init_p, int64_t init_p_numel, const float* coeff3,
                              int32_t coeff3_ndim, const int64_t* coeff3_dims, float* P,
                              float* CRLB, float* LL) {
  (void)varmap;
  (void)varmap_numel;  // ignored for fit types 6-8, as in the reference
  return multid_call(imstack, roi_size, roi_size2, nfits, fittype, iterations, coeff, coeff_ndim,
                     coeff_dims, silent, init_p, init_p_numel, coeff3, coeff3_ndim, coeff3_dims, P,
                     CRLB, LL);
}

// ---------------------------------------------------------------------------
// 4Pi fit (GPUmleFit_LM_4Pi_bspline, demo_4pi/bspline_based_4piloc_v4.m:196-216).

int bsfit_model_create_4pi(const float* coeff, int32_t coeff_ndim, const int64_t* coeff_dims,
                           const float* phase_shift, int32_t n_channels, bsfit_model* out) {
  if (!out) return BSFIT_E_INVALID;
  *out = nullptr;
  if (!coeff || !phase_shift) return BSFIT_E_WRONG_DATA_TYPE;
  if (n_channels != bsfit::k4PiChannels) return BSFIT_E_UNSHARED;
  int st = check_coeff(7, coeff_ndim, coeff_dims);  // a 4D array, as for fit type 7
  if (st) return st;
  for (int c = 0; c < bsfit::k4PiChannels; ++c)
    if (!(phase_shift[c] == phase_shift[c]) || phase_shift[c] > 1e6f || phase_shift[c] < -1e6f)
      return BSFIT_E_INVALID;
  bsfit_model_s* m = new (std::nothrow) bsfit_model_s;
  if (!m) return BSFIT_E_NOT_ENOUGH_MEMORY;
  fill_model(m->dev, 7, coeff_dims, nullptr, 0);
  m->dev.fittype = bsfit::kFit4Pi;
  for (int c = 0; c < bsfit::k4PiChannels; ++c) m->dev.shift[c] = phase_shift[c];
  const size_t bytes = (size_t)numel(coeff_ndim, coeff_dims) * sizeof(float);
  cudaError_t e = cudaMalloc(&m->d_coeff, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_coeff, coeff, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(m->d_coeff);
    delete m;
    return cuda_status(e);
  }
  m->dev.coeff = m->d_coeff;
  e = make_zq(m);
  if (e != cudaSuccess) {
    cudaFree(m->d_coeff);
    cudaFree(m->d_zq);
    delete m;
    return cuda_status(e);
  }
  *out = m;
  return BSFIT_OK;
}

int bsfit_fit4pi_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                        int32_t iterations, const float* d_dT, const float* d_initZ,
                        const float* d_initPhi, float* d_P, float* d_CRLB, float* d_LL,
                        void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype != bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_initZ || !d_initPhi || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.out_n = nfits;
  a.dT = d_dT;
  a.z0 = d_initZ;
  a.w0 = d_initPhi;
  return cuda_status(bsfit::launch_fit(a, (cudaStream_t)stream));
}

int bsfit_eval4pi_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                         const float* d_dT, const float* d_theta, int32_t fisher, float* d_out,
                         void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype != bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_theta || !d_out) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.dT = d_dT;
  return cuda_status(bsfit::launch_eval(a, d_theta, d_out, fisher, (cudaStream_t)stream));
}

int bsfit_GPUmleFit_LM_4Pi_bspline(const float* imstack, int64_t roi_size, int64_t roi_size2,
                                   int64_t nfits, int64_t n_channels, const uint32_t* shared,
                                   int64_t shared_numel, int32_t iterations, const float* coeff,
                                   int32_t coeff_ndim, const int64_t* coeff_dims, const float* dT,
                                   int64_t dT_numel, const float* initZ, int64_t initZ_numel,
                                   const float* initPhi, int64_t initPhi_numel,
                                   const float* phase_shift, int64_t phase_shift_numel,
                                   int32_t silent, float* P, float* CRLB, float* LL) {
  constexpr int NV = 6, C = bsfit::k4PiChannels;
  if (!imstack || !coeff || !dT || !initZ || !initPhi || !phase_shift || !shared)
    return BSFIT_E_WRONG_DATA_TYPE;
  if (roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (roi_size2 != roi_size) return BSFIT_E_SUBREGION_SHAPE;
  if (roi_size < 1 || nfits < 0) return BSFIT_E_INVALID;
  if (n_channels != C || phase_shift_numel != C) return BSFIT_E_UNSHARED;
  if (shared_numel != NV) return BSFIT_E_UNSHARED;
  for (int i = 0; i < NV; ++i)
    if (shared[i] != 1u) return BSFIT_E_UNSHARED;
  if (dT_numel != (int64_t)NV * C * nfits || initZ_numel != nfits || initPhi_numel != nfits)
    return BSFIT_E_WRONG_NO_ARGS;
  if (!P || !CRLB || !LL) return BSFIT_E_INVALID;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count < 1) return BSFIT_E_NO_DEVICE;
  if (!silent) {
    std::printf("subregion size: %lld channels: %d\n", (long long)roi_size, C);
    std::printf("Number of fits: %lld no padding\n", (long long)nfits);
  }
  bsfit_model model = nullptr;
  int st = bsfit_model_create_4pi(coeff, coeff_ndim, coeff_dims, phase_shift, C, &model);
  if (st) return st;
  if (nfits == 0) {
    bsfit_model_release(model);
    return BSFIT_OK;
  }
  const size_t s2 = (size_t)roi_size * roi_size;
  const size_t in_floats = (size_t)nfits * (s2 * C + NV * C + 2);
  const size_t out_floats = (size_t)nfits * (2 * NV + 2);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
      (double)((in_floats + out_floats) * sizeof(float)) > 0.95 * (double)free_b) {
    bsfit_model_release(model);
    return BSFIT_E_NOT_ENOUGH_MEMORY;
  }
  cudaStream_t stream = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  float *d_in = nullptr, *d_out = nullptr;
  if (e == cudaSuccess) e = cudaMallocAsync(&d_in, in_floats * sizeof(float), stream);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_out, out_floats * sizeof(float), stream);
  float* d_rois = d_in;
  float* d_dT = d_rois + (size_t)nfits * s2 * C;
  float* d_z = d_dT + (size_t)nfits * NV * C;
  float* d_w = d_z + nfits;
  // MATLAB [s, s, N, 4] and [6, 4, N] are exactly the device layouts.
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_rois, imstack, (size_t)nfits * s2 * C * sizeof(float),
                        cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_dT, dT, (size_t)nfits * NV * C * sizeof(float), cudaMemcpyHostToDevice,
                        stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_z, initZ, (size_t)nfits * sizeof(float), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_w, initPhi, (size_t)nfits * sizeof(float), cudaMemcpyHostToDevice,
                        stream);
  float* d_P = d_out;
  float* d_C = d_P + (size_t)nfits * (NV + 1);
  float* d_L = d_C + (size_t)nfits * NV;
  if (e == cudaSuccess) {
    st = bsfit_fit4pi_device(model, d_rois, roi_size, nfits, iterations, d_dT, d_z, d_w, d_P,
                             d_C, d_L, stream);
    if (st) e = cudaErrorUnknown;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(P, d_P, (size_t)nfits * (NV + 1) * sizeof(float), cudaMemcpyDeviceToHost,
                        stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(CRLB, d_C, (size_t)nfits * NV * sizeof(float), cudaMemcpyDeviceToHost,
                        stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(LL, d_L, (size_t)nfits * sizeof(float), cudaMemcpyDeviceToHost, stream);
  if (d_in) cudaFreeAsync(d_in, stream);
  if (d_out) cudaFreeAsync(d_out, stream);
  cudaError_t e2 = stream ? cudaStreamSynchronize(stream) : cudaSuccess;
  if (stream) cudaStreamDestroy(stream);
  bsfit_model_release(model);
  if (st) return st;
  if (e == cudaSuccess) e = e2;
  return cuda_status(e);
}

// ---------------------------------------------------------------------------
// Multi-start, fused: every ROI fitted from each start in one launch, the ROI
// staged once, the best log-likelihood kept (the callers' loop at
// MultiD_fitter/simplefitter_cspline.m:463-490, demo_orientation/store/fitb5n3.m:15-46,
// demo_4pi/bspline_based_4piloc_v4.m:193-215).

int bsfit_fit_multistart_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                                int64_t nfits, int32_t iterations, const float* init_p_starts,
                                int32_t start_len, int32_t n_starts, int32_t strict, float* d_P,
                                float* d_CRLB, float* d_LL, void* stream) {
  if (!model) return BSFIT_E_INVALID;
  const int ft = model->dev.fittype;
  if (ft != 7 && ft != 8) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0 || n_starts < 1 || n_starts > bsfit::kMaxStarts) return BSFIT_E_INVALID;
  if (!init_p_starts || start_len < (ft == 7 ? 2 : 4) || start_len > 64) return BSFIT_E_INIT_P;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.out_n = nfits;
  a.n_starts = n_starts;
  a.strict = strict ? 1 : 0;
  for (int k = 0; k < n_starts; ++k)
    for (int i = 0; i < 4; ++i)
      a.starts[k][i] = i < start_len ? init_p_starts[(int64_t)k * start_len + i] : 0.0f;
  return cuda_status(bsfit::launch_fit(a, (cudaStream_t)stream));
}

int bsfit_fit4pi_multistart_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                                   int64_t nfits, int32_t iterations, const float* d_dT,
                                   const float* d_initZ, const float* d_initPhi, int32_t n_starts,
                                   int32_t strict, float* d_P, float* d_CRLB, float* d_LL,
                                   void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype != bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0 || n_starts < 1 || n_starts > bsfit::kMaxStarts) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_initZ || !d_initPhi || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.out_n = nfits;
  a.dT = d_dT;
  a.z0 = d_initZ;
  a.w0 = d_initPhi;
  a.n_starts = n_starts;
  a.strict = strict ? 1 : 0;
  return cuda_status(bsfit::launch_fit(a, (cudaStream_t)stream));
}

// ---------------------------------------------------------------------------
// sCMOS likelihood for the B-spline fit types (the variance map, which the
// reference's B-spline branch ignores, applied as its sCMOS kernels of the
// other fit types do, VC/GPUmleFit_LM/GPUmleFit_LM_sCMOS.cu:1045-1046).

int bsfit_fit_scmos_device(bsfit_model model, const float* d_rois, const float* d_var,
                           int64_t roi_size, int64_t nfits, int32_t iterations, float* d_P,
                           float* d_CRLB, float* d_LL, void* stream) {
  if (!model) return BSFIT_E_INVALID;
  const int ft = model->dev.fittype;
  if (ft != 6 && ft != 7 && ft != 8) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_var || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.var = d_var;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.out_n = nfits;
  return cuda_status(bsfit::launch_fit(a, (cudaStream_t)stream));
}

// ---------------------------------------------------------------------------
// FP64 reference-precision fit: the reference method in double with its order
// of operations (the float build of the reference and the FP32 kernels take
// some LM decisions differently from the double build; this one follows it).

}  // extern "C"

namespace {

// The double tables of a model (values and neighbour differences per axis),
// made on first use and kept with the model.
int ensure_f64_tables(bsfit_model model, cudaStream_t st) {
  const ModelDev& m = model->dev;
  const int ft = m.fittype;
  int64_t total = 1;
  for (int i = 0; i < 5; ++i) total *= m.cd[i];
  const int64_t total3 = (int64_t)m.cd[0] * m.cd[1] * m.cd[2];
  {
    std::lock_guard<std::mutex> lock(model->f64_mu);
    if (!model->d_coeff64) {
      double *c = nullptr, *c3 = nullptr;
      const int D = ft == 6 ? 3 : ft == 8 ? 5 : 4;  // 4: fit type 7 and 4Pi
      cudaError_t e = cudaMalloc(&c, (size_t)(D + 1) * total * sizeof(double));
      if (e == cudaSuccess) e = bsfit::widen_to_f64(model->d_coeff, c, total, D, m.st, st);
      if (e == cudaSuccess && ft == 8) {
        e = cudaMalloc(&c3, (size_t)4 * total3 * sizeof(double));
        if (e == cudaSuccess) e = bsfit::widen_to_f64(model->d_coeff3, c3, total3, 3, m.st, st);
      }
      // Other threads may use the copies on other streams once published.
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        cudaFree(c);
        cudaFree(c3);
        return cuda_status(e);
      }
      model->d_coeff3_64 = c3;
      model->d_coeff64 = c;
    }
  }
  return BSFIT_OK;
}

}  // namespace

extern "C" {

int bsfit_fit_f64_device(bsfit_model model, const float* d_rois, const float* d_var,
                         int64_t roi_size, int64_t nfits, int32_t iterations, double* d_P,
                         double* d_CRLB, double* d_LL, void* stream) {
  if (!model) return BSFIT_E_INVALID;
  const int ft = model->dev.fittype;
  if (ft != 6 && ft != 7 && ft != 8) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  const ModelDev& m = model->dev;
  int64_t total = 1;
  for (int i = 0; i < 5; ++i) total *= m.cd[i];
  const int64_t total3 = (int64_t)m.cd[0] * m.cd[1] * m.cd[2];
  cudaStream_t st = (cudaStream_t)stream;
  const int rc = ensure_f64_tables(model, st);
  if (rc != BSFIT_OK) return rc;
  bsfit::Fit64Args a;
  std::memset(&a, 0, sizeof(a));
  a.m = m;
  a.c = model->d_coeff64;
  a.c3 = model->d_coeff3_64;
  a.total = total;
  a.total3 = total3;
  a.rois = d_rois;
  a.var = d_var;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  return cuda_status(bsfit::launch_fit64(a, st));
}

}  // extern "C"

namespace {

// Leading LM steps of the parity-grade fit taken by the FP64 reference-order
// kernel, per fit type (6, 7, 8): fit type 7's initial Hessian is exactly
// singular (its initial pass copies dudt[4] into dudt[5], CPUmleFit_LM.cpp:2893),
// so its first step is set by the rounding of the reference's double sums and
// is taken in that arithmetic.
int default_exact_steps(int fittype) { return fittype == 7 ? 1 : 0; }

int parity_fit(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
               int32_t iterations, int32_t exact_steps, float* d_P, float* d_CRLB, float* d_LL,
               void* stream) {
  if (!model) return BSFIT_E_INVALID;
  const int ft = model->dev.fittype;
  if (ft != 6 && ft != 7 && ft != 8) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0 || exact_steps < -1) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  if (exact_steps < 0) exact_steps = default_exact_steps(ft);
  cudaStream_t st = (cudaStream_t)stream;
  FitArgs a;
  std::memset(&a, 0, sizeof(a));
  a.m = model->dev;
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.out_n = nfits;
  a.flags = bsfit::FLAG_PARITY;
  if (exact_steps == 0 || iterations <= 0)
    return cuda_status(bsfit::launch_fit(a, st));
  // FP64 reference-order pre-pass: the initial evaluation and the first
  // exact_steps LM steps of every ROI, handed over through a pooled buffer.
  const int rc = ensure_f64_tables(model, st);
  if (rc != BSFIT_OK) return rc;
  const ModelDev& m = model->dev;
  double* handoff = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&handoff),
                                  (size_t)nfits * bsfit::kHandoffStride * sizeof(double), st);
  if (e != cudaSuccess) return cuda_status(e);
  bsfit::Fit64Args f;
  std::memset(&f, 0, sizeof(f));
  f.m = m;
  f.c = model->d_coeff64;
  f.c3 = model->d_coeff3_64;
  f.total = 1;
  for (int i = 0; i < 5; ++i) f.total *= m.cd[i];
  f.total3 = (int64_t)m.cd[0] * m.cd[1] * m.cd[2];
  f.rois = d_rois;
  f.s = (int)roi_size;
  f.nfits = nfits;
  f.iterations = iterations;
  f.handoff = handoff;
  f.handoff_iters = exact_steps;
  e = bsfit::launch_fit64(f, st);
  if (e == cudaSuccess) {
    a.handoff = handoff;
    e = bsfit::launch_fit(a, st);
  }
  cudaFreeAsync(handoff, st);
  return cuda_status(e);
}

}  // namespace

extern "C" {

int bsfit_fit_parity_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                            int64_t nfits, int32_t iterations, float* d_P, float* d_CRLB,
                            float* d_LL, void* stream) {
  return parity_fit(model, d_rois, roi_size, nfits, iterations, -1, d_P, d_CRLB, d_LL, stream);
}

int bsfit_fit_parity_steps_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                                  int64_t nfits, int32_t iterations, int32_t exact_steps,
                                  float* d_P, float* d_CRLB, float* d_LL, void* stream) {
  return parity_fit(model, d_rois, roi_size, nfits, iterations, exact_steps, d_P, d_CRLB, d_LL,
                    stream);
}

// The drop-in call of the parity-grade fit: the arguments and checks of
// bsfit_GPUmleFit_LM_multiD, float outputs from bsfit_fit_parity_device.
int bsfit_GPUmleFit_LM_multiD_parity(const float* imstack, int64_t roi_size, int64_t roi_size2,
                                     int64_t nfits, int32_t fittype, int32_t iterations,
                                     const float* coeff, int32_t coeff_ndim,
                                     const int64_t* coeff_dims, const float* varmap,
                                     int64_t varmap_numel, int32_t silent, const float* init_p,
                                     int64_t init_p_numel, const float* coeff3,
                                     int32_t coeff3_ndim, const int64_t* coeff3_dims, float* P,
                                     float* CRLB, float* LL) {
  (void)varmap;
  (void)varmap_numel;
  int st = call_checks(imstack, roi_size, roi_size2, nfits, fittype, P && CRLB && LL);
  if (st) return st;
  const int nv = num_params(fittype);
  if (!silent) {
    std::printf("subregion size: %lld fittype: %d\n", (long long)roi_size, fittype);
    std::printf("Number of fits: %lld no padding\n", (long long)nfits);
  }
  bsfit_model model = nullptr;
  st = bsfit_model_create(fittype, coeff, coeff_ndim, coeff_dims, coeff3, coeff3_ndim,
                          coeff3_dims, init_p, init_p_numel, &model);
  if (st) return st;
  if (nfits == 0) return bsfit_model_release(model);
  CallStreams* cs = call_streams();
  if (!cs) {
    bsfit_model_release(model);
    return BSFIT_E_CUDA;
  }
  cudaStream_t cst = cs->comp[0];
  const size_t s2 = (size_t)roi_size * roi_size;
  const size_t in_bytes = (size_t)nfits * s2 * sizeof(float);
  const size_t nout = (size_t)nfits * (2 * nv + 2);
  float* d_rois = nullptr;
  float* d_out = nullptr;
  cudaError_t e = cudaMallocAsync(&d_rois, in_bytes, cst);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_out, nout * sizeof(float), cst);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_rois, imstack, in_bytes, cudaMemcpyHostToDevice, cst);
  int rc = BSFIT_OK;
  float* dP = d_out;
  float* dC = d_out + (size_t)nfits * (nv + 1);
  float* dL = dC + (size_t)nfits * nv;
  if (e == cudaSuccess) rc = parity_fit(model, d_rois, roi_size, nfits, iterations, -1, dP, dC, dL, cst);
  if (e == cudaSuccess && rc == BSFIT_OK)
    e = cudaMemcpyAsync(P, dP, (size_t)nfits * (nv + 1) * sizeof(float), cudaMemcpyDeviceToHost, cst);
  if (e == cudaSuccess && rc == BSFIT_OK)
    e = cudaMemcpyAsync(CRLB, dC, (size_t)nfits * nv * sizeof(float), cudaMemcpyDeviceToHost, cst);
  if (e == cudaSuccess && rc == BSFIT_OK)
    e = cudaMemcpyAsync(LL, dL, (size_t)nfits * sizeof(float), cudaMemcpyDeviceToHost, cst);
  if (d_rois) cudaFreeAsync(d_rois, cst);
  if (d_out) cudaFreeAsync(d_out, cst);
  cudaError_t e2 = cudaStreamSynchronize(cst);
  bsfit_model_release(model);
  if (rc != BSFIT_OK) return rc;
  if (e == cudaSuccess) e = e2;
  return cuda_status(e);
}

// The drop-in call with double results from the FP64 reference-precision
// kernel: same arguments and checks as bsfit_GPUmleFit_LM_multiD (varmap
// ignored likewise), double outputs in the same column-major layout.
int bsfit_GPUmleFit_LM_multiD_f64(const float* imstack, int64_t roi_size, int64_t roi_size2,
                                  int64_t nfits, int32_t fittype, int32_t iterations,
                                  const float* coeff, int32_t coeff_ndim,
                                  const int64_t* coeff_dims, const float* varmap,
                                  int64_t varmap_numel, int32_t silent, const float* init_p,
                                  int64_t init_p_numel, const float* coeff3, int32_t coeff3_ndim,
                                  const int64_t* coeff3_dims, double* P, double* CRLB,
                                  double* LL) {
  (void)varmap;
  (void)varmap_numel;
  int st = call_checks(imstack, roi_size, roi_size2, nfits, fittype, P && CRLB && LL);
  if (st) return st;
  const int nv = num_params(fittype);
  if (!silent) {
    std::printf("subregion size: %lld fittype: %d\n", (long long)roi_size, fittype);
    std::printf("Number of fits: %lld no padding\n", (long long)nfits);
  }
  bsfit_model model = nullptr;
  st = bsfit_model_create(fittype, coeff, coeff_ndim, coeff_dims, coeff3, coeff3_ndim,
                          coeff3_dims, init_p, init_p_numel, &model);
  if (st) return st;
  if (nfits == 0) return bsfit_model_release(model);
  CallStreams* cs = call_streams();
  if (!cs) {
    bsfit_model_release(model);
    return BSFIT_E_CUDA;
  }
  cudaStream_t cst = cs->comp[0];
  const size_t s2 = (size_t)roi_size * roi_size;
  const size_t in_bytes = (size_t)nfits * s2 * sizeof(float);
  const size_t nout = (size_t)nfits * (2 * nv + 2);
  float* d_rois = nullptr;
  double* d_out = nullptr;
  cudaError_t e = cudaMallocAsync(&d_rois, in_bytes, cst);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_out, nout * sizeof(double), cst);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_rois, imstack, in_bytes, cudaMemcpyHostToDevice, cst);
  int rc = BSFIT_OK;
  double* dP = d_out;
  double* dC = d_out + (size_t)nfits * (nv + 1);
  double* dL = dC + (size_t)nfits * nv;
  if (e == cudaSuccess)
    rc = bsfit_fit_f64_device(model, d_rois, nullptr, roi_size, nfits, iterations, dP, dC, dL,
                              cst);
  if (e == cudaSuccess && rc == BSFIT_OK)
    e = cudaMemcpyAsync(P, dP, (size_t)nfits * (nv + 1) * sizeof(double), cudaMemcpyDeviceToHost,
                        cst);
  if (e == cudaSuccess && rc == BSFIT_OK)
    e = cudaMemcpyAsync(CRLB, dC, (size_t)nfits * nv * sizeof(double), cudaMemcpyDeviceToHost, cst);
  if (e == cudaSuccess && rc == BSFIT_OK)
    e = cudaMemcpyAsync(LL, dL, (size_t)nfits * sizeof(double), cudaMemcpyDeviceToHost, cst);
  if (d_rois) cudaFreeAsync(d_rois, cst);
  if (d_out) cudaFreeAsync(d_out, cst);
  cudaError_t e2 = cudaStreamSynchronize(cst);
  bsfit_model_release(model);
  if (rc != BSFIT_OK) return rc;
  if (e == cudaSuccess) e = e2;
  return cuda_status(e);
}

// 4Pi in double: the restated 4Pi fit (oracle/bsfit_oracle.cpp fit_4pi_roi)
// in its order of operations, as bsfit_fit_f64_device does for fit types 6-8;
// arguments as bsfit_fit4pi_device with double outputs.
int bsfit_fit4pi_f64_device(bsfit_model model, const float* d_rois, int64_t roi_size,
                            int64_t nfits, int32_t iterations, const float* d_dT,
                            const float* d_initZ, const float* d_initPhi, double* d_P,
                            double* d_CRLB, double* d_LL, void* stream) {
  if (!model) return BSFIT_E_INVALID;
  if (model->dev.fittype != bsfit::kFit4Pi) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 0) return BSFIT_E_INVALID;
  if (nfits == 0) return BSFIT_OK;
  if (!d_rois || !d_dT || !d_initZ || !d_initPhi || !d_P || !d_CRLB || !d_LL)
    return BSFIT_E_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  const int rc = ensure_f64_tables(model, st);
  if (rc != BSFIT_OK) return rc;
  const ModelDev& m = model->dev;
  bsfit::Fit64Args a;
  std::memset(&a, 0, sizeof(a));
  a.m = m;
  a.c = model->d_coeff64;
  a.total = (int64_t)m.cd[0] * m.cd[1] * m.cd[2] * m.cd[3];
  a.rois = d_rois;
  a.s = (int)roi_size;
  a.nfits = nfits;
  a.iterations = iterations;
  a.P = d_P;
  a.CRLB = d_CRLB;
  a.LL = d_LL;
  a.dT = d_dT;
  a.z0 = d_initZ;
  a.w0 = d_initPhi;
  return cuda_status(bsfit::launch_fit64(a, st));
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner (bsfit_tune.cu holds the configuration table and the kernel
// variants).

extern "C" {

int bsfit_tune_num_variants(int32_t fittype) { return bsfit::tune_num_variants(fittype); }

int bsfit_tune_min_blocks(int32_t fittype, int32_t variant) {
  return bsfit::tune_min_blocks(fittype, variant);
}

int bsfit_tune_rois_per_warp(int32_t fittype, int32_t variant) {
  if (variant < 0 || variant >= bsfit::tune_num_variants(fittype)) return 0;
  return bsfit::tune_rois_per_warp(fittype, variant);
}

int bsfit_tune_set(int32_t fittype, int64_t roi_size, int32_t variant, int32_t warps_per_block) {
  if (num_params(fittype) == 0) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BSFIT_E_NO_DEVICE;
  if (variant < 0) {
    bsfit::tune_clear(fittype, (int)roi_size, dev);
    return BSFIT_OK;
  }
  if (!bsfit::tune_store(fittype, (int)roi_size, dev, bsfit::TuneConfig{variant, warps_per_block}))
    return BSFIT_E_INVALID;
  return BSFIT_OK;
}

int bsfit_tune_get(int32_t fittype, int64_t roi_size, int32_t* variant, int32_t* warps_per_block) {
  if (!variant || !warps_per_block) return BSFIT_E_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BSFIT_E_NO_DEVICE;
  bsfit::TuneConfig c{0, 0};
  const bool found = bsfit::tune_lookup(fittype, (int)roi_size, dev, &c);
  *variant = found ? c.variant : -1;
  *warps_per_block = found ? c.wpb : 0;
  return BSFIT_OK;
}

int bsfit_autotune_device(bsfit_model model, const float* d_rois, int64_t roi_size, int64_t nfits,
                          int32_t iterations, float* d_P, float* d_CRLB, float* d_LL, int32_t reps,
                          int32_t* best_variant, int32_t* best_wpb, double* best_ms,
                          double* all_ms, void* stream) {
  if (!model || !best_variant || !best_wpb) return BSFIT_E_INVALID;
  const int ft = model->dev.fittype;
  if (ft != 6 && ft != 7 && ft != 8) return BSFIT_E_UNSUPPORTED_FITTYPE;
  if (roi_size < 1 || roi_size > kMaxRoi) return BSFIT_E_SUBREGION_SIZE;
  if (nfits < 1 || reps < 1 || !d_rois || !d_P || !d_CRLB || !d_LL) return BSFIT_E_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BSFIT_E_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return cuda_status(e);
  }
  const int nv = bsfit::tune_num_variants(ft);
  const int wpbs[3] = {4, 2, 1};
  double best = -1.0;
  bsfit::TuneConfig bc{0, 0};
  int rc = BSFIT_OK;
  for (int v = 0; v < nv && rc == BSFIT_OK; ++v)
    for (int w = 0; w < 3 && rc == BSFIT_OK; ++w) {
      bsfit::tune_store(ft, (int)roi_size, dev, bsfit::TuneConfig{v, wpbs[w]});
      double ms = -1.0;  // infeasible (shared memory or occupancy)
      int r = bsfit_fit_device(model, d_rois, roi_size, nfits, iterations, d_P, d_CRLB, d_LL, st);
      if (r == BSFIT_OK) {
        cudaEventRecord(e0, st);
        for (int k = 0; k < reps && r == BSFIT_OK; ++k)
          r = bsfit_fit_device(model, d_rois, roi_size, nfits, iterations, d_P, d_CRLB, d_LL, st);
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) rc = cuda_status(e);
        float t = 0.0f;
        if (r == BSFIT_OK && e == cudaSuccess && cudaEventElapsedTime(&t, e0, e1) == cudaSuccess)
          ms = (double)t / reps;
      } else if (r != BSFIT_E_CUDA) {
        rc = r;
      }
      if (all_ms) all_ms[v * 3 + w] = ms;
      if (ms > 0.0 && (best < 0.0 || ms < best)) {
        best = ms;
        bc = bsfit::TuneConfig{v, wpbs[w]};
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != BSFIT_OK || best < 0.0) {
    bsfit::tune_clear(ft, (int)roi_size, dev);
    return rc != BSFIT_OK ? rc : BSFIT_E_CUDA;
  }
  bsfit::tune_store(ft, (int)roi_size, dev, bc);
  *best_variant = bc.variant;
  *best_wpb = bc.wpb;
  if (best_ms) *best_ms = best;
  return BSFIT_OK;
}

}  // extern "C"
