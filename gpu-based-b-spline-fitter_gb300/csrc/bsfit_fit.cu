// Host side of the FP32 fitter kernels (bsfit_fit_kernels.cuh): launch shapes,
// the plain, batched and evaluation launches, and the FP32 peak probe.
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "bsfit_fit_kernels.cuh"

namespace bsfit {

// ---------------------------------------------------------------------------
// Stage-A gather table (ModelDev::zq). Entry i of a table with P lateral
// nodes per plane and nq = n[2] z knots (knot k = 1 .. n[2] reads planes
// k - 1 .. k + 2):
//   4Pi: i = (wi * nq + kq) * P + lat holds planes kq .. kq + 3 of w layer wi
//     at lateral node lat;
//   fit type 8: i = kq * P + lat, the same for the 3D table of the mixture;
//   fit type 7: i = ((wi * nq + kq) * 2 + h) * P + lat holds planes kq + 2h and
//     kq + 2h + 1 of layers wi and wi + 1, as (plane 0 layer wi, plane 0 layer
//     wi + 1, plane 1 layer wi, plane 1 layer wi + 1), for first layers
//     wi = 0 .. nW - 2 (the kernel pairs w layers kw - 1, kw and kw + 1, kw + 2).
// Every read stays inside the table: kq + 3 <= n[2] + 2 = nZ - 1, wi + 1 <= nW - 1.
// The 3D kernels read the coefficient table itself (a table of this kind
// measured no faster there), and so does the 5D part of fit type 8 (at 4x its
// 56 MB it would not stay L2-resident).

__global__ void build_zq_kernel(const float* __restrict__ c, float4* __restrict__ q,
                                int64_t total, int64_t plane, int nq, int64_t sz, int64_t sw,
                                int paired) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lat = i % plane;
    int64_t r = i / plane;
    if (!paired) {
      const int64_t kq = r % nq, wi = r / nq;
      const float* p = c + wi * sw + kq * sz + lat;
      q[i] = make_float4(p[0], p[sz], p[2 * sz], p[3 * sz]);
    } else {
      const int64_t h = r % 2;
      r /= 2;
      const int64_t kq = r % nq, wi = r / nq;
      const float* p = c + wi * sw + (kq + 2 * h) * sz + lat;
      q[i] = make_float4(p[0], p[sw], p[sz], p[sz + sw]);
    }
  }
}

int64_t zq_entries(const ModelDev& m) {
  const int64_t plane = (int64_t)m.cd[0] * m.cd[1], nq = m.n[2];
  if (nq < 1) return 0;
  switch (m.fittype) {
    case kFit4Pi: return (int64_t)m.cd[3] * nq * plane;
    case 8: return nq * plane;
    case 7: return (int64_t)(m.cd[3] - 1) * nq * 2 * plane;
    default: return 0;
  }
}

void set_zq(ModelDev& m, float4* zq) {
  const int64_t plane = (int64_t)m.cd[0] * m.cd[1], nq = m.n[2];
  m.zq = zq;
  m.zq_kz = m.zq_w = 0;
  if (!zq) return;
  if (m.fittype == 7) {
    m.zq_kz = 2 * plane;
    m.zq_w = 2 * nq * plane;
  } else {
    m.zq_kz = plane;
    m.zq_w = nq * plane;
  }
}

cudaError_t build_zq(const ModelDev& m, float4* zq, cudaStream_t stream) {
  const int64_t total = zq_entries(m);
  if (total <= 0) return cudaSuccess;
  const int64_t blocks = (total + 255) / 256;
  build_zq_kernel<<<(unsigned)(blocks < 8192 ? blocks : 8192), 256, 0, stream>>>(
      m.fittype == 8 ? m.coeff3 : m.coeff, zq, total, (int64_t)m.cd[0] * m.cd[1], m.n[2],
      m.st[2], m.st[3], m.fittype == 7 ? 1 : 0);
  return cudaGetLastError();
}

int warp_smem_floats(int mode, int s, bool var, int stg) {
  return make_layout(mode, s, var, stg).total();
}

// Launch shape of a fitter kernel for a per-warp shared-memory size: the warps
// per block among 4, 2, 1 that keep the most warps resident per SM, with the
// blocks per SM and the SM count. Computed once per (kernel, size, device) and
// cached; the kernel's dynamic shared-memory limit is raised to the device's
// opt-in maximum on its first use, so launches of any size need no further
// attribute call.
namespace {
struct LaunchChoice {
  const void* kern;
  int per_warp, dev, force, wpb, bps, sms;
};
std::mutex g_choice_mu;
constexpr int kMaxChoices = 128;
LaunchChoice g_choices[kMaxChoices];
int g_nchoices = 0;
struct RaisedKernel {
  const void* kern;
  int dev;
};
RaisedKernel g_raised[128];
int g_nraised = 0;
}  // namespace

cudaError_t pick_launch(const void* kern, int per_warp, int* wpb, int* bps, int* sms) {
  return pick_launch_wpb(kern, per_warp, 0, wpb, bps, sms);
}

cudaError_t pick_launch_wpb(const void* kern, int per_warp, int force_wpb, int* wpb, int* bps,
                            int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_choice_mu);
  for (int i = 0; i < g_nchoices; ++i) {
    const LaunchChoice& c = g_choices[i];
    if (c.kern == kern && c.per_warp == per_warp && c.dev == dev && c.force == force_wpb) {
      *wpb = c.wpb;
      *bps = c.bps;
      *sms = c.sms;
      return cudaSuccess;
    }
  }
  int optin = 0, nsm = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  bool raised = false;
  for (int i = 0; i < g_nraised; ++i) raised |= (g_raised[i].kern == kern && g_raised[i].dev == dev);
  if (!raised) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return e;
    if (g_nraised < 128) g_raised[g_nraised++] = RaisedKernel{kern, dev};
  }
  int best = -1, bw = 4, bb = 0;
  for (int cand = 4; cand >= 1; cand >>= 1) {
    if (force_wpb && cand != force_wpb) continue;
    const int sm = per_warp * cand;
    if (sm > optin) continue;
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 32 * cand, sm) != cudaSuccess) continue;
    if (b * cand > best) {
      best = b * cand;
      bw = cand;
      bb = b;
    }
  }
  if (best <= 0) return cudaErrorInvalidConfiguration;
  const LaunchChoice c{kern, per_warp, dev, force_wpb, bw, bb, nsm};
  if (g_nchoices < kMaxChoices) g_choices[g_nchoices++] = c;
  else g_choices[(per_warp + dev) % kMaxChoices] = c;
  *wpb = bw;
  *bps = bb;
  *sms = nsm;
  return cudaSuccess;
}

cudaError_t launch_batch(const BatchArgs& a, int mode, bool multi, cudaStream_t stream) {
  if (a.nseg <= 0) return cudaSuccess;
  void (*kern)(const BatchArgs) = nullptr;
  const bool cap = a.warp_rois > 0;
  constexpr int M6 = BSFIT_MINBLOCKS(6), M7 = BSFIT_MINBLOCKS(7), M8 = BSFIT_MINBLOCKS(8);
  if (cap) {
    // the capped form of the default kernel (the serving loop's priority launches)
    if (mode == 6 && !multi) kern = batch_kernel<6, false, M6, 0, true>;
    else if (mode == 7) kern = multi ? batch_kernel<7, true, M7, 0, true> : batch_kernel<7, false, M7, 0, true>;
    else if (mode == 8) kern = multi ? batch_kernel<8, true, M8, 0, true> : batch_kernel<8, false, M8, 0, true>;
    else return cudaErrorInvalidValue;
  } else if (mode == 6 && !multi) {
    kern = batch_kernel<6>;
  } else if (mode == 7) {
    kern = multi ? batch_kernel<7, true> : batch_kernel<7>;
  } else if (mode == 8) {
    kern = multi ? batch_kernel<8, true> : batch_kernel<8>;
  } else {
    return cudaErrorInvalidValue;
  }
  // the autotuner's configuration for the largest ROI size of the batch (the
  // capped form keeps the default kernel and takes the tuner's warps per block)
  TuneConfig tc{0, 0};
  int dev = 0;
  if (!multi && cudaGetDevice(&dev) == cudaSuccess && tune_lookup(mode, a.s_max, dev, &tc) &&
      tc.variant > 0) {
    if (cap) tc.variant = 0;
    else kern = batch_variant(mode, tc.variant);
  }
  if (!kern) return cudaErrorInvalidValue;
  const int rpw = tune_rois_per_warp(mode, tc.variant);
  const int per_warp = tune_warp_floats(mode, tc.variant, a.s_max, false) * 4;
  int wpb = 4, blocks_per_sm = 0, sms = 0;
  cudaError_t e = pick_launch_wpb((const void*)kern, per_warp, multi ? 0 : tc.wpb, &wpb,
                                  &blocks_per_sm, &sms);
  if (e != cudaSuccess) return e;
  const int smem = per_warp * wpb;
  int64_t total = 0;
  for (int i = 0; i < a.nseg; ++i) total += a.seg[i].n;
  int64_t grid = (int64_t)sms * blocks_per_sm;
  const int64_t need = (total + rpw * wpb - 1) / (rpw * wpb);
  if (need < grid) grid = need;
  // capped: enough blocks that every ROI is fitted
  if (cap) {
    const int64_t cover = (total + (int64_t)a.warp_rois * wpb - 1) / ((int64_t)a.warp_rois * wpb);
    if (cover > grid) grid = cover;
    if (grid > 0x7fffffff) return cudaErrorInvalidValue;
  }
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, 32 * wpb, smem, stream>>>(a);
  return cudaGetLastError();
}

// One evaluation per ROI at caller-given parameters: writes, per ROI, the
// deviance, the gradient (NV) and the packed upper-triangle Hessian (NH), or
// with fisher set the log-likelihood, zeros and the Fisher information.
template <int MODE>
__global__ void __launch_bounds__(128) eval_kernel(FitArgs a, const float* theta, float* out,
                                                   int fisher) {
  using TR = ModeTraits<MODE>;
  constexpr int NV = TR::NV;
  constexpr int NH = NV * (NV + 1) / 2;
  extern __shared__ float4 smem4[];
  float* smem = reinterpret_cast<float*>(smem4);
  const WarpLayout L = make_layout(MODE, a.s);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  float* ws = smem + wib * L.total();
  const int64_t total_warps = (int64_t)gridDim.x * wpb;
  for (int64_t roi = (int64_t)blockIdx.x * wpb + wib; roi < a.nfits; roi += total_warps) {
    load_roi<MODE>(a, L, ws, lane, roi);
    float th[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) th[i] = theta[i * a.nfits + roi];
    FPair e;
    float gl, hr[NV];
    evaluate<MODE>(a, L, ws, lane, th, false, fisher != 0, e, gl, hr);
    float* o = out + roi * (1 + NV + NH);
    if (lane == 0) o[0] = e.hi + e.lo;
    if (lane < NV) {
      o[1 + lane] = fisher ? 0.0f : gl;
#pragma unroll
      for (int k = 0; k < NV; ++k)
        if (k >= lane) o[1 + NV + hidx<NV>(lane, k)] = hr[k];
    }
    __syncwarp();
  }
}

cudaError_t launch_eval(const FitArgs& a, const float* theta, float* out, int fisher,
                        cudaStream_t stream) {
  if (a.nfits <= 0) return cudaSuccess;
  const int mode = a.m.fittype;
  const int per_warp = warp_smem_floats(mode, a.s) * 4;
  int wpb = 4;
  while (wpb > 1 && per_warp * wpb > 200 * 1024) wpb >>= 1;
  const int smem = per_warp * wpb;
  void (*kern)(FitArgs, const float*, float*, int) = nullptr;
  if (mode == 6) kern = eval_kernel<6>;
  else if (mode == 7) kern = eval_kernel<7>;
  else if (mode == 8) kern = eval_kernel<8>;
  else if (mode == kFit4Pi) kern = eval_kernel<kFit4Pi>;
  else return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int64_t grid = (a.nfits + wpb - 1) / wpb;
  if (grid > 65535) grid = 65535;
  kern<<<(unsigned)grid, 32 * wpb, smem, stream>>>(a, theta, out, fisher);
  return cudaGetLastError();
}

// FP32 FMA throughput probe: the denominator of the fitter's roofline
// (an FP32-pipe-bound kernel), measured on the same device and clocks.
__global__ void fp32_peak_kernel(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
  float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// The same with paired FP32 FMAs (FFMA2): 8 independent float2 chains.
__global__ void fp32x2_peak_kernel(float* out, int iters, float a, float b) {
  const float t = threadIdx.x * 1e-3f;
  float2 x0 = make_float2(t, t + 0.5f), x1 = make_float2(t + 1.f, t + 1.5f);
  float2 x2 = make_float2(t + 2.f, t + 2.5f), x3 = make_float2(t + 3.f, t + 3.5f);
  float2 x4 = make_float2(t + 4.f, t + 4.5f), x5 = make_float2(t + 5.f, t + 5.5f);
  float2 x6 = make_float2(t + 6.f, t + 6.5f), x7 = make_float2(t + 7.f, t + 7.5f);
  const float2 A = make_float2(a, a), B = make_float2(b, b);
  for (int i = 0; i < iters; ++i) {
    x0 = __ffma2_rn(x0, A, B); x1 = __ffma2_rn(x1, A, B); x2 = __ffma2_rn(x2, A, B);
    x3 = __ffma2_rn(x3, A, B); x4 = __ffma2_rn(x4, A, B); x5 = __ffma2_rn(x5, A, B);
    x6 = __ffma2_rn(x6, A, B); x7 = __ffma2_rn(x7, A, B);
  }
  const float2 sum = make_float2(x0.x + x1.x + x2.x + x3.x + x4.x + x5.x + x6.x + x7.x,
                                 x0.y + x1.y + x2.y + x3.y + x4.y + x5.y + x6.y + x7.y);
  out[blockIdx.x * blockDim.x + threadIdx.x] = sum.x + sum.y;
}

cudaError_t measure_fp32_peak2(double* scalar, double* paired) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  float* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(float) * blocks * threads);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best[2] = {1e30f, 1e30f};
  for (int kind = 0; kind < 2; ++kind) {
    if (kind == 0) fp32_peak_kernel<<<blocks, threads>>>(out, 256, 0.999f, 1e-4f);
    else fp32x2_peak_kernel<<<blocks, threads>>>(out, 256, 0.999f, 1e-4f);
    for (int r = 0; r < 5; ++r) {
      cudaEventRecord(e0);
      if (kind == 0) fp32_peak_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-4f);
      else fp32x2_peak_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-4f);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best[kind] = ms < best[kind] ? ms : best[kind];
    }
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flop = 2.0 * 8.0 * (double)iters * blocks * threads;  // scalar: 8 chains x 2 FLOP
  *scalar = flop / (best[0] * 1e-3) * 1e-12;
  *paired = 2.0 * flop / (best[1] * 1e-3) * 1e-12;                  // 2 FMAs per paired op
  return e;
}

cudaError_t measure_fp32_peak(double* tflops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  float* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(float) * blocks * threads);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp32_peak_kernel<<<blocks, threads>>>(out, 256, 0.999f, 1e-4f);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    fp32_peak_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-4f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (best * 1e-3) * 1e-12;
  return e;
}

// ---------------------------------------------------------------------------

cudaError_t launch_fit(const FitArgs& a, cudaStream_t stream) {
  if (a.nfits <= 0) return cudaSuccess;
  if (a.flags & FLAG_PARITY) {
    // double-float kernels: plain EMCCD fits of fit types 6, 7, 8, one start
    if (a.var || a.n_starts > 1 || a.trace || a.m.fittype == kFit4Pi) return cudaErrorInvalidValue;
    return launch_fitdd(a, stream);
  }
  const int mode = a.m.fittype;
  const bool var = a.var != nullptr;
  void (*kern)(FitArgs) = nullptr;
  const bool multi = a.n_starts > 1;
  if (var && multi) return cudaErrorInvalidValue;  // not combined
  if (mode == 6) kern = var ? fit_kernel<6, false, true> : fit_kernel<6, false>;
  else if (mode == 7) kern = var ? fit_kernel<7, false, true> : multi ? fit_kernel<7, true> : fit_kernel<7, false>;
  else if (mode == 8) kern = var ? fit_kernel<8, false, true> : multi ? fit_kernel<8, true> : fit_kernel<8, false>;
  else if (mode == kFit4Pi && !var) kern = multi ? fit_kernel<kFit4Pi, true> : fit_kernel<kFit4Pi, false>;
  else return cudaErrorInvalidValue;
  // The autotuner's configuration (kernel variant, warps per block) for this
  // fit type and ROI size on this device, where one was chosen; otherwise the
  // warps per block among 4, 2, 1 that keep the most warps resident per SM
  // (shared memory per warp grows with s and the model).
  TuneConfig tc{0, 0};
  int dev = 0;
  const bool tunable = !var && !multi && mode != kFit4Pi;
  if (tunable && cudaGetDevice(&dev) == cudaSuccess && tune_lookup(mode, a.s, dev, &tc) &&
      tc.variant > 0)
    kern = fit_variant(mode, tc.variant);
  if (!kern) return cudaErrorInvalidValue;
  // ROIs per warp: 2 for the pair and packed variants of fit type 6
  const int rpw = tunable ? tune_rois_per_warp(mode, tc.variant) : 1;
  const int per_warp =
      (tunable ? tune_warp_floats(mode, tc.variant, a.s, var) : warp_smem_floats(mode, a.s, var)) * 4;
  int wpb = 4, blocks_per_sm = 0, sms = 0;
  cudaError_t e = pick_launch_wpb((const void*)kern, per_warp, tunable ? tc.wpb : 0, &wpb,
                                  &blocks_per_sm, &sms);
  if (e != cudaSuccess) return e;
  const int smem = per_warp * wpb;
  int64_t need = (a.nfits + rpw * wpb - 1) / (rpw * wpb);
  int64_t grid = (int64_t)sms * blocks_per_sm;
  if (need < grid) grid = need;
  // More ROIs than resident warps: claim them dynamically (iteration counts
  // vary per ROI, and a fixed share per warp leaves the launch waiting on its
  // slowest warp). The counter comes from the stream-ordered pool; without it
  // the fixed schedule runs.
  FitArgs b = a;
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
    // A failed pool allocation or memset leaves the fixed schedule; only then
    // is the error it recorded cleared (an error the caller's earlier
    // asynchronous work left pending is not touched otherwise).
    if (ea != cudaSuccess) (void)cudaGetLastError();
  }
  kern<<<(unsigned)grid, 32 * wpb, smem, stream>>>(b);
  e = cudaGetLastError();
  if (claim) cudaFreeAsync(claim, stream);
  return e;
}

}  // namespace bsfit

#ifdef BSFIT_PHASE_TIMING
extern "C" int bsfit_debug_phase_cycles(unsigned long long* out, int reset) {
  cudaError_t e = cudaMemcpyFromSymbol(out, bsfit::g_phase_cycles, sizeof(unsigned long long) * 16);
  if (reset) {
    unsigned long long z[16] = {0};
    cudaMemcpyToSymbol(bsfit::g_phase_cycles, z, sizeof(z));
  }
  return (int)e;
}
#endif
