// Cubic B-spline coefficient builder on the device: the reference's bsarray
// for degree 3 without smoothing, which produces the fitter's coefficient input
// from a sampled PSF stack.
//
// Per axis (MultiD_bspline/bsarray/directFilter.m:200-282, symExpFilt.m:27-44,
// getBSplineFiltCoeffs.m:45-50), every 1-D line x[0..n-1] is filtered with the
// symmetric exponential filter of pole z = sqrt(3) - 2 and gain 6:
//   y[0]   = sum_{k < K0} z^k x[m(k)], m the whole-sample mirror sequence
//            0..n-1, n-2..1 repeated, K0 = ceil(log(eps) / log|z|);
//   y[k]   = x[k] + z y[k-1];
//   y[n-1] = (2 y[n-1] - x[n-1]) (-z / (1 - z^2));
//   y[k]   = (y[k+1] - y[k]) z, k = n-2 .. 0;  then y *= 6.
// Lines of length 1 are left unchanged. Then every axis is padded by one sample
// on each side by whole-sample mirroring (directFilter.m:286-298): c[-1] = c[1],
// c[n] = c[n-2] (c[0] for n = 1), so the coefficients are two larger than the
// samples along every axis. Arithmetic is double, as in the MATLAB builder; the
// fitter's input is the float copy.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/bsfit.h"
#include "bsfit_internal.h"

namespace bsfit {
namespace {

constexpr int kMaxK0 = 64;
__constant__ double c_zpow[kMaxK0];

// One thread per line along the axis of length n and stride `stride` (the
// product of the faster axes' sizes); lines enumerate (outer, inner) with
// inner < stride, so consecutive threads touch consecutive addresses whenever
// stride > 1.
__global__ void prefilter_axis(double* data, int64_t n, int64_t stride, int64_t lines, int k0,
                               double z, double c0, double gain) {
  const int64_t line = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= lines) return;
  const int64_t outer = line / stride, inner = line - outer * stride;
  double* x = data + outer * n * stride + inner;
  // causal initial value from the original samples, mirror sequence of period 2n - 2
  const int64_t period = 2 * n - 2;
  double y0 = 0.0;
  int64_t m = 0;  // position in the mirror sequence
  for (int k = 0; k < k0; ++k) {
    const int64_t idx = (m < n) ? m : period - m;
    y0 = (k == 0) ? c_zpow[0] * x[idx * stride] : y0 + c_zpow[k] * x[idx * stride];
    if (++m == period) m = 0;
  }
  const double x_last = x[(n - 1) * stride];
  double y = y0;
  x[0] = y0;
  for (int64_t k = 1; k < n; ++k) {
    y = x[k * stride] + z * y;
    x[k * stride] = y;
  }
  y = (2.0 * y - x_last) * c0;
  x[(n - 1) * stride] = y;
  for (int64_t k = n - 2; k >= 0; --k) {
    y = (y - x[k * stride]) * z;
    x[k * stride] = y;
  }
  for (int64_t k = 0; k < n; ++k) x[k * stride] *= gain;
}

struct PadDims {
  int ndim;
  int64_t n[5];     // sample sizes
  int64_t sn[5];    // sample strides
  int64_t pn[5];    // padded sizes
};

__global__ void mirror_pad(const double* y, PadDims d, int64_t total, float* out32, double* out64) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  int64_t rem = i, src = 0;
  for (int a = 0; a < d.ndim; ++a) {
    const int64_t p = rem % d.pn[a];
    rem /= d.pn[a];
    const int64_t n = d.n[a];
    int64_t s;
    if (n == 1) s = 0;
    else if (p == 0) s = 1;
    else if (p == n + 1) s = n - 2;
    else s = p - 1;
    src += s * d.sn[a];
  }
  const double v = y[src];
  if (out32) out32[i] = (float)v;
  if (out64) out64[i] = v;
}

}  // namespace
}  // namespace bsfit

extern "C" {

int bsfit_bsarray_coeffs_device(const double* d_samples, int32_t ndim, const int64_t* dims,
                                double* d_work, float* d_coeff, double* d_coeff64,
                                void* stream) {
  if (!d_samples || !dims || !d_work || (!d_coeff && !d_coeff64)) return BSFIT_E_INVALID;
  if (ndim < 1 || ndim > 5) return BSFIT_E_INVALID;
  int64_t total = 1, padded = 1;
  for (int a = 0; a < ndim; ++a) {
    if (dims[a] < 1 || dims[a] > (1 << 20)) return BSFIT_E_INVALID;
    total *= dims[a];
    padded *= dims[a] + 2;
  }
  if (total > ((int64_t)1 << 34)) return BSFIT_E_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  const double z = std::sqrt(3.0) - 2.0;
  const int k0 = (int)std::ceil(std::log(2.220446049250313e-16) / std::log(std::fabs(z)));
  if (k0 > bsfit::kMaxK0) return BSFIT_E_INVALID;
  double zp[bsfit::kMaxK0];
  for (int k = 0; k < k0; ++k) zp[k] = std::pow(z, (double)k);
  cudaError_t e = cudaMemcpyToSymbolAsync(bsfit::c_zpow, zp, sizeof(double) * k0, 0,
                                          cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_work, d_samples, (size_t)total * sizeof(double),
                        cudaMemcpyDeviceToDevice, st);
  const double c0 = -z / (1.0 - z * z);
  int64_t stride = 1;
  for (int a = 0; a < ndim && e == cudaSuccess; ++a) {
    const int64_t n = dims[a];
    if (n > 1) {
      const int64_t lines = total / n;
      const int threads = 128;
      const int64_t blocks = (lines + threads - 1) / threads;
      bsfit::prefilter_axis<<<(unsigned)blocks, threads, 0, st>>>(d_work, n, stride, lines, k0, z,
                                                                  c0, 6.0);
      e = cudaGetLastError();
    }
    stride *= n;
  }
  if (e == cudaSuccess) {
    bsfit::PadDims pd;
    std::memset(&pd, 0, sizeof(pd));
    pd.ndim = ndim;
    int64_t s = 1;
    for (int a = 0; a < ndim; ++a) {
      pd.n[a] = dims[a];
      pd.sn[a] = s;
      pd.pn[a] = dims[a] + 2;
      s *= dims[a];
    }
    const int threads = 256;
    const int64_t blocks = (padded + threads - 1) / threads;
    bsfit::mirror_pad<<<(unsigned)blocks, threads, 0, st>>>(d_work, pd, padded, d_coeff, d_coeff64);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) return BSFIT_OK;
  return e == cudaErrorMemoryAllocation ? BSFIT_E_NOT_ENOUGH_MEMORY : BSFIT_E_CUDA;
}

int bsfit_bsarray_coeffs(const double* samples, int32_t ndim, const int64_t* dims, float* coeff) {
  if (!samples || !dims || !coeff || ndim < 1 || ndim > 5) return BSFIT_E_INVALID;
  int64_t total = 1, padded = 1;
  for (int a = 0; a < ndim; ++a) {
    if (dims[a] < 1 || dims[a] > (1 << 20)) return BSFIT_E_INVALID;
    total *= dims[a];
    padded *= dims[a] + 2;
  }
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  double *d_in = nullptr, *d_work = nullptr;
  float* d_out = nullptr;
  if (e == cudaSuccess) e = cudaMallocAsync(&d_in, (size_t)total * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_work, (size_t)total * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_out, (size_t)padded * sizeof(float), st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_in, samples, (size_t)total * sizeof(double), cudaMemcpyHostToDevice, st);
  int rc = BSFIT_OK;
  if (e == cudaSuccess) rc = bsfit_bsarray_coeffs_device(d_in, ndim, dims, d_work, d_out, nullptr, st);
  if (e == cudaSuccess && rc == BSFIT_OK)
    e = cudaMemcpyAsync(coeff, d_out, (size_t)padded * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (d_in) cudaFreeAsync(d_in, st);
  if (d_work) cudaFreeAsync(d_work, st);
  if (d_out) cudaFreeAsync(d_out, st);
  cudaError_t e2 = st ? cudaStreamSynchronize(st) : cudaSuccess;
  if (st) cudaStreamDestroy(st);
  if (rc != BSFIT_OK) return rc;
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) return BSFIT_OK;
  return e == cudaErrorMemoryAllocation ? BSFIT_E_NOT_ENOUGH_MEMORY : BSFIT_E_CUDA;
}

}  // extern "C"
