// Frame -> ROI front end on the device: the step before the fitter in the
// reference's acquisition loop (MultiD_fitter/simplefitter_cspline.m:197-319):
//   imphot = (frame - offset) * conversion                       (:226)
//   impf   = filter2(h, imphot [- min(imphot(:, 1))])            (:240-246)
//   strict 3x3 local maxima of impf in raster order, columns outer
//            (MultiD_fitter/shared/maximumfind2.c:18-66)
//   keep value > cutoff, dx < x <= W - dx, dx < y <= H - dx      (:249-251)
//   ROI k = imphot(y-dx:y+dx, x-dx:x+dx), x reversed if mirrored  (:295-301)
// Frames are MATLAB [H, W, F] (y fastest). The maxima are counted per
// (frame, column), prefix-summed in order and written in the reference's scan
// order, so the ROI list is deterministic and equal to the reference's.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/bsfit.h"
#include "bsfit_internal.h"

namespace bsfit {
namespace {

constexpr int kMaxKernel = 31;
__constant__ float c_filter[kMaxKernel * kMaxKernel];  // h(u, v) at [u + k v]

struct FrontArgs {
  const float* frames;
  int64_t nframes, H, W;
  float offset, conversion;
  int k;              // kernel size
  int sub_min;        // subtract the first column's minimum before filtering
  double cutoff;
  int dx, s, mirror;
  float* impf;        // [F][W][H]
  float* colmin;      // [F]
  int* counts;        // [F * W]
  long long* offsets; // [F * W + 1]
  float* coords;      // [capacity * 3]: x, y, frame (1-based), column-major
  float* rois;        // [capacity][s][s]
  int64_t capacity;
};

__device__ __forceinline__ float imphot(const FrontArgs& a, int64_t f, int64_t x, int64_t y) {
  return (__ldg(a.frames + (f * a.W + x) * a.H + y) - a.offset) * a.conversion;
}

// min over the first column (x = 0) of imphot, one block per frame
__global__ void first_column_min(FrontArgs a) {
  __shared__ float red[32];
  const int64_t f = blockIdx.x;
  float m = INFINITY;
  for (int64_t y = threadIdx.x; y < a.H; y += blockDim.x) m = fminf(m, imphot(a, f, 0, y));
  for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : INFINITY;
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) a.colmin[f] = m;
  }
}

// 'same'-size correlation with zero padding: Y(y, x) = sum_{u,v} h(u, v)
// X(y + u - o, x + v - o), o = (k - 1) / 2. Block: 32 rows (y) x 8 columns (x)
// of one frame, the input tile with its halo staged in shared memory.
constexpr int TY = 32, TX = 8;
__global__ void filter_frames(FrontArgs a) {
  extern __shared__ float tile[];
  const int k = a.k, o = (k - 1) / 2;
  const int ty = TY + k - 1, tx = TX + k - 1;
  const int64_t f = blockIdx.z;
  const int64_t y0 = (int64_t)blockIdx.x * TY, x0 = (int64_t)blockIdx.y * TX;
  const float sub = a.sub_min ? a.colmin[f] : 0.0f;
  for (int i = threadIdx.y * TY + threadIdx.x; i < ty * tx; i += TY * TX) {
    const int cx = i / ty, cy = i - cx * ty;
    const int64_t gy = y0 + cy - o, gx = x0 + cx - o;
    float v = 0.0f;
    if (gy >= 0 && gy < a.H && gx >= 0 && gx < a.W) v = imphot(a, f, gx, gy) - sub;
    tile[cx * ty + cy] = v;
  }
  __syncthreads();
  const int64_t y = y0 + threadIdx.x, x = x0 + threadIdx.y;
  if (y >= a.H || x >= a.W) return;
  float acc = 0.0f;
  for (int v = 0; v < k; ++v) {
    const float* col = tile + (threadIdx.y + v) * ty + threadIdx.x;
    for (int u = 0; u < k; ++u) acc = fmaf(c_filter[u + k * v], col[u], acc);
  }
  a.impf[(f * a.W + x) * a.H + y] = acc;
}

// Strict 3x3 maximum at interior pixel (x, y) that passes the keep filter.
__device__ __forceinline__ bool kept_max(const FrontArgs& a, const float* img, int64_t x, int64_t y) {
  if (x < 1 || x > a.W - 2 || y < 1 || y > a.H - 2) return false;
  const float c = img[x * a.H + y];
  const float* l = img + (x - 1) * a.H + y;
  const float* m = img + x * a.H + y;
  const float* r = img + (x + 1) * a.H + y;
  if (!(c > l[-1] && c > l[0] && c > l[1] && c > m[-1] && c > m[1] && c > r[-1] && c > r[0] &&
        c > r[1]))
    return false;
  const int64_t x1 = x + 1, y1 = y + 1;  // the reference's 1-based coordinates
  return (double)c > a.cutoff && x1 > a.dx && x1 <= a.W - a.dx && y1 > a.dx && y1 <= a.H - a.dx;
}

// One warp per (frame, column): count (pass 0) or write (pass 1) the kept maxima.
template <int PASS>
__global__ void nms_columns(FrontArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= a.nframes * a.W) return;
  const int64_t f = warp / a.W, x = warp - f * a.W;
  const float* img = a.impf + f * a.W * a.H;
  long long base = (PASS == 1) ? a.offsets[warp] : 0;
  int count = 0;
  for (int64_t y0 = 0; y0 < a.H; y0 += 32) {
    const int64_t y = y0 + lane;
    const bool hit = (y < a.H) && kept_max(a, img, x, y);
    const unsigned b = __ballot_sync(0xffffffffu, hit);
    if (PASS == 1 && hit) {
      const long long idx = base + count + __popc(b & ((1u << lane) - 1u));
      if (idx < a.capacity) {
        a.coords[idx] = (float)(x + 1);
        a.coords[a.capacity + idx] = (float)(y + 1);
        a.coords[2 * a.capacity + idx] = (float)(f + 1);
      }
    }
    count += __popc(b);
  }
  if (PASS == 0 && lane == 0) a.counts[warp] = count;
}

// Exclusive prefix sum of the per-column counts (one block); offsets[n] = total.
__global__ void scan_counts(const int* counts, long long* offsets, int64_t n) {
  __shared__ long long part[1024];
  const int t = threadIdx.x, nt = blockDim.x;
  const int64_t chunk = (n + nt - 1) / nt;
  const int64_t b = t * chunk, e = (b + chunk < n) ? b + chunk : n;
  long long s = 0;
  for (int64_t i = b; i < e; ++i) s += counts[i];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    long long run = 0;
    for (int i = 0; i < nt; ++i) {
      const long long v = part[i];
      part[i] = run;
      run += v;
    }
    offsets[n] = run;
  }
  __syncthreads();
  long long run = part[t];
  for (int64_t i = b; i < e; ++i) {
    offsets[i] = run;
    run += counts[i];
  }
}

// Cut-out: one warp per kept maximum (persistent), the count read on the device.
__global__ void cut_rois(FrontArgs a, const long long* total) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const long long n = *total < a.capacity ? *total : a.capacity;
  const int s = a.s, s2 = s * s, dx = a.dx;
  for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += warps) {
    const int64_t x0 = (int64_t)a.coords[k] - 1, y0 = (int64_t)a.coords[a.capacity + k] - 1;
    const int64_t f = (int64_t)a.coords[2 * a.capacity + k] - 1;
    float* roi = a.rois + k * s2;
    for (int p = lane; p < s2; p += 32) {
      const int jj = p / s, ii = p - jj * s;
      const int64_t x = a.mirror ? x0 + dx - jj : x0 - dx + jj;
      roi[p] = imphot(a, f, x, y0 - dx + ii);
    }
  }
}

}  // namespace
}  // namespace bsfit

extern "C" {

int bsfit_peak_kernel(int32_t mode, double sigma, float* kernel, int32_t* ksize) {
  if (!kernel || !ksize || !(sigma > 0.0) || (mode != 0 && mode != 1)) return BSFIT_E_INVALID;
  auto gauss = [](int k, double sg, double* h) {
    const double half = (k - 1) / 2.0;
    double mx = 0.0, sum = 0.0;
    for (int v = 0; v < k; ++v)
      for (int u = 0; u < k; ++u) {
        const double x = v - half, y = u - half;
        h[u + k * v] = std::exp(-(x * x + y * y) / (2.0 * sg * sg));
        mx = h[u + k * v] > mx ? h[u + k * v] : mx;
      }
    for (int i = 0; i < k * k; ++i) {
      if (h[i] < 2.220446049250313e-16 * mx) h[i] = 0.0;
      sum += h[i];
    }
    if (sum != 0.0)
      for (int i = 0; i < k * k; ++i) h[i] /= sum;
  };
  // fspecial('gaussian') kernels of simplefitter_cspline.m:197-211
  const int k = mode == 0 ? (int)std::fmax(3.0, std::ceil(3.0 * sigma + 1.0))
                          : (int)std::fmax(std::ceil(6.0 * sigma + 1.0), 3.0);
  if (k > bsfit::kMaxKernel) return BSFIT_E_INVALID;
  double h1[bsfit::kMaxKernel * bsfit::kMaxKernel], h2[bsfit::kMaxKernel * bsfit::kMaxKernel];
  gauss(k, sigma, h1);
  if (mode == 1) {
    gauss(k, std::fmax(1.0, 2.5 * sigma), h2);
    for (int i = 0; i < k * k; ++i) h1[i] -= h2[i];
  }
  for (int i = 0; i < k * k; ++i) kernel[i] = (float)h1[i];
  *ksize = k;
  return BSFIT_OK;
}

int64_t bsfit_find_rois_scratch_bytes(int64_t nframes, int64_t height, int64_t width) {
  if (nframes < 0 || height < 0 || width < 0) return 0;
  const int64_t cols = nframes * width;
  int64_t b = 0;
  b += (cols * 4 + 255) / 256 * 256;             // counts
  b += ((cols + 1) * 8 + 255) / 256 * 256;       // offsets and the total
  b += (nframes * 4 + 255) / 256 * 256;          // first-column minima
  b += (nframes * height * width * 4 + 255) / 256 * 256;  // filtered frames
  return b;
}

int bsfit_find_rois_device(const float* d_frames, int64_t nframes, int64_t height, int64_t width,
                           const bsfit_frontend* fe, float* d_rois, float* d_coords,
                           int64_t capacity, int64_t* n_found, float* d_filtered, void* d_scratch,
                           int64_t scratch_bytes, void* stream) {
  if (!fe || !n_found || nframes < 0 || capacity < 0) return BSFIT_E_INVALID;
  *n_found = 0;
  if (nframes == 0) return BSFIT_OK;
  if (!d_frames || !d_scratch || !fe->kernel) return BSFIT_E_INVALID;
  if (height < 3 || width < 3 || height > (1 << 20) || width > (1 << 20)) return BSFIT_E_INVALID;
  // launch limits of the filter grid (frames on z, column tiles on y)
  if (nframes > 65535 || (width + 7) / 8 > 65535) return BSFIT_E_INVALID;
  if (fe->ksize < 1 || fe->ksize > bsfit::kMaxKernel) return BSFIT_E_INVALID;
  if (fe->roi_size < 1 || fe->roi_size > 51 || fe->roi_size % 2 == 0) return BSFIT_E_SUBREGION_SIZE;
  if (capacity > 0 && (!d_rois || !d_coords)) return BSFIT_E_INVALID;
  if (scratch_bytes < bsfit_find_rois_scratch_bytes(nframes, height, width)) return BSFIT_E_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  bsfit::FrontArgs a;
  std::memset(&a, 0, sizeof(a));
  a.frames = d_frames;
  a.nframes = nframes;
  a.H = height;
  a.W = width;
  a.offset = fe->offset;
  a.conversion = fe->conversion;
  a.k = fe->ksize;
  a.sub_min = fe->subtract_first_column_min ? 1 : 0;
  a.cutoff = fe->cutoff;
  a.dx = fe->roi_size / 2;
  a.s = fe->roi_size;
  a.mirror = fe->mirror ? 1 : 0;
  a.capacity = capacity;
  a.coords = d_coords;
  a.rois = d_rois;
  char* p = (char*)d_scratch;
  const int64_t cols = nframes * width;
  a.counts = (int*)p;
  p += (cols * 4 + 255) / 256 * 256;
  a.offsets = (long long*)p;
  p += ((cols + 1) * 8 + 255) / 256 * 256;
  a.colmin = (float*)p;
  p += (nframes * 4 + 255) / 256 * 256;
  a.impf = d_filtered ? d_filtered : (float*)p;
  cudaError_t e = cudaMemcpyToSymbolAsync(bsfit::c_filter, fe->kernel,
                                          sizeof(float) * fe->ksize * fe->ksize, 0,
                                          cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && a.sub_min) {
    bsfit::first_column_min<<<(unsigned)nframes, 256, 0, st>>>(a);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    const int k = a.k;
    const size_t smem = sizeof(float) * (bsfit::TY + k - 1) * (bsfit::TX + k - 1);
    dim3 grid((unsigned)((height + bsfit::TY - 1) / bsfit::TY),
              (unsigned)((width + bsfit::TX - 1) / bsfit::TX), (unsigned)nframes);
    bsfit::filter_frames<<<grid, dim3(bsfit::TY, bsfit::TX), smem, st>>>(a);
    e = cudaGetLastError();
  }
  const int64_t nms_blocks = (cols * 32 + 255) / 256;
  if (e == cudaSuccess) {
    bsfit::nms_columns<0><<<(unsigned)nms_blocks, 256, 0, st>>>(a);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    bsfit::scan_counts<<<1, 1024, 0, st>>>(a.counts, a.offsets, cols);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && capacity > 0) {
    bsfit::nms_columns<1><<<(unsigned)nms_blocks, 256, 0, st>>>(a);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && capacity > 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    bsfit::cut_rois<<<(unsigned)(sms * 8), 256, 0, st>>>(a, a.offsets + cols);
    e = cudaGetLastError();
  }
  long long total = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&total, a.offsets + cols, sizeof(long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? BSFIT_E_NOT_ENOUGH_MEMORY : BSFIT_E_CUDA;
  *n_found = total;
  return BSFIT_OK;
}

}  // extern "C"
