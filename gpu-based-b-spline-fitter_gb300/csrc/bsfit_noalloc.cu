// Allocation-free variant of the batched fit.
//
// Some callers cannot allocate device memory at the moment they want a fit:
// an acquisition loop that must run at a fixed frame rate (cudaMalloc can
// synchronise the device and take unpredictable time), or a host application
// that reserved the GPU's memory for its own pool up front, so that any further
// allocation can fail. bsfit_batch_fit_device already takes caller-provided
// scratch; this entry point removes even that requirement by keeping the
// work-queue counters in a fixed device array of this library.
//
// The array belongs to the library and is shared by every call on a device:
//  - it holds counters for at most BSFIT_STATIC_MAX_SEGMENTS segments; larger
//    calls are rejected with BSFIT_E_STATIC_LIMIT;
//  - each call zeroes the counters it uses (stream-ordered) before its launch,
//    and the array keeps that call's final counts afterwards;
//  - two calls whose work overlaps on the GPU (different streams, or host
//    threads) race on the same counters: serialise them.
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (once per device, with that device current); make that
// first call before any stream capture. No call allocates or frees memory.
#include <cstdint>
#include <mutex>

#include "../../include/bsfit.h"

namespace {

// Two 64-bit counters (claimed, finished) per segment.
static __device__ __align__(256) unsigned long long g_static_batch_scratch[2 * BSFIT_STATIC_MAX_SEGMENTS];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the static array on the current device (looked up once per
// device). Returns a bsfit status.
int static_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BSFIT_E_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_batch_scratch);
    if (e != cudaSuccess || !p) return BSFIT_E_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return BSFIT_OK;
}

}  // namespace

extern "C" int bsfit_batch_fit_device_static(const bsfit_segment* segs, int32_t nseg,
                                             void* stream) {
  if (nseg < 0) return BSFIT_E_INVALID;
  if (nseg > BSFIT_STATIC_MAX_SEGMENTS) return BSFIT_E_STATIC_LIMIT;
  if (nseg == 0) return BSFIT_OK;
  void* scratch = nullptr;
  int st = static_scratch(&scratch);
  if (st != BSFIT_OK) return st;
  // The batched entry point zeroes the counters of this call on the stream
  // before its launches and allocates nothing itself.
  return bsfit_batch_fit_device(segs, nseg, scratch,
                                (int64_t)sizeof(unsigned long long) * 2 * BSFIT_STATIC_MAX_SEGMENTS,
                                stream);
}
