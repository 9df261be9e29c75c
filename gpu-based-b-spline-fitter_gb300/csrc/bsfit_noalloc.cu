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
// cudaGetSymbolAddress (once per device and CUDA context, with that device
// current); make that first call before any stream capture. The address is
// kept together with the context it belongs to: after a device reset the
// primary context is a new one, the array may sit elsewhere, and the next call
// repeats the look-up (make it, too, before any capture). No call allocates or
// frees memory.
#include <cstdint>
#include <mutex>

#include "../../include/bsfit.h"

namespace {

static_assert(BSFIT_STATIC_MAX_SEGMENTS <= BSFIT_MAX_SEGMENTS,
              "the static entry forwards to the batched entry, which takes at most "
              "BSFIT_MAX_SEGMENTS segments");

// Two 64-bit counters (claimed, finished) per segment.
static __device__ __align__(256) unsigned long long g_static_batch_scratch[2 * BSFIT_STATIC_MAX_SEGMENTS];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct ScratchAddr {
  void* ctx;   // the CUDA context the address belongs to
  void* addr;  // device address of g_static_batch_scratch in that context
};
ScratchAddr g_scratch[kMaxDevices] = {};

// cuCtxGetCurrent through the runtime's driver entry-point query (the library
// links only the runtime). Null where the query fails: the address is then
// looked up on every call, which stays correct.
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current() {
  static const CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

void* current_ctx() {
  void* c = nullptr;
  const CtxGetCurrentFn fn = ctx_get_current();
  if (!fn || fn(&c) != 0) return nullptr;
  return c;
}

// Device address of the static array in the current device's context (looked
// up once per device and context). Returns a bsfit status.
int static_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BSFIT_E_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  ScratchAddr& c = g_scratch[dev];
  void* ctx = current_ctx();
  if (!c.addr || !ctx || ctx != c.ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_batch_scratch);
    if (e != cudaSuccess || !p) return BSFIT_E_CUDA;
    c.addr = p;
    c.ctx = current_ctx();  // the look-up made the device's context current
  }
  *out = c.addr;
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
