// Serving form: a continuous-batching request loop over the batched fitter.
//
// The reference's GUI fits blocks of ROIs synchronously, one mex call at a time
// (MultiD_fitter/simplefitter_cspline.m:309-313, 463-524). Here requests (the
// ROI batches of acquired frames, each with its own PSF model) are submitted
// while others run:
//  - a fixed pool of slots, one CUDA stream each, bounds the requests in flight;
//  - device memory for ROIs, results and work-queue counters comes from one
//    arena reserved when the server is created (the HBM budget); a request is
//    admitted when a slot and enough arena space are free, otherwise it waits
//    in submission order;
//  - an admitted request runs host-to-device copies, one persistent batched
//    launch and device-to-host copies on its slot's stream, so requests in
//    flight overlap on the GPU (a new request's blocks start as the running
//    ones retire);
//  - optionally (bsfit_server_set_merge), a free slot takes several queued
//    single-start requests at once and fits all their segments in one
//    persistent launch, each request still copied back and completed on its
//    own;
//  - optionally (bsfit_server_set_priority), a launch goes to one of three
//    streams of its slot by its estimated device time (short, medium, long:
//    highest priority first), and its warps end after a few ROIs each, so its
//    blocks retire while the launch runs: a short request (a 3D frame)
//    submitted while a long one (a 5D frame) runs gets the SMs as the long
//    launch's blocks retire instead of after the whole launch;
//  - a host callback at the end of the stream marks the request done with its
//    completion time, so results are returned per request as soon as they are
//    ready and the latency (submit to completion) is exact.
// No device-side wait exists anywhere: progress is driven by the host calls
// (submit / poll / wait), and waits are bounded by the caller's timeout.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/bsfit.h"
#include "bsfit_internal.h"

namespace bsfit {
// The batched fit with per-fit-type caps on the ROIs a warp fits before it ends
// (bsfit_api.cu).
int batch_fit_capped(const bsfit_segment* segs, const bsfit_starts* starts, int32_t nseg,
                     void* d_scratch, int64_t scratch_bytes, void* stream, bool capped);
}  // namespace bsfit

namespace {

using Clock = std::chrono::steady_clock;

int cuda_status_s(cudaError_t e) {
  if (e == cudaSuccess) return BSFIT_OK;
  if (e == cudaErrorMemoryAllocation) return BSFIT_E_NOT_ENOUGH_MEMORY;
  return BSFIT_E_CUDA;
}

// First-fit allocator over [0, size) with coalescing free list, 256-byte units.
class Arena {
 public:
  void init(int64_t size) {
    size_ = size;
    free_.clear();
    free_[0] = size;
  }
  int64_t alloc(int64_t bytes) {
    bytes = (bytes + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        int64_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > bytes) free_[off + bytes] = len - bytes;
        return off;
      }
    }
    return -1;
  }
  void release(int64_t off, int64_t bytes) {
    bytes = (bytes + 255) / 256 * 256;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  int64_t size() const { return size_; }

 private:
  int64_t size_ = 0;
  std::map<int64_t, int64_t> free_;
};

struct Request {
  int64_t id = 0;
  std::vector<bsfit_host_segment> segs;
  std::vector<bsfit_starts> starts;  // empty: single start
  int64_t bytes = 0;       // arena bytes
  int64_t offset = -1;     // arena offset
  int slot = -1;
  cudaStream_t stream = nullptr;  // the stream its group was launched on
  int64_t rois = 0;
  Clock::time_point submitted, started;
  std::atomic<int64_t> done_ns{0};  // completion time (ns since epoch of Clock), 0 while running
  std::atomic<int> finished{0};
  int status = BSFIT_OK;
};

void CUDART_CB on_done(void* p) {
  Request* r = static_cast<Request*>(p);
  r->done_ns.store(Clock::now().time_since_epoch().count(), std::memory_order_relaxed);
  r->finished.store(1, std::memory_order_release);
}

// Work-queue counters at the start of a request's arena block: room for a
// merged launch of up to BSFIT_MAX_SEGMENTS segments, so the first request of a
// merged group holds the group's counters.
constexpr int64_t kCounterBytes = 256 + (int64_t)BSFIT_MAX_SEGMENTS * 2 * 8;

int64_t request_bytes(const std::vector<bsfit_host_segment>& segs) {
  int64_t b = kCounterBytes;
  for (const auto& g : segs) {
    const int nv = bsfit_num_params(bsfit_model_fittype(g.model));
    b += (g.nfits * g.roi_size * g.roi_size * 4 + 255) / 256 * 256;
    b += ((int64_t)g.nfits * (2 * nv + 2) * 4 + 255) / 256 * 256;
  }
  return b;
}

}  // namespace

struct bsfit_server_s {
  std::mutex mu;
  char* arena_base = nullptr;
  Arena arena;
  std::vector<cudaStream_t> streams;
  // with priorities on: kLevels streams per slot, highest priority first
  std::vector<cudaStream_t> pstreams;
  std::vector<std::vector<Request*>> slot_req;  // requests running in each slot (empty: free)
  int merge = 1;  // most queued requests fitted by one launch
  bool priority = false;
  std::deque<Request*> pending;
  std::map<int64_t, Request*> all;  // every request not yet collected
  std::vector<double> latencies_ms;
  std::vector<int64_t> latency_ids;  // request id of each latencies_ms entry
  int64_t next_id = 1;
  int64_t rois_done = 0;
  Clock::time_point first_submit;
  Clock::time_point last_done;
  bool any_submit = false;
  int device = 0;
};

namespace {

constexpr int kLevels = 3;

// Priority level of a request by its estimated device time: ROIs weighted by
// their fit type's cost relative to a 3D 13 px fit (4D about 6x, 5D about
// 30x, measured on GB300) and by their pixel count; up to about 1 ms of the
// GPU is short, up to about 5 ms medium. A merged group takes its first
// request's level (admission merges requests of one level only).
int request_level(const Request* r) {
  double cost = 0.0;
  for (const auto& g : r->segs) {
    const int ft = bsfit_model_fittype(g.model);
    const double w = ft == 6 ? 1.0 : ft == 7 ? 6.0 : 30.0;
    cost += (double)g.nfits * w * (double)(g.roi_size * g.roi_size) / 169.0;
  }
  return cost <= 4e4 ? 0 : cost <= 2e5 ? 1 : 2;
}

// Enqueue an admitted group of requests on a stream of its slot (with
// priorities on, the stream of the group's level): every request's uploads,
// one batched launch over all their segments (the first request's block holds
// the group's work-queue counters), then every request's result copies and
// completion callback. Caller holds the mutex.
int launch_group(bsfit_server_s* s, int slot, const std::vector<Request*>& grp) {
  cudaStream_t st = s->priority ? s->pstreams[slot * kLevels + request_level(grp[0])]
                                : s->streams[slot];
  for (Request* r : grp) r->stream = st;
  std::vector<bsfit_segment> dsegs;
  std::vector<bsfit_starts> starts;
  cudaError_t e = cudaSuccess;
  for (Request* r : grp) {
    char* base = s->arena_base + r->offset;
    int64_t off = kCounterBytes;
    for (size_t i = 0; i < r->segs.size(); ++i) {
      const bsfit_host_segment& g = r->segs[i];
      const int nv = bsfit_num_params(bsfit_model_fittype(g.model));
      const int64_t rb = g.nfits * g.roi_size * g.roi_size * 4;
      float* d_rois = (float*)(base + off);
      off += (rb + 255) / 256 * 256;
      float* d_out = (float*)(base + off);
      off += ((int64_t)g.nfits * (2 * nv + 2) * 4 + 255) / 256 * 256;
      if (e == cudaSuccess && rb > 0) e = cudaMemcpyAsync(d_rois, g.rois, rb, cudaMemcpyHostToDevice, st);
      bsfit_segment d;
      d.model = g.model;
      d.d_rois = d_rois;
      d.roi_size = g.roi_size;
      d.nfits = g.nfits;
      d.iterations = g.iterations;
      d.d_P = d_out;
      d.d_CRLB = d_out + g.nfits * (nv + 1);
      d.d_LL = d.d_CRLB + g.nfits * nv;
      dsegs.push_back(d);
    }
    for (const auto& q : r->starts) starts.push_back(q);
  }
  if (e != cudaSuccess) return cuda_status_s(e);
  void* scratch = s->arena_base + grp[0]->offset;
  const int64_t sb = bsfit_batch_scratch_bytes((int32_t)dsegs.size());
  int stt = bsfit::batch_fit_capped(dsegs.data(), starts.empty() ? nullptr : starts.data(),
                                    (int32_t)dsegs.size(), scratch, sb, st, s->priority);
  if (stt != BSFIT_OK) return stt;
  size_t k = 0;
  for (Request* r : grp) {
    for (size_t i = 0; i < r->segs.size(); ++i, ++k) {
      const bsfit_host_segment& g = r->segs[i];
      const int nv = bsfit_num_params(bsfit_model_fittype(g.model));
      if (g.nfits == 0) continue;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.P, dsegs[k].d_P, (size_t)g.nfits * (nv + 1) * 4, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.CRLB, dsegs[k].d_CRLB, (size_t)g.nfits * nv * 4, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.LL, dsegs[k].d_LL, (size_t)g.nfits * 4, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaLaunchHostFunc(st, on_done, r);
  }
  return cuda_status_s(e);
}

// Admit pending requests while slots and arena space allow (submission order).
// A free slot takes the oldest request and, with merging on, the next queued
// single-start requests that fit the arena, up to `merge` requests and
// BSFIT_MAX_SEGMENTS segments per launch.
void admit(bsfit_server_s* s) {
  while (!s->pending.empty()) {
    int slot = -1;
    for (size_t i = 0; i < s->slot_req.size(); ++i)
      if (s->slot_req[i].empty()) {
        slot = (int)i;
        break;
      }
    if (slot < 0) return;
    std::vector<Request*> grp;
    size_t nseg = 0;
    while (!s->pending.empty() && (int)grp.size() < s->merge) {
      Request* r = s->pending.front();
      if (!grp.empty() && (!r->starts.empty() || !grp[0]->starts.empty() ||
                           nseg + r->segs.size() > (size_t)BSFIT_MAX_SEGMENTS ||
                           (s->priority && request_level(r) != request_level(grp[0]))))
        break;
      int64_t off = s->arena.alloc(r->bytes);
      if (off < 0) break;  // wait for memory to free up
      s->pending.pop_front();
      r->offset = off;
      r->slot = slot;
      r->started = Clock::now();
      grp.push_back(r);
      nseg += r->segs.size();
    }
    if (grp.empty()) return;
    s->slot_req[slot] = grp;
    int st = launch_group(s, slot, grp);
    if (st != BSFIT_OK) {
      // The group failed to launch: complete its requests with the error.
      cudaStreamSynchronize(grp[0]->stream);
      for (Request* r : grp) {
        r->status = st;
        r->done_ns.store(Clock::now().time_since_epoch().count());
        r->finished.store(1);
      }
    }
  }
}

// Retire finished groups: free their slot and their requests' arena space.
void retire(bsfit_server_s* s) {
  for (size_t i = 0; i < s->slot_req.size(); ++i) {
    std::vector<Request*>& grp = s->slot_req[i];
    if (grp.empty()) continue;
    bool all = true;
    for (Request* r : grp) all = all && r->finished.load(std::memory_order_acquire);
    if (!all) continue;
    for (Request* r : grp) {
      s->arena.release(r->offset, r->bytes);
      const Clock::time_point done{Clock::duration(r->done_ns.load())};
      s->latencies_ms.push_back(std::chrono::duration<double, std::milli>(done - r->submitted).count());
      s->latency_ids.push_back(r->id);
      s->rois_done += r->rois;
      if (done > s->last_done) s->last_done = done;
    }
    grp.clear();
  }
}

bool running(const bsfit_server_s* s, const Request* r) {
  for (const auto& grp : s->slot_req)
    for (const Request* q : grp)
      if (q == r) return true;
  return false;
}

}  // namespace

extern "C" {

int bsfit_server_create(int32_t max_inflight, int64_t arena_bytes, bsfit_server* out) {
  if (!out || max_inflight < 1 || max_inflight > 64 || arena_bytes < (1 << 20)) return BSFIT_E_INVALID;
  *out = nullptr;
  bsfit_server_s* s = new (std::nothrow) bsfit_server_s;
  if (!s) return BSFIT_E_NOT_ENOUGH_MEMORY;
  cudaGetDevice(&s->device);
  cudaError_t e = cudaMalloc(&s->arena_base, (size_t)arena_bytes);
  if (e != cudaSuccess) {
    delete s;
    return cuda_status_s(e);
  }
  s->arena.init(arena_bytes);
  s->streams.resize(max_inflight, nullptr);
  s->slot_req.assign(max_inflight, {});
  for (int i = 0; i < max_inflight && e == cudaSuccess; ++i)
    e = cudaStreamCreateWithFlags(&s->streams[i], cudaStreamNonBlocking);
  // the priority streams: levels spread over the device's priority range
  int least = 0, greatest = 0;
  if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
  s->pstreams.resize((size_t)max_inflight * kLevels, nullptr);
  for (int i = 0; i < max_inflight * kLevels && e == cudaSuccess; ++i) {
    const int lv = i % kLevels;  // 0: greatest priority
    const int pr = greatest + (least - greatest) * lv / (kLevels - 1);
    e = cudaStreamCreateWithPriority(&s->pstreams[i], cudaStreamNonBlocking, pr);
  }
  if (e != cudaSuccess) {
    for (auto st : s->streams)
      if (st) cudaStreamDestroy(st);
    for (auto st : s->pstreams)
      if (st) cudaStreamDestroy(st);
    cudaFree(s->arena_base);
    delete s;
    return cuda_status_s(e);
  }
  *out = s;
  return BSFIT_OK;
}

int bsfit_server_set_merge(bsfit_server s, int32_t max_requests_per_launch) {
  if (!s || max_requests_per_launch < 1 || max_requests_per_launch > BSFIT_MAX_SEGMENTS)
    return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  s->merge = max_requests_per_launch;
  return BSFIT_OK;
}

int bsfit_server_set_priority(bsfit_server s, int32_t enable) {
  if (!s) return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  s->priority = enable != 0;
  return BSFIT_OK;
}

int bsfit_server_destroy(bsfit_server s) {
  if (!s) return BSFIT_E_INVALID;
  for (auto st : s->streams) cudaStreamSynchronize(st);
  for (auto st : s->pstreams) cudaStreamSynchronize(st);
  for (auto st : s->streams) cudaStreamDestroy(st);
  for (auto st : s->pstreams) cudaStreamDestroy(st);
  cudaFree(s->arena_base);
  for (auto& kv : s->all) delete kv.second;
  delete s;
  return BSFIT_OK;
}

int bsfit_server_submit(bsfit_server s, const bsfit_host_segment* segs, int32_t nseg,
                        int64_t* request_id) {
  return bsfit_server_submit_multistart(s, segs, nullptr, nseg, request_id);
}

int bsfit_server_submit_multistart(bsfit_server s, const bsfit_host_segment* segs,
                                   const bsfit_starts* starts, int32_t nseg,
                                   int64_t* request_id) {
  if (!s || !segs || nseg < 1 || nseg > BSFIT_MAX_SEGMENTS || !request_id) return BSFIT_E_INVALID;
  for (int i = 0; i < nseg; ++i) {
    const bsfit_host_segment& g = segs[i];
    if (!g.model || g.nfits < 0 || (g.nfits > 0 && (!g.rois || !g.P || !g.CRLB || !g.LL)))
      return BSFIT_E_INVALID;
    if (g.roi_size < 1 || g.roi_size > 51) return BSFIT_E_SUBREGION_SIZE;
    if (starts) {
      if (starts[i].n_starts < 0 || starts[i].n_starts > BSFIT_MAX_STARTS) return BSFIT_E_INVALID;
      if (bsfit_model_fittype(g.model) == 6 && starts[i].n_starts > 1)
        return BSFIT_E_UNSUPPORTED_FITTYPE;
    }
  }
  std::lock_guard<std::mutex> lock(s->mu);
  Request* r = new (std::nothrow) Request;
  if (!r) return BSFIT_E_NOT_ENOUGH_MEMORY;
  r->segs.assign(segs, segs + nseg);
  if (starts) r->starts.assign(starts, starts + nseg);
  r->bytes = request_bytes(r->segs);
  if (r->bytes > s->arena.size()) {
    delete r;
    return BSFIT_E_NOT_ENOUGH_MEMORY;  // can never fit the HBM budget
  }
  for (const auto& g : r->segs) r->rois += g.nfits;
  r->id = s->next_id++;
  r->submitted = Clock::now();
  if (!s->any_submit) {
    s->first_submit = r->submitted;
    s->last_done = r->submitted;
    s->any_submit = true;
  }
  s->all[r->id] = r;
  s->pending.push_back(r);
  retire(s);
  admit(s);
  *request_id = r->id;
  return BSFIT_OK;
}

int bsfit_server_poll(bsfit_server s, int64_t* done_ids, int32_t max_ids, int32_t* n_done) {
  if (!s || !n_done || (max_ids > 0 && !done_ids)) return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  retire(s);
  admit(s);
  int n = 0;
  for (auto it = s->all.begin(); it != s->all.end() && n < max_ids;) {
    Request* r = it->second;
    if (r->finished.load(std::memory_order_acquire) && !running(s, r)) {
      done_ids[n++] = r->id;
      delete r;
      it = s->all.erase(it);
    } else {
      ++it;
    }
  }
  *n_done = n;
  return BSFIT_OK;
}

int bsfit_server_wait(bsfit_server s, int64_t request_id, double timeout_s) {
  if (!s) return BSFIT_E_INVALID;
  const Clock::time_point limit = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                                      std::chrono::duration<double>(timeout_s));
  for (;;) {
    {
      std::lock_guard<std::mutex> lock(s->mu);
      retire(s);
      admit(s);
      auto it = s->all.find(request_id);
      if (it == s->all.end()) return BSFIT_E_INVALID;  // unknown or already collected
      Request* r = it->second;
      if (r->finished.load(std::memory_order_acquire) && !running(s, r)) {
        int st = r->status;
        delete r;
        s->all.erase(it);
        return st;
      }
    }
    if (Clock::now() > limit) return BSFIT_E_TIMEOUT;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

int bsfit_server_stats(bsfit_server s, double* p50_ms, double* p99_ms, double* fits_per_s,
                       int64_t* completed, int64_t* in_flight, int64_t* queued) {
  if (!s) return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  retire(s);
  std::vector<double> v = s->latencies_ms;
  std::sort(v.begin(), v.end());
  auto q = [&](double f) {
    if (v.empty()) return 0.0;
    size_t i = (size_t)std::min<double>((double)v.size() - 1, std::ceil(f * (double)v.size()) - 1);
    return v[i];
  };
  if (p50_ms) *p50_ms = q(0.50);
  if (p99_ms) *p99_ms = q(0.99);
  if (fits_per_s) {
    double span = std::chrono::duration<double>(s->last_done - s->first_submit).count();
    *fits_per_s = span > 0 ? (double)s->rois_done / span : 0.0;
  }
  if (completed) *completed = (int64_t)s->latencies_ms.size();
  int64_t fl = 0;
  for (const auto& grp : s->slot_req) fl += (int64_t)grp.size();
  if (in_flight) *in_flight = fl;
  if (queued) *queued = (int64_t)s->pending.size();
  return BSFIT_OK;
}

int bsfit_server_latencies(bsfit_server s, int64_t* ids, double* ms, int32_t max_n,
                           int32_t* n) {
  if (!s || !n || max_n < 0 || (max_n > 0 && (!ids || !ms))) return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  retire(s);
  const size_t k = std::min<size_t>((size_t)max_n, s->latencies_ms.size());
  for (size_t i = 0; i < k; ++i) {
    ids[i] = s->latency_ids[i];
    ms[i] = s->latencies_ms[i];
  }
  *n = (int32_t)k;
  return BSFIT_OK;
}

int bsfit_server_reset_stats(bsfit_server s) {
  if (!s) return BSFIT_E_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  s->latencies_ms.clear();
  s->latency_ids.clear();
  s->rois_done = 0;
  s->any_submit = false;
  return BSFIT_OK;
}

}  // extern "C"
