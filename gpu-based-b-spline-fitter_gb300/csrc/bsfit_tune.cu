// Launch configurations of the FP32 fit kernels chosen by the autotuner.
//
// The reference launches every fit with one fixed shape (64-thread blocks, one
// thread per ROI: VC/GPUmleFit_LM/mexFunction.cpp:407, BlockSize = BSZ). Here
// the shape of a fit launch has two free parameters whose best values depend on
// the fit type, the ROI size and the device:
//  - the kernel variant: the minimum number of resident 4-warp blocks per SM
//    the kernel is compiled for (__launch_bounds__), which sets its register
//    budget and so trades registers (and spills) against resident warps;
//  - the warps per block (4, 2 or 1), which sets how finely the per-warp
//    shared memory (ROI pixels and maps, growing with the ROI size) packs into
//    the SM's shared memory;
//  - for fit type 8, the staging of stage A's gathers: into registers, or into
//    shared memory with asynchronous copies one round of 32 nodes ahead;
//  - for fit type 6, the ROIs per warp: one (32 lanes per ROI), or two, either
//    one per half-warp (bsfit_pair.cuh), which shares the per-evaluation work
//    that does not grow with the ROI between two ROIs at twice the shared
//    memory per warp, or both on all 32 lanes in the two halves of paired FP32
//    operations (bsfit_pack.cuh), which shares the whole evaluation.
// Variant 0 is the default kernel (bsfit_fit.cu); this file instantiates the
// others. Every variant runs the same code, so results are bit-identical
// across configurations. A table per (fit type, ROI size, device) holds the
// chosen configuration; launch_fit and launch_batch consult it.
#include <mutex>

#include "bsfit_fit_kernels.cuh"
#include "bsfit_pack.cuh"
#include "bsfit_pair.cuh"

namespace bsfit {

namespace {

// fit type 6: variants 3 to 5 fit two ROIs per warp on its halves, 6 and 7
// two ROIs per warp in paired operations
constexpr int kNumVariants6 = 8;
constexpr int kMinBlocks6[kNumVariants6] = {BSFIT_MINBLOCKS(6), 5, 4, 6, 5, 4, 4, 3};
constexpr int kRoisPerWarp6[kNumVariants6] = {1, 1, 1, 2, 2, 2, 2, 2};
constexpr bool kPacked6[kNumVariants6] = {false, false, false, false, false, false, true, true};
constexpr int kMinBlocks7[3] = {BSFIT_MINBLOCKS(7), 3, 5};
// fit type 8: variants 2 and 3 stage the 5D gathers through shared memory
// (cp.async, two rounds of 32 nodes in flight per warp)
constexpr int kMinBlocks8[4] = {BSFIT_MINBLOCKS(8), 2, 2, 1};
constexpr bool kStaged8[4] = {false, false, true, true};

struct Entry {
  int mode, s, dev;
  TuneConfig c;
};
std::mutex g_tune_mu;
constexpr int kMaxEntries = 512;
Entry g_tune[kMaxEntries];
int g_ntune = 0;

}  // namespace

int tune_num_variants(int mode) {
  return mode == 6 ? kNumVariants6 : mode == 7 ? 3 : mode == 8 ? 4 : 0;
}

int tune_rois_per_warp(int mode, int variant) {
  return (mode == 6 && variant >= 0 && variant < kNumVariants6) ? kRoisPerWarp6[variant] : 1;
}

int tune_warp_floats(int mode, int variant, int s, bool var) {
  if (mode == 6 && variant >= 0 && variant < kNumVariants6 && kPacked6[variant])
    return make_pack_layout(s).total();
  return tune_rois_per_warp(mode, variant) * warp_smem_floats(mode, s, var, tune_staged(mode, variant));
}

int tune_staged(int mode, int variant) {
  return (mode == 8 && variant >= 0 && variant < 4 && kStaged8[variant]) ? 1 : 0;
}

int tune_min_blocks(int mode, int variant) {
  if (variant < 0 || variant >= tune_num_variants(mode)) return 0;
  return mode == 6 ? kMinBlocks6[variant] : mode == 7 ? kMinBlocks7[variant] : kMinBlocks8[variant];
}

FitKern fit_variant(int mode, int variant) {
  switch (mode * 10 + variant) {
    case 61: return fit_kernel<6, false, false, kMinBlocks6[1]>;
    case 62: return fit_kernel<6, false, false, kMinBlocks6[2]>;
    case 63: return fit_pair_kernel<kMinBlocks6[3]>;
    case 64: return fit_pair_kernel<kMinBlocks6[4]>;
    case 65: return fit_pair_kernel<kMinBlocks6[5]>;
    case 66: return fit_pack_kernel<kMinBlocks6[6]>;
    case 67: return fit_pack_kernel<kMinBlocks6[7]>;
    case 71: return fit_kernel<7, false, false, kMinBlocks7[1]>;
    case 72: return fit_kernel<7, false, false, kMinBlocks7[2]>;
    case 81: return fit_kernel<8, false, false, kMinBlocks8[1]>;
    case 82: return fit_kernel<8, false, false, kMinBlocks8[2], 1>;
    case 83: return fit_kernel<8, false, false, kMinBlocks8[3], 1>;
    default: return nullptr;
  }
}

BatchKern batch_variant(int mode, int variant) {
  switch (mode * 10 + variant) {
    case 61: return batch_kernel<6, false, kMinBlocks6[1]>;
    case 62: return batch_kernel<6, false, kMinBlocks6[2]>;
    case 63: return batch_pair_kernel<kMinBlocks6[3]>;
    case 64: return batch_pair_kernel<kMinBlocks6[4]>;
    case 65: return batch_pair_kernel<kMinBlocks6[5]>;
    case 66: return batch_pack_kernel<kMinBlocks6[6]>;
    case 67: return batch_pack_kernel<kMinBlocks6[7]>;
    case 71: return batch_kernel<7, false, kMinBlocks7[1]>;
    case 72: return batch_kernel<7, false, kMinBlocks7[2]>;
    case 81: return batch_kernel<8, false, kMinBlocks8[1]>;
    case 82: return batch_kernel<8, false, kMinBlocks8[2], 1>;
    case 83: return batch_kernel<8, false, kMinBlocks8[3], 1>;
    default: return nullptr;
  }
}

bool tune_lookup(int mode, int s, int dev, TuneConfig* out) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (int i = 0; i < g_ntune; ++i)
    if (g_tune[i].mode == mode && g_tune[i].s == s && g_tune[i].dev == dev) {
      *out = g_tune[i].c;
      return true;
    }
  return false;
}

bool tune_store(int mode, int s, int dev, TuneConfig c) {
  if (c.variant < 0 || c.variant >= tune_num_variants(mode)) return false;
  if (c.wpb != 0 && c.wpb != 1 && c.wpb != 2 && c.wpb != 4) return false;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (int i = 0; i < g_ntune; ++i)
    if (g_tune[i].mode == mode && g_tune[i].s == s && g_tune[i].dev == dev) {
      g_tune[i].c = c;
      return true;
    }
  if (g_ntune >= kMaxEntries) return false;
  g_tune[g_ntune++] = Entry{mode, s, dev, c};
  return true;
}

void tune_clear(int mode, int s, int dev) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (int i = 0; i < g_ntune; ++i)
    if (g_tune[i].mode == mode && g_tune[i].s == s && g_tune[i].dev == dev) {
      g_tune[i] = g_tune[--g_ntune];
      return;
    }
}

}  // namespace bsfit
