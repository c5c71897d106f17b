// monte_internal.h -- shared host-side plumbing of libmonte: the context,
// error reporting, and grow-only device scratch buffers.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/monte.h"
#include "bp_footprints.h"

namespace monte {

// A device allocation owned by a context, grown on demand, never shrunk
// until the context is destroyed.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct ViewCache;  // per-geometry device tables (fdk_api.cu)

}  // namespace monte

struct monte_ctx {
  int device = 0;
  int sm_count = 0;
  int cc_major = 0, cc_minor = 0;
  size_t smem_optin = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;  // own_stream or a caller-provided one
  std::string last_error;
  // named scratch buffers
  monte::DevBuf scratch[16];
  // cached FDK device tables for the last geometry seen
  std::vector<uint8_t> fdk_key;
  monte::DevBuf fdk_views, fdk_viewsd, fdk_weights, fdk_taps, fdk_bsplit;
  // cached MC device tables
  std::vector<uint8_t> mc_key;
  // what the local-majorant tables in mc_mclass were built from (phantom
  // grid, label materials and densities, attenuation tables, and for host
  // labels the cells' label sets): a call with the same key reuses them.
  // For device labels the label volume itself is kept in mc_label_copy
  // (mc_label_bytes of it) and compared on the device.
  std::vector<uint8_t> mc_macro_key;
  monte::DevBuf mc_tables, mc_views, mc_pixels, mc_mclass, mc_label_copy;
  size_t mc_label_bytes = 0;
  // device-side error flag word for bounded waits / kernel status
  int* d_status = nullptr;
  // autotuned backprojection tile choice, keyed by geometry
  std::vector<uint8_t> bp_tune_key;
  int bp_tune_choice = -1;
  int last_bp_variant = -1;  // tile variant of the last backprojection, -1: plain kernel
  // host-memory FDK pipeline (created on first use): upload and download
  // streams, a high-priority stream for the filter of each view range, and
  // the events that order them against `stream`
  cudaStream_t copy_in = nullptr, copy_out = nullptr, filter_stream = nullptr;
  // footprint table of the tiled backprojector's last geometry and shape
  monte::BpFootprints bp_footprints;
  cudaEvent_t pipe_ev[24] = {};
  bool pipe_ready = false;
  int last_host_ranges = 0;  // view ranges of the last pipelined monte_fdk, 0: unpipelined
};

namespace monte {

// Scratch slots used by the entry points.
enum ScratchSlot {
  kScratchProj = 0,
  kScratchFiltered = 1,
  kScratchVolXY = 2,
  kScratchVolZY = 3,
  kScratchMcPrimary = 4,
  kScratchMcScatter = 5,
  kScratchLabels = 6,
  kScratchAux0 = 7,
  kScratchAux1 = 8,
  kScratchAux2 = 9,
  kScratchAux3 = 10,
  kScratchStats = 11,
  kScratchFbp2 = 12,
  kScratchBpPad = 13,  // filtered projections with rows padded to 16 bytes (TMA)
  kScratchSiddon = 14,  // the Siddon adjoint's fixed-point sums and scale
};

int set_error(monte_ctx* ctx, int code, const char* fmt, ...);
int cuda_fail(monte_ctx* ctx, cudaError_t e, const char* what);
// Ensure the slot holds at least `bytes` bytes; returns status.
int ensure(monte_ctx* ctx, DevBuf& b, size_t bytes, const char* what);
inline int ensure_slot(monte_ctx* ctx, int slot, size_t bytes, const char* what) {
  return ensure(ctx, ctx->scratch[slot], bytes, what);
}
void release(DevBuf& b);

// Make the context's device current for this thread.
int enter(monte_ctx* ctx);

// Checked multiplication of sizes.
inline bool mul_ok(size_t a, size_t b, size_t* out) {
  if (a != 0 && b > SIZE_MAX / a) return false;
  *out = a * b;
  return true;
}

}  // namespace monte

#define MONTE_CUDA(ctx, expr)                                  \
  do {                                                         \
    cudaError_t e_ = (expr);                                   \
    if (e_ != cudaSuccess) return monte::cuda_fail(ctx, e_, #expr); \
  } while (0)

#define MONTE_TRY(expr)             \
  do {                              \
    int s_ = (expr);                \
    if (s_ != MONTE_OK) return s_;  \
  } while (0)
