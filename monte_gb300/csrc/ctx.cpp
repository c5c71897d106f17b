// ctx.cpp -- context lifetime, streams, error text, scratch buffers.
//
// The reference has no runtime around its kernel: host main() calls
// cudaMalloc/cudaMemcpy directly and never checks a return code
// (monte_cu/CBCT_real325im.cu:94-111,235-248).  Here every CUDA call is
// checked and reported through the context.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "monte_internal.h"

namespace {
std::mutex g_err_mu;
std::string g_create_error = "no error";
}  // namespace

namespace monte {

int set_error(monte_ctx* ctx, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (ctx) {
    ctx->last_error = buf;
  } else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_error = buf;
  }
  return code;
}

int cuda_fail(monte_ctx* ctx, cudaError_t e, const char* what) {
  return set_error(ctx, MONTE_ECUDA, "%s failed: %s (%s)", what, cudaGetErrorName(e),
                   cudaGetErrorString(e));
}

int ensure(monte_ctx* ctx, DevBuf& b, size_t bytes, const char* what) {
  if (bytes <= b.bytes && b.ptr) return MONTE_OK;
  if (b.ptr) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
  }
  size_t want = bytes < 256 ? 256 : bytes;
  cudaError_t e = cudaMalloc(&b.ptr, want);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    cudaGetLastError();
    return set_error(ctx, MONTE_ENOMEM, "device allocation of %zu bytes for %s failed: %s", want,
                     what, cudaGetErrorString(e));
  }
  b.bytes = want;
  return MONTE_OK;
}

void release(DevBuf& b) {
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
}

int enter(monte_ctx* ctx) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_CUDA(ctx, cudaSetDevice(ctx->device));
  return MONTE_OK;
}

}  // namespace monte

extern "C" {

int monte_abi_version(void) { return MONTE_ABI_VERSION; }

int monte_ctx_create(monte_ctx** out, int device) {
  if (!out) return monte::set_error(nullptr, MONTE_EINVAL, "monte_ctx_create: out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return monte::set_error(nullptr, MONTE_ECUDA, "no usable CUDA device (%s)",
                            e == cudaSuccess ? "device count 0" : cudaGetErrorString(e));
  }
  if (device < 0 || device >= n)
    return monte::set_error(nullptr, MONTE_EINVAL, "device %d out of range [0,%d)", device, n);
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) return monte::set_error(nullptr, MONTE_ECUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
  if (prop.major < 10)
    return monte::set_error(nullptr, MONTE_EUNSUPPORTED,
                            "device %d is sm_%d%d; this library is built for sm_103a", device,
                            prop.major, prop.minor);
  monte_ctx* ctx = new monte_ctx();
  ctx->device = device;
  ctx->sm_count = prop.multiProcessorCount;
  ctx->cc_major = prop.major;
  ctx->cc_minor = prop.minor;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, 64 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, 64 * sizeof(int));
  if (e != cudaSuccess) {
    int rc = monte::set_error(nullptr, MONTE_ECUDA, "context set-up failed: %s", cudaGetErrorString(e));
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->d_status) cudaFree(ctx->d_status);
    delete ctx;
    return rc;
  }
  ctx->stream = ctx->own_stream;
  *out = ctx;
  return MONTE_OK;
}

int monte_ctx_destroy(monte_ctx* ctx) {
  if (!ctx) return MONTE_OK;
  cudaSetDevice(ctx->device);
  if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
  if (ctx->stream && ctx->stream != ctx->own_stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->copy_in) cudaStreamSynchronize(ctx->copy_in);
  if (ctx->copy_out) cudaStreamSynchronize(ctx->copy_out);
  if (ctx->filter_stream) cudaStreamSynchronize(ctx->filter_stream);
  for (auto& b : ctx->scratch) monte::release(b);
  monte::release(ctx->fdk_views);
  monte::release(ctx->fdk_viewsd);
  monte::release(ctx->fdk_weights);
  monte::release(ctx->fdk_taps);
  monte::release(ctx->fdk_bsplit);
  monte::release(ctx->mc_tables);
  monte::release(ctx->mc_views);
  monte::release(ctx->mc_mclass);
  monte::release(ctx->mc_label_copy);
  monte::release(ctx->mc_pixels);
  monte::fdk_bp_footprints_release(&ctx->bp_footprints);
  if (ctx->d_status) cudaFree(ctx->d_status);
  for (cudaEvent_t ev : ctx->pipe_ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->copy_in) cudaStreamDestroy(ctx->copy_in);
  if (ctx->copy_out) cudaStreamDestroy(ctx->copy_out);
  if (ctx->filter_stream) cudaStreamDestroy(ctx->filter_stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return MONTE_OK;
}

const char* monte_last_error(const monte_ctx* ctx) {
  if (ctx) return ctx->last_error.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  static thread_local std::string copy;
  copy = g_create_error;
  return copy.c_str();
}

// The context's scratch buffers and tables are reused by the next call,
// which nothing would order after work still queued on the old stream: a
// switch waits for that work first.
static int switch_stream(monte_ctx* ctx, cudaStream_t next) {
  if (next == ctx->stream) return MONTE_OK;
  MONTE_TRY(monte::enter(ctx));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->stream = next;
  return MONTE_OK;
}

int monte_ctx_set_stream(monte_ctx* ctx, void* cuda_stream) {
  if (!ctx) return MONTE_EINVAL;
  return switch_stream(ctx, (cudaStream_t)cuda_stream);
}

int monte_ctx_use_own_stream(monte_ctx* ctx) {
  if (!ctx) return MONTE_EINVAL;
  return switch_stream(ctx, ctx->own_stream);
}

int monte_ctx_synchronize(monte_ctx* ctx) {
  MONTE_TRY(monte::enter(ctx));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

int monte_ctx_check_status(monte_ctx* ctx) {
  MONTE_TRY(monte::enter(ctx));
  int h = 0;
  MONTE_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h != 0) {
    MONTE_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return monte::set_error(ctx, MONTE_ETIMEOUT,
                            "a bounded device wait gave up (kernel status %d); results of the "
                            "affected launch are invalid",
                            h);
  }
  return MONTE_OK;
}

}  // extern "C"
