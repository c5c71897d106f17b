// mc_noalloc.cu -- the Monte Carlo entry point for callers that cannot
// allocate device memory.
//
// monte_mc_run keeps its scratch (the device copies of the interaction
// tables, the per-view and per-pixel aim tables, the persistent kernel's
// history counter and the run statistics) in buffers it cudaMallocs inside
// a context.  Some callers cannot let a library do that: services that
// reserve all of the GPU's memory for their own pool at start-up, hosts
// whose framework owns every device allocation through a caching
// allocator, and latency-critical loops where a cudaMalloc -- which may
// synchronize the device -- is not acceptable.  monte_mc_run_noalloc runs
// the same persistent kernel with all of that scratch in one file-scope
// __device__ array, reserved when the library is loaded, so the call
// itself allocates nothing.  The caller passes its own device arrays for
// the label volume and the two tallies.
//
// Facts a caller must know:
//  * The array is g_noalloc_scratch below: sizeof(NoallocScratch), about
//    280 KB, on every GPU that loads the library, held until the process
//    exits.  It fixes the limits: at most MONTE_NOALLOC_MAX_VIEWS views and
//    MONTE_NOALLOC_MAX_PIXELS detector pixels along each axis; larger
//    requests are rejected with MONTE_EINVAL.
//  * The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and keeps it for the
//    life of the process; a cudaDeviceReset on that device between calls
//    would leave it stale, so do not reset a device this entry point has
//    used.
//  * The call cannot be captured into a CUDA graph: its tables go up from
//    host staging that the next call overwrites, and with statistics it
//    waits for the stream.  A call on a capturing stream returns
//    MONTE_EUNSUPPORTED before it issues any work.
//  * labels, primary and scatter must be device memory (or managed);
//    anything else is rejected with MONTE_EINVAL.
//  * Every call on a device shares the array and leaves the last call's
//    tables in it.  Each call re-initialises what it needs (tables, counter
//    and statistics are written before its kernel starts), but two calls
//    whose work overlaps on the GPU -- on different streams, or issued from
//    different host threads -- race on the array and both results are
//    invalid.  Serialize them.
#include <cstddef>
#include <cstring>
#include <mutex>

#include "mc.cuh"
#include "mc_setup.h"
#include "monte_internal.h"

namespace monte {
namespace {

struct NoallocScratch {
  mc_tables tables;
  mc_view views[MONTE_NOALLOC_MAX_VIEWS];
  mc_pixel pixels[2 * MONTE_NOALLOC_MAX_PIXELS];
  unsigned long long stats[12];
  unsigned long long counter[8];
};

// The scratch of monte_mc_run_noalloc (see the file comment).  In host code
// this name is only a handle for the runtime: the device address comes from
// cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoallocScratch)];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device, looked up once per
// device.
int scratch_address(int dev, NoallocScratch** out) {
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(nullptr, MONTE_EUNSUPPORTED, "device %d beyond the %d this build tracks", dev,
                     kMaxDevices);
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return set_error(nullptr, MONTE_ECUDA, "cudaGetSymbolAddress of the scratch array: %s",
                       cudaGetErrorString(e));
    }
    g_addr[dev] = p;
  }
  *out = reinterpret_cast<NoallocScratch*>(g_addr[dev]);
  return MONTE_OK;
}

// Whether p is memory the GPU can address directly (device or managed).
bool device_addressable(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Host staging for the tables: per thread, static storage (no allocation).
thread_local mc_tables tl_tables;
thread_local mc_view tl_views[MONTE_NOALLOC_MAX_VIEWS];
thread_local mc_pixel tl_pixels[2 * MONTE_NOALLOC_MAX_PIXELS];

}  // namespace
}  // namespace monte

using namespace monte;

extern "C" int monte_mc_run_noalloc(const monte_mc_geom* g, const monte_mc_phantom* ph,
                                    const monte_xcom* xcom, const monte_spectrum* spec,
                                    const monte_mc_request* run, int64_t* primary,
                                    int64_t* scatter, monte_mc_stats* stats, void* cuda_stream) {
  if (!g || !ph || !xcom || !spec || !run || !primary || !scatter || !ph->labels)
    return set_error(nullptr, MONTE_EINVAL, "monte_mc_run_noalloc: null argument");
  if (g->n_views > MONTE_NOALLOC_MAX_VIEWS || g->nu > MONTE_NOALLOC_MAX_PIXELS ||
      g->nv > MONTE_NOALLOC_MAX_PIXELS)
    return set_error(nullptr, MONTE_EINVAL,
                     "monte_mc_run_noalloc: %d views of %d x %d pixels exceed its static scratch "
                     "(at most %d views and %d pixels per axis)",
                     g->n_views, g->nu, g->nv, MONTE_NOALLOC_MAX_VIEWS, MONTE_NOALLOC_MAX_PIXELS);
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing((cudaStream_t)cuda_stream, &cs);
    if (ce != cudaSuccess) {
      cudaGetLastError();
      return cuda_fail(nullptr, ce, "monte_mc_run_noalloc: stream query");
    }
    if (cs != cudaStreamCaptureStatusNone)
      return set_error(nullptr, MONTE_EUNSUPPORTED,
                       "monte_mc_run_noalloc: the stream is being captured; this call cannot "
                       "be part of a CUDA graph");
  }
  if (!device_addressable(ph->labels) || !device_addressable(primary) ||
      !device_addressable(scatter))
    return set_error(nullptr, MONTE_EINVAL,
                     "monte_mc_run_noalloc: labels, primary and scatter must be device memory");
  if (g->flags & MONTE_MC_LOCAL_MAJORANT)
    return set_error(nullptr, MONTE_EUNSUPPORTED,
                     "monte_mc_run_noalloc: MONTE_MC_LOCAL_MAJORANT needs per-phantom tables "
                     "that its static scratch does not hold");
  mc_params P;
  const char* why = "";
  if (mc_setup_params(g, ph, run, &P, &why) != MONTE_OK)
    return set_error(nullptr, MONTE_EINVAL, "monte_mc_run_noalloc: %s", why);
  if (mc_setup_tables(ph, xcom, spec, &tl_tables, &why) != MONTE_OK)
    return set_error(nullptr, MONTE_EINVAL, "monte_mc_run_noalloc: %s", why);
  mc_setup_views(g, tl_views);
  mc_setup_pixels(g, tl_pixels, tl_pixels + g->nu);
  const unsigned long long npix =
      (unsigned long long)(run->u_end - run->u_begin) * (unsigned long long)(run->v_end - run->v_begin);
  const unsigned long long nview = (unsigned long long)(run->view_end - run->view_begin);
  unsigned long long total = 0;
  if (npix && nview && run->histories_per_pixel) {
    if (npix * nview > (1ull << 62) / run->histories_per_pixel)
      return set_error(nullptr, MONTE_EOVERFLOW, "monte_mc_run_noalloc: too many histories");
    total = npix * nview * run->histories_per_pixel;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "monte_mc_run_noalloc: device query");
  NoallocScratch* S = nullptr;
  MONTE_TRY(scratch_address(dev, &S));
  cudaStream_t st = (cudaStream_t)cuda_stream;
  // tables from this thread's static staging (pageable: the copy has read
  // them when cudaMemcpyAsync returns), then a zeroed counter and statistics
  e = cudaMemcpyAsync(&S->tables, &tl_tables, sizeof(mc_tables), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(S->views, tl_views, sizeof(mc_view) * g->n_views, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(S->pixels, tl_pixels, sizeof(mc_pixel) * (g->nu + g->nv),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->stats, 0, sizeof(S->stats) + sizeof(S->counter), st);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "monte_mc_run_noalloc: table upload");
  McDev d;
  memset(&d, 0, sizeof(d));
  d.P = P;
  d.T = &S->tables;
  d.V = S->views;
  d.U = S->pixels;
  d.W = S->pixels + g->nu;
  d.labels = ph->labels;
  d.prim = (unsigned long long*)primary;
  d.scat = (unsigned long long*)scatter;
  d.stats = S->stats;
  d.counter = S->counter;
  d.total = total;
  if (total) {
    e = launch_mc(d, run->kernel, sms, st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "monte_mc_run_noalloc: launch");
  }
  if (stats) {
    unsigned long long h[kMcStats];
    e = cudaMemcpyAsync(h, S->stats, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "monte_mc_run_noalloc: statistics");
    mc_stats_from(h, stats);
  }
  return MONTE_OK;
}
