// batch.cu -- batched scans: Monte Carlo of many phantoms followed by the FDK
// reconstruction of each (include/monte.h, monte_batch_*).
//
// The reference runs one phantom per program invocation: the projection
// launch and post-processing of monte_cu/CBCT_real325im.cu:235-294, then
// recon/bp3d20.cpp:15-194 on the map it wrote.  A plan here holds every
// table of every job in one device arena and runs the batch in one of two
// forms:
//   FUSED       one persistent Monte Carlo launch over the histories of all
//               jobs (lanes refill from any job), then per job finalize ->
//               filter -> backprojection on one of kLanes streams, all
//               captured once into a CUDA graph and replayed by
//               monte_batch_run;
//   SEQUENTIAL  per job, in order, the plain one-thread-per-pixel Monte
//               Carlo kernel, finalize, FP32 filter and plain backprojector:
//               the one-instance form the batch is measured against.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fdk.cuh"
#include "mc.cuh"
#include "mc_setup.h"
#include "monte_internal.h"

namespace monte {
namespace {

constexpr int kLanes = 4;
constexpr size_t kAlign = 256;

size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

struct BatchJob {
  monte_batch_job job;
  FdkDev fdk;
  McDev mc;                      // device pointers filled after the arena exists
  size_t ncell = 0;              // n_views * nu * nv
  unsigned long long histories = 0;
  double log_per = 0.0;
  int filter_mode = MONTE_FILTER_FP32;
  int bp_variant = -1;           // -1: plain backprojector
  int lane = 0;
  double cost = 0.0;
  // arena offsets
  size_t o_tables = 0, o_views = 0, o_pixels = 0;
  size_t o_bpv = 0, o_bpvd = 0, o_weights = 0, o_taps = 0, o_bsplit = 0;
  size_t o_filtered = 0, o_map = 0;
  size_t o_local = 0;            // local-majorant tables + class grid (MONTE_MC_LOCAL_MAJORANT)
  // device pointers
  const BpView* bpv = nullptr;
  const BpViewD* bpvd = nullptr;
  const float* weights = nullptr;
  const float* taps = nullptr;
  const uint16_t* bsplit = nullptr;
  float* filtered = nullptr;
  float* map = nullptr;
};

}  // namespace
}  // namespace monte

struct monte_batch {
  monte_ctx* ctx = nullptr;
  int mode = MONTE_BATCH_FUSED;
  std::vector<monte::BatchJob> jobs;
  monte::DevBuf arena;
  size_t o_mcdev = 0, o_starts = 0, o_counters = 0;
  unsigned long long total = 0;
  bool mc_all_local = false;               // every job uses MONTE_MC_LOCAL_MAJORANT
  unsigned long long* counters = nullptr;  // [0] batch counter, [4..13] stats, [16+j] per job
  cudaStream_t lanes[monte::kLanes] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[monte::kLanes] = {};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace monte {
namespace {

int job_error(monte_ctx* ctx, int j, int code, const char* why) {
  return set_error(ctx, code, "batch job %d: %s", j, why);
}

// Checks one job, fills the host-side parts of its plan and its sizes.
int plan_job(monte_ctx* ctx, const monte_xcom* xcom, int j, BatchJob* b) {
  const monte_batch_job& J = b->job;
  const monte_mc_geom& g = J.mc;
  if (!J.phantom.labels || !J.primary || !J.scatter || !J.vol_xy)
    return job_error(ctx, j, MONTE_EINVAL, "null labels/primary/scatter/vol_xy");
  if (J.histories_per_pixel == 0 || J.histories_per_pixel > (uint64_t)INT32_MAX)
    return job_error(ctx, j, MONTE_EINVAL, "histories_per_pixel must be 1..2^31-1");
  if (J.recon_total != 0 && J.recon_total != 1)
    return job_error(ctx, j, MONTE_EINVAL, "recon_total must be 0 or 1");
  if (J.fdk.n_views != g.n_views || J.fdk.nu != g.nu || J.fdk.nv != g.nv)
    return job_error(ctx, j, MONTE_EINVAL, "FDK detector differs from the Monte Carlo detector");
  MONTE_TRY(fdk_validate(ctx, &J.fdk, true));
  monte_mc_request r;
  memset(&r, 0, sizeof(r));
  r.seed = J.seed;
  r.histories_per_pixel = J.histories_per_pixel;
  r.view_begin = 0;
  r.view_end = g.n_views;
  r.u_begin = 0;
  r.u_end = g.nu;
  r.v_begin = 0;
  r.v_end = g.nv;
  r.kernel = MONTE_MC_PERSISTENT;
  r.job = (uint32_t)j;
  const char* why = "";
  memset(&b->mc, 0, sizeof(b->mc));
  if (mc_setup_params(&g, &J.phantom, &r, &b->mc.P, &why) != MONTE_OK)
    return job_error(ctx, j, MONTE_EINVAL, why);
  // the XCOM/spectrum/label tables are checked here and rebuilt at upload
  std::vector<mc_tables> T(1);
  if (mc_setup_tables(&J.phantom, xcom, &J.spectrum, T.data(), &why) != MONTE_OK)
    return job_error(ctx, j, MONTE_EINVAL, why);
  b->ncell = (size_t)g.n_views * g.nu * g.nv;
  if (b->ncell > ((size_t)1 << 40) / J.histories_per_pixel)
    return job_error(ctx, j, MONTE_EOVERFLOW, "too many histories");
  b->histories = (unsigned long long)b->ncell * J.histories_per_pixel;
  b->log_per = (double)(float)std::log((double)J.histories_per_pixel);
  b->fdk = make_fdk_dev(J.fdk);
  const double upd = (double)(J.fdk.s_end - J.fdk.s_begin) * J.fdk.ny * J.fdk.nz * J.fdk.n_views;
  b->cost = upd + 4.0 * (double)b->ncell * g.nu;
  return MONTE_OK;
}

int upload(monte_ctx* ctx, const void* host, void* dev, size_t bytes) {
  if (!bytes) return MONTE_OK;
  MONTE_CUDA(ctx, cudaMemcpyAsync(dev, host, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return MONTE_OK;
}

// Queue job b's finalize -> filter -> backprojection on stream st.
int enqueue_fdk(monte_ctx* ctx, const BatchJob& b, int* status, cudaStream_t st) {
  const monte_batch_job& J = b.job;
  const bool total = J.recon_total != 0;
  cudaError_t e = launch_mc_finalize(b.ncell, J.histories_per_pixel, b.log_per,
                                     (const long long*)J.primary, (const long long*)J.scatter,
                                     nullptr, total ? nullptr : b.map, nullptr,
                                     total ? b.map : nullptr, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch finalize launch");
  if (b.filter_mode == MONTE_FILTER_BF16X3)
    e = launch_fdk_filter_bf16x3(b.fdk, b.map, b.weights, b.bsplit, b.filtered, status,
                                 ctx->sm_count, st);
  else
    e = launch_fdk_filter_fp32(b.fdk, b.map, b.weights, b.taps, b.filtered, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch filter launch");
  if (J.fdk.s_begin != 0 || J.fdk.s_end != J.fdk.nx)
    MONTE_CUDA(ctx, cudaMemsetAsync(J.vol_xy, 0, (size_t)J.fdk.nx * J.fdk.ny * J.fdk.nz * 4, st));
  if (b.bp_variant >= 0)
    e = launch_fdk_bp_tiled(b.fdk, b.bpv, b.bpvd, b.filtered, J.vol_xy, nullptr, b.bp_variant,
                            status, st);
  else
    e = launch_fdk_bp_plain(b.fdk, b.bpv, b.bpvd, b.filtered, J.vol_xy, nullptr, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch backprojection launch");
  return MONTE_OK;
}

// Capture the fused form into b->graph and instantiate it.
int capture(monte_batch* B) {
  monte_ctx* ctx = B->ctx;
  const int n = (int)B->jobs.size();
  cudaStream_t s0 = B->lanes[0];
  MONTE_CUDA(ctx, cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
  int st = MONTE_OK;
  auto fail = [&](int code) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(s0, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return code;
  };
  cudaError_t e = cudaMemsetAsync(B->counters, 0, (16 + n) * sizeof(unsigned long long), s0);
  for (int j = 0; j < n && e == cudaSuccess; j++) {
    const BatchJob& b = B->jobs[j];
    e = cudaMemsetAsync(b.job.primary, 0, b.ncell * 8, s0);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.job.scatter, 0, b.ncell * 8, s0);
  }
  if (e != cudaSuccess) return fail(cuda_fail(ctx, e, "batch capture (zero tallies)"));
  if (B->total) {
    unsigned char* base = (unsigned char*)B->arena.ptr;
    e = launch_mc_batch((const McDev*)(base + B->o_mcdev),
                        (const unsigned long long*)(base + B->o_starts), n, B->total, B->counters,
                        B->counters + 4, B->mc_all_local, ctx->sm_count, s0);
    if (e != cudaSuccess) return fail(cuda_fail(ctx, e, "batch Monte Carlo launch"));
  }
  e = cudaEventRecord(B->fork, s0);
  for (int l = 1; l < kLanes && e == cudaSuccess; l++) e = cudaStreamWaitEvent(B->lanes[l], B->fork, 0);
  if (e != cudaSuccess) return fail(cuda_fail(ctx, e, "batch capture (fork)"));
  for (int j = 0; j < n; j++) {
    const BatchJob& b = B->jobs[j];
    st = enqueue_fdk(ctx, b, ctx->d_status, B->lanes[b.lane]);
    if (st != MONTE_OK) return fail(st);
  }
  for (int l = 1; l < kLanes && e == cudaSuccess; l++) {
    e = cudaEventRecord(B->join[l], B->lanes[l]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s0, B->join[l], 0);
  }
  if (e != cudaSuccess) return fail(cuda_fail(ctx, e, "batch capture (join)"));
  MONTE_CUDA(ctx, cudaStreamEndCapture(s0, &B->graph));
  MONTE_CUDA(ctx, cudaGraphInstantiate(&B->exec, B->graph, 0));
  return MONTE_OK;
}

void destroy_plan(monte_batch* B) {
  if (!B) return;
  if (B->ctx) cudaSetDevice(B->ctx->device);
  if (B->ctx && B->ctx->stream) cudaStreamSynchronize(B->ctx->stream);
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  for (int l = 0; l < kLanes; l++) {
    if (B->lanes[l]) cudaStreamDestroy(B->lanes[l]);
    if (B->join[l]) cudaEventDestroy(B->join[l]);
  }
  if (B->fork) cudaEventDestroy(B->fork);
  release(B->arena);
  delete B;
}

int create_plan(monte_ctx* ctx, const monte_xcom* xcom, const monte_batch_job* jobs, int n,
                int mode, int options, monte_batch* B) {
  B->ctx = ctx;
  B->mode = mode;
  B->jobs.resize(n);
  for (int j = 0; j < n; j++) {
    B->jobs[j].job = jobs[j];
    MONTE_TRY(plan_job(ctx, xcom, j, &B->jobs[j]));
  }
  // arena layout
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align_up(bytes);
    return o;
  };
  std::vector<FdkHostTables> ft(n);
  for (int j = 0; j < n; j++) {
    BatchJob& b = B->jobs[j];
    const monte_batch_job& J = b.job;
    build_fdk_tables(&J.fdk, &ft[j]);
    b.o_tables = take(sizeof(mc_tables));
    b.o_views = take((size_t)J.mc.n_views * sizeof(mc_view));
    b.o_pixels = take((size_t)(J.mc.nu + J.mc.nv) * sizeof(mc_pixel));
    b.o_bpv = take(ft[j].views.size() * sizeof(BpView));
    b.o_bpvd = take(ft[j].viewsd.size() * sizeof(BpViewD));
    b.o_weights = take(ft[j].weights.size() * 4);
    b.o_taps = take(ft[j].taps.size() * 4);
    b.o_bsplit = take(ft[j].bsplit.size() * 2);
    b.o_filtered = take(b.ncell * 4);
    if (J.mc.flags & MONTE_MC_LOCAL_MAJORANT)
      b.o_local = take(sizeof(mc_local_tables) +
                       (size_t)b.mc.P.mgx * b.mc.P.mgy * b.mc.P.mgz * sizeof(uint16_t));
    b.o_map = J.map ? 0 : take(b.ncell * 4);
    b.filter_mode = (mode == MONTE_BATCH_FUSED && !ft[j].bsplit.empty()) ? MONTE_FILTER_BF16X3
                                                                           : MONTE_FILTER_FP32;
  }
  B->o_mcdev = take((size_t)n * sizeof(McDev));
  B->o_starts = take((size_t)(n + 1) * sizeof(unsigned long long));
  B->o_counters = take((size_t)(16 + n) * sizeof(unsigned long long));
  MONTE_TRY(enter(ctx));
  MONTE_TRY(ensure(ctx, B->arena, off, "batch arena"));
  unsigned char* base = (unsigned char*)B->arena.ptr;
  B->counters = (unsigned long long*)(base + B->o_counters);
  // tables
  std::vector<McDev> devs(n);
  std::vector<unsigned long long> starts(n + 1, 0);
  std::vector<mc_tables> T(1);
  for (int j = 0; j < n; j++) {
    BatchJob& b = B->jobs[j];
    const monte_batch_job& J = b.job;
    const char* why = "";
    mc_setup_tables(&J.phantom, xcom, &J.spectrum, T.data(), &why);
    std::vector<mc_view> V(J.mc.n_views);
    std::vector<mc_pixel> UW(J.mc.nu + J.mc.nv);
    mc_setup_views(&J.mc, V.data());
    mc_setup_pixels(&J.mc, UW.data(), UW.data() + J.mc.nu);
    MONTE_TRY(upload(ctx, T.data(), base + b.o_tables, sizeof(mc_tables)));
    MONTE_TRY(upload(ctx, V.data(), base + b.o_views, V.size() * sizeof(mc_view)));
    MONTE_TRY(upload(ctx, UW.data(), base + b.o_pixels, UW.size() * sizeof(mc_pixel)));
    MONTE_TRY(upload(ctx, ft[j].views.data(), base + b.o_bpv, ft[j].views.size() * sizeof(BpView)));
    MONTE_TRY(upload(ctx, ft[j].viewsd.data(), base + b.o_bpvd, ft[j].viewsd.size() * sizeof(BpViewD)));
    MONTE_TRY(upload(ctx, ft[j].weights.data(), base + b.o_weights, ft[j].weights.size() * 4));
    MONTE_TRY(upload(ctx, ft[j].taps.data(), base + b.o_taps, ft[j].taps.size() * 4));
    MONTE_TRY(upload(ctx, ft[j].bsplit.data(), base + b.o_bsplit, ft[j].bsplit.size() * 2));
    std::vector<mc_local_tables> Lt;
    std::vector<uint16_t> cls;
    if (J.mc.flags & MONTE_MC_LOCAL_MAJORANT) {
      Lt.resize(1);
      MONTE_TRY(mc_build_macro(ctx, &J.phantom, xcom, true, b.mc.P, Lt.data(), &cls, nullptr));
      MONTE_TRY(upload(ctx, Lt.data(), base + b.o_local, sizeof(mc_local_tables)));
      MONTE_TRY(upload(ctx, cls.data(), base + b.o_local + sizeof(mc_local_tables),
                       cls.size() * sizeof(uint16_t)));
    }
    // the uploads read host vectors that die at the end of this iteration
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    b.bpv = (const BpView*)(base + b.o_bpv);
    b.bpvd = (const BpViewD*)(base + b.o_bpvd);
    b.weights = (const float*)(base + b.o_weights);
    b.taps = (const float*)(base + b.o_taps);
    b.bsplit = (const uint16_t*)(base + b.o_bsplit);
    b.filtered = (float*)(base + b.o_filtered);
    b.map = J.map ? J.map : (float*)(base + b.o_map);
    McDev& d = b.mc;
    d.T = (const mc_tables*)(base + b.o_tables);
    d.V = (const mc_view*)(base + b.o_views);
    d.U = (const mc_pixel*)(base + b.o_pixels);
    d.W = d.U + J.mc.nu;
    d.labels = J.phantom.labels;
    if (J.mc.flags & MONTE_MC_LOCAL_MAJORANT) {
      d.L = (const mc_local_tables*)(base + b.o_local);
      d.mclass = (const uint16_t*)(base + b.o_local + sizeof(mc_local_tables));
    }
    d.prim = (unsigned long long*)J.primary;
    d.scat = (unsigned long long*)J.scatter;
    d.stats = B->counters + 4;
    d.counter = B->counters + 16 + j;
    d.total = b.histories;
    devs[j] = d;
    starts[j + 1] = starts[j] + b.histories;
  }
  B->total = starts[n];
  B->mc_all_local = true;
  for (int j = 0; j < n; j++)
    B->mc_all_local = B->mc_all_local && (B->jobs[j].job.mc.flags & MONTE_MC_LOCAL_MAJORANT);
  MONTE_TRY(upload(ctx, devs.data(), base + B->o_mcdev, devs.size() * sizeof(McDev)));
  MONTE_TRY(upload(ctx, starts.data(), base + B->o_starts, starts.size() * sizeof(unsigned long long)));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (mode == MONTE_BATCH_SEQUENTIAL) return MONTE_OK;
  // backprojector tile shapes: the autotuner per distinct geometry, else the
  // context's choice or the default shape where it fits
  std::vector<std::pair<std::vector<uint8_t>, int>> tuned;
  for (int j = 0; j < n; j++) {
    BatchJob& b = B->jobs[j];
    int v = -1;
    if (options & MONTE_BATCH_AUTOTUNE) {
      std::vector<uint8_t> key(sizeof(monte_fdk_geom));
      memcpy(key.data(), &b.job.fdk, sizeof(monte_fdk_geom));
      bool found = false;
      for (auto& t : tuned)
        if (t.first == key) {
          v = t.second;
          found = true;
        }
      if (!found) {
        MONTE_CUDA(ctx, cudaMemsetAsync(b.filtered, 0, b.ncell * 4, ctx->stream));
        MONTE_TRY(fdk_tune_bp(ctx, &b.job.fdk, b.bpv, b.bpvd, b.filtered, b.job.vol_xy, &v,
                              kBpQuickCandidates, kBpQuickCandidatesN, 2));
        tuned.push_back({key, v});
      }
    } else {
      v = fdk_bp_pick(b.fdk, ctx->bp_tune_choice);
    }
    b.bp_variant = v;
  }
  // spread the FDK chains over the lanes, longest first
  std::vector<int> order(n);
  for (int j = 0; j < n; j++) order[j] = j;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return B->jobs[a].cost > B->jobs[c].cost; });
  double load[kLanes] = {0, 0, 0, 0};
  for (int j : order) {
    int l = (int)(std::min_element(load, load + kLanes) - load);
    B->jobs[j].lane = l;
    load[l] += B->jobs[j].cost;
  }
  for (int l = 0; l < kLanes; l++) {
    MONTE_CUDA(ctx, cudaStreamCreateWithFlags(&B->lanes[l], cudaStreamNonBlocking));
    MONTE_CUDA(ctx, cudaEventCreateWithFlags(&B->join[l], cudaEventDisableTiming));
  }
  MONTE_CUDA(ctx, cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming));
  return capture(B);
}

}  // namespace
}  // namespace monte

using namespace monte;

extern "C" {

int monte_batch_create(monte_ctx* ctx, const monte_xcom* xcom, const monte_batch_job* jobs,
                       int n_jobs, int mode, int options, monte_batch** out) {
  if (!ctx) return MONTE_EINVAL;
  if (!out) return set_error(ctx, MONTE_EINVAL, "null output handle");
  *out = nullptr;
  if (!jobs || !xcom) return set_error(ctx, MONTE_EINVAL, "null jobs or XCOM tables");
  if (n_jobs <= 0 || n_jobs > kMaxBatchJobs)
    return set_error(ctx, MONTE_EINVAL, "n_jobs must be 1..%d (got %d)", kMaxBatchJobs, n_jobs);
  if (mode != MONTE_BATCH_FUSED && mode != MONTE_BATCH_SEQUENTIAL)
    return set_error(ctx, MONTE_EINVAL, "unknown batch mode %d", mode);
  if (options & ~MONTE_BATCH_AUTOTUNE)
    return set_error(ctx, MONTE_EINVAL, "unknown batch options 0x%x", options);
  monte_batch* B = new monte_batch();
  int st = create_plan(ctx, xcom, jobs, n_jobs, mode, options, B);
  if (st != MONTE_OK) {
    destroy_plan(B);
    return st;
  }
  *out = B;
  return MONTE_OK;
}

int monte_batch_run(monte_batch* B) {
  if (!B) return MONTE_EINVAL;
  monte_ctx* ctx = B->ctx;
  MONTE_TRY(enter(ctx));
  if (B->mode == MONTE_BATCH_FUSED) {
    MONTE_CUDA(ctx, cudaGraphLaunch(B->exec, ctx->stream));
    return MONTE_OK;
  }
  const int n = (int)B->jobs.size();
  MONTE_CUDA(ctx, cudaMemsetAsync(B->counters, 0, (16 + n) * sizeof(unsigned long long), ctx->stream));
  for (int j = 0; j < n; j++) {
    const BatchJob& b = B->jobs[j];
    MONTE_CUDA(ctx, cudaMemsetAsync(b.job.primary, 0, b.ncell * 8, ctx->stream));
    MONTE_CUDA(ctx, cudaMemsetAsync(b.job.scatter, 0, b.ncell * 8, ctx->stream));
    cudaError_t e = launch_mc(b.mc, MONTE_MC_PLAIN, ctx->sm_count, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch Monte Carlo launch");
    MONTE_TRY(enqueue_fdk(ctx, b, ctx->d_status, ctx->stream));
  }
  return MONTE_OK;
}

int monte_batch_stats(monte_batch* B, monte_mc_stats* stats) {
  if (!B) return MONTE_EINVAL;
  monte_ctx* ctx = B->ctx;
  if (!stats) return set_error(ctx, MONTE_EINVAL, "null stats");
  MONTE_TRY(enter(ctx));
  unsigned long long h[kMcStats];
  MONTE_CUDA(ctx, cudaMemcpyAsync(h, B->counters + 4, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  mc_stats_from(h, stats);
  return MONTE_OK;
}

int monte_batch_bp_variant(const monte_batch* B, int job) {
  if (!B || job < 0 || job >= (int)B->jobs.size()) return -1;
  return B->jobs[job].bp_variant;
}

int monte_batch_destroy(monte_batch* B) {
  if (!B) return MONTE_EINVAL;
  destroy_plan(B);
  return MONTE_OK;
}

}  // extern "C"
