// fdk_api.cu -- C-ABI entry points of the FDK path (include/monte.h):
// argument checks, per-geometry device tables, host staging, launches.
//
// Reference programs: recon/bp3d20.cpp (65x65 detector) and
// recon/bp3d20_325.cpp (325x325), whose main() reads the projection file,
// weights, filters, backprojects and writes three raw files
// (recon/bp3d20.cpp:15-194).  Here the same three stages run on the GPU
// behind monte_fdk_filter / monte_fdk_backproject / monte_fdk.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fdk.cuh"
#include "monte_internal.h"

namespace monte {

FdkDev make_fdk_dev(const monte_fdk_geom& g) {
  FdkDev d{};  // every byte defined: the tile caches compare FdkDev bytes
  d.x0d = g.x0;
  d.y0d = g.y0;
  d.z0d = g.z0;
  d.dvoxd = g.dvox;
  d.sddd = g.sdd;
  d.Dd = g.wdist;
  d.half_ud = g.half_u;
  d.half_vd = g.half_v;
  d.inv_dud = 1.0 / g.du;
  d.inv_dvd = 1.0 / g.dv;
  d.n_views = g.n_views;
  d.nu = g.nu;
  d.nv = g.nv;
  d.nx = g.nx;
  d.ny = g.ny;
  d.nz = g.nz;
  d.s_begin = g.s_begin;
  d.s_end = g.s_end;
  d.mask_r2 = g.mask_radius > 0 ? g.mask_radius * g.mask_radius : 0;
  d.cs = g.nx / 2;
  d.ct = g.ny / 2;
  d.cz = g.nz / 2;
  d.flags = g.flags;
  d.x0 = (float)g.x0;
  d.y0 = (float)g.y0;
  d.z0 = (float)g.z0;
  d.dvox = (float)g.dvox;
  d.sdd = (float)g.sdd;
  d.D = (float)g.wdist;
  d.sod = (float)g.sod;
  d.half_u = (float)g.half_u;
  d.half_v = (float)g.half_v;
  d.inv_du = (float)(1.0 / g.du);
  d.inv_dv = (float)(1.0 / g.dv);
  d.inv_du_lo = (float)(1.0 / g.du - (double)d.inv_du);
  d.inv_dv_lo = (float)(1.0 / g.dv - (double)d.inv_dv);
  d.dvox_inv_dv = (float)(g.dvox / g.dv);
  d.dvox_inv_dv_lo = (float)(g.dvox / g.dv - (double)d.dvox_inv_dv);
  // recon/bp3d20.cpp:116 rejects |u'|>half_u, |v'|>half_v; :152 then needs
  // 0 <= x <= nv and 0 <= y <= nu.
  d.xmax = (float)std::fmin((double)g.nv, 2.0 * g.half_v / g.dv);
  d.ymax = (float)std::fmin((double)g.nu, 2.0 * g.half_u / g.du);
  auto split = [](double v, float* h, float* l) {
    *h = (float)v;
    *l = (float)(v - (double)*h);
  };
  split(g.half_u / g.du, &d.yc_h, &d.yc_l);
  split(g.half_v / g.dv, &d.xc_h, &d.xc_l);
  split(g.sdd / g.dv, &d.kv_h, &d.kv_l);
  split(g.sdd * g.dvox / g.dv, &d.kb_h, &d.kb_l);
  split(g.z0, &d.z0_h, &d.z0_l);
  split(g.dvox, &d.dz_h, &d.dz_l);
  return d;
}

int fdk_validate(monte_ctx* ctx, const monte_fdk_geom* g, bool need_grid) {
  if (!g) return set_error(ctx, MONTE_EINVAL, "geometry is NULL");
  if (g->n_views <= 0 || g->nu <= 0 || g->nv <= 0)
    return set_error(ctx, MONTE_EINVAL, "bad detector size views=%d nu=%d nv=%d", g->n_views,
                     g->nu, g->nv);
  if (!(g->du > 0) || !(g->dv > 0) || !(g->sdd > 0) || !(g->sod > 0) || !(g->half_u > 0) ||
      !(g->half_v > 0))
    return set_error(ctx, MONTE_EINVAL, "non-positive detector pitch/extent or distance");
  if (g->flags & ~(MONTE_FDK_TAN_DEGREES | MONTE_FDK_FLAT_EDGE))
    return set_error(ctx, MONTE_EINVAL, "unknown FDK flags 0x%x", g->flags);
  size_t n;
  if (!mul_ok((size_t)g->n_views, (size_t)g->nu, &n) || !mul_ok(n, (size_t)g->nv, &n) ||
      n > ((size_t)1 << 40))
    return set_error(ctx, MONTE_EOVERFLOW, "projection stack too large");
  if ((size_t)g->nu * g->nv > (size_t)INT32_MAX)
    return set_error(ctx, MONTE_EOVERFLOW, "detector too large");
  if (need_grid) {
    if (g->nx <= 0 || g->ny <= 0 || g->nz <= 0)
      return set_error(ctx, MONTE_EINVAL, "bad grid %d x %d x %d", g->nx, g->ny, g->nz);
    if (g->s_begin < 0 || g->s_end > g->nx || g->s_begin > g->s_end)
      return set_error(ctx, MONTE_EINVAL, "bad slab [%d,%d) for nx=%d", g->s_begin, g->s_end,
                       g->nx);
    if (!(g->dvox > 0)) return set_error(ctx, MONTE_EINVAL, "non-positive voxel pitch");
    if (!mul_ok((size_t)g->nx, (size_t)g->ny, &n) || !mul_ok(n, (size_t)g->nz, &n) ||
        n > ((size_t)1 << 40))
      return set_error(ctx, MONTE_EOVERFLOW, "volume too large");
  }
  return MONTE_OK;
}

namespace {
// a + i b + j c for integer 0 <= i < ni, 0 <= j < nj, split as exact parts
// (multiples of one power of two q, large enough that every partial sum
// a_h + j c_h + i b_h is a float: |sum| < 2^24 q) plus float remainders.
void split_affine(double a, double b, double c, int ni, int nj, float* ah, float* bh, float* ch,
                  float* al, float* bl, float* cl) {
  const double m = std::fabs(a) + (ni - 1) * std::fabs(b) + (nj - 1) * std::fabs(c);
  // one bit of headroom for the rounding of the parts to multiples of q
  const double q = std::ldexp(1.0, (m > 0 ? (int)std::ceil(std::log2(m)) : 0) + 1 - 24);
  const double a_h = std::nearbyint(a / q) * q, b_h = std::nearbyint(b / q) * q,
               c_h = std::nearbyint(c / q) * q;
  *ah = (float)a_h;
  *bh = (float)b_h;
  *ch = (float)c_h;
  *al = (float)(a - a_h);
  *bl = (float)(b - b_h);
  *cl = (float)(c - c_h);
}
}  // namespace

void build_fdk_tables(const monte_fdk_geom* g, FdkHostTables* t) {
  const int nv_ = g->n_views, nu = g->nu, nv = g->nv;
  std::vector<BpView>& views = t->views;
  std::vector<BpViewD>& viewsd = t->viewsd;
  views.assign(nv_, BpView());
  viewsd.assign(nv_, BpViewD());
  float beta_span = (float)(360.0 / nv_);
  for (int k = 0; k < nv_; k++) {
    double beta = (double)k * 360.0 / nv_;
    double a = M_PI * beta / 180;
    double c = cos(a), s = sin(a);
    float start_x = (float)(-g->sod);
    double tanb = (g->flags & MONTE_FDK_TAN_DEGREES) ? tan(beta) : tan(a);
    BpView& v = views[k];
    v.c = (float)c;
    v.s = (float)s;
    v.px = (float)(start_x * c);
    v.py = (float)(start_x * s);
    v.tanb = (float)tanb;
    v.rs = (float)(1.0 / sqrt(1 + tanb * tanb));
    v.factor = (float)(beta_span * 2 * M_PI / 360 * g->scale * g->scale2);
    v.pad = 0.f;
    // Vx = X c + Y s - start_x and W = (sdd / du) (Y c - X s) at
    // X = x0 + i dvox, Y = y0 - j dvox: the reference's (X - px) c +
    // (Y - py) s and (Y - py) c - (X - px) s (recon/bp3d20.cpp:103-110)
    // with px = start_x c, py = start_x s
    const double K = g->sdd / g->du;
    split_affine(g->x0 * c + g->y0 * s - (double)start_x, g->dvox * c, -g->dvox * s, g->nx,
                 g->ny, &v.ah, &v.bh, &v.ch, &v.al, &v.bl, &v.cl);
    split_affine(K * (g->y0 * c - g->x0 * s), -K * g->dvox * s, -K * g->dvox * c, g->nx, g->ny,
                 &v.dh, &v.eh, &v.fh, &v.dl, &v.el, &v.fl);
    viewsd[k].c = c;
    viewsd[k].s = s;
    viewsd[k].px = start_x * c - 0.f * s;  // recon/bp3d20.cpp:87-88
    viewsd[k].py = start_x * s + 0.f * c;
    viewsd[k].tanb = tanb;
  }
  // cosine weights w[u][v] (recon/bp3d20.cpp:40)
  std::vector<float>& w = t->weights;
  w.assign((size_t)nu * nv, 0.f);
  for (int a = 0; a < nu; a++)
    for (int b = 0; b < nv; b++) {
      double D = g->wdist;
      double pu = -1 * (a * g->du) + g->half_u;
      double pv = (b * g->dv) - g->half_v;
      w[(size_t)a * nv + b] = (float)(D / sqrt(D * D + pu * pu + pv * pv));
    }
  // taps 0.5*h[n] at index nu-1+n (recon/bp3d20.cpp:48-60,68)
  std::vector<float>& taps = t->taps;
  taps.assign(2 * nu - 1, 0.f);
  taps[nu - 1] = 0.125f;
  for (int n = 1; n < nu; n++) {
    float h = 0.f;
    if (n % 2 == 1) {
      double x = n * M_PI;
      h = (float)(-1. / (x * x));
    }
    taps[nu - 1 + n] = taps[nu - 1 - n] = 0.5f * h;
  }
  t->bsplit.clear();
  if (bf16x3_supported(make_fdk_dev(*g))) {
    t->bsplit.resize(bf16x3_bsplit_bytes(nu) / 2);
    bf16x3_build_bsplit(nu, taps.data(), t->bsplit.data());
  }
}

int fdk_tune_bp(monte_ctx* ctx, const monte_fdk_geom* g, const BpView* views,
                const BpViewD* viewsd, const float* df, float* dv, int* best,
                const int* candidates, int n_candidates, int reps, const float* padded,
                BpFootprints* footprints) {
  FdkDev d = make_fdk_dev(*g);
  if (reps < 2) reps = 2;
  cudaEvent_t e0, e1;
  MONTE_CUDA(ctx, cudaEventCreate(&e0));
  MONTE_CUDA(ctx, cudaEventCreate(&e1));
  int pick = -1;
  float best_ms = 3.0e38f;
  const int n = candidates ? n_candidates : fdk_bp_tiled_variants();
  for (int i = 0; i < n; i++) {
    const int v = candidates ? candidates[i] : i;
    if (!fdk_bp_tiled_supported(d, v, padded != nullptr)) continue;
    float ms_min = 3.0e38f;
    for (int rep = 0; rep < reps; rep++) {
      cudaEventRecord(e0, ctx->stream);
      cudaError_t e = launch_fdk_bp_tiled(d, views, viewsd, df, dv, nullptr, v, ctx->d_status,
                                          ctx->stream, nullptr, padded, footprints);
      cudaEventRecord(e1, ctx->stream);
      if (e != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return cuda_fail(ctx, e != cudaSuccess ? e : cudaGetLastError(), "autotune launch");
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < ms_min) ms_min = ms;  // first run warms up
    }
    // a later shape must win by more than 1 %: timing noise does not flip
    // the choice between near-equal shapes, and the candidate lists put
    // the shapes with the least DRAM traffic first
    if (ms_min < best_ms * 0.99f) {
      best_ms = ms_min;
      pick = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *best = pick;
  return MONTE_OK;
}

namespace {

// Upload per-view constants, weight table and taps for geometry g (cached).
int prepare_tables(monte_ctx* ctx, const monte_fdk_geom* g) {
  std::vector<uint8_t> key(sizeof(monte_fdk_geom));
  memcpy(key.data(), g, sizeof(monte_fdk_geom));
  if (key == ctx->fdk_key && ctx->fdk_views.ptr) return MONTE_OK;
  FdkHostTables t;
  build_fdk_tables(g, &t);
  const std::vector<BpView>& views = t.views;
  const std::vector<BpViewD>& viewsd = t.viewsd;
  const std::vector<float>& w = t.weights;
  const std::vector<float>& taps = t.taps;
  MONTE_TRY(ensure(ctx, ctx->fdk_views, views.size() * sizeof(BpView), "view table"));
  MONTE_TRY(ensure(ctx, ctx->fdk_viewsd, viewsd.size() * sizeof(BpViewD), "view table"));
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->fdk_viewsd.ptr, viewsd.data(),
                                  viewsd.size() * sizeof(BpViewD), cudaMemcpyHostToDevice,
                                  ctx->stream));
  MONTE_TRY(ensure(ctx, ctx->fdk_weights, w.size() * sizeof(float), "weight table"));
  MONTE_TRY(ensure(ctx, ctx->fdk_taps, taps.size() * sizeof(float), "tap table"));
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->fdk_views.ptr, views.data(), views.size() * sizeof(BpView),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->fdk_weights.ptr, w.data(), w.size() * sizeof(float),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->fdk_taps.ptr, taps.data(), taps.size() * sizeof(float),
                                  cudaMemcpyHostToDevice, ctx->stream));
  if (!t.bsplit.empty()) {
    MONTE_TRY(ensure(ctx, ctx->fdk_bsplit, t.bsplit.size() * 2, "split Toeplitz operand"));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->fdk_bsplit.ptr, t.bsplit.data(), t.bsplit.size() * 2,
                                    cudaMemcpyHostToDevice, ctx->stream));
  }
  // the host vectors die at return: make the copies complete first
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->fdk_key = key;
  return MONTE_OK;
}

int run_filter(monte_ctx* ctx, const monte_fdk_geom* g, const float* d_proj, float* d_filtered,
               int filter_mode, cudaStream_t st = nullptr) {
  if (!st) st = ctx->stream;
  FdkDev d = make_fdk_dev(*g);
  cudaError_t e;
  if (filter_mode == MONTE_FILTER_FP32) {
    e = launch_fdk_filter_fp32(d, d_proj, (const float*)ctx->fdk_weights.ptr,
                               (const float*)ctx->fdk_taps.ptr, d_filtered, st);
  } else if (filter_mode == MONTE_FILTER_BF16X3) {
    if (!bf16x3_supported(d))
      return set_error(ctx, MONTE_EUNSUPPORTED,
                       "BF16x3 filter needs nu %% 64 == 0 and nv %% 128 == 0 (got %d, %d)", g->nu,
                       g->nv);
    e = launch_fdk_filter_bf16x3(d, d_proj, (const float*)ctx->fdk_weights.ptr,
                                 (const uint16_t*)ctx->fdk_bsplit.ptr, d_filtered, ctx->d_status,
                                 ctx->sm_count, st);
  } else {
    return set_error(ctx, MONTE_EINVAL, "unknown filter mode %d", filter_mode);
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "filter launch");
  return MONTE_OK;
}

int run_bp(monte_ctx* ctx, const monte_fdk_geom* g, const float* d_filtered, float* d_xy,
           float* d_zy, int bp_mode) {
  FdkDev d = make_fdk_dev(*g);
  const size_t vol = (size_t)g->nx * g->ny * g->nz * sizeof(float);
  if (g->s_begin != 0 || g->s_end != g->nx) {
    MONTE_CUDA(ctx, cudaMemsetAsync(d_xy, 0, vol, ctx->stream));
    if (d_zy) MONTE_CUDA(ctx, cudaMemsetAsync(d_zy, 0, vol, ctx->stream));
  }
  cudaError_t e;
  const BpView* views = (const BpView*)ctx->fdk_views.ptr;
  const BpViewD* viewsd = (const BpViewD*)ctx->fdk_viewsd.ptr;
  if (bp_mode == MONTE_BP_PLAIN) {
    e = launch_fdk_bp_plain(d, views, viewsd, d_filtered, d_xy, d_zy, ctx->stream);
    ctx->last_bp_variant = -1;
  } else if (bp_mode == MONTE_BP_TILED) {
    // rows that are not a multiple of 16 bytes: the tiles come from a
    // padded copy (TMA row strides are multiples of 16 bytes)
    const float* padded = nullptr;
    if (d.nu % 4 != 0) {
      const size_t pbytes = (size_t)g->n_views * g->nv * fdk_bp_pad_pitch(g->nu) * sizeof(float);
      MONTE_TRY(ensure_slot(ctx, kScratchBpPad, pbytes, "padded filtered projections"));
      padded = (const float*)ctx->scratch[kScratchBpPad].ptr;
      cudaError_t ep = launch_fdk_bp_pad_rows(d, d_filtered, (float*)padded, ctx->stream);
      if (ep != cudaSuccess) return cuda_fail(ctx, ep, "row padding launch");
    }
    const bool pad = padded != nullptr;
    const int variant = fdk_bp_pick(d, ctx->bp_tune_choice, pad);
    if (variant < 0) {
      // the footprint of a voxel block does not fit a shared-memory box:
      // the one-voxel-per-thread kernel handles any geometry
      e = launch_fdk_bp_plain(d, views, viewsd, d_filtered, d_xy, d_zy, ctx->stream);
      ctx->last_bp_variant = -1;
    } else {
      e = launch_fdk_bp_tiled(d, views, viewsd, d_filtered, d_xy, d_zy, variant, ctx->d_status,
                              ctx->stream, nullptr, padded, &ctx->bp_footprints);
      ctx->last_bp_variant = variant;
    }
  } else {
    return set_error(ctx, MONTE_EINVAL, "unknown backprojection mode %d", bp_mode);
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "backprojection launch");
  return MONTE_OK;
}

size_t proj_bytes(const monte_fdk_geom* g) {
  return (size_t)g->n_views * g->nu * g->nv * sizeof(float);
}
size_t vol_bytes(const monte_fdk_geom* g) {
  return (size_t)g->nx * g->ny * g->nz * sizeof(float);
}

// ---- FDK from and to host memory, pipelined -------------------------------
//
// The views are cut into two ranges, the first 2/15 of the scan (360
// views: 0-48, 48-360): on the 325^3 workload a view uploads in 3.7 us (786
// KB at 210 GB/s) and backprojects in 23 us, so the second range's upload
// (1.2 ms at 210 GB/s, 1.4 ms at 170) hides, or nearly, under the first
// range's backprojection (1.2 ms), and the first range's upload and filter
// (0.25 ms) stay exposed.  Measured end to end at 202 GB/s: 9.22 ms, against
// 9.33 ms with a first range of 1/6 and 9.40 ms with three ranges growing
// fivefold from 1/31 (0-12, 12-72, 72-360): every extra backprojection
// launch costs more than a smaller first upload saves.  Range i is
// uploaded on copy_in, filtered as soon as it has landed on filter_stream
// (the greatest priority, so that its blocks take the SMs the previous
// range's backprojection frees, alongside that launch's last waves), and
// backprojected on the context's stream into the running per-voxel sums
// (BpPart; one view behind, as the flat-edge reads of a view's last row
// reach into the next view); the upload of range i+1 runs under the
// backprojection of range i, so of the upload only the first, small range
// stays on the critical path.  The last range's backprojection stores its
// sums straight into the caller's pinned volume, which spreads the download
// over that launch instead of appending it.  Filtered projections, when
// asked for, go back range by range on copy_out.  The values are those of
// the unsplit path bit for bit: the filter is per view, and every voxel sums
// its views in index order.
constexpr int kPipeMaxRanges = 8;
enum { kEvStart = 0, kEvIn = 1, kEvFilt = 1 + kPipeMaxRanges, kEvOut = 1 + 2 * kPipeMaxRanges };
static_assert(kEvOut < 24, "pipeline events");

// Device address of pinned (page-locked, mapped) host memory, else null.
void* host_mapped(const void* h) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int pipe_init(monte_ctx* ctx) {
  if (ctx->pipe_ready) return MONTE_OK;
  if (!ctx->copy_in)
    MONTE_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
  if (!ctx->copy_out)
    MONTE_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
  if (!ctx->filter_stream) {
    // the greatest priority: a range's filter takes the SMs that the
    // previous range's backprojection frees, ahead of that launch's
    // remaining blocks
    int least = 0, greatest = 0;
    MONTE_CUDA(ctx, cudaDeviceGetStreamPriorityRange(&least, &greatest));
    MONTE_CUDA(ctx, cudaStreamCreateWithPriority(&ctx->filter_stream, cudaStreamNonBlocking,
                                                 greatest));
  }
  for (cudaEvent_t& ev : ctx->pipe_ev)
    if (!ev) MONTE_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  ctx->pipe_ready = true;
  return MONTE_OK;
}

// View ranges [r[i], r[i+1]) of the pipeline; returns their number.
int pipe_ranges(int n_views, int* r) {
  const int first = std::max(1, (2 * n_views + 14) / 15);
  int nr = 0;
  r[0] = 0;
  r[++nr] = std::min(n_views, first);
  if (first < n_views) r[++nr] = n_views;
  return nr;
}

// The stages a pipelined call runs.
enum { kPipeFilter = 1, kPipeBackproject = 2 };

// src: the host input, projections (kPipeFilter) or filtered projections
// (backprojection alone); filtered: host output of the filter or null;
// dvol_xy/dvol_zy: device addresses of the pinned host volumes.
int fdk_host_pipelined_body(monte_ctx* ctx, const monte_fdk_geom* g, int stages,
                            const float* src, float* filtered, float* dvol_xy, float* dvol_zy,
                            int filter_mode, int variant) {
  const bool do_filter = (stages & kPipeFilter) != 0, do_bp = (stages & kPipeBackproject) != 0;
  const size_t view_elems = (size_t)g->nu * g->nv;
  const size_t pb = proj_bytes(g), vb = vol_bytes(g);
  int r[kPipeMaxRanges + 1];
  const int nr = pipe_ranges(g->n_views, r);
  if (do_filter) MONTE_TRY(ensure_slot(ctx, kScratchProj, pb, "projection staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "filtered staging"));
  if (do_bp && nr > 1) MONTE_TRY(ensure_slot(ctx, kScratchVolXY, vb, "partial sums"));
  // rows that are not a multiple of 16 bytes: every backprojection range
  // first copies its views into the padded layout its tiles load from
  float* padded = nullptr;
  if (do_bp && g->nu % 4 != 0) {
    const size_t pbytes = (size_t)g->n_views * g->nv * fdk_bp_pad_pitch(g->nu) * sizeof(float);
    MONTE_TRY(ensure_slot(ctx, kScratchBpPad, pbytes, "padded filtered projections"));
    padded = (float*)ctx->scratch[kScratchBpPad].ptr;
  }
  float* dp = do_filter ? (float*)ctx->scratch[kScratchProj].ptr : nullptr;
  float* df = (float*)ctx->scratch[kScratchFiltered].ptr;
  float* dsum = (float*)ctx->scratch[kScratchVolXY].ptr;
  float* din = do_filter ? dp : df;  // where the uploads land
  cudaEvent_t* ev = ctx->pipe_ev;
  // the copies start after the work already queued on the stream (which
  // may still read the staging buffers)
  MONTE_CUDA(ctx, cudaEventRecord(ev[kEvStart], ctx->stream));
  MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_in, ev[kEvStart], 0));
  MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_out, ev[kEvStart], 0));
  MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->filter_stream, ev[kEvStart], 0));
  for (int i = 0; i < nr; i++) {
    const size_t off = (size_t)r[i] * view_elems;
    MONTE_CUDA(ctx, cudaMemcpyAsync(din + off, src + off,
                                    (size_t)(r[i + 1] - r[i]) * view_elems * sizeof(float),
                                    cudaMemcpyHostToDevice, ctx->copy_in));
    MONTE_CUDA(ctx, cudaEventRecord(ev[kEvIn + i], ctx->copy_in));
  }
  const FdkDev d = make_fdk_dev(*g);
  const BpView* views = (const BpView*)ctx->fdk_views.ptr;
  const BpViewD* viewsd = (const BpViewD*)ctx->fdk_viewsd.ptr;
  bool have_sum = false;  // dsum holds the sums of the views before this range
  for (int i = 0; i < nr; i++) {
    const size_t off = (size_t)r[i] * view_elems;
    const size_t bytes = (size_t)(r[i + 1] - r[i]) * view_elems * sizeof(float);
    if (do_filter) {
      // filtered on its own stream as soon as it has landed, alongside the
      // previous range's backprojection; the stream waits for it before
      // the next backprojection (and before returning)
      monte_fdk_geom gr = *g;  // the range's views as a scan of their own
      gr.n_views = r[i + 1] - r[i];
      MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->filter_stream, ev[kEvIn + i], 0));
      MONTE_TRY(run_filter(ctx, &gr, dp + off, df + off, filter_mode, ctx->filter_stream));
      MONTE_CUDA(ctx, cudaEventRecord(ev[kEvFilt + i], ctx->filter_stream));
      MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev[kEvFilt + i], 0));
      if (filtered) {
        MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_out, ev[kEvFilt + i], 0));
        MONTE_CUDA(ctx, cudaMemcpyAsync(filtered + off, df + off, bytes, cudaMemcpyDeviceToHost,
                                        ctx->copy_out));
      }
    } else {
      MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev[kEvIn + i], 0));
    }
    if (!do_bp) continue;
    // the backprojection ranges trail the filtered ones by a view: with
    // the flat-edge reads (MONTE_FDK_FLAT_EDGE) view k's last row and
    // column read on into view k + 1
    const bool last = i == nr - 1;
    const int kb = i == 0 ? 0 : r[i] - 1, ke = last ? g->n_views : r[i + 1] - 1;
    if (ke == kb && !last) continue;
    const BpPart part{kb, ke, have_sum ? dsum : nullptr};
    if (padded) {
      cudaError_t ep = launch_fdk_bp_pad_rows(d, df, padded, ctx->stream, kb, ke);
      if (ep != cudaSuccess) return cuda_fail(ctx, ep, "row padding launch");
    }
    cudaError_t e = launch_fdk_bp_tiled(d, views, viewsd, df, last ? dvol_xy : dsum,
                                        last ? dvol_zy : nullptr, variant, ctx->d_status,
                                        ctx->stream, &part, padded, &ctx->bp_footprints);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "backprojection launch");
    have_sum = true;
  }
  if (do_bp) ctx->last_bp_variant = variant;
  ctx->last_host_ranges = nr;
  MONTE_CUDA(ctx, cudaEventRecord(ev[kEvOut], ctx->copy_out));
  MONTE_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ev[kEvOut], 0));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

// Runs the pipelined path and returns 1 when the call qualifies for it, 0
// (nothing done) otherwise.  It qualifies with every host buffer pinned,
// and for the backprojection a tiled shape that fits and a full-width
// volume.  stages as above; src: projections when filtering, else the
// filtered projections.
int fdk_host_pipelined(monte_ctx* ctx, const monte_fdk_geom* g, int stages, const float* src,
                       float* filtered, float* vol_xy, float* vol_zy, int filter_mode,
                       int bp_mode, int* rc) {
  const bool do_filter = (stages & kPipeFilter) != 0, do_bp = (stages & kPipeBackproject) != 0;
  if (do_filter && filter_mode != MONTE_FILTER_FP32 && filter_mode != MONTE_FILTER_BF16X3)
    return 0;
  if (!host_mapped(src) || (filtered && !host_mapped(filtered))) return 0;
  int variant = -1;
  float *mxy = nullptr, *mzy = nullptr;
  if (do_bp) {
    if (bp_mode != MONTE_BP_TILED || g->s_begin != 0 || g->s_end != g->nx) return 0;
    const FdkDev d = make_fdk_dev(*g);
    const bool pad = g->nu % 4 != 0;  // tiles from a padded copy
    variant = fdk_bp_pick(d, ctx->bp_tune_choice, pad);
    if (variant < 0) return 0;
    mxy = (float*)host_mapped(vol_xy);
    mzy = vol_zy ? (float*)host_mapped(vol_zy) : nullptr;
    if (!mxy || (vol_zy && !mzy)) return 0;
  }
  *rc = pipe_init(ctx);
  if (*rc == MONTE_OK)
    *rc = fdk_host_pipelined_body(ctx, g, stages, src, filtered, mxy, mzy, filter_mode, variant);
  if (*rc != MONTE_OK) {
    // nothing may still read or write the caller's buffers after the return
    cudaStreamSynchronize(ctx->copy_in);
    cudaStreamSynchronize(ctx->copy_out);
    if (ctx->filter_stream) cudaStreamSynchronize(ctx->filter_stream);
    cudaStreamSynchronize(ctx->stream);
  }
  return 1;
}

}  // namespace
}  // namespace monte

using namespace monte;

extern "C" {

void monte_fdk_geom_reference65(monte_fdk_geom* g) {
  if (!g) return;
  memset(g, 0, sizeof(*g));
  g->n_views = 360;  // recon/bp3d20.cpp:19
  g->nu = g->nv = 65;  // :17
  g->flags = MONTE_FDK_TAN_DEGREES | MONTE_FDK_FLAT_EDGE;
  g->du = g->dv = 0.5;  // :40,123-124
  g->half_u = g->half_v = 16.25;
  g->sod = 160;  // :85
  g->sdd = 220;  // :107
  g->wdist = 60;  // :40,159
  g->nx = g->ny = g->nz = 256;  // :18
  g->s_begin = 125;  // :93
  g->s_end = 130;
  g->dvox = 0.1;  // :96-98
  g->x0 = -12.8;
  g->y0 = 12.8;
  g->z0 = 12.8;
  g->mask_radius = 118;  // :145
  g->scale = 2.7;  // :160
  g->scale2 = 1.0;
}

void monte_fdk_geom_reference325(monte_fdk_geom* g) {
  if (!g) return;
  monte_fdk_geom_reference65(g);
  g->nu = g->nv = 325;  // recon/bp3d20_325.cpp:17
  g->du = g->dv = 0.1;  // :43,134-135
  g->mask_radius = 0;   // the sphere test of bp3d20.cpp:145 is dropped
  g->scale = 2.7;       // :170
  g->scale2 = 5.0;
}

int monte_fdk_filter(monte_ctx* ctx, const monte_fdk_geom* g, const float* proj, float* filtered,
                     int filter_mode, int mem) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(fdk_validate(ctx, g, false));
  if (!proj || !filtered) return set_error(ctx, MONTE_EINVAL, "null projection/filtered pointer");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST)
    return set_error(ctx, MONTE_EINVAL, "bad mem %d", mem);
  MONTE_TRY(enter(ctx));
  MONTE_TRY(prepare_tables(ctx, g));
  if (mem == MONTE_MEM_DEVICE) return run_filter(ctx, g, proj, filtered, filter_mode);
  int rc = MONTE_OK;
  ctx->last_host_ranges = 0;
  if (fdk_host_pipelined(ctx, g, kPipeFilter, proj, filtered, nullptr, nullptr, filter_mode,
                         MONTE_BP_TILED, &rc))
    return rc;
  const size_t pb = proj_bytes(g);
  MONTE_TRY(ensure_slot(ctx, kScratchProj, pb, "projection staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "filtered staging"));
  float* dp = (float*)ctx->scratch[kScratchProj].ptr;
  float* df = (float*)ctx->scratch[kScratchFiltered].ptr;
  MONTE_CUDA(ctx, cudaMemcpyAsync(dp, proj, pb, cudaMemcpyHostToDevice, ctx->stream));
  MONTE_TRY(run_filter(ctx, g, dp, df, filter_mode));
  MONTE_CUDA(ctx, cudaMemcpyAsync(filtered, df, pb, cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

int monte_fdk_backproject(monte_ctx* ctx, const monte_fdk_geom* g, const float* filtered,
                          float* vol_xy, float* vol_zy, int bp_mode, int mem) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(fdk_validate(ctx, g, true));
  if (!filtered || !vol_xy) return set_error(ctx, MONTE_EINVAL, "null filtered/volume pointer");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST)
    return set_error(ctx, MONTE_EINVAL, "bad mem %d", mem);
  MONTE_TRY(enter(ctx));
  MONTE_TRY(prepare_tables(ctx, g));
  if (mem == MONTE_MEM_DEVICE) return run_bp(ctx, g, filtered, vol_xy, vol_zy, bp_mode);
  int rc = MONTE_OK;
  ctx->last_host_ranges = 0;
  if (fdk_host_pipelined(ctx, g, kPipeBackproject, filtered, nullptr, vol_xy, vol_zy,
                         MONTE_FILTER_FP32, bp_mode, &rc))
    return rc;
  const size_t pb = proj_bytes(g), vb = vol_bytes(g);
  MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "filtered staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchVolXY, vb, "volume staging"));
  if (vol_zy) MONTE_TRY(ensure_slot(ctx, kScratchVolZY, vb, "volume staging"));
  float* df = (float*)ctx->scratch[kScratchFiltered].ptr;
  float* dxy = (float*)ctx->scratch[kScratchVolXY].ptr;
  float* dzy = vol_zy ? (float*)ctx->scratch[kScratchVolZY].ptr : nullptr;
  MONTE_CUDA(ctx, cudaMemcpyAsync(df, filtered, pb, cudaMemcpyHostToDevice, ctx->stream));
  MONTE_TRY(run_bp(ctx, g, df, dxy, dzy, bp_mode));
  MONTE_CUDA(ctx, cudaMemcpyAsync(vol_xy, dxy, vb, cudaMemcpyDeviceToHost, ctx->stream));
  if (vol_zy) MONTE_CUDA(ctx, cudaMemcpyAsync(vol_zy, dzy, vb, cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

int monte_fdk(monte_ctx* ctx, const monte_fdk_geom* g, const float* proj, float* filtered,
              float* vol_xy, float* vol_zy, int filter_mode, int bp_mode, int mem) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(fdk_validate(ctx, g, true));
  if (!proj || !vol_xy) return set_error(ctx, MONTE_EINVAL, "null projection/volume pointer");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST)
    return set_error(ctx, MONTE_EINVAL, "bad mem %d", mem);
  MONTE_TRY(enter(ctx));
  MONTE_TRY(prepare_tables(ctx, g));
  const size_t pb = proj_bytes(g), vb = vol_bytes(g);
  if (mem == MONTE_MEM_DEVICE) {
    float* df = filtered;
    if (!df) {
      MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "filtered scratch"));
      df = (float*)ctx->scratch[kScratchFiltered].ptr;
    }
    MONTE_TRY(run_filter(ctx, g, proj, df, filter_mode));
    return run_bp(ctx, g, df, vol_xy, vol_zy, bp_mode);
  }
  int rc = MONTE_OK;
  ctx->last_host_ranges = 0;
  if (fdk_host_pipelined(ctx, g, kPipeFilter | kPipeBackproject, proj, filtered, vol_xy, vol_zy,
                         filter_mode, bp_mode, &rc))
    return rc;
  // pageable buffers, the plain backprojector or a column window: one
  // upload, the two stages, one download
  MONTE_TRY(ensure_slot(ctx, kScratchProj, pb, "projection staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "filtered staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchVolXY, vb, "volume staging"));
  if (vol_zy) MONTE_TRY(ensure_slot(ctx, kScratchVolZY, vb, "volume staging"));
  float* dp = (float*)ctx->scratch[kScratchProj].ptr;
  float* df = (float*)ctx->scratch[kScratchFiltered].ptr;
  float* dxy = (float*)ctx->scratch[kScratchVolXY].ptr;
  float* dzy = vol_zy ? (float*)ctx->scratch[kScratchVolZY].ptr : nullptr;
  MONTE_CUDA(ctx, cudaMemcpyAsync(dp, proj, pb, cudaMemcpyHostToDevice, ctx->stream));
  MONTE_TRY(run_filter(ctx, g, dp, df, filter_mode));
  MONTE_TRY(run_bp(ctx, g, df, dxy, dzy, bp_mode));
  if (filtered)
    MONTE_CUDA(ctx, cudaMemcpyAsync(filtered, df, pb, cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(vol_xy, dxy, vb, cudaMemcpyDeviceToHost, ctx->stream));
  if (vol_zy) MONTE_CUDA(ctx, cudaMemcpyAsync(vol_zy, dzy, vb, cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

int monte_fdk_autotune(monte_ctx* ctx, const monte_fdk_geom* g, int* best) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(fdk_validate(ctx, g, true));
  MONTE_TRY(enter(ctx));
  MONTE_TRY(prepare_tables(ctx, g));
  const size_t pb = proj_bytes(g), vb = vol_bytes(g);
  MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "autotune filtered"));
  MONTE_TRY(ensure_slot(ctx, kScratchVolXY, vb, "autotune volume"));
  MONTE_CUDA(ctx, cudaMemsetAsync(ctx->scratch[kScratchFiltered].ptr, 0, pb, ctx->stream));
  const float* df = (const float*)ctx->scratch[kScratchFiltered].ptr;
  float* dv = (float*)ctx->scratch[kScratchVolXY].ptr;
  const float* padded = nullptr;
  if (g->nu % 4 != 0) {  // as run_bp: tiles from a copy with padded rows (zeros here)
    const size_t pbytes = (size_t)g->n_views * g->nv * fdk_bp_pad_pitch(g->nu) * sizeof(float);
    MONTE_TRY(ensure_slot(ctx, kScratchBpPad, pbytes, "autotune padded projections"));
    MONTE_CUDA(ctx, cudaMemsetAsync(ctx->scratch[kScratchBpPad].ptr, 0, pbytes, ctx->stream));
    padded = (const float*)ctx->scratch[kScratchBpPad].ptr;
  }
  const BpView* views = (const BpView*)ctx->fdk_views.ptr;
  const BpViewD* viewsd = (const BpViewD*)ctx->fdk_viewsd.ptr;
  // every shape, the quick list's first (the leaders, in order of
  // preference: a later shape has to be 1 % faster to displace one)
  std::vector<int> order(kBpQuickCandidates, kBpQuickCandidates + kBpQuickCandidatesN);
  for (int v = 0; v < fdk_bp_tiled_variants(); v++)
    if (std::find(order.begin(), order.end(), v) == order.end()) order.push_back(v);
  int pick = -1;
  MONTE_TRY(fdk_tune_bp(ctx, g, views, viewsd, df, dv, &pick, order.data(), (int)order.size(), 3,
                        padded, &ctx->bp_footprints));
  ctx->bp_tune_choice = pick;
  if (best) *best = pick;
  return monte_ctx_check_status(ctx);
}

int monte_fdk_last_bp_variant(const monte_ctx* ctx) { return ctx ? ctx->last_bp_variant : -1; }

int monte_fdk_exact_counts(monte_ctx* ctx, uint64_t* counts, int reset) {
  if (!ctx) return MONTE_EINVAL;
  if (!counts) return set_error(ctx, MONTE_EINVAL, "null counts");
  MONTE_TRY(enter(ctx));
  unsigned long long* dc = reinterpret_cast<unsigned long long*>(ctx->d_status + kBpExactSlot);
  unsigned long long h[2];
  MONTE_CUDA(ctx, cudaMemcpyAsync(h, dc, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  if (reset) MONTE_CUDA(ctx, cudaMemsetAsync(dc, 0, sizeof(h), ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  counts[0] = h[0];
  counts[1] = h[1];
  return MONTE_OK;
}

int monte_fdk_last_host_ranges(const monte_ctx* ctx) { return ctx ? ctx->last_host_ranges : 0; }

int monte_fdk_forward_project(monte_ctx* ctx, const monte_fdk_geom* g, const float* vol_xy,
                              float* filtered_out, int mem) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(fdk_validate(ctx, g, true));
  if (!vol_xy || !filtered_out) return set_error(ctx, MONTE_EINVAL, "null volume/output pointer");
  if (g->flags & MONTE_FDK_FLAT_EDGE)
    return set_error(ctx, MONTE_EUNSUPPORTED,
                     "the adjoint is defined for the operator without MONTE_FDK_FLAT_EDGE");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST)
    return set_error(ctx, MONTE_EINVAL, "bad mem %d", mem);
  MONTE_TRY(enter(ctx));
  MONTE_TRY(prepare_tables(ctx, g));
  FdkDev d = make_fdk_dev(*g);
  const size_t pb = proj_bytes(g), vb = vol_bytes(g);
  const float* dv = vol_xy;
  float* dout = filtered_out;
  if (mem == MONTE_MEM_HOST) {
    MONTE_TRY(ensure_slot(ctx, kScratchVolXY, vb, "volume staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "projection staging"));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchVolXY].ptr, vol_xy, vb,
                                    cudaMemcpyHostToDevice, ctx->stream));
    dv = (const float*)ctx->scratch[kScratchVolXY].ptr;
    dout = (float*)ctx->scratch[kScratchFiltered].ptr;
  }
  // z-major copy of the volume: the projector reads a voxel column along z
  MONTE_TRY(ensure_slot(ctx, kScratchVolZY, fdk_fp_scratch_bytes(*g), "z-major volume copy"));
  cudaError_t e = launch_fdk_forward_project(d, (const BpView*)ctx->fdk_views.ptr,
                                             (const BpViewD*)ctx->fdk_viewsd.ptr, dv,
                                             (float*)ctx->scratch[kScratchVolZY].ptr, dout,
                                             ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "forward projection launch");
  if (mem == MONTE_MEM_HOST) {
    MONTE_CUDA(ctx, cudaMemcpyAsync(filtered_out, dout, pb, cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return MONTE_OK;
}

int monte_fdk_backward(monte_ctx* ctx, const monte_fdk_geom* g, const float* grad_vol,
                       float* grad_proj, int mem) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(fdk_validate(ctx, g, true));
  if (!grad_vol || !grad_proj) return set_error(ctx, MONTE_EINVAL, "null gradient pointer");
  if (g->flags & MONTE_FDK_FLAT_EDGE)
    return set_error(ctx, MONTE_EUNSUPPORTED,
                     "the adjoint is defined for the operator without MONTE_FDK_FLAT_EDGE");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST)
    return set_error(ctx, MONTE_EINVAL, "bad mem %d", mem);
  MONTE_TRY(enter(ctx));
  MONTE_TRY(prepare_tables(ctx, g));
  FdkDev d = make_fdk_dev(*g);
  const size_t pb = proj_bytes(g), vb = vol_bytes(g);
  MONTE_TRY(ensure_slot(ctx, kScratchAux0, pb, "adjoint scratch"));
  float* tmp = (float*)ctx->scratch[kScratchAux0].ptr;
  const float* dv = grad_vol;
  float* dout = grad_proj;
  if (mem == MONTE_MEM_HOST) {
    MONTE_TRY(ensure_slot(ctx, kScratchVolXY, vb, "volume staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchProj, pb, "projection staging"));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchVolXY].ptr, grad_vol, vb,
                                    cudaMemcpyHostToDevice, ctx->stream));
    dv = (const float*)ctx->scratch[kScratchVolXY].ptr;
    dout = (float*)ctx->scratch[kScratchProj].ptr;
  }
  MONTE_TRY(ensure_slot(ctx, kScratchVolZY, fdk_fp_scratch_bytes(*g), "z-major volume copy"));
  cudaError_t e = launch_fdk_forward_project(d, (const BpView*)ctx->fdk_views.ptr,
                                             (const BpViewD*)ctx->fdk_viewsd.ptr, dv,
                                             (float*)ctx->scratch[kScratchVolZY].ptr, tmp,
                                             ctx->stream);
  if (e == cudaSuccess)
    e = launch_fdk_filter_adjoint(d, tmp, (const float*)ctx->fdk_weights.ptr,
                                  (const float*)ctx->fdk_taps.ptr, dout, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "FDK backward launch");
  if (mem == MONTE_MEM_HOST) {
    MONTE_CUDA(ctx, cudaMemcpyAsync(grad_proj, dout, pb, cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return MONTE_OK;
}

int monte_fdk_set_bp_variant(monte_ctx* ctx, int variant) {
  if (!ctx) return MONTE_EINVAL;
  if (variant < -1 || variant >= fdk_bp_tiled_variants())
    return set_error(ctx, MONTE_EINVAL, "tile shape %d out of range [-1,%d)", variant,
                     fdk_bp_tiled_variants());
  ctx->bp_tune_choice = variant;
  return MONTE_OK;
}

}  // extern "C"
