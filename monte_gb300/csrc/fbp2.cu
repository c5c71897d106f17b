// fbp2.cu -- the reference's 2-D fan-beam FBP (recon/fbp2.cpp) on the GPU,
// behind monte_fbp2 (include/monte.h).
//
// The problem is small (65 detector elements x 360 views -> a 256^2 image,
// 2.4e7 pixel-view updates), so the kernels keep the reference's double
// arithmetic, operation by operation, and its float accumulation order:
//   * per-view constants (cos, sin of the angle and of its negative, tan as
//     the reference evaluates it, sqrt(1 + tan^2), the rotated source) and
//     the per-element weights are computed on the host with the C library
//     the reference program uses;
//   * fbp2_filter_kernel: one thread per (view, element): the weighted
//     projection in float, then the Ram-Lak convolution summed in double in
//     the reference's order (recon/fbp2.cpp:36-73);
//   * fbp2_bp_kernel: one thread per pixel, views in ascending order, double
//     geometry, nearest detector element, float image accumulated in a
//     register as the reference accumulates image_xy (:86-150).
// The library is compiled with -fmad=false, so no multiply-add is fused
// that the reference keeps separate.
#include <cmath>
#include <cstring>
#include <vector>

#include "monte_internal.h"

namespace monte {
namespace {

struct Fbp2View {
  double c, s;      // cos, sin of the view angle
  double cn, sn;    // cos, sin of minus the angle (the reference's rotation)
  double px, py;    // rotated source
  double tb, rden;  // tan as evaluated, sqrt(1 + tan^2)
};

struct Fbp2Dev {
  int n_views, n_det, view_begin, view_end, nx, ny;
  double pitch_inv, half, sdd, d2, wdist, pix, x0, y0, scale, dfac;
};

__global__ void fbp2_filter_kernel(Fbp2Dev g, const float* __restrict__ proj,
                                   const double* __restrict__ wt,
                                   const double* __restrict__ ramp, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n_views * g.n_det) return;
  const int d = i / g.n_det, b = i % g.n_det, H = g.n_det;
  double tmp = 0.;
  for (int c = 0; c < H; c++) {
    const float pw = (float)((double)proj[d * H + c] * wt[c]);  // :38
    tmp = __dadd_rn(tmp, __dmul_rn(__dmul_rn((double)pw, 0.5), ramp[H - 1 - b + c]));  // :66
  }
  out[i] = (float)tmp;
}

__global__ void fbp2_bp_kernel(Fbp2Dev g, const Fbp2View* __restrict__ views,
                               const float* __restrict__ filt, float* __restrict__ image) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nx * g.ny) return;
  const int t = i / g.nx, s = i % g.nx;
  const size_t n_total = (size_t)g.n_views * g.n_det;
  const double X = __dadd_rn(g.x0, __dmul_rn((double)s, g.pix));
  const double Y = __dsub_rn(g.y0, __dmul_rn((double)t, g.pix));
  float acc = 0.f;
  for (int beta = g.view_begin; beta < g.view_end; beta++) {
    const Fbp2View v = views[beta];
    double v0 = __dsub_rn(X, v.px), v1 = __dsub_rn(Y, v.py);
    const double tx = v0;
    v0 = __dsub_rn(__dmul_rn(v0, v.cn), __dmul_rn(v1, v.sn));
    v1 = __dadd_rn(__dmul_rn(tx, v.sn), __dmul_rn(v1, v.cn));
    const double k = __ddiv_rn(g.sdd, v0);
    v1 = __dmul_rn(v1, k);
    if (fabs(v1) > g.half) continue;  // :120
    const int iy = (int)__dmul_rn(-g.pitch_inv, __dsub_rn(v1, g.half));  // :126
    const double ts = __dsub_rn(__dmul_rn(X, v.c), __dmul_rn(Y, v.s));
    const double tt = __dadd_rn(__dmul_rn(X, v.s), __dmul_rn(Y, v.c));
    double dd = __ddiv_rn(fabs(__dadd_rn(__dmul_rn(__dmul_rn(-1.0, v.tb), tt), ts)), v.rden);
    if (ts < 0) dd = -dd;
    const size_t idx = (size_t)beta * g.n_det + iy;
    const double q = idx < n_total ? (double)filt[idx] : 0.0;
    const double e = __dsub_rn(g.wdist, dd);
    const double w = __ddiv_rn(g.d2, __dmul_rn(e, e));
    const double out = __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(w, q), g.dfac), 2.0 * M_PI),
                                 360.0);
    acc = (float)__dadd_rn((double)acc, __dmul_rn(out, g.scale));  // :148
  }
  image[i] = acc;
}

int validate(monte_ctx* ctx, const monte_fbp2_geom* g) {
  if (!g) return set_error(ctx, MONTE_EINVAL, "geometry is NULL");
  if (g->n_views <= 0 || g->n_det <= 0 || g->nx <= 0 || g->ny <= 0)
    return set_error(ctx, MONTE_EINVAL, "bad 2-D FBP sizes");
  if (g->view_begin < 0 || g->view_end > g->n_views || g->view_begin > g->view_end)
    return set_error(ctx, MONTE_EINVAL, "bad view range [%d,%d)", g->view_begin, g->view_end);
  if (!(g->pitch > 0) || !(g->half > 0) || !(g->sdd > 0) || !(g->sod > 0) || !(g->pix > 0))
    return set_error(ctx, MONTE_EINVAL, "non-positive pitch, extent or distance");
  if (g->flags & ~MONTE_FDK_TAN_DEGREES) return set_error(ctx, MONTE_EINVAL, "unknown flags");
  if ((size_t)g->n_views * g->n_det > ((size_t)1 << 31) || (size_t)g->nx * g->ny > ((size_t)1 << 31))
    return set_error(ctx, MONTE_EOVERFLOW, "2-D FBP sizes too large");
  return MONTE_OK;
}

int run(monte_ctx* ctx, const monte_fbp2_geom* g, const float* dproj, float* dfilt,
        float* dimg) {
  const int H = g->n_det, nv = g->n_views;
  // host tables, in the reference's arithmetic (recon/fbp2.cpp:36-60,89-95,135)
  std::vector<double> wt(H), ramp(2 * H - 1, 0.0);
  for (int z = 0; z < H; z++)
    wt[z] = g->wdist / (std::sqrt(std::pow(g->wdist, 2) + std::pow(-g->half + g->pitch * z, 2)));
  ramp[H - 1] = 0.25;
  for (int n = 1; n < H; n++)
    if (n % 2 == 1) ramp[H - 1 + n] = ramp[H - 1 - n] = -1. / std::pow(n * M_PI, 2);
  const float span = 360.0f / (float)nv;
  std::vector<Fbp2View> views(nv);
  for (int beta = 0; beta < nv; beta++) {
    Fbp2View& v = views[beta];
    const double ang = M_PI * (beta * span) / 180;
    const float start_x = (float)(-g->sod);
    v.c = std::cos(ang);
    v.s = std::sin(ang);
    v.cn = std::cos(-1 * ang);
    v.sn = std::sin(-1 * ang);
    v.px = start_x * v.c - 0.f * v.s;
    v.py = start_x * v.s + 0.f * v.c;
    v.tb = (g->flags & MONTE_FDK_TAN_DEGREES) ? std::tan((double)(beta * span)) : std::tan(ang);
    v.rden = std::sqrt(1 + std::pow(v.tb, 2));
  }
  Fbp2Dev d;
  d.n_views = nv;
  d.n_det = H;
  d.view_begin = g->view_begin;
  d.view_end = g->view_end;
  d.nx = g->nx;
  d.ny = g->ny;
  d.pitch_inv = 1.0 / g->pitch;
  d.half = g->half;
  d.sdd = g->sdd;
  d.d2 = std::pow(g->wdist, 2);
  d.wdist = g->wdist;
  d.pix = g->pix;
  d.x0 = g->x0;
  d.y0 = g->y0;
  d.scale = g->scale;
  d.dfac = (double)span;
  const size_t tab = H * sizeof(double) + (2 * H - 1) * sizeof(double) + nv * sizeof(Fbp2View);
  MONTE_TRY(ensure_slot(ctx, kScratchFbp2, tab, "2-D FBP tables"));
  unsigned char* base = (unsigned char*)ctx->scratch[kScratchFbp2].ptr;
  double* d_wt = (double*)base;
  double* d_ramp = d_wt + H;
  Fbp2View* d_views = (Fbp2View*)(d_ramp + 2 * H - 1);
  MONTE_CUDA(ctx, cudaMemcpyAsync(d_wt, wt.data(), H * sizeof(double), cudaMemcpyHostToDevice,
                                  ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(d_ramp, ramp.data(), (2 * H - 1) * sizeof(double),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(d_views, views.data(), nv * sizeof(Fbp2View),
                                  cudaMemcpyHostToDevice, ctx->stream));
  const int nf = nv * H, ni = g->nx * g->ny;
  fbp2_filter_kernel<<<(nf + 127) / 128, 128, 0, ctx->stream>>>(d, dproj, d_wt, d_ramp, dfilt);
  MONTE_CUDA(ctx, cudaGetLastError());
  fbp2_bp_kernel<<<(ni + 127) / 128, 128, 0, ctx->stream>>>(d, d_views, dfilt, dimg);
  MONTE_CUDA(ctx, cudaGetLastError());
  // the host tables must outlive their asynchronous copies
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

}  // namespace
}  // namespace monte

using namespace monte;

extern "C" {

void monte_fbp2_geom_reference(monte_fbp2_geom* g) {
  if (!g) return;
  memset(g, 0, sizeof(*g));
  g->n_views = 360;  // recon/fbp2.cpp:36,63
  g->n_det = 65;     // :17
  g->view_begin = 1; // :89
  g->view_end = 360;
  g->nx = g->ny = 256;  // :18
  g->flags = MONTE_FDK_TAN_DEGREES;
  g->pitch = 0.5;    // :38
  g->half = 16.25;
  g->sod = 160;      // :92
  g->sdd = 220;      // :112
  g->wdist = 60;     // :38,145
  g->pix = 0.1;      // :101-102
  g->x0 = -12.8;
  g->y0 = 12.8;
  g->scale = 1.7;    // :148
}

int monte_fbp2(monte_ctx* ctx, const monte_fbp2_geom* g, const float* proj, float* filtered,
               float* image, int mem) {
  if (!ctx) return MONTE_EINVAL;
  MONTE_TRY(validate(ctx, g));
  if (!proj || !image) return set_error(ctx, MONTE_EINVAL, "null proj or image");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST)
    return set_error(ctx, MONTE_EINVAL, "bad mem %d", mem);
  MONTE_TRY(enter(ctx));
  const size_t pb = (size_t)g->n_views * g->n_det * sizeof(float);
  const size_t ib = (size_t)g->nx * g->ny * sizeof(float);
  if (mem == MONTE_MEM_DEVICE) {
    float* df = filtered;
    if (!df) {
      MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "2-D FBP filtered scratch"));
      df = (float*)ctx->scratch[kScratchFiltered].ptr;
    }
    return run(ctx, g, proj, df, image);
  }
  MONTE_TRY(ensure_slot(ctx, kScratchProj, pb, "2-D FBP projection staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchFiltered, pb, "2-D FBP filtered staging"));
  MONTE_TRY(ensure_slot(ctx, kScratchVolXY, ib, "2-D FBP image staging"));
  float* dp = (float*)ctx->scratch[kScratchProj].ptr;
  float* df = (float*)ctx->scratch[kScratchFiltered].ptr;
  float* di = (float*)ctx->scratch[kScratchVolXY].ptr;
  MONTE_CUDA(ctx, cudaMemcpyAsync(dp, proj, pb, cudaMemcpyHostToDevice, ctx->stream));
  MONTE_TRY(run(ctx, g, dp, df, di));
  if (filtered)
    MONTE_CUDA(ctx, cudaMemcpyAsync(filtered, df, pb, cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(image, di, ib, cudaMemcpyDeviceToHost, ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return MONTE_OK;
}

}  // extern "C"
