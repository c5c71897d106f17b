// siddon.cu -- primary signal exp(-integral mu dl) along the Monte Carlo's
// primary rays and its adjoint d(signal)/d(mu), for the differentiable mode.
//
// The reference has no deterministic projector: its primary image is the
// Monte Carlo tally of unscattered photons (monte_cu/CBCT_real325im.cu:
// 567-590).  The expected value of that tally per history is exactly
// exp(-line integral) along the emission ray (Beer-Lambert), which these
// kernels compute with Siddon's exact voxel traversal:
//  * siddon_forward_kernel: one thread per ray, line integral and
//    transmission;
//  * siddon_backward_kernel: one thread per ray; recomputes the line
//    integral (nothing from the forward pass is stored), then scatters
//    dL/dmu_v = length in v, times the incoming gradient, into grad_mu with
//    float atomics.
#include <cmath>
#include <cstring>
#include <vector>

#include "mc_setup.h"
#include "monte_internal.h"
#include "siddon.cuh"

namespace monte {
namespace {

struct SiddonDev {
  mc_params P;
  const mc_view* V;
  const mc_pixel* U;
  const mc_pixel* W;
  SiddonGrid g;
  int view_begin, view_end;
};

__device__ __forceinline__ bool ray_of(const SiddonDev& s, size_t r, int* view, int* iu, int* iv,
                                       size_t* cell) {
  const size_t per_view = (size_t)s.P.nu * s.P.nv;
  const size_t nrays = (size_t)(s.view_end - s.view_begin) * per_view;
  if (r >= nrays) return false;
  *view = s.view_begin + (int)(r / per_view);
  size_t p = r % per_view;
  *iu = (int)(p / s.P.nv);
  *iv = (int)(p % s.P.nv);
  *cell = (size_t)(*view) * per_view + p;
  return true;
}

// Line integral of mu along the ray, the segments summed with Kahan's
// compensation (the float sum of a few hundred terms otherwise loses ~1e-6).
__device__ __forceinline__ float line_integral(const SiddonDev& s, const float* __restrict__ mu,
                                               const float* o, const float* d) {
  float sum = 0.f, comp = 0.f;
  siddon_walk(s.g, o[0], o[1], o[2], d[0], d[1], d[2], [&](size_t v, float len) {
    const float y = __ldg(mu + v) * len - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
  });
  return sum;
}

__global__ void siddon_forward_kernel(SiddonDev s, const float* __restrict__ mu,
                                      float* __restrict__ line, float* __restrict__ trans) {
  size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int view, iu, iv;
  size_t cell;
  if (!ray_of(s, r, &view, &iu, &iv, &cell)) return;
  float o[3], d[3];
  siddon_ray(s.P, s.V, s.U, s.W, view, iu, iv, o, d);
  const float L = line_integral(s, mu, o, d);
  if (line) line[cell] = L;
  if (trans) trans[cell] = expf(-L);
}

__global__ void siddon_backward_kernel(SiddonDev s, const float* __restrict__ mu,
                                       const float* __restrict__ grad_line,
                                       const float* __restrict__ grad_trans,
                                       float* __restrict__ grad_mu) {
  size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int view, iu, iv;
  size_t cell;
  if (!ray_of(s, r, &view, &iu, &iv, &cell)) return;
  float o[3], d[3];
  siddon_ray(s.P, s.V, s.U, s.W, view, iu, iv, o, d);
  float gL = grad_line ? grad_line[cell] : 0.0f;
  if (grad_trans) gL -= grad_trans[cell] * expf(-line_integral(s, mu, o, d));  // dT/dL = -T
  if (gL == 0.0f) return;
  siddon_walk(s.g, o[0], o[1], o[2], d[0], d[1], d[2],
              [&](size_t v, float len) { atomicAdd(grad_mu + v, gL * len); });
}

int setup(monte_ctx* ctx, const monte_mc_geom* g, const monte_siddon_grid* grid, int vb, int ve,
          SiddonDev* s) {
  if (!g || !grid) return set_error(ctx, MONTE_EINVAL, "null geometry");
  if (grid->nx <= 0 || grid->ny <= 0 || grid->nz <= 0 || !(grid->dx > 0 && grid->dy > 0 && grid->dz > 0))
    return set_error(ctx, MONTE_EINVAL, "bad Siddon grid");
  if (vb < 0 || ve > g->n_views || vb > ve) return set_error(ctx, MONTE_EINVAL, "bad view range");
  monte_mc_phantom ph;
  memset(&ph, 0, sizeof(ph));
  ph.nx = grid->nx;
  ph.ny = grid->ny;
  ph.nz = grid->nz;
  ph.dx = grid->dx;
  ph.dy = grid->dy;
  ph.dz = grid->dz;
  ph.x0 = grid->x0;
  ph.y0 = grid->y0;
  ph.z0 = grid->z0;
  ph.n_labels = 1;
  monte_mc_request rq;
  memset(&rq, 0, sizeof(rq));
  rq.view_begin = vb;
  rq.view_end = ve;
  rq.u_end = g->nu;
  rq.v_end = g->nv;
  rq.histories_per_pixel = 1;
  const char* why;
  if (mc_setup_params(g, &ph, &rq, &s->P, &why) != MONTE_OK)
    return set_error(ctx, MONTE_EINVAL, "%s", why);
  std::vector<mc_view> V(g->n_views);
  std::vector<mc_pixel> U(g->nu), W(g->nv);
  mc_setup_views(g, V.data());
  mc_setup_pixels(g, U.data(), W.data());
  MONTE_TRY(ensure(ctx, ctx->mc_views, V.size() * sizeof(mc_view), "view table"));
  MONTE_TRY(ensure(ctx, ctx->mc_pixels, (U.size() + W.size()) * sizeof(mc_pixel), "pixel table"));
  mc_pixel* dp = (mc_pixel*)ctx->mc_pixels.ptr;
  MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->mc_views.ptr, V.data(), V.size() * sizeof(mc_view),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(dp, U.data(), U.size() * sizeof(mc_pixel),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaMemcpyAsync(dp + U.size(), W.data(), W.size() * sizeof(mc_pixel),
                                  cudaMemcpyHostToDevice, ctx->stream));
  MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // host tables die at return
  s->V = (const mc_view*)ctx->mc_views.ptr;
  s->U = dp;
  s->W = dp + U.size();
  s->g.nx = grid->nx;
  s->g.ny = grid->ny;
  s->g.nz = grid->nz;
  s->g.x0 = grid->x0;
  s->g.y0 = grid->y0;
  s->g.z0 = grid->z0;
  s->g.dx = grid->dx;
  s->g.dy = grid->dy;
  s->g.dz = grid->dz;
  s->view_begin = vb;
  s->view_end = ve;
  return MONTE_OK;
}

size_t n_rays(const monte_mc_geom* g, int vb, int ve) { return (size_t)(ve - vb) * g->nu * g->nv; }

}  // namespace
}  // namespace monte

using namespace monte;

extern "C" {

int monte_siddon_forward(monte_ctx* ctx, const monte_mc_geom* g, const monte_siddon_grid* grid,
                         const float* mu, int view_begin, int view_end, float* line,
                         float* transmission, int mem) {
  if (!ctx) return MONTE_EINVAL;
  if (!mu || (!line && !transmission)) return set_error(ctx, MONTE_EINVAL, "null array");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST) return set_error(ctx, MONTE_EINVAL, "bad mem");
  MONTE_TRY(enter(ctx));
  SiddonDev s;
  MONTE_TRY(setup(ctx, g, grid, view_begin, view_end, &s));
  const size_t nr = n_rays(g, view_begin, view_end);
  const size_t nvox = (size_t)grid->nx * grid->ny * grid->nz;
  const size_t ncell = (size_t)g->n_views * g->nu * g->nv;
  const float* dmu = mu;
  float *dl = line, *dt = transmission;
  if (mem == MONTE_MEM_HOST) {
    MONTE_TRY(ensure_slot(ctx, kScratchAux0, nvox * 4, "mu staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchAux1, ncell * 4, "line staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchAux2, ncell * 4, "transmission staging"));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchAux0].ptr, mu, nvox * 4,
                                    cudaMemcpyHostToDevice, ctx->stream));
    dmu = (const float*)ctx->scratch[kScratchAux0].ptr;
    dl = line ? (float*)ctx->scratch[kScratchAux1].ptr : nullptr;
    dt = transmission ? (float*)ctx->scratch[kScratchAux2].ptr : nullptr;
    if (dl) MONTE_CUDA(ctx, cudaMemcpyAsync(dl, line, ncell * 4, cudaMemcpyHostToDevice, ctx->stream));
    if (dt) MONTE_CUDA(ctx, cudaMemcpyAsync(dt, transmission, ncell * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (nr) {
    siddon_forward_kernel<<<(unsigned)((nr + 127) / 128), 128, 0, ctx->stream>>>(s, dmu, dl, dt);
    MONTE_CUDA(ctx, cudaGetLastError());
  }
  if (mem == MONTE_MEM_HOST) {
    if (dl) MONTE_CUDA(ctx, cudaMemcpyAsync(line, dl, ncell * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (dt) MONTE_CUDA(ctx, cudaMemcpyAsync(transmission, dt, ncell * 4, cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return MONTE_OK;
}

int monte_siddon_backward(monte_ctx* ctx, const monte_mc_geom* g, const monte_siddon_grid* grid,
                          const float* mu, int view_begin, int view_end, const float* grad_line,
                          const float* grad_transmission, float* grad_mu, int mem) {
  if (!ctx) return MONTE_EINVAL;
  if (!mu || !grad_mu || (!grad_line && !grad_transmission))
    return set_error(ctx, MONTE_EINVAL, "null array");
  if (mem != MONTE_MEM_DEVICE && mem != MONTE_MEM_HOST) return set_error(ctx, MONTE_EINVAL, "bad mem");
  MONTE_TRY(enter(ctx));
  SiddonDev s;
  MONTE_TRY(setup(ctx, g, grid, view_begin, view_end, &s));
  const size_t nr = n_rays(g, view_begin, view_end);
  const size_t nvox = (size_t)grid->nx * grid->ny * grid->nz;
  const size_t ncell = (size_t)g->n_views * g->nu * g->nv;
  const float *dmu = mu, *dgl = grad_line, *dgt = grad_transmission;
  float* dg = grad_mu;
  if (mem == MONTE_MEM_HOST) {
    MONTE_TRY(ensure_slot(ctx, kScratchAux0, nvox * 4, "mu staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchAux1, ncell * 4, "gradient staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchAux2, ncell * 4, "gradient staging"));
    MONTE_TRY(ensure_slot(ctx, kScratchAux3, nvox * 4, "grad_mu staging"));
    MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchAux0].ptr, mu, nvox * 4, cudaMemcpyHostToDevice, ctx->stream));
    dmu = (const float*)ctx->scratch[kScratchAux0].ptr;
    if (grad_line) {
      MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchAux1].ptr, grad_line, ncell * 4, cudaMemcpyHostToDevice, ctx->stream));
      dgl = (const float*)ctx->scratch[kScratchAux1].ptr;
    }
    if (grad_transmission) {
      MONTE_CUDA(ctx, cudaMemcpyAsync(ctx->scratch[kScratchAux2].ptr, grad_transmission, ncell * 4, cudaMemcpyHostToDevice, ctx->stream));
      dgt = (const float*)ctx->scratch[kScratchAux2].ptr;
    }
    dg = (float*)ctx->scratch[kScratchAux3].ptr;
    MONTE_CUDA(ctx, cudaMemcpyAsync(dg, grad_mu, nvox * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (nr) {
    siddon_backward_kernel<<<(unsigned)((nr + 127) / 128), 128, 0, ctx->stream>>>(s, dmu, dgl, dgt, dg);
    MONTE_CUDA(ctx, cudaGetLastError());
  }
  if (mem == MONTE_MEM_HOST) {
    MONTE_CUDA(ctx, cudaMemcpyAsync(grad_mu, dg, nvox * 4, cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return MONTE_OK;
}

}  // extern "C"
