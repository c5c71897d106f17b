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
//    dL/dmu_v = length in v, times the incoming gradient, into per-voxel
//    int64 fixed-point sums.  Integer additions commute, so the gradient is
//    the same bit for bit whatever order the rays' atomics land in (float
//    atomics would round differently from run to run).  The scale is a
//    power of two chosen on the device from the largest incoming gradient
//    so that no sum can overflow: with |d exp(-L)/dL| <= 1, every ray adds
//    at most (|grad_line| + |grad_transmission|) times the voxel diagonal
//    to a voxel, and there are at most n_rays of them.
#include <algorithm>
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

// The fixed-point scale of the adjoint's sums, in the scratch words after
// them: [0] the largest |grad_line| + |grad_transmission| over the rays (as
// float bits: non-negative floats order like their bit patterns), [1] the
// scale as float bits, [2..3] 1 / scale as a double.
struct SiddonScale {
  unsigned gmax_bits;
  unsigned scale_bits;
  double inv_scale;
};

__global__ void siddon_gmax_kernel(SiddonDev s, const float* __restrict__ grad_line,
                                   const float* __restrict__ grad_trans, SiddonScale* sc) {
  const size_t nr = (size_t)(s.view_end - s.view_begin) * s.P.nu * s.P.nv;
  float m = 0.f;
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < nr;
       r += (size_t)gridDim.x * blockDim.x) {
    const size_t cell = (size_t)s.view_begin * s.P.nu * s.P.nv + r;
    const float g = (grad_line ? fabsf(grad_line[cell]) : 0.f) +
                    (grad_trans ? fabsf(grad_trans[cell]) : 0.f);
    m = g > m || g != g ? g : m;  // a NaN wins (its bits order above every finite value)
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m || x != x ? x : m;
  }
  if ((threadIdx.x & 31) == 0 && m != 0.f) atomicMax(&sc->gmax_bits, __float_as_uint(m));
}

// scale = 2^e with bound * scale <= 2^62, bound = gmax * diagonal * n_rays:
// no voxel's sum can leave the int64 range.  A zero or non-finite gradient
// leaves the scale at zero (the sums stay zero; a non-finite gradient then
// makes grad_mu NaN in the conversion).
__global__ void siddon_scale_kernel(SiddonScale* sc, double diag, double n_rays) {
  const float g = __uint_as_float(sc->gmax_bits);
  float scale = 0.f;
  double inv = 0.0;
  if (g > 0.f && isfinite(g)) {
    int e;
    frexp((double)g * diag * n_rays, &e);  // bound < 2^e
    const int k = max(min(62 - e, 126), -126);  // bound * 2^k < 2^62
    scale = ldexpf(1.f, k);
    inv = ldexp(1.0, -k);
  } else if (g != 0.f) {
    inv = __longlong_as_double(0x7ff8000000000000ll);  // NaN
  }
  sc->scale_bits = __float_as_uint(scale);
  sc->inv_scale = inv;
}

__global__ void siddon_backward_kernel(SiddonDev s, const float* __restrict__ mu,
                                       const float* __restrict__ grad_line,
                                       const float* __restrict__ grad_trans,
                                       unsigned long long* __restrict__ acc,
                                       const SiddonScale* __restrict__ sc) {
  size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  int view, iu, iv;
  size_t cell;
  if (!ray_of(s, r, &view, &iu, &iv, &cell)) return;
  const float scale = __uint_as_float(sc->scale_bits);
  if (scale == 0.f) return;
  float o[3], d[3];
  siddon_ray(s.P, s.V, s.U, s.W, view, iu, iv, o, d);
  float gL = grad_line ? grad_line[cell] : 0.0f;
  if (grad_trans) gL -= grad_trans[cell] * expf(-line_integral(s, mu, o, d));  // dT/dL = -T
  if (gL == 0.0f) return;
  const float gs = gL * scale;  // exact: scale is a power of two
  siddon_walk(s.g, o[0], o[1], o[2], d[0], d[1], d[2], [&](size_t v, float len) {
    atomicAdd(acc + v, (unsigned long long)__float2ll_rn(gs * len));
  });
}

// grad_mu += sums / scale
__global__ void siddon_accumulate_kernel(const long long* __restrict__ acc,
                                         const SiddonScale* __restrict__ sc, size_t n,
                                         float* __restrict__ grad_mu) {
  const double inv = sc->inv_scale;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    grad_mu[i] += (float)((double)acc[i] * inv);
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
  // the fixed-point sums (int64 per voxel) and, after them, their scale
  const size_t acc_bytes = nvox * sizeof(long long);
  MONTE_TRY(ensure_slot(ctx, kScratchSiddon, acc_bytes + sizeof(SiddonScale), "gradient sums"));
  unsigned long long* acc = (unsigned long long*)ctx->scratch[kScratchSiddon].ptr;
  SiddonScale* sc = (SiddonScale*)((char*)ctx->scratch[kScratchSiddon].ptr + acc_bytes);
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
    MONTE_CUDA(ctx, cudaMemsetAsync(acc, 0, acc_bytes + sizeof(SiddonScale), ctx->stream));
    const size_t cap = (size_t)std::max(ctx->sm_count, 1) * 8;  // grid-stride loops
    const unsigned gblocks = (unsigned)std::min<size_t>((nr + 255) / 256, cap);
    siddon_gmax_kernel<<<gblocks, 256, 0, ctx->stream>>>(s, dgl, dgt, sc);
    const double diag = std::sqrt(grid->dx * grid->dx + grid->dy * grid->dy + grid->dz * grid->dz);
    siddon_scale_kernel<<<1, 1, 0, ctx->stream>>>(sc, diag, (double)nr);
    siddon_backward_kernel<<<(unsigned)((nr + 127) / 128), 128, 0, ctx->stream>>>(s, dmu, dgl, dgt,
                                                                                  acc, sc);
    const unsigned ablocks = (unsigned)std::min<size_t>((nvox + 255) / 256, cap);
    siddon_accumulate_kernel<<<ablocks, 256, 0, ctx->stream>>>((const long long*)acc, sc, nvox, dg);
    MONTE_CUDA(ctx, cudaGetLastError());
  }
  if (mem == MONTE_MEM_HOST) {
    MONTE_CUDA(ctx, cudaMemcpyAsync(grad_mu, dg, nvox * 4, cudaMemcpyDeviceToHost, ctx->stream));
    MONTE_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return MONTE_OK;
}

}  // extern "C"
