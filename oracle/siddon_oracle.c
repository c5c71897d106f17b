/*
 * siddon_oracle.c -- FP64 CPU oracle for the primary-signal projector and
 * its adjoint.  TEST INFRASTRUCTURE (see oracle/__init__.py).
 *
 * Siddon's original formulation (Med. Phys. 12, 1985): the parametric
 * crossings of the ray with every x-, y- and z-plane of the grid are merged
 * into one sorted list; each interval between consecutive crossings lies in
 * one voxel (found from its midpoint) and contributes its length.  This is
 * a different construction from the GPU's incremental traversal, in double
 * precision, over the same rays (the Monte Carlo's emission rays, built
 * from the same float tables).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../monte_gb300/csrc/mc_setup.h"

static int cmp_double(const void* a, const void* b) {
  double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

/* Visit (voxel, length) pairs of the ray o + t d, t >= 0. */
typedef void (*visit_fn)(void* ctx, size_t v, double len);

static void siddon_ray_d(const monte_siddon_grid* g, const double o[3], const double d[3],
                         double* buf, visit_fn f, void* ctx) {
  const int n[3] = {g->nx, g->ny, g->nz};
  const double lo[3] = {g->x0, g->y0, g->z0};
  const double h[3] = {g->dx, g->dy, g->dz};
  double t0 = 0.0, t1 = INFINITY;
  for (int a = 0; a < 3; a++) {
    if (d[a] == 0.0) {
      if (o[a] < lo[a] || o[a] >= lo[a] + n[a] * h[a]) return;
    } else {
      double ta = (lo[a] - o[a]) / d[a], tb = (lo[a] + n[a] * h[a] - o[a]) / d[a];
      double tn = ta < tb ? ta : tb, tf = ta < tb ? tb : ta;
      if (tn > t0) t0 = tn;
      if (tf < t1) t1 = tf;
    }
  }
  if (!(t0 < t1)) return;
  int m = 0;
  buf[m++] = t0;
  for (int a = 0; a < 3; a++) {
    if (d[a] == 0.0) continue;
    for (int i = 0; i <= n[a]; i++) {
      double t = (lo[a] + i * h[a] - o[a]) / d[a];
      if (t > t0 && t < t1) buf[m++] = t;
    }
  }
  buf[m++] = t1;
  qsort(buf, m, sizeof(double), cmp_double);
  for (int k = 0; k + 1 < m; k++) {
    double len = buf[k + 1] - buf[k];
    if (len <= 0) continue;
    double tm = 0.5 * (buf[k] + buf[k + 1]);
    int idx[3];
    for (int a = 0; a < 3; a++) {
      int i = (int)floor((o[a] + tm * d[a] - lo[a]) / h[a]);
      idx[a] = i < 0 ? 0 : (i >= n[a] ? n[a] - 1 : i);
    }
    f(ctx, ((size_t)idx[2] * g->ny + idx[1]) * g->nx + idx[0], len);
  }
}

typedef struct {
  const float* mu;
  double acc;
  double g;
  double* grad;
} ray_ctx;

static void add_line(void* c, size_t v, double len) {
  ray_ctx* r = (ray_ctx*)c;
  r->acc += (double)r->mu[v] * len;
}

static void add_grad(void* c, size_t v, double len) {
  ray_ctx* r = (ray_ctx*)c;
#pragma omp atomic
  r->grad[v] += r->g * len;
}

/* The Monte Carlo's emission ray of pixel (iu, iv) in view `view`
 * (monte_gb300/csrc/siddon.cuh siddon_ray), in double. */
static void mc_ray(const mc_params* P, const mc_view* V, const mc_pixel* U, const mc_pixel* W,
                   int view, int iu, int iv, double o[3], double d[3]) {
  float cp = U[iu].cos_a * V[view].c - U[iu].sin_a * V[view].s;
  float sp = U[iu].sin_a * V[view].c + U[iu].cos_a * V[view].s;
  o[0] = (double)(-P->sod * V[view].c);
  o[1] = (double)(-P->sod * V[view].s);
  o[2] = 0.0;
  d[0] = (double)(W[iv].sin_t * cp);
  d[1] = (double)(W[iv].sin_t * sp);
  d[2] = (double)W[iv].cos_t;
}

static int setup(const monte_mc_geom* g, const monte_siddon_grid* grid, mc_params* P,
                 mc_view** V, mc_pixel** U, mc_pixel** W) {
  monte_mc_phantom ph;
  memset(&ph, 0, sizeof(ph));
  ph.nx = grid->nx;
  ph.ny = grid->ny;
  ph.nz = grid->nz;
  ph.dx = grid->dx;
  ph.dy = grid->dy;
  ph.dz = grid->dz;
  ph.n_labels = 1;
  monte_mc_request rq;
  memset(&rq, 0, sizeof(rq));
  rq.view_end = g->n_views;
  rq.u_end = g->nu;
  rq.v_end = g->nv;
  const char* why;
  if (mc_setup_params(g, &ph, &rq, P, &why) != MONTE_OK) return MONTE_EINVAL;
  *V = (mc_view*)malloc(sizeof(mc_view) * g->n_views);
  *U = (mc_pixel*)malloc(sizeof(mc_pixel) * g->nu);
  *W = (mc_pixel*)malloc(sizeof(mc_pixel) * g->nv);
  mc_setup_views(g, *V);
  mc_setup_pixels(g, *U, *W);
  return MONTE_OK;
}

/* line[view][iu][iv] (double) for views [vb, ve). */
int oracle_siddon_forward(const monte_mc_geom* g, const monte_siddon_grid* grid, const float* mu,
                          int vb, int ve, double* line) {
  mc_params P;
  mc_view* V;
  mc_pixel *U, *W;
  if (setup(g, grid, &P, &V, &U, &W) != MONTE_OK) return MONTE_EINVAL;
  const int nbuf = grid->nx + grid->ny + grid->nz + 8;
  const long nrays = (long)(ve - vb) * g->nu * g->nv;
#pragma omp parallel
  {
    double* buf = (double*)malloc(sizeof(double) * nbuf);
#pragma omp for schedule(dynamic, 64)
    for (long r = 0; r < nrays; r++) {
      int view = vb + (int)(r / ((long)g->nu * g->nv));
      long p = r % ((long)g->nu * g->nv);
      int iu = (int)(p / g->nv), iv = (int)(p % g->nv);
      double o[3], d[3];
      mc_ray(&P, V, U, W, view, iu, iv, o, d);
      ray_ctx c = {mu, 0.0, 0.0, NULL};
      siddon_ray_d(grid, o, d, buf, add_line, &c);
      line[(size_t)view * g->nu * g->nv + p] = c.acc;
    }
    free(buf);
  }
  free(V);
  free(U);
  free(W);
  return MONTE_OK;
}

/* grad_mu[v] += sum_rays (grad_line + grad_trans * (-exp(-L))) * len. */
int oracle_siddon_backward(const monte_mc_geom* g, const monte_siddon_grid* grid, const float* mu,
                           int vb, int ve, const double* grad_line, const double* grad_trans,
                           double* grad_mu) {
  mc_params P;
  mc_view* V;
  mc_pixel *U, *W;
  if (setup(g, grid, &P, &V, &U, &W) != MONTE_OK) return MONTE_EINVAL;
  const int nbuf = grid->nx + grid->ny + grid->nz + 8;
  const long nrays = (long)(ve - vb) * g->nu * g->nv;
#pragma omp parallel
  {
    double* buf = (double*)malloc(sizeof(double) * nbuf);
#pragma omp for schedule(dynamic, 64)
    for (long r = 0; r < nrays; r++) {
      int view = vb + (int)(r / ((long)g->nu * g->nv));
      long p = r % ((long)g->nu * g->nv);
      size_t cell = (size_t)view * g->nu * g->nv + p;
      int iu = (int)(p / g->nv), iv = (int)(p % g->nv);
      double o[3], d[3];
      mc_ray(&P, V, U, W, view, iu, iv, o, d);
      ray_ctx c = {mu, 0.0, 0.0, grad_mu};
      double gl = grad_line ? grad_line[cell] : 0.0;
      if (grad_trans) {
        siddon_ray_d(grid, o, d, buf, add_line, &c);
        gl -= grad_trans[cell] * exp(-c.acc);
      }
      c.g = gl;
      if (gl != 0.0) siddon_ray_d(grid, o, d, buf, add_grad, &c);
    }
    free(buf);
  }
  free(V);
  free(U);
  free(W);
  return MONTE_OK;
}
