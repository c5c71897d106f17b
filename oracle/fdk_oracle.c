/*
 * fdk_oracle.c -- CPU oracle for the FDK hot path.  TEST INFRASTRUCTURE:
 * only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * it, and only to check results or time the CPU form; the product never links
 * or calls it.
 *
 * A restatement of recon/bp3d20.cpp and recon/bp3d20_325.cpp with their
 * hard-coded constants turned into monte_fdk_geom fields.  Two modes:
 *
 *   faithful (precise == 0): the reference's own arithmetic -- weights and
 *     products in double, the filter accumulator and the output volume in
 *     float, taps rounded to float -- so on x86-64 the result is bit-equal
 *     to the compiled reference programs on the same input (pinned by
 *     tests/golden, generated by tests/golden/make_golden.py).
 *   precise (precise == 1): everything in double, outputs in double.  This is
 *     the FP64 oracle that the GPU filter variants are measured against.
 *
 * Build: oracle/Makefile (-ffp-contract=off so aarch64 does not fuse
 * multiply-adds the reference does not fuse).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/monte.h"

/* Ram-Lak taps h[n], n in [-(nu-1), nu-1], stored at taps[nu-1+n], rounded
 * to float as the reference stores them (recon/bp3d20.cpp:48-60). */
void oracle_fdk_taps(int nu, float* taps) {
  taps[nu - 1] = 0.25f;
  for (int n = 1; n < nu; n++) {
    if (n % 2 == 0) {
      taps[nu - 1 + n] = 0.0f;
      taps[nu - 1 - n] = 0.0f;
    } else {
      double x = n * M_PI;
      double v = -1. / (x * x);
      taps[nu - 1 + n] = (float)v;
      taps[nu - 1 - n] = (float)v;
    }
  }
}

/* Cosine weight of detector element (a, b) (recon/bp3d20.cpp:40). */
static double fdk_weight(const monte_fdk_geom* g, int a, int b) {
  double D = g->wdist;
  double pu = -1 * (a * g->du) + g->half_u;
  double pv = (b * g->dv) - g->half_v;
  return D / sqrt(D * D + pu * pu + pv * pv);
}

/* Weighting + ramp filter, faithful mode (recon/bp3d20.cpp:36-73):
 *   Pw[n][a][b]       = float(P[n][a][b] * w(a,b))
 *   Q[n][b][c]        = sum_a float-accumulated  Pw[n][a][b] * 0.5 * h[a-c]
 * proj is [n_views][nu][nv]; filtered is [n_views][nv][nu]. */
void oracle_fdk_filter(const monte_fdk_geom* g, const float* proj, float* filtered) {
  const int nu = g->nu, nv = g->nv;
  float* taps = (float*)malloc(sizeof(float) * (2 * nu - 1));
  oracle_fdk_taps(nu, taps);
  double* wt = (double*)malloc(sizeof(double) * nu * nv);
  for (int a = 0; a < nu; a++)
    for (int b = 0; b < nv; b++) wt[a * nv + b] = fdk_weight(g, a, b);
#pragma omp parallel
  {
    float* pw = (float*)malloc(sizeof(float) * nu * nv);
#pragma omp for schedule(static)
    for (int n = 0; n < g->n_views; n++) {
      const float* p = proj + (size_t)n * nu * nv;
      for (int i = 0; i < nu * nv; i++) pw[i] = (float)(p[i] * wt[i]);
      float* q = filtered + (size_t)n * nu * nv;
      for (int d = 0; d < nv; d++) {
        for (int b = 0; b < nu; b++) {
          float tmp = 0.f;
          for (int c = 0; c < nu; c++) tmp += pw[c * nv + d] * 0.5 * taps[nu - 1 - b + c];
          q[d * nu + b] = tmp;
        }
      }
    }
    free(pw);
  }
  free(wt);
  free(taps);
}

/* Same operator entirely in double (the FP64 oracle); filtered64 is
 * [n_views][nv][nu]. */
void oracle_fdk_filter_f64(const monte_fdk_geom* g, const float* proj, double* filtered64) {
  const int nu = g->nu, nv = g->nv;
  double* taps = (double*)malloc(sizeof(double) * (2 * nu - 1));
  taps[nu - 1] = 0.25;
  for (int n = 1; n < nu; n++) {
    double x = n * M_PI;
    double v = (n % 2 == 0) ? 0.0 : -1. / (x * x);
    taps[nu - 1 + n] = v;
    taps[nu - 1 - n] = v;
  }
#pragma omp parallel
  {
    double* pw = (double*)malloc(sizeof(double) * nu * nv);
#pragma omp for schedule(static)
    for (int n = 0; n < g->n_views; n++) {
      const float* p = proj + (size_t)n * nu * nv;
      for (int a = 0; a < nu; a++)
        for (int b = 0; b < nv; b++) pw[a * nv + b] = p[a * nv + b] * fdk_weight(g, a, b);
      double* q = filtered64 + (size_t)n * nu * nv;
      for (int d = 0; d < nv; d++)
        for (int b = 0; b < nu; b++) {
          double tmp = 0.0;
          for (int c = 0; c < nu; c++) tmp += pw[c * nv + d] * 0.5 * taps[nu - 1 - b + c];
          q[d * nu + b] = tmp;
        }
    }
    free(pw);
  }
  free(taps);
}

/* Per-view constants of the backprojection (recon/bp3d20.cpp:83-88,103-104,
 * 134-137, 159). */
typedef struct {
  double c, s;   /* cos, sin of pi*beta/180 */
  double px, py; /* rotated source position */
  double tanb;   /* tan(beta) as the reference evaluates it */
  double dbeta;  /* angular step factor, beta_span*2*pi/360 */
} bp_view;

static void bp_view_init(const monte_fdk_geom* g, int k, bp_view* v) {
  double beta = (double)k * 360.0 / g->n_views; /* integer degrees for 360 views */
  double a = M_PI * beta / 180;
  v->c = cos(a);
  v->s = sin(a);
  float start_x = (float)(-g->sod), start_y = 0.f;
  v->px = start_x * v->c - start_y * v->s;
  v->py = start_x * v->s + start_y * v->c;
  v->tanb = (g->flags & MONTE_FDK_TAN_DEGREES) ? tan(beta) : tan(a);
  float beta_span = (float)(360.0 / g->n_views);
  v->dbeta = beta_span * 2 * M_PI / 360; /* evaluated left to right below */
  (void)v->dbeta;
}

/* One voxel-view update; returns the value added (before the float store).
 * flat: filtered array, total elements n_total. */
static inline int bp_sample(const monte_fdk_geom* g, const bp_view* v, int k, int s, int t, int z,
                            const float* flat, size_t n_total, double* out) {
  const int nu = g->nu, nv = g->nv;
  double X = (g->x0 + s * g->dvox), Y = (g->y0 - t * g->dvox), Z = (g->z0 - z * g->dvox);
  double pv0 = X - v->px;
  double pv1 = Y - v->py;
  double pv2 = Z;
  double tmp_x = pv0;
  /* rotate by -beta: cos(-a) = cos(a), sin(-a) = -sin(a) exactly in libm */
  pv0 = pv0 * v->c - pv1 * (-v->s);
  pv1 = tmp_x * (-v->s) + pv1 * v->c;
  double to_det = g->sdd / pv0;
  pv0 *= to_det;
  pv1 *= to_det;
  pv2 *= to_det;
  if (fabs(pv1) > g->half_u || fabs(pv2) > g->half_v) return 0;
  double inv_du = 1.0 / g->du, inv_dv = 1.0 / g->dv;
  double y = -1 * (pv1 * inv_du - g->half_u * inv_du);
  double x = -1 * (pv2 * inv_dv - g->half_v * inv_dv);
  int yi = (int)y, xi = (int)x;
  double tmp_s = X * v->c - Y * v->s;
  double tmp_t = X * v->s + Y * v->c;
  double d = fabs(-1 * v->tanb * tmp_t + 1 * tmp_s) / (sqrt(1 + v->tanb * v->tanb));
  if (tmp_s < 0) d *= -1;
  if (g->mask_radius > 0) {
    int cz = g->nz / 2, ct = g->ny / 2, cs = g->nx / 2;
    if ((z - cz) * (z - cz) + (t - ct) * (t - ct) + (s - cs) * (s - cs) >
        g->mask_radius * g->mask_radius)
      return 0;
  }
  double tmp_output = 0;
  if (0 <= x && x <= nv && 0 <= y && y <= nu) {
    size_t base = (size_t)k * nu * nv;
    size_t i00 = base + (size_t)xi * nu + yi;
    size_t i10 = base + (size_t)(xi + 1) * nu + yi;
    size_t i01 = i00 + 1, i11 = i10 + 1;
    int flat_edge = (g->flags & MONTE_FDK_FLAT_EDGE) != 0;
    /* without the flat-edge quirk, neighbours outside the view are zero */
    double f00 = (i00 < n_total && (flat_edge || (xi < nv && yi < nu))) ? flat[i00] : 0.0;
    double f10 = (i10 < n_total && (flat_edge || (xi + 1 < nv && yi < nu))) ? flat[i10] : 0.0;
    double f01 = (i01 < n_total && (flat_edge || (xi < nv && yi + 1 < nu))) ? flat[i01] : 0.0;
    double f11 = (i11 < n_total && (flat_edge || (xi + 1 < nv && yi + 1 < nu))) ? flat[i11] : 0.0;
    double geo_bl = (yi + 1 - y) * ((xi + 1 - x) * f00 + (x - xi) * f10) +
                    (y - yi) * ((xi + 1 - x) * f01 + (x - xi) * f11);
    tmp_output = geo_bl;
  }
  float beta_span = (float)(360.0 / g->n_views);
  double D = g->wdist;
  double output = (D * D / ((D - d) * (D - d))) * tmp_output * beta_span * 2 * M_PI / 360;
  *out = output;
  return 1;
}

/* Backprojection, faithful mode (recon/bp3d20.cpp:81-166): float volumes
 * accumulated view by view in the reference's order.  Only z in
 * [z_begin, z_end) is computed (the CPU baseline times a bounded sample).
 * vol_zy may be NULL. */
void oracle_fdk_backproject(const monte_fdk_geom* g, const float* filtered, float* vol_xy,
                            float* vol_zy, int z_begin, int z_end) {
  const size_t n_total = (size_t)g->n_views * g->nu * g->nv;
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  bp_view* views = (bp_view*)malloc(sizeof(bp_view) * g->n_views);
  for (int k = 0; k < g->n_views; k++) bp_view_init(g, k, &views[k]);
#pragma omp parallel for schedule(dynamic, 1)
  for (int z = z_begin; z < z_end; z++) {
    for (int k = 0; k < g->n_views; k++) {
      for (int t = 0; t < ny; t++) {
        for (int s = g->s_begin; s < g->s_end; s++) {
          double out;
          if (!bp_sample(g, &views[k], k, s, t, z, filtered, n_total, &out)) continue;
          float* pxy = &vol_xy[(size_t)z * ny * nx + (size_t)t * nx + s];
          *pxy = (float)((double)*pxy + out * g->scale * g->scale2);
          if (vol_zy) {
            float* pzy = &vol_zy[(size_t)s * ny * nz + (size_t)t * nz + z];
            *pzy = (float)((double)*pzy + out * g->scale * g->scale2);
          }
        }
      }
    }
  }
  free(views);
}

/* Backprojection entirely in double from double filtered data (FP64
 * oracle).  vol64 is [nz][ny][nx]. */
void oracle_fdk_backproject_f64(const monte_fdk_geom* g, const double* filtered64, double* vol64,
                                int z_begin, int z_end) {
  const size_t n_total = (size_t)g->n_views * g->nu * g->nv;
  const int nx = g->nx, ny = g->ny;
  bp_view* views = (bp_view*)malloc(sizeof(bp_view) * g->n_views);
  for (int k = 0; k < g->n_views; k++) bp_view_init(g, k, &views[k]);
  /* bp_sample reads float data; convert per view on the fly through a
   * double-capable twin would duplicate code, so sample the double array by
   * casting through a small shim: rebuild the float-free path here. */
#pragma omp parallel for schedule(dynamic, 1)
  for (int z = z_begin; z < z_end; z++) {
    for (int k = 0; k < g->n_views; k++) {
      const bp_view* v = &views[k];
      for (int t = 0; t < ny; t++) {
        for (int s = g->s_begin; s < g->s_end; s++) {
          const int nu = g->nu, nv = g->nv;
          double X = (g->x0 + s * g->dvox), Y = (g->y0 - t * g->dvox), Z = (g->z0 - z * g->dvox);
          double pv0 = X - v->px, pv1 = Y - v->py, pv2 = Z, tmp_x = pv0;
          pv0 = pv0 * v->c + pv1 * v->s;
          pv1 = -tmp_x * v->s + pv1 * v->c;
          double to_det = g->sdd / pv0;
          pv1 *= to_det;
          pv2 *= to_det;
          if (fabs(pv1) > g->half_u || fabs(pv2) > g->half_v) continue;
          double y = (g->half_u - pv1) / g->du, x = (g->half_v - pv2) / g->dv;
          int yi = (int)y, xi = (int)x;
          double tmp_s = X * v->c - Y * v->s, tmp_t = X * v->s + Y * v->c;
          double d = fabs(tmp_s - v->tanb * tmp_t) / sqrt(1 + v->tanb * v->tanb);
          if (tmp_s < 0) d = -d;
          if (g->mask_radius > 0) {
            int cz = g->nz / 2, ct = g->ny / 2, cs = g->nx / 2;
            if ((z - cz) * (z - cz) + (t - ct) * (t - ct) + (s - cs) * (s - cs) >
                g->mask_radius * g->mask_radius)
              continue;
          }
          double val = 0;
          if (0 <= x && x <= nv && 0 <= y && y <= nu) {
            size_t base = (size_t)k * nu * nv;
            size_t i00 = base + (size_t)xi * nu + yi, i10 = i00 + nu;
            int fe = (g->flags & MONTE_FDK_FLAT_EDGE) != 0;
            double f00 = (i00 < n_total && (fe || (xi < nv && yi < nu))) ? filtered64[i00] : 0.0;
            double f10 = (i10 < n_total && (fe || (xi + 1 < nv && yi < nu))) ? filtered64[i10] : 0.0;
            double f01 = (i00 + 1 < n_total && (fe || (xi < nv && yi + 1 < nu))) ? filtered64[i00 + 1] : 0.0;
            double f11 = (i10 + 1 < n_total && (fe || (xi + 1 < nv && yi + 1 < nu))) ? filtered64[i10 + 1] : 0.0;
            val = (yi + 1 - y) * ((xi + 1 - x) * f00 + (x - xi) * f10) +
                  (y - yi) * ((xi + 1 - x) * f01 + (x - xi) * f11);
          }
          double D = g->wdist;
          double dbeta = (360.0 / g->n_views) * 2 * M_PI / 360;
          vol64[(size_t)z * ny * nx + (size_t)t * nx + s] +=
              D * D / ((D - d) * (D - d)) * val * dbeta * g->scale * g->scale2;
        }
      }
    }
  }
  free(views);
}

/* Transpose of oracle_fdk_backproject_f64 (needs flags without
 * MONTE_FDK_FLAT_EDGE): out64[view][v][u] = sum over voxels of the same
 * coefficients times vol64[z][t][s].  FP64 reference for the GPU forward
 * projector and the FDK gradient. */
void oracle_fdk_forward_project_f64(const monte_fdk_geom* g, const double* vol64, double* out64) {
  const int nx = g->nx, ny = g->ny, nu = g->nu, nv = g->nv;
  bp_view* views = (bp_view*)malloc(sizeof(bp_view) * g->n_views);
  for (int k = 0; k < g->n_views; k++) bp_view_init(g, k, &views[k]);
  memset(out64, 0, sizeof(double) * (size_t)g->n_views * nu * nv);
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < g->n_views; k++) {
    const bp_view* v = &views[k];
    double* out = out64 + (size_t)k * nu * nv;
    for (int z = 0; z < g->nz; z++)
      for (int t = 0; t < ny; t++)
        for (int s = g->s_begin; s < g->s_end; s++) {
          double r = vol64[(size_t)z * ny * nx + (size_t)t * nx + s];
          if (r == 0.0) continue;
          double X = (g->x0 + s * g->dvox), Y = (g->y0 - t * g->dvox), Z = (g->z0 - z * g->dvox);
          double pv0 = X - v->px, pv1 = Y - v->py, pv2 = Z, tmp_x = pv0;
          pv0 = pv0 * v->c + pv1 * v->s;
          pv1 = -tmp_x * v->s + pv1 * v->c;
          double to_det = g->sdd / pv0;
          pv1 *= to_det;
          pv2 *= to_det;
          if (fabs(pv1) > g->half_u || fabs(pv2) > g->half_v) continue;
          double y = (g->half_u - pv1) / g->du, x = (g->half_v - pv2) / g->dv;
          if (!(0 <= x && x <= nv && 0 <= y && y <= nu)) continue;
          if (g->mask_radius > 0) {
            int cz = g->nz / 2, ct = g->ny / 2, cs = g->nx / 2;
            if ((z - cz) * (z - cz) + (t - ct) * (t - ct) + (s - cs) * (s - cs) >
                g->mask_radius * g->mask_radius)
              continue;
          }
          int yi = (int)y, xi = (int)x;
          double fx = x - xi, fy = y - yi;
          double tmp_s = X * v->c - Y * v->s, tmp_t = X * v->s + Y * v->c;
          double d = fabs(tmp_s - v->tanb * tmp_t) / sqrt(1 + v->tanb * v->tanb);
          if (tmp_s < 0) d = -d;
          double D = g->wdist;
          double dbeta = (360.0 / g->n_views) * 2 * M_PI / 360;
          double c = D * D / ((D - d) * (D - d)) * dbeta * g->scale * g->scale2 * r;
          for (int dx = 0; dx < 2; dx++)
            for (int dy = 0; dy < 2; dy++) {
              int row = xi + dx, col = yi + dy;
              if (row >= nv || col >= nu) continue;
              out[(size_t)row * nu + col] += c * (dx ? fx : 1 - fx) * (dy ? fy : 1 - fy);
            }
        }
  }
  free(views);
}

/* Transpose of the weighting + filter (oracle_fdk_filter_f64):
 * h64[view][u][v] = w(u,v) * sum_b 0.5 h[u-b] g64[view][v][b]. */
void oracle_fdk_filter_adjoint_f64(const monte_fdk_geom* g, const double* g64, double* h64) {
  const int nu = g->nu, nv = g->nv;
  double* taps = (double*)malloc(sizeof(double) * (2 * nu - 1));
  taps[nu - 1] = 0.25;
  for (int n = 1; n < nu; n++) {
    double x = n * M_PI;
    double v = (n % 2 == 0) ? 0.0 : -1. / (x * x);
    taps[nu - 1 + n] = v;
    taps[nu - 1 - n] = v;
  }
#pragma omp parallel for schedule(static)
  for (int n = 0; n < g->n_views; n++) {
    const double* G = g64 + (size_t)n * nu * nv;
    double* H = h64 + (size_t)n * nu * nv;
    for (int c = 0; c < nu; c++)
      for (int d = 0; d < nv; d++) {
        double acc = 0.0;
        for (int b = 0; b < nu; b++) acc += G[(size_t)d * nu + b] * 0.5 * taps[nu - 1 - b + c];
        H[(size_t)c * nv + d] = acc * fdk_weight(g, c, d);
      }
  }
  free(taps);
}
