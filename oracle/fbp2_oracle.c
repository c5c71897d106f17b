/*
 * fbp2_oracle.c -- CPU restatement of the reference's 2-D fan-beam FBP,
 * recon/fbp2.cpp.  TEST INFRASTRUCTURE: only the tests use it; the product
 * never links or calls it.
 *
 * Same arithmetic as the reference program, parameterised by
 * monte_fbp2_geom (include/monte.h):
 *   weighting  pw[v][c] = float(p[v][c] * D / sqrt(D^2 + (-half + pitch*c)^2))
 *              (recon/fbp2.cpp:36-40)
 *   filter     q[v][b] = float(sum_c double(pw[v][c]) * 0.5 * h[c - b]),
 *              Ram-Lak taps h (:44-73)
 *   backprojection over views [view_begin, view_end) (:86-152): rotate the
 *              pixel into the view frame, scale to the detector at sdd, reject
 *              |u| > half, take the NEAREST detector element
 *              int((half - u) / pitch), weight D^2 / (D - d)^2 with d the
 *              signed distance to the line of slope tan(beta) (beta in
 *              degrees passed to tan, as the reference does), and add
 *              float(q * dbeta * scale) to the float image.
 * Detector reads past the end of the filtered array read zero (the
 * reference reads whatever follows its allocation there).
 *
 * Build: oracle/Makefile (-ffp-contract=off).  Pinned to the compiled
 * reference program by tests/golden/fbp2.npz.
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>

#include "../include/monte.h"

void oracle_fbp2(const monte_fbp2_geom* g, const float* proj, float* filtered, float* image) {
  const int H = g->n_det, nview = g->n_views;
  float* pw = (float*)malloc(sizeof(float) * (size_t)H * nview);
  double* ramp = (double*)calloc((size_t)(2 * H - 1), sizeof(double));
  for (int b = 0; b < nview; b++)
    for (int z = 0; z < H; z++)
      pw[b * H + z] = proj[b * H + z] * (g->wdist / (sqrt(pow(g->wdist, 2) +
                                                         pow(-g->half + g->pitch * z, 2))));
  ramp[H - 1] = 0.25;
  for (int n = 1; n < H; n++) {
    if (n % 2 == 0) {
      ramp[H - 1 + n] = 0;
      ramp[H - 1 - n] = 0;
    } else {
      ramp[H - 1 + n] = -1. / pow(n * M_PI, 2);
      ramp[H - 1 - n] = -1. / pow(n * M_PI, 2);
    }
  }
  for (int d = 0; d < nview; d++)
    for (int b = 0; b < H; b++) {
      double tmp = 0.;
      for (int c = 0; c < H; c++) tmp += pw[d * H + c] * 0.5 * ramp[H - 1 - b + c];
      filtered[d * H + b] = (float)tmp;
    }
  const size_t n_total = (size_t)H * nview;
  for (size_t i = 0; i < (size_t)g->nx * g->ny; i++) image[i] = 0.f;
  const float span = 360.0f / (float)nview;
  for (int beta = g->view_begin; beta < g->view_end; beta++) {
    const double ang = M_PI * (beta * span) / 180;
    const float start_x = (float)(-g->sod);
    const double px = start_x * cos(ang) - 0.f * sin(ang);
    const double py = start_x * sin(ang) + 0.f * cos(ang);
    const double tb = (g->flags & MONTE_FDK_TAN_DEGREES) ? tan((double)(beta * span)) : tan(ang);
    for (int t = 0; t < g->ny; t++)
      for (int s = 0; s < g->nx; s++) {
        double v0 = (g->x0 + s * g->pix) - px;
        double v1 = (g->y0 - t * g->pix) - py;
        const double tmp_x = v0;
        v0 = v0 * cos(-1 * ang) - v1 * sin(-1 * ang);
        v1 = tmp_x * sin(-1 * ang) + v1 * cos(-1 * ang);
        const double k = g->sdd / v0;
        v0 *= k;
        v1 *= k;
        if (fabs(v1) > g->half) continue;
        const int iy = (int)(-(1.0 / g->pitch) * (v1 - g->half));
        const double ts = (g->x0 + s * g->pix) * cos(ang) - (g->y0 - g->pix * t) * sin(ang);
        const double tt = (g->x0 + s * g->pix) * sin(ang) + (g->y0 - g->pix * t) * cos(ang);
        double dd = fabs(-1 * tb * tt + 1 * ts) / (sqrt(1 + pow(tb, 2)));
        if (ts < 0) dd *= -1;
        const size_t idx = (size_t)beta * H + iy;
        const double q = idx < n_total ? filtered[idx] : 0.0;
        const double out = (pow(g->wdist, 2) / pow(g->wdist - dd, 2)) * q * span * 2 * M_PI / 360;
        image[(size_t)g->nx * t + s] += out * g->scale;
      }
  }
  free(pw);
  free(ramp);
}
