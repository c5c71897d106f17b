/*
 * mc_setup.h -- host-side interpretation of the public Monte Carlo structs
 * (include/monte.h) into the float tables the history functions of
 * mc_physics.h read.  Plain C, host only; used by the library's entry
 * points and by the CPU replay harness so both start from identical tables.
 *
 * The per-view and per-pixel constants follow monte_cu/CBCT_real325im.cu:
 * 476-512 (aim at the pixel centre, polar angle pi/2 - atan(zl/Dsd),
 * azimuth atan(yl/Dsd) + view angle); the Woodcock and interaction tables
 * follow :217-222, :501-503, :624-656 (mu = table * density, majorant =
 * max over media, ratios as float divisions).
 */
#ifndef MONTE_MC_SETUP_H
#define MONTE_MC_SETUP_H

#include <math.h>
#include <string.h>

#include "../../include/monte.h"
#include "mc_physics.h"

/* Returns MONTE_OK or MONTE_EINVAL; `why` receives a message. */
static inline int mc_setup_params(const monte_mc_geom* g, const monte_mc_phantom* ph,
                                  const monte_mc_request* run, mc_params* P, const char** why) {
  *why = "";
  if (g->n_views <= 0 || g->nu <= 0 || g->nv <= 0) { *why = "bad detector size"; return MONTE_EINVAL; }
  if (!(g->du > 0 && g->dv > 0 && g->half_u > 0 && g->half_v > 0 && g->sod > 0 && g->sdd > g->sod)) {
    *why = "bad detector pitch/extent or distances (need sdd > sod > 0)";
    return MONTE_EINVAL;
  }
  if (g->max_interactions < 0 || g->max_interactions > 1000) { *why = "bad max_interactions"; return MONTE_EINVAL; }
  if (g->flags & ~(unsigned)(MONTE_MC_STALE_SIN_PHI | MONTE_MC_FIRST_COMPTON_Z | MONTE_MC_NO_RAYLEIGH_TALLY)) {
    *why = "unknown MC flags";
    return MONTE_EINVAL;
  }
  if (ph->nx <= 0 || ph->ny <= 0 || ph->nz <= 0 || !(ph->dx > 0 && ph->dy > 0 && ph->dz > 0)) {
    *why = "bad phantom grid";
    return MONTE_EINVAL;
  }
  if (ph->n_labels <= 0 || ph->n_labels > MC_MAX_LABELS) { *why = "n_labels must be 1..256"; return MONTE_EINVAL; }
  if (run->view_begin < 0 || run->view_end > g->n_views || run->view_begin > run->view_end ||
      run->u_begin < 0 || run->u_end > g->nu || run->u_begin > run->u_end || run->v_begin < 0 ||
      run->v_end > g->nv || run->v_begin > run->v_end) {
    *why = "view/pixel range outside the detector";
    return MONTE_EINVAL;
  }
  if (run->kernel != MONTE_MC_PLAIN && run->kernel != MONTE_MC_PERSISTENT) { *why = "unknown kernel"; return MONTE_EINVAL; }
  memset(P, 0, sizeof(*P));
  P->n_views = g->n_views;
  P->nu = g->nu;
  P->nv = g->nv;
  P->max_int = g->max_interactions;
  P->flags = g->flags;
  P->du = (float)g->du;
  P->dv = (float)g->dv;
  P->half_u = (float)g->half_u;
  P->half_v = (float)g->half_v;
  P->inv_du = (float)(1.0 / g->du);
  P->inv_dv = (float)(1.0 / g->dv);
  P->sod = (float)g->sod;
  P->sdd = (float)g->sdd;
  P->dod = (float)(g->sdd - g->sod);
  P->to = (float)((g->sod - g->start_plane) / g->sdd);
  P->nx = ph->nx;
  P->ny = ph->ny;
  P->nz = ph->nz;
  P->x0 = (float)ph->x0;
  P->y0 = (float)ph->y0;
  P->z0 = (float)ph->z0;
  P->inv_dx = (float)(1.0 / ph->dx);
  P->inv_dy = (float)(1.0 / ph->dy);
  P->inv_dz = (float)(1.0 / ph->dz);
  P->clip_r2 = ph->clip_radius > 0 ? (float)(ph->clip_radius * ph->clip_radius) : 0.0f;
  P->clip_hz = (float)ph->clip_half_z;
  P->seed = run->seed;
  monte_philox_schedule(run->seed, &P->keys);
  P->job = run->job;
  P->per = run->histories_per_pixel;
  P->view_begin = run->view_begin;
  P->view_end = run->view_end;
  P->u_begin = run->u_begin;
  P->u_end = run->u_end;
  P->v_begin = run->v_begin;
  P->v_end = run->v_end;
  return MONTE_OK;
}

static inline int mc_setup_tables(const monte_mc_phantom* ph, const monte_xcom* x,
                                  const monte_spectrum* sp, mc_tables* T, const char** why) {
  *why = "";
  if (!x || x->n_materials <= 0 || x->n_materials > 8 || !x->coherent || !x->incoherent ||
      !x->photoelectric || !x->total) {
    *why = "bad XCOM tables (1..8 materials, four arrays)";
    return MONTE_EINVAL;
  }
  if (!sp || sp->n_lines <= 0 || sp->n_lines > MC_MAX_LINES || !sp->energy_kev || !sp->weight) {
    *why = "bad spectrum (1..512 lines)";
    return MONTE_EINVAL;
  }
  if (!ph->label_material || !ph->label_density) { *why = "null label tables"; return MONTE_EINVAL; }
  memset(T, 0, sizeof(*T));
  for (int l = 0; l < ph->n_labels; l++) {
    int m = ph->label_material[l];
    if (m < -1 || m >= x->n_materials) { *why = "label material out of range"; return MONTE_EINVAL; }
    if (m >= 0 && !(ph->label_density[l] >= 0)) { *why = "negative density"; return MONTE_EINVAL; }
    T->label_material[l] = (int8_t)m;
  }
  for (int l = ph->n_labels; l < MC_MAX_LABELS; l++) T->label_material[l] = -1;
  for (int k = 0; k < MC_NBINS; k++) {
    float mu_max = 0.0f;
    float mu[MC_MAX_LABELS];
    for (int l = 0; l < ph->n_labels; l++) {
      int m = T->label_material[l];
      mu[l] = m < 0 ? 0.0f : x->total[m * MC_NBINS + k] * (float)ph->label_density[l];
      if (mu[l] > mu_max) mu_max = mu[l];
    }
    /* a phantom of air only: one huge step leaves the box */
    T->inv_mu_max[k] = mu_max > 0.0f ? 1.0f / mu_max : 1.0e6f;
    for (int l = 0; l < ph->n_labels; l++) T->ratio[l][k] = mu_max > 0.0f ? mu[l] / mu_max : 0.0f;
  }
  for (int m = 0; m < x->n_materials; m++) {
    for (int k = 0; k < MC_NBINS; k++) {
      float ab = x->photoelectric[m * MC_NBINS + k];
      float coh = x->coherent[m * MC_NBINS + k];
      float mu = x->total[m * MC_NBINS + k];
      T->p_photo[m][k] = mu > 0.0f ? ab / mu : 1.0f;
      T->p_photo_coh[m][k] = mu > 0.0f ? (ab + coh) / mu : 1.0f;
    }
  }
  double wsum = 0.0;
  for (int i = 0; i < sp->n_lines; i++) {
    if (!(sp->weight[i] >= 0) || !(sp->energy_kev[i] > 0 && sp->energy_kev[i] <= 200)) {
      *why = "spectrum lines need weight >= 0 and 0 < E <= 200 keV";
      return MONTE_EINVAL;
    }
    wsum += sp->weight[i];
  }
  if (!(wsum > 0)) { *why = "spectrum weights sum to zero"; return MONTE_EINVAL; }
  double acc = 0.0;
  for (int i = 0; i < sp->n_lines; i++) {
    acc += sp->weight[i];
    T->cdf[i] = (float)(acc / wsum);
    T->energy[i] = (float)sp->energy_kev[i];
  }
  T->cdf[sp->n_lines - 1] = 1.0f;
  T->n_lines = sp->n_lines;
  return MONTE_OK;
}

static inline void mc_setup_views(const monte_mc_geom* g, mc_view* V) {
  for (int k = 0; k < g->n_views; k++) {
    double a = M_PI * ((double)k * 360.0 / g->n_views) / 180.;
    V[k].c = (float)cos(a);
    V[k].s = (float)sin(a);
  }
}

static inline void mc_setup_pixels(const monte_mc_geom* g, mc_pixel* U, mc_pixel* W) {
  for (int i = 0; i < g->nu; i++) {
    double yl = g->half_u - g->du * (i + 0.5);
    double phia = atan(yl / g->sdd);
    memset(&U[i], 0, sizeof(mc_pixel));
    U[i].a = (float)yl;
    U[i].sin_a = (float)sin(phia);
    U[i].cos_a = (float)cos(phia);
  }
  for (int j = 0; j < g->nv; j++) {
    double zl = g->half_v - g->dv * (j + 0.5);
    double th = 0.5 * M_PI - atan(zl / g->sdd);
    memset(&W[j], 0, sizeof(mc_pixel));
    W[j].b = (float)zl;
    W[j].sin_t = (float)sin(th);
    W[j].cos_t = (float)cos(th);
  }
}

#endif /* MONTE_MC_SETUP_H */
