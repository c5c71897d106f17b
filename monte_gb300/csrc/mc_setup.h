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
#include <stdlib.h>
#include <string.h>

#include "../../include/monte.h"
#include "mc_physics.h"

/* Macro-cell grid of the local majorants: cells of 2^mshift voxels per
 * axis, the smallest power of two >= 2 that leaves at most 96 cells along
 * the longest axis (a leg then spans ~1% of the phantom; on the 325^3
 * workload 4-voxel cells measured 12 % faster than 8-voxel ones, 16-voxel
 * ones 2x slower).  `leg` is 2^mshift times the smallest voxel edge,
 * rounded down. */
static inline void mc_macro_dims(const monte_mc_phantom* ph, mc_params* P) {
  int n = ph->nx > ph->ny ? ph->nx : ph->ny;
  if (ph->nz > n) n = ph->nz;
  int sh = 1;
  while (sh < 20 && ((n + (1 << sh) - 1) >> sh) > 96) sh++;
  P->mshift = sh;
  P->mgx = (ph->nx + (1 << sh) - 1) >> sh;
  P->mgy = (ph->ny + (1 << sh) - 1) >> sh;
  P->mgz = (ph->nz + (1 << sh) - 1) >> sh;
  double d = ph->dx < ph->dy ? ph->dx : ph->dy;
  if (ph->dz < d) d = ph->dz;
  P->leg = (float)(ldexp(d, sh) * (1.0 - 1e-6));
}

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
  if (g->flags & ~(unsigned)(MONTE_MC_STALE_SIN_PHI | MONTE_MC_FIRST_COMPTON_Z |
                             MONTE_MC_NO_RAYLEIGH_TALLY | MONTE_MC_LOCAL_MAJORANT)) {
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
  mc_macro_dims(ph, P);
  return MONTE_OK;
}

/* Spectrum lines -> energies and Walker's alias table (Vose's
 * construction in double): n slots of probability 1/n each; slot i keeps
 * line i with probability alias_p[i] and gives line alias_i[i] otherwise.
 * Lines of zero weight are never drawn. */
static inline int mc_setup_spectrum(const monte_spectrum* sp, mc_tables* T, const char** why) {
  *why = "";
  if (!sp || sp->n_lines <= 0 || sp->n_lines > MC_MAX_LINES || !sp->energy_kev || !sp->weight) {
    *why = "bad spectrum (1..512 lines)";
    return MONTE_EINVAL;
  }
  const int n = sp->n_lines;
  double wsum = 0.0;
  for (int i = 0; i < n; i++) {
    if (!(sp->weight[i] >= 0) || !(sp->energy_kev[i] > 0 && sp->energy_kev[i] <= 200)) {
      *why = "spectrum lines need weight >= 0 and 0 < E <= 200 keV";
      return MONTE_EINVAL;
    }
    wsum += sp->weight[i];
  }
  if (!(wsum > 0)) { *why = "spectrum weights sum to zero"; return MONTE_EINVAL; }
  double q[MC_MAX_LINES];
  int small[MC_MAX_LINES], large[MC_MAX_LINES];
  int ns = 0, nl = 0;
  for (int i = 0; i < n; i++) {
    T->energy[i] = (float)sp->energy_kev[i];
    q[i] = sp->weight[i] / wsum * n;
    T->alias_i[i] = (int16_t)i;
    if (q[i] < 1.0) small[ns++] = i; else large[nl++] = i;
  }
  while (ns > 0 && nl > 0) {
    const int s = small[--ns], l = large[nl - 1];
    T->alias_p[s] = (float)q[s];
    T->alias_i[s] = (int16_t)l;
    q[l] = (q[l] + q[s]) - 1.0;
    if (q[l] < 1.0) {
      nl--;
      small[ns++] = l;
    }
  }
  /* what is left is 1 up to rounding: keep the slot's own line */
  while (nl > 0) T->alias_p[large[--nl]] = 1.0f;
  while (ns > 0) {
    const int s = small[--ns];
    T->alias_p[s] = q[s] > 0.0 ? 1.0f : 0.0f;
    if (q[s] <= 0.0) {  /* a zero-weight slot left over: give it the heaviest line */
      int best = 0;
      for (int i = 1; i < n; i++) if (sp->weight[i] > sp->weight[best]) best = i;
      T->alias_i[s] = (int16_t)best;
    }
  }
  T->n_lines = n;
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
  return mc_setup_spectrum(sp, T, why);
}

/* Labels present in each macro cell, as 256-bit sets (4 words per cell,
 * cell (cx, cy, cz) at ((cz mgy + cy) mgx + cx) * 4), from host labels.
 * The library computes the same sets on the GPU for device labels. */
static inline void mc_macro_bits_host(const monte_mc_phantom* ph, const uint8_t* labels,
                                      const mc_params* P, uint64_t* bits) {
  memset(bits, 0, (size_t)P->mgx * P->mgy * P->mgz * 4 * sizeof(uint64_t));
  for (int z = 0; z < ph->nz; z++)
    for (int y = 0; y < ph->ny; y++)
      for (int x = 0; x < ph->nx; x++) {
        const int l = labels[((size_t)z * ph->ny + y) * ph->nx + x];
        const size_t c = (((size_t)(z >> P->mshift) * P->mgy + (size_t)(y >> P->mshift)) *
                              P->mgx + (size_t)(x >> P->mshift));
        bits[c * 4 + (l >> 6)] |= 1ull << (l & 63);
      }
}

typedef struct {
  float curve[MC_NBINS];
  int id;
} mc_class_curve;

static int mc_cmp_curve(const void* a, const void* b) {
  return memcmp(((const mc_class_curve*)a)->curve, ((const mc_class_curve*)b)->curve,
                sizeof(float) * MC_NBINS);
}

static int mc_cmp_curve_level(const void* a, const void* b) {
  /* order by the mean majorant */
  double sa = 0, sb = 0;
  for (int k = 0; k < MC_NBINS; k++) {
    sa += ((const mc_class_curve*)a)->curve[k];
    sb += ((const mc_class_curve*)b)->curve[k];
  }
  return sa < sb ? -1 : (sa > sb ? 1 : 0);
}

/* Attenuation per label and bin for the local majorants: the same float
 * products as mc_setup_tables' Woodcock tables (tables checked there). */
static inline void mc_setup_local(const monte_mc_phantom* ph, const monte_xcom* x,
                                  mc_local_tables* L) {
  memset(L, 0, sizeof(*L));
  for (int l = 0; l < ph->n_labels; l++) {
    const int m = ph->label_material[l];
    for (int k = 0; k < MC_NBINS; k++)
      L->mu[l][k] = m < 0 ? 0.0f : x->total[m * MC_NBINS + k] * (float)ph->label_density[l];
  }
}

/* Majorant classes and leg lengths (MC_F_LOCAL_MAJORANT).
 *
 * Class: each cell stands for itself and its 26 neighbours; its majorant
 * curve is, bin by bin, the largest mu of any label present there (L->mu,
 * filled by mc_setup_local).  Cells with the same curve share a class;
 * beyond MC_MAX_CLASSES classes, classes of neighbouring levels are merged
 * (bin-wise maxima: still majorants).
 *
 * Leg: the class's curve also bounds mu over the cells within Chebyshev
 * distance R of the cell, for the largest R <= MC_MAX_LEG_CELLS such that
 * no label above the curve lies there (found with one prefix-sum grid per
 * class of "holds a label the class does not bound"); a photon in the cell
 * may then move R legs of P->leg cm under that majorant.  Far from bone a
 * leg reaches across many cells.
 *
 * Fills L->maj and cls[cell] = class | R << 8.  Returns MONTE_OK, or
 * MONTE_ENOMEM. */
#define MC_MAX_LEG_CELLS 32
static inline int mc_macro_classes(const mc_params* P, mc_local_tables* L, const uint64_t* bits,
                                   uint16_t* cls) {
  const int gx = P->mgx, gy = P->mgy, gz = P->mgz;
  const size_t nc = (size_t)gx * gy * gz;
  /* distinct dilated label sets, found by open addressing on their four
   * words (set ids in order of first appearance), each with its curve */
  size_t cap = 64;
  while (cap < 2 * nc) cap <<= 1;
  size_t ucap = 64, nsets = 0;
  int32_t* table = (int32_t*)malloc(sizeof(int32_t) * cap);
  uint64_t* uniq = (uint64_t*)malloc(ucap * 4 * sizeof(uint64_t));
  mc_class_curve* cur = (mc_class_curve*)malloc(sizeof(mc_class_curve) * ucap);
  int* set_class = (int*)malloc(sizeof(int) * nc);
  int* set_to_class = (int*)malloc(sizeof(int) * (nc + 1));
  int* remap = (int*)malloc(sizeof(int) * (nc + 1));
  const size_t np = (size_t)(gx + 1) * (gy + 1) * (gz + 1);
  int32_t* pre = (int32_t*)malloc(sizeof(int32_t) * np);
  int oom = !table || !uniq || !cur || !set_class || !set_to_class || !remap || !pre;
  if (!oom) memset(table, 0xff, sizeof(int32_t) * cap);
  for (int z = 0; z < gz && !oom; z++)
    for (int y = 0; y < gy && !oom; y++)
      for (int x = 0; x < gx && !oom; x++) {
        uint64_t w[4] = {0, 0, 0, 0};
        for (int a = z > 0 ? z - 1 : 0; a <= (z + 1 < gz ? z + 1 : z); a++)
          for (int b = y > 0 ? y - 1 : 0; b <= (y + 1 < gy ? y + 1 : y); b++)
            for (int c = x > 0 ? x - 1 : 0; c <= (x + 1 < gx ? x + 1 : x); c++) {
              const uint64_t* q = bits + (((size_t)a * gy + b) * gx + c) * 4;
              for (int i = 0; i < 4; i++) w[i] |= q[i];
            }
        uint64_t h = (w[0] * 0x9E3779B97F4A7C15ull) ^ (w[1] * 0xC2B2AE3D27D4EB4Full) ^
                     (w[2] * 0x165667B19E3779F9ull) ^ (w[3] * 0xD6E8FEB86659FD93ull);
        h ^= h >> 29;
        size_t e = (size_t)h & (cap - 1);
        while (table[e] >= 0 && memcmp(uniq + (size_t)table[e] * 4, w, sizeof(w)) != 0)
          e = (e + 1) & (cap - 1);
        if (table[e] < 0) {
          if (nsets == ucap) {
            ucap *= 2;
            uint64_t* u2 = (uint64_t*)realloc(uniq, ucap * 4 * sizeof(uint64_t));
            mc_class_curve* c2 = (mc_class_curve*)realloc(cur, sizeof(mc_class_curve) * ucap);
            if (u2) uniq = u2;
            if (c2) cur = c2;
            if (!u2 || !c2) {
              oom = 1;
              break;
            }
          }
          memcpy(uniq + nsets * 4, w, sizeof(w));
          mc_class_curve* c = &cur[nsets];
          for (int k = 0; k < MC_NBINS; k++) c->curve[k] = 0.0f;
          for (int l = 0; l < MC_MAX_LABELS; l++)
            if (w[l >> 6] >> (l & 63) & 1)
              for (int k = 0; k < MC_NBINS; k++)
                if (L->mu[l][k] > c->curve[k]) c->curve[k] = L->mu[l][k];
          c->id = (int)nsets;
          table[e] = (int32_t)nsets++;
        }
        set_class[((size_t)z * gy + y) * gx + x] = table[e];  /* per cell: its set, for now */
      }
  free(table);
  free(uniq);
  if (oom) {
    free(cur);
    free(set_class);
    free(set_to_class);
    free(remap);
    free(pre);
    return MONTE_ENOMEM;
  }
  /* sets with equal curves -> one class */
  qsort(cur, nsets, sizeof(mc_class_curve), mc_cmp_curve);
  int ncls = 0;
  for (size_t i = 0; i < nsets; i++) {
    if (i == 0 || mc_cmp_curve(&cur[i], &cur[i - 1]) != 0) {
      if (ncls != (int)i) cur[ncls] = cur[i];
      ncls++;
    }
    set_to_class[cur[i].id] = ncls - 1;
    cur[ncls - 1].id = ncls - 1;
  }
  /* too many: merge runs of classes ordered by level */
  for (int c = 0; c < ncls; c++) remap[c] = c;
  if (ncls > MC_MAX_CLASSES) {
    qsort(cur, ncls, sizeof(mc_class_curve), mc_cmp_curve_level);
    mc_class_curve* merged = (mc_class_curve*)malloc(sizeof(mc_class_curve) * MC_MAX_CLASSES);
    if (!merged) {
      free(cur);
      free(set_class);
      free(set_to_class);
      free(remap);
      free(pre);
      return MONTE_ENOMEM;
    }
    for (int g = 0; g < MC_MAX_CLASSES; g++) {
      const int lo = (int)((long long)g * ncls / MC_MAX_CLASSES);
      const int hi = (int)((long long)(g + 1) * ncls / MC_MAX_CLASSES);
      for (int k = 0; k < MC_NBINS; k++) merged[g].curve[k] = 0.0f;
      for (int c = lo; c < hi; c++) {
        remap[cur[c].id] = g;
        for (int k = 0; k < MC_NBINS; k++)
          if (cur[c].curve[k] > merged[g].curve[k]) merged[g].curve[k] = cur[c].curve[k];
      }
    }
    for (int g = 0; g < MC_MAX_CLASSES; g++) cur[g] = merged[g];
    free(merged);
    ncls = MC_MAX_CLASSES;
  }
  for (int c = 0; c < MC_MAX_CLASSES; c++)
    for (int k = 0; k < MC_NBINS; k++) {
      const float m = c < ncls ? cur[c].curve[k] : 0.0f;
      L->maj[c][k].maj = m;
      L->maj[c][k].inv = m > 0.0f ? 1.0f / m : 3.0e38f;
    }
  for (size_t i = 0; i < nc; i++) cls[i] = (uint16_t)remap[set_to_class[set_class[i]]];
  /* leg lengths: pre = prefix sums over the grid of "the cell holds a
   * label above the class's curve", one grid per distinct set of such
   * labels (classes that share it share the grid) */
  uint64_t bad[MC_MAX_CLASSES][4];
  int present[MC_MAX_CLASSES];
  for (int c = 0; c < ncls; c++) {
    present[c] = 0;
    for (int i = 0; i < 4; i++) bad[c][i] = 0;
    for (int l = 0; l < MC_MAX_LABELS; l++)
      for (int k = 0; k < MC_NBINS; k++)
        if (L->mu[l][k] > cur[c].curve[k]) {
          bad[c][l >> 6] |= 1ull << (l & 63);
          break;
        }
  }
  for (size_t i = 0; i < nc; i++) present[cls[i] & 0xff] = 1;
  for (int c = 0; c < ncls; c++) {
    if (!present[c]) continue;
    uint64_t group = 0;  /* present classes with c's set, c first */
    for (int c2 = c; c2 < ncls; c2++)
      if (present[c2] && memcmp(bad[c2], bad[c], sizeof(bad[c])) == 0) {
        group |= 1ull << c2;
        if (c2 != c) present[c2] = 0;
      }
    const uint64_t* bd = bad[c];
#define MC_PRE(x, y, z) pre[((size_t)(z) * (gy + 1) + (size_t)(y)) * (gx + 1) + (size_t)(x)]
    for (int z = 0; z <= gz; z++)
      for (int y = 0; y <= gy; y++)
        for (int x = 0; x <= gx; x++) {
          if (!x || !y || !z) {
            MC_PRE(x, y, z) = 0;
            continue;
          }
          const uint64_t* q = bits + (((size_t)(z - 1) * gy + (y - 1)) * gx + (x - 1)) * 4;
          const int32_t v = ((q[0] & bd[0]) | (q[1] & bd[1]) | (q[2] & bd[2]) | (q[3] & bd[3])) != 0;
          MC_PRE(x, y, z) = v + MC_PRE(x - 1, y, z) + MC_PRE(x, y - 1, z) + MC_PRE(x, y, z - 1) -
                            MC_PRE(x - 1, y - 1, z) - MC_PRE(x - 1, y, z - 1) -
                            MC_PRE(x, y - 1, z - 1) + MC_PRE(x - 1, y - 1, z - 1);
        }
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++) {
          const size_t i = ((size_t)z * gy + y) * gx + x;
          const int ci = cls[i] & 0xff;
          if (!(group >> ci & 1)) continue;
          /* the box of radius 1 is clean by construction and cleanness only
           * shrinks with the radius: bisect for the largest clean one */
          int r = 1, hi = MC_MAX_LEG_CELLS;
          while (r < hi) {
            const int q = (r + hi + 1) >> 1;
            const int x0 = x - q > 0 ? x - q : 0, x1 = x + q + 1 < gx ? x + q + 1 : gx;
            const int y0 = y - q > 0 ? y - q : 0, y1 = y + q + 1 < gy ? y + q + 1 : gy;
            const int z0 = z - q > 0 ? z - q : 0, z1 = z + q + 1 < gz ? z + q + 1 : gz;
            const int32_t n = MC_PRE(x1, y1, z1) - MC_PRE(x0, y1, z1) - MC_PRE(x1, y0, z1) -
                              MC_PRE(x1, y1, z0) + MC_PRE(x0, y0, z1) + MC_PRE(x0, y1, z0) +
                              MC_PRE(x1, y0, z0) - MC_PRE(x0, y0, z0);
            if (n) hi = q - 1; else r = q;
          }
          cls[i] = (uint16_t)(ci | (r << 8));
        }
#undef MC_PRE
  }
  free(remap);
  free(set_to_class);
  free(cur);
  free(set_class);
  free(pre);
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
