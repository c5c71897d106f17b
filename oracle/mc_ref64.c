/*
 * mc_ref64.c -- an independent FP64 restatement of the reference's photon
 * transport for the CBCT Monte Carlo.  TEST INFRASTRUCTURE: only the tests
 * use it; the product never links or calls it.
 *
 * Unlike mc_oracle.c (which replays the GPU kernels' own step functions
 * and Philox streams bit for bit), this file shares no code with the
 * product: it is written from monte_cu/CBCT_real325im.cu in double
 * arithmetic, with its own random streams (xoshiro256** seeded by
 * splitmix64 per history), its own inverse-CDF spectrum sampling and its
 * own Woodcock loop.  The GPU tallies must agree with its tallies in
 * distribution (per-pixel chi-square), which pins the physics the replay
 * harness cannot: the source aim, delta tracking, the interaction
 * selection, Kahn's Klein-Nishina sampler, the direction rotation and the
 * detector tally.
 *
 * Model (the reference's `projection` kernel, :425-860, with the
 * deviations the product documents):
 *   - a history aims at the centre of its pixel: polar angle
 *     pi/2 - atan(zl / Dsd), azimuth atan(yl / Dsd) + view angle
 *     (:476-503), and starts on the line from the rotated source through
 *     the pixel centre at fraction (Dso - start_plane) / Dsd (:506-540);
 *   - in air nothing interacts, so the photon streams to the phantom box
 *     and a photon leaving the box is done (the reference keeps sampling
 *     Woodcock steps through air until |x|, |y| >= 62 or |z| >= 17, :929);
 *   - delta tracking at the majorant mu_max(E) = max over the labels of
 *     total(E) * density (photon::delta_sampling, :862-976), a real
 *     collision with probability mu(label) / mu_max;
 *   - at a real collision (up to max_interactions of them, :599): a uniform
 *     u selects photoelectric (u <= photo / total: absorbed), Rayleigh
 *     (u <= (photo + coh) / total: direction kept) or Compton (:649-660),
 *     the mass coefficients of the site's material at bin (int)(E + 0.5);
 *   - Compton: Kahn's rejection sampling of lambda' (:701-736),
 *     cos(theta) = 1 - (lambda' - lambda) clamped at -1, E' = 511 /
 *     lambda', phi = 2 pi u, and the rotation of (:768-781) with the
 *     reference's stale sin(phi) of the emission direction from the
 *     second Compton on (MONTE_MC_STALE_SIN_PHI) and the CPU program's
 *     first turn about +z (MONTE_MC_FIRST_COMPTON_Z,
 *     monte_cpp/CBCT_real2.cpp:193,460-463);
 *   - an escaping photon is tallied where its line meets the detector plane
 *     x' = Dod of its view (:567-585, :672-692, :823-841): primary with no
 *     interaction, scatter otherwise (none after a Rayleigh event with
 *     MONTE_MC_NO_RAYLEIGH_TALLY), out-of-detector hits dropped.
 *
 * Build: oracle/Makefile.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/monte.h"

#define R64_NBINS 201
#define R64_MAX_LABELS 256

typedef struct {
  uint64_t s[4];
} r64_rng;

static uint64_t r64_splitmix(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t r64_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* xoshiro256** (Blackman and Vigna, 2018) */
static uint64_t r64_next(r64_rng* r) {
  const uint64_t out = r64_rotl(r->s[1] * 5, 7) * 9;
  const uint64_t t = r->s[1] << 17;
  r->s[2] ^= r->s[0];
  r->s[3] ^= r->s[1];
  r->s[1] ^= r->s[2];
  r->s[0] ^= r->s[3];
  r->s[2] ^= t;
  r->s[3] = r64_rotl(r->s[3], 45);
  return out;
}

/* uniform in (0, 1], 53 bits (curand_uniform's range) */
static double r64_u(r64_rng* r) { return ((double)(r64_next(r) >> 11) + 1.0) * 0x1.0p-53; }

static void r64_seed(r64_rng* r, uint64_t seed, uint64_t history) {
  uint64_t x = seed ^ (history * 0xD1342543DE82EF95ull);
  for (int i = 0; i < 4; i++) r->s[i] = r64_splitmix(&x);
}

typedef struct {
  const monte_mc_geom* g;
  const monte_mc_phantom* ph;
  const monte_xcom* x;
  double mu[R64_MAX_LABELS][R64_NBINS];   /* 1/cm */
  double mu_max[R64_NBINS];
  double cdf[512];
  int n_lines;
  const double* energies;
} r64_run;

static int r64_bin(double E) {
  int k = (int)(E + 0.5);
  return k < 1 ? 1 : (k > R64_NBINS - 1 ? R64_NBINS - 1 : k);
}

/* label at (x, y, z), or -1 outside the phantom box */
static int r64_label(const r64_run* R, double x, double y, double z) {
  const monte_mc_phantom* ph = R->ph;
  const double fx = (x - ph->x0) / ph->dx, fy = (y - ph->y0) / ph->dy, fz = (z - ph->z0) / ph->dz;
  if (!(fx >= 0 && fx < ph->nx && fy >= 0 && fy < ph->ny && fz >= 0 && fz < ph->nz)) return -1;
  if (ph->clip_radius > 0 &&
      (x * x + y * y > ph->clip_radius * ph->clip_radius || fabs(z) > ph->clip_half_z))
    return 0;
  return ph->labels[((size_t)(int)fz * ph->ny + (size_t)(int)fy) * ph->nx + (size_t)(int)fx];
}

/* entry distance of the ray into the phantom box, -1 if it misses */
static double r64_box_entry(const r64_run* R, const double o[3], const double d[3]) {
  const monte_mc_phantom* ph = R->ph;
  const double lo_b[3] = {ph->x0, ph->y0, ph->z0};
  const double hi_b[3] = {ph->x0 + ph->nx * ph->dx, ph->y0 + ph->ny * ph->dy,
                          ph->z0 + ph->nz * ph->dz};
  double lo = 0.0, hi = 1e300;
  for (int i = 0; i < 3; i++) {
    if (d[i] == 0.0) {
      if (o[i] < lo_b[i] || o[i] >= hi_b[i]) return -1.0;
    } else {
      double a = (lo_b[i] - o[i]) / d[i], b = (hi_b[i] - o[i]) / d[i];
      if (a > b) { double t = a; a = b; b = t; }
      if (a > lo) lo = a;
      if (b < hi) hi = b;
    }
  }
  return lo < hi ? lo : -1.0;
}

/* detector cell [view][u][v] hit by the line (p, d) in view k, or -1 */
static long long r64_detector(const r64_run* R, int k, const double p[3], const double d[3]) {
  const monte_mc_geom* g = R->g;
  const double a = M_PI * ((double)k * 360.0 / g->n_views) / 180.0;
  const double c = cos(a), s = sin(a);
  const double xr = p[0] * c + p[1] * s, yr = p[1] * c - p[0] * s;
  const double dxr = d[0] * c + d[1] * s, dyr = d[1] * c - d[0] * s;
  if (!(dxr > 0)) return -1;
  const double t = ((g->sdd - g->sod) - xr) / dxr;
  if (t < 0) return -1;
  const double fu = (g->half_u - (yr + t * dyr)) / g->du;
  const double fv = (g->half_v - (p[2] + t * d[2])) / g->dv;
  if (!(fu >= 0 && fu < g->nu && fv >= 0 && fv < g->nv)) return -1;
  return ((long long)k * g->nu + (int)fu) * g->nv + (int)fv;
}

typedef struct {
  uint64_t histories, steps, interactions, primary, scatter, rayleigh, compton, photo;
} r64_stats;

static void r64_history(const r64_run* R, int k, int iu, int iv, uint64_t seed, uint64_t hid,
                        int64_t* prim, int64_t* scat, r64_stats* st) {
  const monte_mc_geom* g = R->g;
  r64_rng rng;
  r64_seed(&rng, seed, hid);
  st->histories++;
  /* energy: inverse CDF over the lines */
  double E = R->energies[0];
  if (R->n_lines > 1) {
    const double u = r64_u(&rng);
    int i = 0;
    while (i < R->n_lines - 1 && u > R->cdf[i]) i++;
    E = R->energies[i];
  }
  const double va = M_PI * ((double)k * 360.0 / g->n_views) / 180.0;
  const double c = cos(va), s = sin(va);
  const double yl = g->half_u - g->du * (iu + 0.5), zl = g->half_v - g->dv * (iv + 0.5);
  const double th = 0.5 * M_PI - atan(zl / g->sdd), ph = atan(yl / g->sdd) + va;
  double st_ = sin(th), ct = cos(th), sp = sin(ph), cp = cos(ph);
  const double sp_aim = sp;
  const double dod = g->sdd - g->sod, to = (g->sod - g->start_plane) / g->sdd;
  const double sx = -g->sod * c, sy = -g->sod * s;
  double p[3] = {sx + (dod * c - yl * s - sx) * to, sy + (dod * s + yl * c - sy) * to, zl * to};
  double d[3] = {st_ * cp, st_ * sp, ct};
  const double t0 = r64_box_entry(R, p, d);
  int n_int = 0, n_compton = 0, last = 0, label = 0;
  if (t0 >= 0) {
    for (int i = 0; i < 3; i++) p[i] += t0 * d[i];
    for (;;) {
      /* one flight: delta tracking until a real collision or the box exit */
      int escaped = 0;
      for (;;) {
        const int kb = r64_bin(E);
        const double r = -log(r64_u(&rng)) / R->mu_max[kb];
        for (int i = 0; i < 3; i++) p[i] += r * d[i];
        const double nu = r64_u(&rng);
        st->steps++;
        const int lab = r64_label(R, p[0], p[1], p[2]);
        if (lab < 0) { escaped = 1; break; }
        if (nu <= R->mu[lab][kb] / R->mu_max[kb]) { label = lab; break; }
      }
      if (escaped) break;
      if (n_int >= g->max_interactions) return;  /* the last allowed interaction was used */
      const int mat = R->ph->label_material[label];
      const int kb = r64_bin(E);
      const double tot = R->x->total[mat * R64_NBINS + kb];
      const double pe = R->x->photoelectric[mat * R64_NBINS + kb];
      const double coh = R->x->coherent[mat * R64_NBINS + kb];
      const double u = r64_u(&rng);
      n_int++;
      st->interactions++;
      if (u <= pe / tot) { st->photo++; return; }
      if (u <= (pe + coh) / tot) { st->rayleigh++; last = 1; continue; }
      st->compton++;
      last = 2;
      /* Kahn's sampler of lambda' = rho lambda */
      const double lam = 511.0 / E;
      double rho = 1.0;
      for (;;) {
        if (r64_u(&rng) < (lam + 2.0) / (9.0 * lam + 2.0)) {
          rho = 1.0 + (2.0 / lam) * r64_u(&rng);
          if (r64_u(&rng) <= 4.0 * (1.0 / rho - 1.0 / (rho * rho))) break;
        } else {
          rho = (lam + 2.0) / (lam + 2.0 * (1.0 - r64_u(&rng)));
          const double q = lam - rho * lam + 1.0;
          if (r64_u(&rng) <= 0.5 * (q * q + 1.0 / rho)) break;
        }
      }
      double cth = 1.0 - (rho * lam - lam);
      if (cth < -1.0) cth = -1.0;
      const double sth = sqrt(1.0 - cth * cth);
      E = 511.0 / (rho * lam);
      const double phi = 2.0 * M_PI * r64_u(&rng);
      double ist = st_, ict = ct, isp = sp, icp = cp;
      if ((g->flags & MONTE_MC_FIRST_COMPTON_Z) && n_compton == 0) {
        ist = 0.0; ict = 1.0; isp = 1.0; icp = 0.0;
      } else if ((g->flags & MONTE_MC_STALE_SIN_PHI) && n_compton > 0) {
        isp = sp_aim;
      }
      double cn = ict * cth - ist * sth * cos(phi);
      if (cn < -1.0) cn = -1.0;
      if (cn > 1.0) return;
      const double sn = sqrt(1.0 - cn * cn);
      if (sn == 0.0) return;
      cp = (ict * icp * sth * cos(phi) + ist * icp * cth - isp * sth * sin(phi)) / sn;
      sp = (ict * isp * sth * cos(phi) + ist * isp * cth + icp * sth * sin(phi)) / sn;
      st_ = sn;
      ct = cn;
      d[0] = st_ * cp;
      d[1] = st_ * sp;
      d[2] = ct;
      n_compton++;
    }
  }
  if (n_int > 0 && last == 1 && (g->flags & MONTE_MC_NO_RAYLEIGH_TALLY)) return;
  const long long cell = r64_detector(R, k, p, d);
  if (cell < 0) return;
  if (n_int == 0) {
#pragma omp atomic
    prim[cell] += 1;
    st->primary++;
  } else {
#pragma omp atomic
    scat[cell] += 1;
    st->scatter++;
  }
}

/* histories_per_pixel histories at every pixel of views [view_begin,
 * view_end); history (view, u, v, k) seeds its stream with id
 * ((view * nu + u) * nv + v) * per + k.  stats_out: histories, steps,
 * interactions, primary, scatter, rayleigh, compton, photo. */
int oracle_mc_ref64(const monte_mc_geom* g, const monte_mc_phantom* ph, const monte_xcom* x,
                    const monte_spectrum* sp, uint64_t seed, uint64_t per, int view_begin,
                    int view_end, int64_t* prim, int64_t* scat, uint64_t* stats_out) {
  if (!g || !ph || !x || !sp || sp->n_lines < 1 || sp->n_lines > 512 || ph->n_labels < 1 ||
      ph->n_labels > R64_MAX_LABELS || view_begin < 0 || view_end > g->n_views)
    return MONTE_EINVAL;
  r64_run* R = (r64_run*)calloc(1, sizeof(r64_run));
  R->g = g;
  R->ph = ph;
  R->x = x;
  for (int k = 0; k < R64_NBINS; k++) {
    double m = 0.0;
    for (int l = 0; l < ph->n_labels; l++) {
      const int mat = ph->label_material[l];
      R->mu[l][k] = mat < 0 ? 0.0 : (double)x->total[mat * R64_NBINS + k] * ph->label_density[l];
      if (R->mu[l][k] > m) m = R->mu[l][k];
    }
    R->mu_max[k] = m > 0 ? m : 1e-6;
  }
  double wsum = 0.0, acc = 0.0;
  for (int i = 0; i < sp->n_lines; i++) wsum += sp->weight[i];
  for (int i = 0; i < sp->n_lines; i++) {
    acc += sp->weight[i];
    R->cdf[i] = acc / wsum;
  }
  R->n_lines = sp->n_lines;
  R->energies = sp->energy_kev;
  r64_stats tot;
  memset(&tot, 0, sizeof(tot));
  const int npix = g->nu * g->nv;
  for (int k = view_begin; k < view_end; k++) {
#pragma omp parallel
    {
      r64_stats st;
      memset(&st, 0, sizeof(st));
#pragma omp for schedule(dynamic, 16)
      for (int pix = 0; pix < npix; pix++) {
        const int iu = pix / g->nv, iv = pix % g->nv;
        for (uint64_t h = 0; h < per; h++)
          r64_history(R, k, iu, iv, seed,
                      (((uint64_t)k * g->nu + iu) * g->nv + iv) * per + h, prim, scat, &st);
      }
#pragma omp critical
      {
        tot.histories += st.histories;
        tot.steps += st.steps;
        tot.interactions += st.interactions;
        tot.primary += st.primary;
        tot.scatter += st.scatter;
        tot.rayleigh += st.rayleigh;
        tot.compton += st.compton;
        tot.photo += st.photo;
      }
    }
  }
  if (stats_out) {
    const uint64_t v[8] = {tot.histories, tot.steps, tot.interactions, tot.primary,
                           tot.scatter, tot.rayleigh, tot.compton, tot.photo};
    memcpy(stats_out, v, sizeof(v));
  }
  free(R);
  return MONTE_OK;
}
