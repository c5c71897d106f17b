/*
 * mc_physics.h -- one photon history of the CBCT Monte Carlo, as step
 * functions shared by the CUDA kernels (mc_kernels.cu) and the CPU replay
 * harness.  Plain C, float arithmetic in a fixed order, every fused
 * multiply-add explicit, so host and device produce identical histories.
 *
 * Reference: monte_cu/CBCT_real325im.cu (voxel phantom) and
 * monte_cu/CBCT_real325.cu (analytic phantom), kernel `projection`
 * (:425-860) and photon::delta_sampling (:862-976); CPU variant
 * monte_cpp/CBCT_real2.cpp:145-595,733-815.
 *
 * State of a photon (photon class, CBCT_real325im.cu:47-58): position,
 * energy, and the direction as the reference carries it -- polar and
 * azimuthal sines/cosines (sin_theta_a, cos_theta_a, sin_phi_a,
 * cos_phi_a), the Cartesian step being (s_t c_p, s_t s_p, c_t).
 */
#ifndef MONTE_MC_PHYSICS_H
#define MONTE_MC_PHYSICS_H

#include "monte_rng.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MC_NBINS 201         /* XCOM rows, index = keV (CBCT_real2.cpp:633-668) */
#define MC_MAX_LABELS 256
#define MC_MAX_LINES 512
#define MC_MAX_STEPS (1 << 22)   /* Woodcock steps per flight before a history is dropped */
#define MC_MAX_KN_TRIES 4096     /* Kahn rejection attempts before a history is dropped */
#define MC_MAX_CLASSES 64        /* majorant classes of the macro-cell grid */

/* physics switches (public values in include/monte.h) */
#define MC_F_STALE_SIN_PHI 0x1u    /* 2nd+ Compton keeps the emission sin_phi_a (CBCT_real325im.cu:768-773) */
#define MC_F_FIRST_COMPTON_Z 0x2u  /* 1st Compton turns about +z (CBCT_real2.cpp:193,460-463) */
#define MC_F_NO_RAYLEIGH_TALLY 0x4u /* flights after a Rayleigh event are not tallied (CBCT_real2.cpp:373-397) */
#define MC_F_LOCAL_MAJORANT 0x8u   /* majorants per macro cell (mc_flight_leg) */

/* Majorant of a macro-cell class at one energy bin, and its reciprocal. */
typedef struct {
  float maj, inv;
} mc_majorant;

/* Tables of one run, built on the host. */
typedef struct {
  /* Woodcock: per label and keV bin, mu_label / mu_max (float division,
   * exactly the reference's `mu_H2O/mu_max`, CBCT_real325im.cu:941) */
  float ratio[MC_MAX_LABELS][MC_NBINS];
  float inv_mu_max[MC_NBINS];     /* 1/max over present labels of mu (1/cm) */
  /* interaction selection per material and bin (CBCT_real325im.cu:651-656):
   * photo if u <= p_photo, Rayleigh if u <= p_photo_coh, else Compton */
  float p_photo[8][MC_NBINS];
  float p_photo_coh[8][MC_NBINS];
  int8_t label_material[MC_MAX_LABELS];  /* -1: air */
  /* spectrum: Walker's alias table over the lines (slot i keeps line i
   * with probability alias_p[i], else gives line alias_i[i]) */
  float alias_p[MC_MAX_LINES];
  int16_t alias_i[MC_MAX_LINES];
  float energy[MC_MAX_LINES];
  int n_lines;
  int pad_;
} mc_tables;

/* Tables of the local majorants (MC_F_LOCAL_MAJORANT), built on the host:
 * attenuation per label and bin (1/cm, table * density), and per
 * macro-cell class the largest mu over the labels of the cells it stands
 * for ({0, 3e38} for air only). */
typedef struct {
  float mu[MC_MAX_LABELS][MC_NBINS];
  mc_majorant maj[MC_MAX_CLASSES][MC_NBINS];
} mc_local_tables;

/* Geometry and run parameters (float as the kernels use them). */
typedef struct {
  int n_views, nu, nv, max_int;
  unsigned flags;
  float du, dv, half_u, half_v, inv_du, inv_dv;
  float sod, sdd, dod, to;  /* to = (sod - start_plane) / sdd */
  int nx, ny, nz;
  float x0, y0, z0;          /* phantom low corner */
  float inv_dx, inv_dy, inv_dz;
  float clip_r2, clip_hz;    /* clip_r2 <= 0: no clip cylinder */
  uint64_t seed;
  monte_philox_keys keys;    /* round keys of seed (monte_philox_schedule) */
  uint32_t job;
  uint64_t per;              /* histories per pixel per view */
  /* macro-cell grid of the local majorants: cells of 2^mshift voxels per
   * axis, mgx x mgy x mgz of them; `leg` (cm) = 2^mshift times the
   * smallest voxel edge, the longest move from a point of a cell that
   * stays within the cell and its neighbours */
  int mgx, mgy, mgz, mshift;
  float leg;
  int view_begin, view_end, u_begin, u_end, v_begin, v_end;
} mc_params;

/* Per-view and per-pixel constants, computed on the host in double and
 * rounded to float (CBCT_real325im.cu:476-512). */
typedef struct {
  float c, s;  /* cos, sin of the view angle */
} mc_view;
typedef struct {
  float a, sin_a, cos_a; /* u pixel: yl, sin/cos(atan(yl/sdd)) */
  float b, sin_t, cos_t; /* v pixel: zl, sin/cos(pi/2 - atan(zl/sdd)) */
} mc_pixel;

enum { MC_FLY = 0, MC_COLLIDED = 1, MC_ESCAPED = 2, MC_DEAD = 3, MC_COMPTON = 4 };
enum { MC_EV_NONE = 0, MC_EV_RAYLEIGH = 1, MC_EV_COMPTON = 2, MC_EV_PHOTO = 3 };

typedef struct {
  float x, y, z;
  float st, ct, sp, cp;  /* direction: sin/cos theta, sin/cos phi */
  float sp_aim;          /* emission sin_phi_a (for MC_F_STALE_SIN_PHI) */
  float E;
  int kb;                /* energy bin (int)(E+0.5) */
  int label;             /* label at the last real collision */
  int n_int;             /* interactions done */
  int last;              /* kind of the last interaction: 0 none, 1 Rayleigh, 2 Compton,
                            3 photoelectric (MC_EV_*) */
  int n_compton;         /* Compton events so far */
  int view, iu, iv;
  int state;
  uint32_t steps;        /* Woodcock steps (and majorant legs) in the current flight */
  float tau;             /* optical depth left of the current exponential draw (local
                            majorants; 0: draw a new one) */
  monte_stream rng;
} mc_photon;

MONTE_HD int mc_bin(float E) {
  int k = (int)(E + 0.5f);
  return k < 1 ? 1 : (k > MC_NBINS - 1 ? MC_NBINS - 1 : k);
}

/* History id of (view, iu, iv, k): the stream address. */
MONTE_HD uint64_t mc_history_id(const mc_params* P, int view, int iu, int iv, uint64_t k) {
  return (((uint64_t)view * (uint64_t)P->nu + (uint64_t)iu) * (uint64_t)P->nv + (uint64_t)iv) *
             P->per + k;
}

/* Direction cosines of the step (CBCT_real325im.cu:892-894). */
MONTE_HD void mc_dir(const mc_photon* p, float* dx, float* dy, float* dz) {
  *dx = p->st * p->cp;
  *dy = p->st * p->sp;
  *dz = p->ct;
}

/* Entry/exit parameters of the ray o + t d through the phantom box in
 * voxel index space; returns 0 when the ray misses it. */
MONTE_HD int mc_box_span(const mc_params* P, float ox, float oy, float oz, float dx, float dy,
                         float dz, float* t0, float* t1) {
  float lo = 0.0f, hi = 3.0e38f;
  float o[3], d[3], n[3];
  o[0] = (ox - P->x0) * P->inv_dx;
  o[1] = (oy - P->y0) * P->inv_dy;
  o[2] = (oz - P->z0) * P->inv_dz;
  d[0] = dx * P->inv_dx;
  d[1] = dy * P->inv_dy;
  d[2] = dz * P->inv_dz;
  n[0] = (float)P->nx;
  n[1] = (float)P->ny;
  n[2] = (float)P->nz;
  for (int i = 0; i < 3; i++) {
    if (d[i] == 0.0f) {
      if (o[i] < 0.0f || o[i] >= n[i]) return 0;
    } else {
      float ta = (0.0f - o[i]) / d[i];
      float tb = (n[i] - o[i]) / d[i];
      float tn = ta < tb ? ta : tb, tf = ta < tb ? tb : ta;
      lo = tn > lo ? tn : lo;
      hi = tf < hi ? tf : hi;
    }
  }
  *t0 = lo;
  *t1 = hi;
  return lo < hi;
}

/* Source energy from a uniform u in (0, 1] by the alias table: slot
 * i = floor(n u), kept with probability alias_p[i] (the fraction n u - i
 * decides), else its alias -- the same distribution as the reference's
 * inverse-CDF search (CBCT_real325.cu:479-486) in constant time, with no
 * data-dependent loop. */
MONTE_HD float mc_sample_energy(const mc_tables* T, float u) {
  const float x = u * (float)T->n_lines;
  int i = (int)x;
  if (i >= T->n_lines) i = T->n_lines - 1;
  const float f = x - (float)i;
  return T->energy[f < T->alias_p[i] ? i : (int)T->alias_i[i]];
}

/* Start a history: energy, emission direction aimed at pixel (iu, iv) of
 * view `view`, position on the start plane, then straight to the phantom
 * box (air streaming is exact: nothing interacts in air).
 * CBCT_real325im.cu:466-540. */
MONTE_HD void mc_start(const mc_params* P, const mc_tables* T, const mc_view* V,
                       const mc_pixel* U, const mc_pixel* W, int view, int iu, int iv,
                       uint64_t k, mc_photon* p) {
  monte_stream_init(&p->rng, P->seed, mc_history_id(P, view, iu, iv, k), P->job);
  p->view = view;
  p->iu = iu;
  p->iv = iv;
  p->n_int = 0;
  p->last = 0;
  p->n_compton = 0;
  p->steps = 0;
  p->tau = 0.0f;
  p->label = 0;
  /* spectrum (CBCT_real325im.cu:491-498): one uniform per history */
  p->E = T->n_lines > 1 ? mc_sample_energy(T, monte_uniform_keys(&p->rng, &P->keys))
                        : T->energy[0];
  p->kb = mc_bin(p->E);
  const mc_view* v = &V[view];
  const mc_pixel* pu = &U[iu];
  const mc_pixel* pv = &W[iv];
  /* polar angle from the axial pixel offset, azimuth from the in-plane
   * offset plus the view angle (:485-512) */
  p->st = pv->sin_t;
  p->ct = pv->cos_t;
  p->cp = pu->cos_a * v->c - pu->sin_a * v->s;
  p->sp = pu->sin_a * v->c + pu->cos_a * v->s;
  p->sp_aim = p->sp;
  /* source rotated by the view angle, moved along the ray through the
   * pixel centre to the start plane (:516-540) */
  float sx = -P->sod * v->c, sy = -P->sod * v->s;
  float ax = P->dod * v->c - pu->a * v->s - sx;
  float ay = P->dod * v->s + pu->a * v->c - sy;
  float az = pv->b;
  p->x = fmaf(ax, P->to, sx);
  p->y = fmaf(ay, P->to, sy);
  p->z = az * P->to;
  float dx, dy, dz, t0, t1;
  mc_dir(p, &dx, &dy, &dz);
  if (mc_box_span(P, p->x, p->y, p->z, dx, dy, dz, &t0, &t1)) {
    if (t0 > 0.0f) {
      p->x = fmaf(t0, dx, p->x);
      p->y = fmaf(t0, dy, p->y);
      p->z = fmaf(t0, dz, p->z);
    }
    p->state = MC_FLY;
  } else {
    p->state = MC_ESCAPED;
  }
}

/* Label at a point, or -1 outside the phantom box (then the photon has
 * left it for good: the box is convex and nothing outside interacts).
 * Index as CBCT_real325im.cu:921, optional clip cylinder as :904. */
MONTE_HD int mc_label_at(const mc_params* P, const uint8_t* labels, float x, float y, float z) {
  float fx = (x - P->x0) * P->inv_dx;
  float fy = (y - P->y0) * P->inv_dy;
  float fz = (z - P->z0) * P->inv_dz;
  if (!(fx >= 0.0f && fx < (float)P->nx && fy >= 0.0f && fy < (float)P->ny && fz >= 0.0f &&
        fz < (float)P->nz))
    return -1;
  if (P->clip_r2 > 0.0f && (fmaf(x, x, y * y) > P->clip_r2 || z < -P->clip_hz || z > P->clip_hz))
    return 0;
  int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  return (int)labels[((size_t)iz * (size_t)P->ny + (size_t)iy) * (size_t)P->nx + (size_t)ix];
}

/* One Woodcock step (photon::delta_sampling, CBCT_real325im.cu:886-962):
 * exponential step at the majorant, then accept a real collision with
 * probability mu(label)/mu_max.  Updates p->state. */
MONTE_HD void mc_flight_step(const mc_params* P, const mc_tables* T, const uint8_t* labels,
                             mc_photon* p) {
  float beta = monte_uniform_keys(&p->rng, &P->keys);
  float r = -monte_logf(beta) * T->inv_mu_max[p->kb];
  float dx, dy, dz;
  mc_dir(p, &dx, &dy, &dz);
  p->x = fmaf(r, dx, p->x);
  p->y = fmaf(r, dy, p->y);
  p->z = fmaf(r, dz, p->z);
  float nu = monte_uniform_keys(&p->rng, &P->keys);
  int lab = mc_label_at(P, labels, p->x, p->y, p->z);
  p->steps++;
  if (lab < 0) {
    p->state = MC_ESCAPED;
  } else if (nu <= T->ratio[lab][p->kb]) {
    p->label = lab;
    p->state = MC_COLLIDED;
  } else if (p->steps >= MC_MAX_STEPS) {
    p->state = MC_DEAD;
  }
}

/* One event of a flight with majorants local to macro cells
 * (MC_F_LOCAL_MAJORANT; the reference's single majorant is mc_flight_step):
 * delta tracking with a piecewise-constant majorant.  The photon carries
 * tau, the optical depth left of its current exponential draw.  In the
 * macro cell holding it, the majorant m of the cell's class bounds mu over
 * every cell within R cells of it (R >= 1 is stored with the class), so
 * over the next R legs of P->leg cm at least: a leg is shorter than a
 * cell's smallest edge.  If tau / m fits in those R legs the photon moves
 * there and makes a tentative collision, accepted with probability
 * mu(label) / m (a Woodcock step); otherwise it moves the R legs and
 * spends m times their length of tau (nothing can collide there beyond
 * what m accounts for; exponential flights are memoryless).  Air-only
 * cells (m = 0) are crossed R legs at a time.
 * Returns 1 after a tentative collision, 0 after a leg; updates p->state. */
MONTE_HD int mc_flight_leg(const mc_params* P, const mc_local_tables* L, const uint8_t* labels,
                           const uint16_t* mclass, mc_photon* p) {
  /* A photon that enters the box sits on a face (mc_start), and rounding
   * can put it a hair outside: positions within half a voxel of the box
   * count as inside, with the cell index clamped to the grid (nothing
   * outside the box interacts; a tentative collision there escapes
   * through mc_label_at).  Farther out the photon has left: the box is
   * convex. */
  const float fx = (p->x - P->x0) * P->inv_dx;
  const float fy = (p->y - P->y0) * P->inv_dy;
  const float fz = (p->z - P->z0) * P->inv_dz;
  if (!(fx > -0.5f && fx < (float)P->nx + 0.5f && fy > -0.5f && fy < (float)P->ny + 0.5f &&
        fz > -0.5f && fz < (float)P->nz + 0.5f)) {
    p->state = MC_ESCAPED;
    return 0;
  }
  int cx = (int)(fx > 0.0f ? fx : 0.0f) >> P->mshift;
  int cy = (int)(fy > 0.0f ? fy : 0.0f) >> P->mshift;
  int cz = (int)(fz > 0.0f ? fz : 0.0f) >> P->mshift;
  cx = cx < P->mgx ? cx : P->mgx - 1;
  cy = cy < P->mgy ? cy : P->mgy - 1;
  cz = cz < P->mgz ? cz : P->mgz - 1;
  const unsigned cr =
      mclass[((size_t)cz * (size_t)P->mgy + (size_t)cy) * (size_t)P->mgx + (size_t)cx];
  const mc_majorant m = L->maj[cr & 0xffu][p->kb];
  const float leg = (float)(cr >> 8) * P->leg;  /* R legs: the class bounds mu that far */
  if (p->tau <= 0.0f) p->tau = -monte_logf(monte_uniform_keys(&p->rng, &P->keys));
  float dx, dy, dz;
  mc_dir(p, &dx, &dy, &dz);
  const float s = p->tau * m.inv;
  p->steps++;
  if (!(s <= leg)) {
    p->x = fmaf(leg, dx, p->x);
    p->y = fmaf(leg, dy, p->y);
    p->z = fmaf(leg, dz, p->z);
    p->tau = fmaf(-m.maj, leg, p->tau);
    if (p->steps >= MC_MAX_STEPS) p->state = MC_DEAD;
    return 0;
  }
  p->x = fmaf(s, dx, p->x);
  p->y = fmaf(s, dy, p->y);
  p->z = fmaf(s, dz, p->z);
  p->tau = 0.0f;
  const float nu = monte_uniform_keys(&p->rng, &P->keys);
  const int lab = mc_label_at(P, labels, p->x, p->y, p->z);
  if (lab < 0) {
    p->state = MC_ESCAPED;
  } else if (nu * m.maj <= L->mu[lab][p->kb]) {
    p->label = lab;
    p->state = MC_COLLIDED;
  } else if (p->steps >= MC_MAX_STEPS) {
    p->state = MC_DEAD;
  }
  return 1;
}

/* One event of a flight, by the run's transport: returns 1 for a
 * Woodcock step, 0 for a majorant leg (local majorants only). */
MONTE_HD int mc_flight_event(const mc_params* P, const mc_tables* T, const mc_local_tables* L,
                             const uint8_t* labels, const uint16_t* mclass, mc_photon* p) {
  if (P->flags & MC_F_LOCAL_MAJORANT) return mc_flight_leg(P, L, labels, mclass, p);
  mc_flight_step(P, T, labels, p);
  return 1;
}

/* Detector pixel hit by an escaped photon, as a flat index into the
 * [view][u][v] tally, or -1.  The line through the last position along the
 * current direction, in the view frame, meets the detector plane x' = dod
 * (primary: CBCT_real325im.cu:567-585; scatter: :672-692, :823-841); the
 * pixel is floor((half - coord) / pitch) (the reference's
 * -int(10 d - 162.5), bounds-checked here). */
MONTE_HD long long mc_detector_index(const mc_params* P, const mc_view* V, const mc_photon* p) {
  const mc_view* v = &V[p->view];
  float dx, dy, dz;
  mc_dir(p, &dx, &dy, &dz);
  float xr = p->x * v->c + p->y * v->s;
  float yr = p->y * v->c - p->x * v->s;
  float dxr = dx * v->c + dy * v->s;
  float dyr = dy * v->c - dx * v->s;
  if (!(dxr > 0.0f)) return -1;
  float t = (P->dod - xr) / dxr;
  if (t < 0.0f) return -1;
  float hy = fmaf(t, dyr, yr);
  float hz = fmaf(t, dz, p->z);
  float fu = (P->half_u - hy) * P->inv_du;
  float fv = (P->half_v - hz) * P->inv_dv;
  if (!(fu >= 0.0f && fu < (float)P->nu && fv >= 0.0f && fv < (float)P->nv)) return -1;
  int iu = (int)fu, iv = (int)fv;
  return ((long long)p->view * P->nu + iu) * P->nv + iv;
}

/* Interaction at a real collision (CBCT_real325im.cu:649-795).  Returns
 * the new state: MC_DEAD (photo-absorption or numerical failure) or MC_FLY
 * (Rayleigh: direction kept, :656-671; Compton: Kahn sampling of
 * Klein-Nishina, :701-736, energy 511/lambda', rotation :768-781). */
/* The first part of an interaction, its type: MC_DEAD (photoelectric
 * absorption, or a label without a material), MC_FLY (Rayleigh: the
 * direction is kept), or MC_COMPTON, for which mc_compton follows.  Split
 * so that a kernel can settle the short outcomes at once and run the long
 * Compton sampling for several lanes together; the draws are the same
 * either way. */
MONTE_HD int mc_interact_type(const mc_params* P, const mc_tables* T, mc_photon* p) {
  int mat = T->label_material[p->label];
  if (mat < 0) return MC_DEAD;
  float sc = monte_uniform_keys(&p->rng, &P->keys);
  p->n_int++;
  if (sc <= T->p_photo[mat][p->kb]) {
    p->last = MC_EV_PHOTO;
    return MC_DEAD;
  }
  if (sc <= T->p_photo_coh[mat][p->kb]) {
    p->last = MC_EV_RAYLEIGH;
    p->steps = 0;
    return MC_FLY;
  }
  p->last = MC_EV_COMPTON;
  return MC_COMPTON;
}

/* The Compton part of an interaction (after mc_interact_type). */
MONTE_HD int mc_compton(const mc_params* P, mc_photon* p) {
  /* Kahn's rejection sampling of lambda' = rho * lambda (:701-736) */
  float lambda = 511.0f / p->E;
  float lam2 = lambda + 2.0f;
  float thr = lam2 / fmaf(9.0f, lambda, 2.0f);
  float ro = 1.0f;
  int ok = 0;
  for (int tries = 0; tries < MC_MAX_KN_TRIES; tries++) {
    float r1 = monte_uniform_keys(&p->rng, &P->keys);
    if (r1 < thr) {
      float r2 = monte_uniform_keys(&p->rng, &P->keys);
      ro = fmaf(2.0f / lambda, r2, 1.0f);
      float r3 = monte_uniform_keys(&p->rng, &P->keys);
      float inv = 1.0f / ro;
      if (r3 <= 4.0f * (inv - inv * inv)) {
        ok = 1;
        break;
      }
    } else {
      float r2 = monte_uniform_keys(&p->rng, &P->keys);
      ro = lam2 / fmaf(2.0f, 1.0f - r2, lambda);
      float r3 = monte_uniform_keys(&p->rng, &P->keys);
      float q = lambda - ro * lambda + 1.0f;
      if (r3 <= 0.5f * fmaf(q, q, 1.0f / ro)) {
        ok = 1;
        break;
      }
    }
  }
  if (!ok) return MC_DEAD;
  float lam_d = ro * lambda;
  float cth = 1.0f - (lam_d - lambda);
  if (cth < -1.0f) cth = -1.0f;
  float sth = sqrtf(1.0f - cth * cth);
  p->E = 511.0f / lam_d;
  p->kb = mc_bin(p->E);
  float sphi, cphi;
  monte_sincos_2pi(monte_uniform_keys(&p->rng, &P->keys), &sphi, &cphi);
  /* incoming direction (:768-773; CBCT_real2.cpp:460-463) */
  float st = p->st, ct = p->ct, sp = p->sp, cp = p->cp;
  if ((P->flags & MC_F_FIRST_COMPTON_Z) && p->n_compton == 0) {
    st = 0.0f; /* the CPU program starts from sin_theta_a_new = 0, cos = 1, */
    ct = 1.0f; /* sin_phi_a_new = 1, cos_phi_a_new = 0 (CBCT_real2.cpp:193) */
    sp = 1.0f;
    cp = 0.0f;
  } else if ((P->flags & MC_F_STALE_SIN_PHI) && p->n_compton > 0) {
    sp = p->sp_aim; /* sin_phi_a is never refreshed (CBCT_real325im.cu:768-773) */
  }
  float cn = ct * cth - st * sth * cphi;
  if (cn < -1.0f) cn = -1.0f;
  if (cn > 1.0f) return MC_DEAD; /* the reference's sqrt goes NaN and it stops (:782-791) */
  float sn = sqrtf(1.0f - cn * cn);
  if (sn == 0.0f) return MC_DEAD;
  float cpn = (ct * cp * sth * cphi + st * cp * cth - sp * sth * sphi) / sn;
  float spn = (ct * sp * sth * cphi + st * sp * cth + cp * sth * sphi) / sn;
  p->st = sn;
  p->ct = cn;
  p->cp = cpn;
  p->sp = spn;
  p->n_compton++;
  p->steps = 0;
  return MC_FLY;
}

MONTE_HD int mc_interact(const mc_params* P, const mc_tables* T, mc_photon* p) {
  const int s = mc_interact_type(P, T, p);
  return s == MC_COMPTON ? mc_compton(P, p) : s;
}

/* Whether an escaped photon is tallied, and into which tally:
 * 0 primary, 1 scatter, -1 not tallied. */
MONTE_HD int mc_tally_kind(const mc_params* P, const mc_photon* p) {
  if (p->n_int == 0) return 0;
  if (p->last == MC_EV_RAYLEIGH && (P->flags & MC_F_NO_RAYLEIGH_TALLY)) return -1;
  return 1;
}

/* After a flight ends in a real collision: interact, unless the history
 * already used its max_int interactions (the `for a < ScatterNUM` loop of
 * CBCT_real325im.cu:599). */
MONTE_HD int mc_after_collision(const mc_params* P, const mc_tables* T, mc_photon* p) {
  if (p->n_int >= P->max_int) return MC_DEAD;
  return mc_interact(P, T, p);
}

#ifdef __cplusplus
}
#endif
#endif /* MONTE_MC_PHYSICS_H */
