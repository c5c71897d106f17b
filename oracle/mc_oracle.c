/*
 * mc_oracle.c -- CPU replay harness for the Monte Carlo hot path.  TEST
 * INFRASTRUCTURE: only the tests, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use it; the product never links or calls it.
 *
 * It restates the control flow of the reference kernel `projection`
 * (monte_cu/CBCT_real325im.cu:462-847) on the host, history by history in
 * the reference's loop order (view, pixel, history), and drives each
 * history through the same per-step functions (mc_physics.h) and the same
 * Philox streams (monte_rng.h) as the GPU kernels, so the GPU tallies must
 * equal these bit for bit.  The physics of those step functions is pinned
 * separately: by a chi-square test against the reference CPU program
 * monte_cpp/CBCT_real2.cpp (tests/golden/cbct_real2.npz) and by analytic
 * known answers (Beer-Lambert transmission, Klein-Nishina moments).
 *
 * Build: oracle/Makefile (-ffp-contract=off).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../monte_gb300/csrc/mc_setup.h"

typedef struct {
  uint64_t histories, steps, interactions, primary, scatter, dropped;
  uint64_t rayleigh, compton, photo;  /* interactions by kind */
  uint64_t legs;                      /* majorant legs (local majorants) */
} oracle_mc_stats;

/* the local-majorant tables and class grid of a run (NULL: global) */
typedef struct {
  const mc_local_tables* L;
  const uint16_t* mclass;
} oracle_local;

/* One Woodcock flight: photon::delta_sampling (CBCT_real325im.cu:862-976). */
static void fly(const mc_params* P, const mc_tables* T, const oracle_local* loc,
                const uint8_t* labels, mc_photon* p, oracle_mc_stats* st) {
  while (p->state == MC_FLY) {
    if (mc_flight_event(P, T, loc->L, labels, loc->mclass, p)) st->steps++; else st->legs++;
    if (p->state == MC_DEAD) st->dropped++;
  }
}

static void tally(const mc_params* P, const mc_view* V, const mc_photon* p, int64_t* prim,
                  int64_t* scat, oracle_mc_stats* st) {
  int kind = mc_tally_kind(P, p);
  long long cell = mc_detector_index(P, V, p);
  if (kind < 0 || cell < 0) return;
  if (kind == 0) {
#pragma omp atomic
    prim[cell] += 1;
    st->primary++;
  } else {
#pragma omp atomic
    scat[cell] += 1;
    st->scatter++;
  }
}

/* One history of `projection`: emission (:466-540), first flight (:549),
 * primary tally (:567-590), then up to max_int interactions (:599-846),
 * each followed by a flight and, on escape, a scatter tally. */
static void history(const mc_params* P, const mc_tables* T, const oracle_local* loc,
                    const mc_view* V, const mc_pixel* U, const mc_pixel* W,
                    const uint8_t* labels, int view, int iu, int iv, uint64_t k, int64_t* prim,
                    int64_t* scat, oracle_mc_stats* st) {
  mc_photon p;
  mc_start(P, T, V, U, W, view, iu, iv, k, &p);
  st->histories++;
  fly(P, T, loc, labels, &p, st);
  if (p.state == MC_ESCAPED) {
    tally(P, V, &p, prim, scat, st);
    return;
  }
  for (int a = 0; a < P->max_int && p.state == MC_COLLIDED; a++) {
    p.state = mc_interact(P, T, &p);
    st->interactions++;
    if (p.last == MC_EV_RAYLEIGH) st->rayleigh++;
    else if (p.last == MC_EV_COMPTON) st->compton++;
    else st->photo++;
    if (p.state != MC_FLY) return; /* photo-absorption (:651-655) */
    fly(P, T, loc, labels, &p, st);
    if (p.state == MC_ESCAPED) {
      tally(P, V, &p, prim, scat, st);
      return;
    }
  }
}

/* Same inputs and semantics as monte_mc_run (include/monte.h), on the CPU.
 * Returns MONTE_OK or MONTE_EINVAL. */
int oracle_mc_run(const monte_mc_geom* g, const monte_mc_phantom* ph, const monte_xcom* x,
                  const monte_spectrum* sp, const monte_mc_request* run, int64_t* prim,
                  int64_t* scat, uint64_t* stats_out) {
  mc_params P;
  const char* why;
  if (mc_setup_params(g, ph, run, &P, &why) != MONTE_OK) return MONTE_EINVAL;
  mc_tables* T = (mc_tables*)malloc(sizeof(mc_tables));
  if (mc_setup_tables(ph, x, sp, T, &why) != MONTE_OK) {
    free(T);
    return MONTE_EINVAL;
  }
  mc_view* V = (mc_view*)malloc(sizeof(mc_view) * g->n_views);
  mc_pixel* U = (mc_pixel*)malloc(sizeof(mc_pixel) * g->nu);
  mc_pixel* W = (mc_pixel*)malloc(sizeof(mc_pixel) * g->nv);
  mc_setup_views(g, V);
  mc_setup_pixels(g, U, W);
  oracle_local loc = {NULL, NULL};
  mc_local_tables* L = NULL;
  uint16_t* mclass = NULL;
  if (P.flags & MC_F_LOCAL_MAJORANT) {
    const size_t cells = (size_t)P.mgx * P.mgy * P.mgz;
    uint64_t* bits = (uint64_t*)malloc(cells * 4 * sizeof(uint64_t));
    L = (mc_local_tables*)malloc(sizeof(mc_local_tables));
    mclass = (uint16_t*)malloc(cells * sizeof(uint16_t));
    mc_setup_local(ph, x, L);
    mc_macro_bits_host(ph, ph->labels, &P, bits);
    mc_macro_classes(&P, L, bits, mclass);
    free(bits);
    loc.L = L;
    loc.mclass = mclass;
  }
  const int nvr = run->v_end - run->v_begin;
  const int npix = (run->u_end - run->u_begin) * nvr;
  oracle_mc_stats tot;
  memset(&tot, 0, sizeof(tot));
  for (int view = run->view_begin; view < run->view_end; view++) {
#pragma omp parallel
    {
      oracle_mc_stats st;
      memset(&st, 0, sizeof(st));
#pragma omp for schedule(dynamic, 1)
      for (int pix = 0; pix < npix; pix++) {
        int iu = run->u_begin + pix / nvr, iv = run->v_begin + pix % nvr;
        for (uint64_t k = 0; k < run->histories_per_pixel; k++)
          history(&P, T, &loc, V, U, W, ph->labels, view, iu, iv, k, prim, scat, &st);
      }
#pragma omp critical
      {
        tot.histories += st.histories;
        tot.steps += st.steps;
        tot.interactions += st.interactions;
        tot.primary += st.primary;
        tot.scatter += st.scatter;
        tot.dropped += st.dropped;
        tot.rayleigh += st.rayleigh;
        tot.compton += st.compton;
        tot.photo += st.photo;
        tot.legs += st.legs;
      }
    }
  }
  if (stats_out) {
    stats_out[0] = tot.histories;
    stats_out[1] = tot.steps;
    stats_out[2] = tot.interactions;
    stats_out[3] = tot.primary;
    stats_out[4] = tot.scatter;
    stats_out[5] = tot.dropped;
    stats_out[6] = tot.rayleigh;
    stats_out[7] = tot.compton;
    stats_out[8] = tot.photo;
    stats_out[9] = tot.legs;
  }
  free(L);
  free(mclass);
  free(T);
  free(V);
  free(U);
  free(W);
  return MONTE_OK;
}

/* Draw n uniforms of history `history` (seed, job): exposes the stream to
 * the tests (Philox known answers, uniformity). */
void oracle_stream(uint64_t seed, uint64_t hist, uint32_t job, int n, float* out) {
  monte_stream s;
  monte_stream_init(&s, seed, hist, job);
  for (int i = 0; i < n; i++) out[i] = monte_uniform(&s);
}

void oracle_philox(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  monte_u32x4 c;
  memcpy(c.v, ctr, 16);
  monte_u32x4 r = monte_philox4x32_10(c, k0, k1);
  memcpy(out, r.v, 16);
}

void oracle_logf(const float* x, float* y, int n) {
  for (int i = 0; i < n; i++) y[i] = monte_logf(x[i]);
}

void oracle_sincos_2pi(const float* u, float* s, float* c, int n) {
  for (int i = 0; i < n; i++) monte_sincos_2pi(u[i], &s[i], &c[i]);
}

/* Compton scattering at energy E for n draws of stream (seed, 0): returns
 * cos(theta) and the new energy, with the photon travelling along +x
 * (tests compare against the Klein-Nishina cross section). */
void oracle_compton(float E, uint64_t seed, int n, float* cos_theta, float* e_out) {
  mc_params P;
  memset(&P, 0, sizeof(P));
  mc_tables* T = (mc_tables*)calloc(1, sizeof(mc_tables));
  T->label_material[0] = 0;
  for (int k = 0; k < MC_NBINS; k++) {
    T->p_photo[0][k] = 0.0f;
    T->p_photo_coh[0][k] = 0.0f; /* always Compton */
  }
  P.max_int = 1000;
  P.seed = seed;
  monte_philox_schedule(seed, &P.keys);
  for (int i = 0; i < n; i++) {
    mc_photon p;
    memset(&p, 0, sizeof(p));
    monte_stream_init(&p.rng, seed, (uint64_t)i, 0);
    p.E = E;
    p.kb = mc_bin(E);
    p.st = 1.0f; p.ct = 0.0f; p.sp = 0.0f; p.cp = 1.0f; /* +x */
    p.sp_aim = 0.0f;
    p.label = 0;
    int s = mc_interact(&P, T, &p);
    cos_theta[i] = s == MC_FLY ? p.st * p.cp : 2.0f;
    e_out[i] = p.E;
  }
  free(T);
}
