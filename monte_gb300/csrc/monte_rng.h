/*
 * monte_rng.h -- counter-based random streams and elementary float math
 * shared by the CUDA kernels and the CPU replay harness.  Plain C, usable
 * from C, C++ and CUDA; every function rounds identically on host and
 * device provided multiply-adds are not contracted (nvcc -fmad=false,
 * gcc -ffp-contract=off) -- fused operations are written as fmaf().
 *
 * The reference draws from per-pixel cuRAND MRG32k3a states
 * (monte_cu/CBCT_real325im.cu:454,978-991) or one global MT19937
 * (monte_cpp/CBCT_real2.cpp:102), so its histories depend on the launch
 * shape and cannot be replayed.  Here every history owns a Philox4x32-10
 * stream keyed by the run seed and addressed by (history id, job id): any
 * history can be recomputed alone, in any order, on either side.
 */
#ifndef MONTE_RNG_H
#define MONTE_RNG_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define MONTE_HD __host__ __device__ __forceinline__
#else
#define MONTE_HD static inline
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Philox4x32-10 -------------------------------------------------
 * Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2,
 * 3", SC'11: ten rounds of two 32x32->64 multiplies with the published
 * multipliers and Weyl key increments. */
#define MONTE_PHILOX_M0 0xD2511F53u
#define MONTE_PHILOX_M1 0xCD9E8D57u
#define MONTE_PHILOX_W0 0x9E3779B9u
#define MONTE_PHILOX_W1 0xBB67AE85u

typedef struct {
  uint32_t v[4];
} monte_u32x4;

MONTE_HD monte_u32x4 monte_philox4x32_10(monte_u32x4 c, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)MONTE_PHILOX_M0 * c.v[0];
    uint64_t p1 = (uint64_t)MONTE_PHILOX_M1 * c.v[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    monte_u32x4 n;
    n.v[0] = hi1 ^ c.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ c.v[3] ^ k1;
    n.v[3] = lo0;
    c = n;
    k0 += MONTE_PHILOX_W0;
    k1 += MONTE_PHILOX_W1;
  }
  return c;
}

/* The round keys of key (k0, k1): round r uses (k0 + r W0, k1 + r W1).
 * A kernel that runs one key reads them as constants instead of stepping
 * the key in every round of every block; the outputs are the same. */
typedef struct {
  uint32_t k0[10], k1[10];
} monte_philox_keys;

MONTE_HD void monte_philox_schedule(uint64_t seed, monte_philox_keys* K) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; r++) {
    K->k0[r] = k0;
    K->k1[r] = k1;
    k0 += MONTE_PHILOX_W0;
    k1 += MONTE_PHILOX_W1;
  }
}

MONTE_HD monte_u32x4 monte_philox4x32_10_keys(monte_u32x4 c, const monte_philox_keys* K) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)MONTE_PHILOX_M0 * c.v[0];
    uint64_t p1 = (uint64_t)MONTE_PHILOX_M1 * c.v[2];
    monte_u32x4 n;
    n.v[0] = (uint32_t)(p1 >> 32) ^ c.v[1] ^ K->k0[r];
    n.v[1] = (uint32_t)p1;
    n.v[2] = (uint32_t)(p0 >> 32) ^ c.v[3] ^ K->k1[r];
    n.v[3] = (uint32_t)p0;
    c = n;
  }
  return c;
}

/* One history's stream: block b of history h is
 * philox(counter = (b, h_lo, h_hi, job), key = (seed_lo, seed_hi)). */
typedef struct {
  uint32_t k0, k1;      /* key */
  uint32_t h_lo, h_hi;  /* history id */
  uint32_t job;
  uint32_t next;        /* index of the next draw */
  uint32_t buf[4];      /* outputs of block next/4 (valid when next%4 != 0) */
} monte_stream;

MONTE_HD void monte_stream_init(monte_stream* s, uint64_t seed, uint64_t history, uint32_t job) {
  s->k0 = (uint32_t)seed;
  s->k1 = (uint32_t)(seed >> 32);
  s->h_lo = (uint32_t)history;
  s->h_hi = (uint32_t)(history >> 32);
  s->job = job;
  s->next = 0;
  s->buf[0] = s->buf[1] = s->buf[2] = s->buf[3] = 0;
}

MONTE_HD uint32_t monte_stream_u32(monte_stream* s) {
  uint32_t w = s->next & 3u;
  if (w == 0) {
    monte_u32x4 c;
    c.v[0] = s->next >> 2;
    c.v[1] = s->h_lo;
    c.v[2] = s->h_hi;
    c.v[3] = s->job;
    monte_u32x4 r = monte_philox4x32_10(c, s->k0, s->k1);
    s->buf[0] = r.v[0];
    s->buf[1] = r.v[1];
    s->buf[2] = r.v[2];
    s->buf[3] = r.v[3];
  }
  s->next++;
  /* a select, not buf[w]: a run-time index would keep the buffer (and the
   * photon around it) in local memory */
  return w == 0 ? s->buf[0] : w == 1 ? s->buf[1] : w == 2 ? s->buf[2] : s->buf[3];
}

/* monte_stream_u32 with the key's round keys precomputed (K must be the
 * schedule of the stream's key). */
MONTE_HD uint32_t monte_stream_u32_keys(monte_stream* s, const monte_philox_keys* K) {
  uint32_t w = s->next & 3u;
  if (w == 0) {
    monte_u32x4 c;
    c.v[0] = s->next >> 2;
    c.v[1] = s->h_lo;
    c.v[2] = s->h_hi;
    c.v[3] = s->job;
    monte_u32x4 r = monte_philox4x32_10_keys(c, K);
    s->buf[0] = r.v[0];
    s->buf[1] = r.v[1];
    s->buf[2] = r.v[2];
    s->buf[3] = r.v[3];
  }
  s->next++;
  return w == 0 ? s->buf[0] : w == 1 ? s->buf[1] : w == 2 ? s->buf[2] : s->buf[3];
}

/* Uniform on (0, 1] with 24-bit resolution, like curand_uniform's range
 * (the reference's -log(beta) needs beta > 0, CBCT_real325im.cu:888-889). */
MONTE_HD float monte_u01(uint32_t x) { return (float)((x >> 8) + 1u) * 5.9604644775390625e-8f; }

MONTE_HD float monte_uniform(monte_stream* s) { return monte_u01(monte_stream_u32(s)); }

MONTE_HD float monte_uniform_keys(monte_stream* s, const monte_philox_keys* K) {
  return monte_u01(monte_stream_u32_keys(s, K));
}

/* ---- elementary functions ------------------------------------------ */

MONTE_HD uint32_t monte_f2u(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
MONTE_HD float monte_u2f(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

/* Natural log of a positive normal float.  x = 2^e * m, m in
 * [sqrt(1/2), sqrt(2)); log m = 2 atanh(s) with s = (m-1)/(m+1), summed as
 * the atanh Taylor series 2(s + s^3/3 + ... + s^11/11) (|s| <= 0.1716, the
 * truncation error is below 2e-11); e*ln2 is added in two parts (a
 * high part exact for |e| < 2^8 and the remainder).  Error about 1 ulp. */
MONTE_HD float monte_logf(float x) {
  uint32_t b = monte_f2u(x);
  int e = (int)((b >> 23) & 0xffu) - 127;
  uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
  if (mb > 0x3fb504f3u) { /* m > sqrt(2): use m/2 */
    mb -= 0x00800000u;
    e += 1;
  }
  float m = monte_u2f(mb);
  float f = m - 1.0f;
  float s = f / (m + 1.0f);
  float z = s * s;
  float p = 0.18181818181818182f;          /* 2/11 */
  p = fmaf(p, z, 0.22222222222222222f);    /* 2/9 */
  p = fmaf(p, z, 0.28571428571428571f);    /* 2/7 */
  p = fmaf(p, z, 0.4f);                    /* 2/5 */
  p = fmaf(p, z, 0.66666666666666667f);    /* 2/3 */
  float t = s * z;
  float lm = fmaf(t, p, 2.0f * s);
  float fe = (float)e;
  /* ln2 = 0.693145751953125 (exact, 16 significant bits) + 1.428606820e-6 */
  return fmaf(fe, 0.693145751953125f, fmaf(fe, 1.42860682030941723212e-6f, lm));
}

/* sin and cos of x in [0, pi/4] from their Taylor series (truncation
 * below 1.3e-10 for sin to x^11 and cos to x^12). */
MONTE_HD void monte_sincos_small(float x, float* s, float* c) {
  float x2 = x * x;
  float ps = -2.5052108385441720e-8f;          /* -1/11! */
  ps = fmaf(ps, x2, 2.7557319223985893e-6f);   /* 1/9! */
  ps = fmaf(ps, x2, -1.9841269841269841e-4f);  /* -1/7! */
  ps = fmaf(ps, x2, 8.3333333333333333e-3f);   /* 1/5! */
  ps = fmaf(ps, x2, -0.16666666666666667f);    /* -1/3! */
  *s = fmaf(x * x2, ps, x);
  float pc = 2.0876756987868099e-9f;           /* 1/12! */
  pc = fmaf(pc, x2, -2.7557319223985891e-7f);  /* -1/10! */
  pc = fmaf(pc, x2, 2.4801587301587302e-5f);   /* 1/8! */
  pc = fmaf(pc, x2, -1.3888888888888889e-3f);  /* -1/6! */
  pc = fmaf(pc, x2, 4.1666666666666667e-2f);   /* 1/4! */
  pc = fmaf(pc, x2, -0.5f);                    /* -1/2! */
  *c = fmaf(x2, pc, 1.0f);
}

/* sin and cos of 2*pi*u for u in [0, 1]: quadrant q = floor(4u), reflect
 * the remaining fraction into [0, pi/4], then rotate by q quarter turns.
 * For u = k * 2^-24 every reduction step is exact. */
MONTE_HD void monte_sincos_2pi(float u, float* sn, float* cs) {
  float t = 4.0f * u;
  int q = (int)t;
  float f = t - (float)q;
  float s0, c0;
  if (f <= 0.5f) {
    monte_sincos_small(f * 1.5707963267948966f, &s0, &c0);
  } else {
    monte_sincos_small((1.0f - f) * 1.5707963267948966f, &c0, &s0);
  }
  switch (q & 3) {
    case 0: *sn = s0; *cs = c0; break;
    case 1: *sn = c0; *cs = -s0; break;
    case 2: *sn = -s0; *cs = -c0; break;
    default: *sn = -c0; *cs = s0; break;
  }
}

#ifdef __cplusplus
}
#endif
#endif /* MONTE_RNG_H */
