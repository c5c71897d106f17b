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
  uint32_t pf;          /* device kernels only: shared-memory byte address of a
                           16-byte slot that monte_stream_prefetch fills with
                           the block the next wrap of `next` loads, bit 0 set
                           while it holds it; 0 = no slot (the host, and kernels
                           that do not prefetch) */
} monte_stream;

MONTE_HD void monte_stream_init(monte_stream* s, uint64_t seed, uint64_t history, uint32_t job) {
  s->k0 = (uint32_t)seed;
  s->k1 = (uint32_t)(seed >> 32);
  s->h_lo = (uint32_t)history;
  s->h_hi = (uint32_t)(history >> 32);
  s->job = job;
  s->next = 0;
  s->buf[0] = s->buf[1] = s->buf[2] = s->buf[3] = 0;
  s->pf = 0;
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
#if defined(__CUDA_ARCH__)
  if (w == 0 && (s->pf & 1u)) {  /* the block was prefetched */
    asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(s->buf[0]), "=r"(s->buf[1]), "=r"(s->buf[2]), "=r"(s->buf[3])
                 : "r"(s->pf & ~15u));
    s->pf &= ~1u;
  } else
#endif
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

#if defined(__CUDACC__)
/* Compute, ahead of need, the block that the next wrap of s->next loads
 * (block next/4 when next%4 == 0, else the one after it) into the stream's
 * shared-memory slot.  The draws are the same whenever the block is
 * computed; what changes is where the Philox rounds run.  A warp runs a
 * divergent branch once for all of its lanes that take it, so a kernel
 * whose lanes draw at their own pace would run the ten rounds in nearly
 * every step for the few lanes whose block ran out; prefetching for every
 * lane without a block whenever one lane is about to run out makes those
 * passes several steps apart. */
__device__ __forceinline__ void monte_stream_prefetch(monte_stream* s, const monte_philox_keys* K) {
  monte_u32x4 c;
  c.v[0] = (s->next + 3u) >> 2;
  c.v[1] = s->h_lo;
  c.v[2] = s->h_hi;
  c.v[3] = s->job;
  const monte_u32x4 r = monte_philox4x32_10_keys(c, K);
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(s->pf & ~15u), "r"(r.v[0]),
               "r"(r.v[1]), "r"(r.v[2]), "r"(r.v[3])
               : "memory");
  s->pf |= 1u;
}
#endif

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

/* Natural log of a positive normal float, table-driven (the method of
 * P. T. P. Tang, "Table-driven implementation of the logarithm function in
 * IEEE floating-point arithmetic", ACM TOMS 16(4), 1990), with no division.
 * x = 2^e m, m in [sqrt(1/2), sqrt(2)); the exponent and top mantissa bits
 * of m pick one of 65 intervals, each with a float g close to 1/m (g = 1
 * exactly for the two intervals next to 1, so log x keeps its relative
 * accuracy as x -> 1).  Then r = m g - 1 (one fused rounding; |r| < 1/64)
 * and log m = log1p(r) - log(g), log1p by its Taylor series to r^5
 * (truncation below 3e-12 relative), -log(g) from the table as hi + lo
 * floats; e ln2 is added in two parts (a high part exact for |e| < 2^8).
 * Error below 2 ulp.  Row k of MONTE_LOG_TABLE: {g, -log(g) hi, lo, 0} for
 * the m whose float bits b satisfy (b >> 17) == 0x1f9a + k; g = 2 / (m0 + m1)
 * rounded to float over the interval [m0, m1], -log(g) from double. */
#define MONTE_LOG_TABLE \
  {0x1.690f88p+0f, -0x1.601f14p-2f, -0x1.1ac6f4p-28f, 0.0f}, \
  {0x1.661ec8p+0f, -0x1.57bf7ap-2f, 0x1.c6e5c4p-27f, 0.0f}, \
  {0x1.623fa8p+0f, -0x1.4c9e0cp-2f, 0x1.fa34f2p-28f, 0.0f}, \
  {0x1.5e75bcp+0f, -0x1.419b44p-2f, 0x1.ca85dp-28f, 0.0f}, \
  {0x1.5ac058p+0f, -0x1.36b67cp-2f, 0x1.683dep-27f, 0.0f}, \
  {0x1.571ed4p+0f, -0x1.2bef08p-2f, -0x1.f724d4p-28f, 0.0f}, \
  {0x1.539096p+0f, -0x1.21445cp-2f, 0x1.ae28eap-27f, 0.0f}, \
  {0x1.501502p+0f, -0x1.16b5cep-2f, -0x1.a59f6ep-27f, 0.0f}, \
  {0x1.4cab8ap+0f, -0x1.0c42dcp-2f, 0x1.83d3aap-27f, 0.0f}, \
  {0x1.4953ap+0f, -0x1.01eaeap-2f, -0x1.c4d8cap-27f, 0.0f}, \
  {0x1.460cbep+0f, -0x1.ef5ae8p-3f, 0x1.08c01cp-29f, 0.0f}, \
  {0x1.42d664p+0f, -0x1.db13e6p-3f, 0x1.256ee6p-28f, 0.0f}, \
  {0x1.3fb014p+0f, -0x1.c6ffbcp-3f, -0x1.1e01eep-28f, 0.0f}, \
  {0x1.3c995cp+0f, -0x1.b31d9p-3f, -0x1.2b79b8p-28f, 0.0f}, \
  {0x1.3991c4p+0f, -0x1.9f6c48p-3f, -0x1.2112c4p-28f, 0.0f}, \
  {0x1.3698ep+0f, -0x1.8beb04p-3f, 0x1.31c064p-29f, 0.0f}, \
  {0x1.33ae46p+0f, -0x1.7898dap-3f, -0x1.11131cp-29f, 0.0f}, \
  {0x1.30d19p+0f, -0x1.6574ecp-3f, 0x1.2e7d98p-28f, 0.0f}, \
  {0x1.2e025cp+0f, -0x1.527e5ep-3f, -0x1.50dac6p-30f, 0.0f}, \
  {0x1.2b404cp+0f, -0x1.3fb462p-3f, -0x1.e64a22p-29f, 0.0f}, \
  {0x1.288b02p+0f, -0x1.2d1616p-3f, -0x1.30d024p-28f, 0.0f}, \
  {0x1.25e228p+0f, -0x1.1aa2bep-3f, -0x1.447eep-28f, 0.0f}, \
  {0x1.234568p+0f, -0x1.08598ep-3f, -0x1.33c74p-28f, 0.0f}, \
  {0x1.20b472p+0f, -0x1.ec73aap-4f, 0x1.bd7bdep-30f, 0.0f}, \
  {0x1.1e2ef4p+0f, -0x1.c88584p-4f, -0x1.6f12c6p-30f, 0.0f}, \
  {0x1.1bb4a4p+0f, -0x1.a4e764p-4f, 0x1.a721e4p-31f, 0.0f}, \
  {0x1.194538p+0f, -0x1.8197e2p-4f, -0x1.d038fcp-30f, 0.0f}, \
  {0x1.16e06ap+0f, -0x1.5e95bap-4f, 0x1.1a1bc4p-30f, 0.0f}, \
  {0x1.1485f2p+0f, -0x1.3bdf6cp-4f, 0x1.c5c244p-29f, 0.0f}, \
  {0x1.12359p+0f, -0x1.1973d4p-4f, -0x1.46545ep-32f, 0.0f}, \
  {0x1.0fef02p+0f, -0x1.eea338p-5f, -0x1.01adecp-31f, 0.0f}, \
  {0x1.0db20cp+0f, -0x1.aaef5ap-5f, 0x1.c13c3cp-31f, 0.0f}, \
  {0x1.0b7e7p+0f, -0x1.67c976p-5f, 0x1.a568c2p-30f, 0.0f}, \
  {0x1.0953f4p+0f, -0x1.252f4p-5f, -0x1.e34604p-31f, 0.0f}, \
  {0x1.073262p+0f, -0x1.c63d84p-6f, 0x1.7d6b12p-31f, 0.0f}, \
  {0x1.05198p+0f, -0x1.432ab2p-6f, -0x1.66031p-32f, 0.0f}, \
  {0x1.03091cp+0f, -0x1.8244ep-7f, -0x1.c4506ep-34f, 0.0f}, \
  {0x1.0p+0f, 0.0f, 0.0f, 0.0f}, \
  {0x1.0p+0f, 0.0f, 0.0f, 0.0f}, \
  {0x1.f4465cp-1f, 0x1.7b916cp-6f, -0x1.054992p-31f, 0.0f}, \
  {0x1.ecc07ep-1f, 0x1.39e84cp-5f, 0x1.bfd7fp-30f, 0.0f}, \
  {0x1.e573aep-1f, 0x1.b42dbep-5f, 0x1.a32e4ap-30f, 0.0f}, \
  {0x1.de5d7p-1f, 0x1.16536p-4f, -0x1.5c84bp-32f, 0.0f}, \
  {0x1.d77b66p-1f, 0x1.51b06ep-4f, -0x1.7cf3d8p-31f, 0.0f}, \
  {0x1.d0cb5ap-1f, 0x1.8c3454p-4f, 0x1.0c66d2p-30f, 0.0f}, \
  {0x1.ca4b32p-1f, 0x1.c5e53ap-4f, 0x1.5bc7b2p-32f, 0.0f}, \
  {0x1.c3f8f2p-1f, 0x1.fec902p-4f, -0x1.20a598p-35f, 0.0f}, \
  {0x1.bdd2bap-1f, 0x1.1b72a6p-3f, 0x1.c5ecfap-28f, 0.0f}, \
  {0x1.b7d6c6p-1f, 0x1.371fb8p-3f, 0x1.1e8fd8p-31f, 0.0f}, \
  {0x1.b20366p-1f, 0x1.526e54p-3f, 0x1.d43692p-28f, 0.0f}, \
  {0x1.ac5704p-1f, 0x1.6d60f4p-3f, -0x1.5cc5acp-28f, 0.0f}, \
  {0x1.a6d01cp-1f, 0x1.87f9fep-3f, 0x1.64192ap-28f, 0.0f}, \
  {0x1.a16d4p-1f, 0x1.a23bcp-3f, -0x1.d4a99p-35f, 0.0f}, \
  {0x1.9c2d16p-1f, 0x1.bc2862p-3f, -0x1.a4e61cp-32f, 0.0f}, \
  {0x1.970e5p-1f, 0x1.d5c214p-3f, 0x1.a7ddccp-30f, 0.0f}, \
  {0x1.920fb6p-1f, 0x1.ef0ad6p-3f, -0x1.48e9a6p-29f, 0.0f}, \
  {0x1.8d301ap-1f, 0x1.040256p-2f, 0x1.0d3414p-28f, 0.0f}, \
  {0x1.886e6p-1f, 0x1.1058bep-2f, -0x1.ca36a4p-27f, 0.0f}, \
  {0x1.83c978p-1f, 0x1.1c898cp-2f, -0x1.92cccp-27f, 0.0f}, \
  {0x1.7f406p-1f, 0x1.2895ap-2f, 0x1.7bd0d4p-27f, 0.0f}, \
  {0x1.7ad222p-1f, 0x1.347dd6p-2f, -0x1.f3c146p-29f, 0.0f}, \
  {0x1.767ddp-1f, 0x1.404304p-2f, -0x1.5e55fcp-28f, 0.0f}, \
  {0x1.72428ap-1f, 0x1.4be5f4p-2f, -0x1.4221c8p-28f, 0.0f}, \
  {0x1.6e1f78p-1f, 0x1.57676ep-2f, -0x1.5d52bcp-29f, 0.0f}, \
  {0x1.6b0f96p-1f, 0x1.600112p-2f, 0x1.71fdcp-30f, 0.0f}

#if defined(__CUDACC__)
static __device__ const float4 monte_log_tbl_d[65] = {MONTE_LOG_TABLE};
#endif
static const float monte_log_tbl_h[65][4] = {MONTE_LOG_TABLE};

MONTE_HD float monte_logf(float x) {
  uint32_t b = monte_f2u(x);
  int e = (int)((b >> 23) & 0xffu) - 127;
  uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
  if (mb > 0x3fb504f3u) { /* m > sqrt(2): use m/2 */
    mb -= 0x00800000u;
    e += 1;
  }
  const uint32_t k = (mb >> 17) - 0x1f9au;
#if defined(__CUDA_ARCH__)
  const float4 t = monte_log_tbl_d[k];
  const float g = t.x, thi = t.y, tlo = t.z;
#else
  const float g = monte_log_tbl_h[k][0], thi = monte_log_tbl_h[k][1], tlo = monte_log_tbl_h[k][2];
#endif
  float m = monte_u2f(mb);
  float r = fmaf(m, g, -1.0f);
  float q = fmaf(r, 0.2f, -0.25f);
  q = fmaf(q, r, 0.33333333333333333f);
  q = fmaf(q, r, -0.5f);
  float lm = thi + (tlo + fmaf(r * r, q, r));
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
