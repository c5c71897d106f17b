// siddon.cuh -- exact radiological path through a voxel grid (Siddon,
// "Fast calculation of the exact radiological path for a three-dimensional
// CT array", Med. Phys. 12 (1985); incremental traversal as in Jacobs et
// al., Med. Phys. 25 (1998)), shared by the forward and adjoint kernels.
//
// The rays are the Monte Carlo's primary rays: from the source of view k
// along the emission direction of pixel (i, j) (monte_cu/CBCT_real325im.cu:
// 476-512), so exp(-integral) is the expected primary fraction of that
// pixel's histories.
#pragma once

#include <cuda_runtime.h>

#include "mc_physics.h"

namespace monte {

struct SiddonGrid {
  int nx, ny, nz;
  double x0, y0, z0;       // low corner (cm)
  double dx, dy, dz;       // voxel pitch (cm)
};

// Float-float numbers (value = hi + lo, |lo| <= ulp(hi) / 2) for the walk:
// sums and products with their exact float errors (Knuth's two-sum, the
// FMA two-product; T. J. Dekker, "A floating-point technique for extending
// the available precision", Numer. Math. 18, 1971).  FP64 runs at a small
// fraction of the FP32 rate on this GPU; these keep ~44 bits in FP32 work.
struct SidFF {
  float hi, lo;
};

__device__ __forceinline__ SidFF sid_ff(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}

// p * b + c for an integer-valued float p (a plane index, exact in float)
__device__ __forceinline__ SidFF sid_ff_fma(float p, SidFF b, SidFF c) {
  const float ph = p * b.hi;
  const float pe = fmaf(p, b.hi, -ph);  // p * b.hi = ph + pe exactly
  const float s = ph + c.hi;            // two-sum of ph and c.hi
  const float bb = s - ph;
  const float se = (ph - (s - bb)) + (c.hi - bb);
  const float lo = se + pe + fmaf(p, b.lo, c.lo);
  const float hi = s + lo;              // renormalise
  return {hi, lo - (hi - s)};
}

__device__ __forceinline__ bool sid_le(SidFF a, SidFF b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}

// Visit the voxels a ray o + t*d (|d| = 1, t in cm) crosses inside the
// grid, calling f(voxel index, segment length in cm).  Crossing parameters
// are recomputed from integer plane indices at every step, never
// accumulated.
//
// The parameters reach the ray's length (tens of cm) while segments are a
// fraction of a voxel: in plain float every segment length would carry an
// absolute error of ~1 ulp(t), about 5e-5 of a 0.8 mm segment, and a line
// integral across a few strong boundaries would drift by more than 1e-5
// relative.  So the per-ray set-up (the entry point, a small difference of
// large numbers: the source sits hundreds of voxels from the grid) runs in
// double, and the walk in float-float: a segment length, the difference of
// two neighbouring crossings, is then exact to ~1e-13 cm before it is
// rounded to float.
template <typename F>
__device__ __forceinline__ void siddon_walk(const SiddonGrid& g, float ox, float oy, float oz,
                                            float dx, float dy, float dz, F&& f) {
  const double invd[3] = {1.0 / g.dx, 1.0 / g.dy, 1.0 / g.dz};
  const double od[3] = {((double)ox - g.x0) * invd[0], ((double)oy - g.y0) * invd[1],
                        ((double)oz - g.z0) * invd[2]};
  const double dd[3] = {(double)dx * invd[0], (double)dy * invd[1], (double)dz * invd[2]};
  const int n[3] = {g.nx, g.ny, g.nz};
  double t0 = 0.0, t1 = 1.0e300;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (dd[a] == 0.0) {
      if (od[a] < 0.0 || od[a] >= (double)n[a]) return;
    } else {
      double ta = -od[a] / dd[a], tb = ((double)n[a] - od[a]) / dd[a];
      t0 = fmax(t0, fmin(ta, tb));
      t1 = fmin(t1, fmax(ta, tb));
    }
  }
  if (!(t0 < t1)) return;
  // voxel at the entry: evaluate 1e-4 voxel inside the grid; crossing of
  // plane p along axis a at t = p * inv[a] + c[a]
  int idx[3], step[3];
  SidFF tnext[3], inv[3], c[3];
  const double dmax = fmax(fabs(dd[0]), fmax(fabs(dd[1]), fabs(dd[2])));
  const double tm = t0 + 1e-4 / dmax;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double p = od[a] + tm * dd[a];
    const int i = (int)floor(p);
    idx[a] = min(max(i, 0), n[a] - 1);
    step[a] = dd[a] > 0.0 ? 1 : -1;
    if (dd[a] == 0.0) {
      inv[a] = {0.f, 0.f};
      c[a] = {0.f, 0.f};
      tnext[a] = {3.0e38f, 0.f};  // never
    } else {
      const double ia = 1.0 / dd[a];
      inv[a] = sid_ff(ia);
      c[a] = sid_ff(-od[a] * ia);
      tnext[a] = sid_ff_fma((float)(idx[a] + (step[a] > 0 ? 1 : 0)), inv[a], c[a]);
    }
  }
  SidFF t = sid_ff(t0);
  const SidFF tend = sid_ff(t1);
  const int max_steps = g.nx + g.ny + g.nz + 3;
  for (int it = 0; it < max_steps && !sid_le(tend, t); it++) {
    const int a = sid_le(tnext[0], tnext[1]) ? (sid_le(tnext[0], tnext[2]) ? 0 : 2)
                                             : (sid_le(tnext[1], tnext[2]) ? 1 : 2);
    const SidFF tn = sid_le(tnext[a], tend) ? tnext[a] : tend;
    if (!sid_le(tn, t)) {
      // neighbouring crossings: the difference of the high parts is exact
      const float len = (tn.hi - t.hi) + (tn.lo - t.lo);
      f(((size_t)idx[2] * g.ny + idx[1]) * g.nx + idx[0], len);
    }
    t = tn;
    idx[a] += step[a];
    if (idx[a] < 0 || idx[a] >= n[a]) break;
    tnext[a] = sid_ff_fma((float)(idx[a] + (step[a] > 0 ? 1 : 0)), inv[a], c[a]);
  }
}

// Source point and unit emission direction of pixel (iu, iv) of view k,
// as mc_start() aims its histories.
__device__ __forceinline__ void siddon_ray(const mc_params& P, const mc_view* V, const mc_pixel* U,
                                           const mc_pixel* W, int view, int iu, int iv, float* o,
                                           float* d) {
  const mc_view& v = V[view];
  const mc_pixel& pu = U[iu];
  const mc_pixel& pv = W[iv];
  float cp = pu.cos_a * v.c - pu.sin_a * v.s;
  float sp = pu.sin_a * v.c + pu.cos_a * v.s;
  o[0] = -P.sod * v.c;
  o[1] = -P.sod * v.s;
  o[2] = 0.0f;
  d[0] = pv.sin_t * cp;
  d[1] = pv.sin_t * sp;
  d[2] = pv.cos_t;
}

}  // namespace monte
