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

// Visit the voxels a ray o + t*d (|d| = 1, t in cm) crosses inside the
// grid, calling f(voxel index, segment length in cm, as a double).
// Crossing parameters are recomputed from integer plane indices at every
// step, never accumulated.
//
// The walk runs in double.  Its parameters reach the ray's length inside the
// grid (tens of cm) while segments are a fraction of a voxel, so in float
// every segment length would carry an absolute error of ~1 ulp(t) -- about
// 5e-5 of a 0.8 mm segment -- and the line integral of a ray crossing a few
// strong boundaries would drift by more than 1e-5 relative.  The ray's entry
// point (a small difference of large numbers: the source sits hundreds of
// voxels from the grid) is likewise computed in double.
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
  double tnext[3], inv[3], c[3];
  const double dmax = fmax(fabs(dd[0]), fmax(fabs(dd[1]), fabs(dd[2])));
  const double tm = t0 + 1e-4 / dmax;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double p = od[a] + tm * dd[a];
    const int i = (int)floor(p);
    idx[a] = min(max(i, 0), n[a] - 1);
    step[a] = dd[a] > 0.0 ? 1 : -1;
    if (dd[a] == 0.0) {
      inv[a] = 0.0;
      c[a] = 0.0;
      tnext[a] = 1.0e300;
    } else {
      inv[a] = 1.0 / dd[a];
      c[a] = -od[a] * inv[a];
      tnext[a] = fma((double)(idx[a] + (step[a] > 0 ? 1 : 0)), inv[a], c[a]);
    }
  }
  double t = t0;
  const int max_steps = g.nx + g.ny + g.nz + 3;
  for (int it = 0; it < max_steps && t < t1; it++) {
    int a = (tnext[0] <= tnext[1]) ? ((tnext[0] <= tnext[2]) ? 0 : 2) : ((tnext[1] <= tnext[2]) ? 1 : 2);
    double tn = fmin(tnext[a], t1);
    if (tn > t) {
      size_t v = ((size_t)idx[2] * g.ny + idx[1]) * g.nx + idx[0];
      f(v, tn - t);
    }
    t = tn;
    idx[a] += step[a];
    if (idx[a] < 0 || idx[a] >= n[a]) break;
    tnext[a] = fma((double)(idx[a] + (step[a] > 0 ? 1 : 0)), inv[a], c[a]);
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
