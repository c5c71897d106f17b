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
  float x0, y0, z0;        // low corner (cm)
  float dx, dy, dz;        // voxel pitch (cm)
};

// Visit the voxels a ray o + t*d (|d| = 1, t in cm) crosses inside the
// grid, calling f(voxel index, segment length).  Crossing parameters are
// recomputed from integer plane indices at every step, never accumulated.
template <typename F>
__device__ __forceinline__ void siddon_walk(const SiddonGrid& g, float ox, float oy, float oz,
                                            float dx, float dy, float dz, F&& f) {
  // Per-ray set-up in double: the source sits hundreds of voxels from the
  // grid, and in float the entry point (a small difference of large
  // numbers) would shift the ray by ~1e-5 voxel -- enough to move the plane
  // crossings of rays that graze a plane.  The walk itself runs in float
  // from the entry point, where all parameters stay within the grid's extent.
  const double invd[3] = {1.0 / (double)g.dx, 1.0 / (double)g.dy, 1.0 / (double)g.dz};
  const double od[3] = {((double)ox - (double)g.x0) * invd[0], ((double)oy - (double)g.y0) * invd[1],
                        ((double)oz - (double)g.z0) * invd[2]};
  const double dd[3] = {(double)dx * invd[0], (double)dy * invd[1], (double)dz * invd[2]};
  const int n[3] = {g.nx, g.ny, g.nz};
  double t0d = 0.0, t1d = 1.0e300;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (dd[a] == 0.0) {
      if (od[a] < 0.0 || od[a] >= (double)n[a]) return;
    } else {
      double ta = -od[a] / dd[a], tb = ((double)n[a] - od[a]) / dd[a];
      t0d = fmax(t0d, fmin(ta, tb));
      t1d = fmin(t1d, fmax(ta, tb));
    }
  }
  if (!(t0d < t1d)) return;
  float e[3], dir[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    e[a] = (float)(od[a] + t0d * dd[a]);
    dir[a] = (float)dd[a];
  }
  float t1 = (float)(t1d - t0d);
  // voxel at the entry: evaluate 1e-4 voxel inside the grid
  int idx[3], step[3];
  float tnext[3];
  const float dmax = fmaxf(fabsf(dir[0]), fmaxf(fabsf(dir[1]), fabsf(dir[2])));
  const float tm = 1e-4f / dmax;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    float p = fmaf(tm, dir[a], e[a]);
    int i = (int)floorf(p);
    idx[a] = min(max(i, 0), n[a] - 1);
    step[a] = dir[a] > 0.0f ? 1 : -1;
    if (dir[a] == 0.0f) {
      tnext[a] = 3.0e38f;
    } else {
      float plane = (float)(idx[a] + (step[a] > 0 ? 1 : 0));
      tnext[a] = (plane - e[a]) / dir[a];
    }
  }
  float t = 0.0f;
  const int max_steps = g.nx + g.ny + g.nz + 3;
  for (int it = 0; it < max_steps && t < t1; it++) {
    int a = (tnext[0] <= tnext[1]) ? ((tnext[0] <= tnext[2]) ? 0 : 2) : ((tnext[1] <= tnext[2]) ? 1 : 2);
    float tn = fminf(tnext[a], t1);
    if (tn > t) {
      size_t v = ((size_t)idx[2] * g.ny + idx[1]) * g.nx + idx[0];
      f(v, tn - t);
    }
    t = tn;
    idx[a] += step[a];
    if (idx[a] < 0 || idx[a] >= n[a]) break;
    float plane = (float)(idx[a] + (step[a] > 0 ? 1 : 0));
    tnext[a] = (plane - e[a]) / dir[a];
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
