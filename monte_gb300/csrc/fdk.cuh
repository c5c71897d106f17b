// fdk.cuh -- device-side description of one FDK problem and the kernel
// launchers shared by fdk_filter.cu, fdk_bp.cu and fdk_api.cu.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/monte.h"

namespace monte {

// Per-view constants of the backprojector, computed on the host in double
// (recon/bp3d20.cpp:85-88,103-104,134-137,159) and rounded to float.
struct BpView {
  float c, s;     // cos, sin of the view angle
  float px, py;   // rotated source position
  float tanb;     // tan() as the distance term evaluates it
  float rs;       // 1/sqrt(1+tanb^2)
  float factor;   // dbeta * scale * scale2
  float pad;
};

// Geometry as the kernels use it (float), derived from monte_fdk_geom.
struct FdkDev {
  int n_views, nu, nv, nx, ny, nz;
  int s_begin, s_end;
  int mask_r2;           // <=0: no mask
  int cs, ct, cz;        // mask centre
  int flags;
  float x0, y0, z0, dvox;
  float sdd, D;
  float half_u, half_v;
  float inv_du, inv_dv;
  float xmax, ymax;      // accepted detector coordinate ranges [0,xmax], [0,ymax]
};

FdkDev make_fdk_dev(const monte_fdk_geom& g);

// Kernel launchers (return cudaGetLastError()).
cudaError_t launch_fdk_filter_fp32(const FdkDev& d, const float* proj, const float* weights,
                                   const float* taps_half, float* filtered, cudaStream_t st);
cudaError_t launch_fdk_filter_bf16x3(const FdkDev& d, const float* proj, const float* weights,
                                     const uint16_t* bsplit, float* filtered, int* status,
                                     int sm_count, cudaStream_t st);
// Size in bytes of the pre-split, pre-tiled B operand of the BF16x3 filter.
size_t bf16x3_bsplit_bytes(int nu);
// Fill `out` (host) with the pre-split Toeplitz operand for the BF16x3 filter.
void bf16x3_build_bsplit(int nu, const float* taps_half, uint16_t* out);
bool bf16x3_supported(const FdkDev& d);

cudaError_t launch_fdk_bp_plain(const FdkDev& d, const BpView* views, const float* filtered,
                                float* vol_xy, float* vol_zy, cudaStream_t st);
cudaError_t launch_fdk_bp_tiled(const FdkDev& d, const BpView* views, const float* filtered,
                                float* vol_xy, float* vol_zy, int variant, cudaStream_t st);
int fdk_bp_tiled_variants();
bool fdk_bp_tiled_supported(const FdkDev& d, int variant);

#ifdef __CUDACC__
// Shared by the plain and tiled kernels: bilinear read of filtered[view]
// at detector coordinates (x: v row, y: u column), with the reference's
// flat-array semantics for neighbours past the last row/column.
__device__ __forceinline__ float bp_fetch(const float* __restrict__ f, size_t total, size_t idx,
                                          bool ok) {
  return (ok && idx < total) ? __ldg(f + idx) : 0.f;
}

__device__ __forceinline__ float bp_bilinear_global(const FdkDev& d, const float* __restrict__ f,
                                                    int k, float x, float y) {
  const size_t total = (size_t)d.n_views * d.nu * d.nv;
  int xi = (int)x, yi = (int)y;
  float fx = x - (float)xi, fy = y - (float)yi;
  size_t i00 = (size_t)k * d.nu * d.nv + (size_t)xi * d.nu + yi;
  bool flat = (d.flags & MONTE_FDK_FLAT_EDGE) != 0;
  float f00 = bp_fetch(f, total, i00, flat || (xi < d.nv && yi < d.nu));
  float f10 = bp_fetch(f, total, i00 + d.nu, flat || (xi + 1 < d.nv && yi < d.nu));
  float f01 = bp_fetch(f, total, i00 + 1, flat || (xi < d.nv && yi + 1 < d.nu));
  float f11 = bp_fetch(f, total, i00 + d.nu + 1, flat || (xi + 1 < d.nv && yi + 1 < d.nu));
  float r0 = fmaf(fx, f10 - f00, f00);
  float r1 = fmaf(fx, f11 - f01, f01);
  return fmaf(fy, r1 - r0, r0);
}

#endif

}  // namespace monte
