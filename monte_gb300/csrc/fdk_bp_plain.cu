// fdk_bp_plain.cu -- voxel-driven cone-beam backprojection, plain form.
//
// Reference: recon/bp3d20.cpp:81-166 (recon/bp3d20_325.cpp:93-172).  One
// thread per voxel loops over all views; each view maps the voxel onto the
// detector (rotate by -beta, magnify to the detector plane, :95-126),
// applies the distance weight D^2/(D-d)^2 (:134-142,159) and bilinearly
// interpolates the filtered projection (:152-158).  Projections are read
// straight from global memory through L1/L2.  This is the one-instance FP32
// baseline the tiled backprojector (fdk_bp_tiled.cu) is measured against.
#include "fdk.cuh"

namespace monte {

namespace {

__global__ void __launch_bounds__(256) bp_plain_kernel(FdkDev d, const BpView* __restrict__ views,
                                                       const BpViewD* __restrict__ viewsd,
                                                       const float* __restrict__ filtered,
                                                       float* __restrict__ vol_xy,
                                                       float* __restrict__ vol_zy) {
  const int ws = d.s_end - d.s_begin;
  const size_t n_vox = (size_t)ws * d.ny * d.nz;
  size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_vox) return;
  const int s = d.s_begin + (int)(idx % ws);
  const int t = (int)((idx / ws) % d.ny);
  const int z = (int)(idx / ((size_t)ws * d.ny));
  float acc = 0.f;
  bool inside = true;
  if (d.mask_r2 > 0) {
    int a = z - d.cz, b = t - d.ct, c = s - d.cs;
    inside = a * a + b * b + c * c <= d.mask_r2;
  }
  if (inside) {
    const float X = fmaf((float)s, d.dvox, d.x0);
    const float Y = fmaf(-(float)t, d.dvox, d.y0);
    const Fpair m = bp_zterm(d, z);
    for (int k = 0; k < d.n_views; k++) {
      const BpView v = views[k];
      int xi, yi;
      float fx, fy, w;
      if (!bp_coef(d, v, viewsd[k], s, t, z, X, Y, m, &xi, &yi, &fx, &fy, &w)) continue;
      float val = bp_bilinear_at(d, filtered, k, xi, yi, fx, fy);
      acc = fmaf(w * val, v.factor, acc);
    }
  }
  vol_xy[((size_t)z * d.ny + t) * d.nx + s] = acc;
  if (vol_zy) vol_zy[((size_t)s * d.ny + t) * d.nz + z] = acc;
}

}  // namespace

cudaError_t launch_fdk_bp_plain(const FdkDev& d, const BpView* views, const BpViewD* viewsd,
                                const float* filtered, float* vol_xy, float* vol_zy,
                                cudaStream_t st) {
  const size_t n_vox = (size_t)(d.s_end - d.s_begin) * d.ny * d.nz;
  if (n_vox == 0) return cudaSuccess;
  unsigned blocks = (unsigned)((n_vox + 255) / 256);
  bp_plain_kernel<<<blocks, 256, 0, st>>>(d, views, viewsd, filtered, vol_xy, vol_zy);
  return cudaGetLastError();
}

}  // namespace monte
