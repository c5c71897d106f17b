// fdk_adjoint.cu -- exact adjoints of the FDK operator for the
// differentiable mode.
//
//  * Forward projector = transpose of the voxel-driven backprojection
//    (recon/bp3d20.cpp:81-166): G[k][row][col] = sum over voxels of
//    w * factor * (bilinear weight of (row, col)) * R[z][t][s], with the
//    coefficients of bp_column + bp_coef_z, the operations the plain
//    backprojector's bp_coef performs.  A CTA owns one view and a block of
//    32 detector columns; it enumerates the voxel columns in the wedge of
//    source rays that project onto them (for each voxel row along the
//    view's major axis, the range along the other axis follows from the
//    perspective map).  A warp takes one voxel column at a time with its
//    lanes along z: the column's part of the coefficients is computed once,
//    the lanes read 32 consecutive voxels of a z-major copy of the volume,
//    and scatter into consecutive detector rows of a column-major shared
//    accumulator (different banks), stored once, coalesced, at the end.
//  * Adjoint of the weighting + ramp filter (recon/bp3d20.cpp:36-73): the
//    Toeplitz matrix is symmetric, so the transpose filters along u again,
//    reading [view][v][u] and writing [view][u][v], then applies the cosine
//    weight.
#include "fdk.cuh"

namespace monte {
namespace {

constexpr int FP_COLS = 32;    // detector columns per CTA
constexpr int FP_THREADS = 256;

// vol_z: the volume transposed to [s][t][z] (z contiguous).
__global__ void __launch_bounds__(FP_THREADS) fp_kernel(FdkDev d, const BpView* __restrict__ views,
                                                        const BpViewD* __restrict__ viewsd,
                                                        const float* __restrict__ vol,
                                                        const float* __restrict__ vol_z,
                                                        const unsigned char* __restrict__ occ,
                                                        float* __restrict__ out) {
  extern __shared__ float G[];  // [FP_COLS][nv]: column-major, then nz z-terms
  Fpair* zterm = reinterpret_cast<Fpair*>(G + FP_COLS * d.nv);
  const int k = blockIdx.y;
  const int c0 = blockIdx.x * FP_COLS;
  const int ncols = min(FP_COLS, d.nu - c0);
  for (int i = threadIdx.x; i < d.nv * FP_COLS; i += FP_THREADS) G[i] = 0.f;
  for (int z = threadIdx.x; z < d.nz; z += FP_THREADS) zterm[z] = bp_zterm(d, z);
  __syncthreads();
  const BpView v = views[k];
  const BpViewD& vd = viewsd[k];
  // u' range of the detector columns [c0 - 1, c0 + ncols] (one column of
  // margin either side), as y = (half_u - u') / du
  const float ua = d.half_u - (float)(c0 + ncols + 1) * (1.0f / d.inv_du);
  const float ub = d.half_u - (float)(c0 - 2) * (1.0f / d.inv_du);
  const bool x_major = fabsf(v.c) >= fabsf(v.s);
  const int n_major = x_major ? (d.s_end - d.s_begin) : d.ny;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int m = warp; m < n_major; m += FP_THREADS / 32) {
    // minor-axis range of the wedge on this voxel row
    int lo, hi;
    if (x_major) {
      const int s = d.s_begin + m;
      const float X = fmaf((float)s, d.dvox, d.x0);
      const float ax = X - v.px;
      float Ys[2];
      for (int e = 0; e < 2; e++) {
        float u = e ? ub : ua;
        float den = u * v.s - d.sdd * v.c;
        Ys[e] = v.py - ax * (u * v.c + d.sdd * v.s) / den;
      }
      float tA = (d.y0 - Ys[0]) / d.dvox, tB = (d.y0 - Ys[1]) / d.dvox;
      lo = max((int)floorf(fminf(tA, tB)) - 2, 0);
      hi = min((int)ceilf(fmaxf(tA, tB)) + 2, d.ny - 1);
    } else {
      const int t = m;
      const float Y = fmaf(-(float)t, d.dvox, d.y0);
      const float ay = Y - v.py;
      float Xs[2];
      for (int e = 0; e < 2; e++) {
        float u = e ? ub : ua;
        float den = u * v.c + d.sdd * v.s;
        Xs[e] = v.px - ay * (u * v.s - d.sdd * v.c) / den;
      }
      float sA = (Xs[0] - d.x0) / d.dvox, sB = (Xs[1] - d.x0) / d.dvox;
      lo = max((int)floorf(fminf(sA, sB)) - 2, d.s_begin);
      hi = min((int)ceilf(fmaxf(sA, sB)) + 2, d.s_end - 1);
    }
    for (int q = lo; q <= hi; q++) {  // warp-uniform: one voxel column at a time
      const int s = x_major ? d.s_begin + m : q;
      const int t = x_major ? q : m;
      if (!occ[(size_t)s * d.ny + t]) continue;  // an empty voxel column adds nothing
      const float X = fmaf((float)s, d.dvox, d.x0);
      const float Y = fmaf(-(float)t, d.dvox, d.y0);
      // the column's part of the coefficients, once; does it project near
      // our detector columns (margin 2)?
      BpColumn col;
      bp_column(d, v, vd, s, t, X, Y, &col);
      if (!(col.y >= (float)(c0 - 2) && col.y < (float)(c0 + ncols + 1))) continue;
      const float* src = vol_z + ((size_t)s * d.ny + t) * d.nz;
      for (int z = lane; z < d.nz; z += 32) {
        if (d.mask_r2 > 0) {
          int a = z - d.cz, b = t - d.ct, c = s - d.cs;
          if (a * a + b * b + c * c > d.mask_r2) continue;
        }
        // an empty voxel contributes nothing: skip it before its
        // coefficients (most voxels of a phantom in air are empty)
        const float r = __ldg(src + z);
        if (r == 0.f) continue;
        int xi, yi;
        float fx, fy, w;
        if (!bp_coef_z(d, col, vd, s, t, z, zterm[z], &xi, &yi, &fx, &fy, &w)) continue;
        const float c = w * r * v.factor;
#pragma unroll
        for (int dy = 0; dy < 2; dy++) {
          const int cl = yi + dy - c0;
          if (cl < 0 || cl >= ncols || yi + dy >= d.nu) continue;
          const float wy = dy ? fy : 1.f - fy;
#pragma unroll
          for (int dx = 0; dx < 2; dx++) {
            const int row = xi + dx;
            if (row >= d.nv) continue;
            const float wx = dx ? fx : 1.f - fx;
            atomicAdd(&G[cl * d.nv + row], c * wx * wy);
          }
        }
      }
    }
  }
  __syncthreads();
  float* dst = out + (size_t)k * d.nu * d.nv;
  for (int i = threadIdx.x; i < d.nv * FP_COLS; i += FP_THREADS) {
    int row = i / FP_COLS, cl = i % FP_COLS;
    if (cl < ncols) dst[(size_t)row * d.nu + c0 + cl] = G[cl * d.nv + row];
  }
}

// occ[s][t] = whether voxel column (s, t) of the z-major volume holds a
// nonzero voxel (a warp per column)
__global__ void column_occupancy_kernel(int ncols, int nz, const float* __restrict__ vol_z,
                                        unsigned char* __restrict__ occ) {
  const int col = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (col >= ncols) return;  // warp-uniform
  const float* c = vol_z + (size_t)col * nz;
  bool any = false;
  for (int z = lane; z < nz && !any; z += 32) any = c[z] != 0.f;
  any = __any_sync(0xffffffffu, any);
  if (lane == 0) occ[col] = any ? 1 : 0;
}

// out[s][t][z] = in[z][t][s]: per t, a 32 x 32 tile of the (z, s) plane
// through shared memory, read along s and written along z
__global__ void transpose_zs_kernel(int nx, int ny, int nz, const float* __restrict__ in,
                                    float* __restrict__ out) {
  __shared__ float tile[32][33];
  const int t = blockIdx.z;
  const int s0 = blockIdx.x * 32, z0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int z = z0 + i, s = s0 + threadIdx.x;
    if (z < nz && s < nx) tile[i][threadIdx.x] = in[((size_t)z * ny + t) * nx + s];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += 8) {
    const int s = s0 + i, z = z0 + threadIdx.x;
    if (z < nz && s < nx) out[((size_t)s * ny + t) * nz + z] = tile[threadIdx.x][i];
  }
}

// H[n][c][v] = w[c][v] * sum_b T[b][c] * G[n][v][b]  (T symmetric)
constexpr int TM = 64, TN = 64, TK = 16;
__global__ void __launch_bounds__(256) filter_adjoint_kernel(int nu, int nv,
                                                             const float* __restrict__ g,
                                                             const float* __restrict__ weights,
                                                             const float* __restrict__ taps_half,
                                                             float* __restrict__ h) {
  __shared__ __align__(16) float As[TK][TM];  // [b][v]
  __shared__ __align__(16) float Bs[TK][TN];  // [b][c]
  const int n = blockIdx.z;
  const int v0 = blockIdx.y * TM;
  const int c0 = blockIdx.x * TN;
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const float* G = g + (size_t)n * nu * nv;
  float acc[4][4] = {};
  for (int b0 = 0; b0 < nu; b0 += TK) {
#pragma unroll
    for (int i = 0; i < (TK * TM) / 256; i++) {
      int e = tid + i * 256;
      int r = e % TK, col = e / TK;  // r: b offset (fastest in memory), col: v
      int b = b0 + r, v = v0 + col;
      As[r][col] = (b < nu && v < nv) ? G[(size_t)v * nu + b] : 0.f;
      int e2 = tid + i * 256;
      int r2 = e2 / TN, cc = e2 % TN;
      int bb = b0 + r2, c = c0 + cc;
      Bs[r2][cc] = (bb < nu && c < nu) ? taps_half[bb - c + nu - 1] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      float4 a4 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      float4 b4 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      float a[4] = {a4.x, a4.y, a4.z, a4.w};
      float bb[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* H = h + (size_t)n * nu * nv;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    int c = c0 + tx * 4 + j;
    if (c >= nu) continue;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      int v = v0 + ty * 4 + i;
      if (v < nv) H[(size_t)c * nv + v] = acc[i][j] * weights[(size_t)c * nv + v];
    }
  }
}

}  // namespace

cudaError_t launch_fdk_forward_project(const FdkDev& d, const BpView* views, const BpViewD* viewsd,
                                       const float* vol, float* vol_z, float* out,
                                       cudaStream_t st) {
  if (!vol_z) return cudaErrorInvalidValue;
  dim3 tg((d.nx + 31) / 32, (d.nz + 31) / 32, d.ny);
  transpose_zs_kernel<<<tg, dim3(32, 8), 0, st>>>(d.nx, d.ny, d.nz, vol, vol_z);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  unsigned char* occ = reinterpret_cast<unsigned char*>(vol_z + (size_t)d.nx * d.ny * d.nz);
  const int ncols = d.nx * d.ny;
  column_occupancy_kernel<<<(unsigned)((ncols * 32ull + 255) / 256), 256, 0, st>>>(ncols, d.nz,
                                                                                 vol_z, occ);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  size_t smem = (size_t)d.nv * FP_COLS * sizeof(float) + (size_t)d.nz * sizeof(Fpair);
  e = cudaFuncSetAttribute(fp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((d.nu + FP_COLS - 1) / FP_COLS, d.n_views);
  fp_kernel<<<grid, FP_THREADS, smem, st>>>(d, views, viewsd, vol, vol_z, occ, out);
  return cudaGetLastError();
}

cudaError_t launch_fdk_filter_adjoint(const FdkDev& d, const float* g, const float* weights,
                                      const float* taps_half, float* h, cudaStream_t st) {
  dim3 grid((d.nu + TN - 1) / TN, (d.nv + TM - 1) / TM, d.n_views);
  filter_adjoint_kernel<<<grid, 256, 0, st>>>(d.nu, d.nv, g, weights, taps_half, h);
  return cudaGetLastError();
}

}  // namespace monte
