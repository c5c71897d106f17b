// fdk_filter_fp32.cu -- cosine weighting + Ram-Lak ramp filter on the FP32
// CUDA cores.
//
// Reference: recon/bp3d20.cpp:36-73 (weights :40, taps :48-60, convolution
// :63-73).  The convolution along the in-plane detector axis u is a
// Toeplitz product per view:
//
//     Q_n[v][b] = sum_c  (P_n[c][v] * w[c][v]) * 0.5*h[c-b]
//
// with the output transposed to [view][v][u] as the reference writes it.
// This kernel runs it as a tiled SIMT GEMM (M = v rows, N = b, K = c), the
// weight applied while the A tile is staged, the Toeplitz tile generated
// from the tap vector.  It is the "plain FP32" filter; fdk_filter_bf16x3.cu
// holds the tensor-core variant.
#include "fdk.cuh"

namespace monte {
namespace {

constexpr int TM = 64;   // v rows per CTA
constexpr int TN = 64;   // b columns per CTA
constexpr int TK = 16;   // c per stage

__global__ void __launch_bounds__(256) filter_fp32_kernel(int nu, int nv,
                                                          const float* __restrict__ proj,
                                                          const float* __restrict__ weights,
                                                          const float* __restrict__ taps_half,
                                                          float* __restrict__ out) {
  __shared__ __align__(16) float As[TK][TM];
  __shared__ __align__(16) float Bs[TK][TN];
  const int n = blockIdx.z;
  const int v0 = blockIdx.y * TM;
  const int b0 = blockIdx.x * TN;
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const float* P = proj + (size_t)n * nu * nv;
  float acc[4][4] = {};
  for (int c0 = 0; c0 < nu; c0 += TK) {
#pragma unroll
    for (int i = 0; i < (TK * TM) / 256; i++) {
      int e = tid + i * 256;
      int r = e / TM, col = e % TM;
      int c = c0 + r, v = v0 + col;
      float a = 0.f;
      if (c < nu && v < nv) a = P[(size_t)c * nv + v] * weights[(size_t)c * nv + v];
      As[r][col] = a;
      int b = b0 + col;
      float t = 0.f;
      if (c < nu && b < nu) t = taps_half[c - b + nu - 1];
      Bs[r][col] = t;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      float4 a4 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      float4 b4 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      float a[4] = {a4.x, a4.y, a4.z, a4.w};
      float b[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* Q = out + (size_t)n * nu * nv;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int v = v0 + ty * 4 + i;
    if (v >= nv) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int b = b0 + tx * 4 + j;
      if (b < nu) Q[(size_t)v * nu + b] = acc[i][j];
    }
  }
}

}  // namespace

cudaError_t launch_fdk_filter_fp32(const FdkDev& d, const float* proj, const float* weights,
                                   const float* taps_half, float* filtered, cudaStream_t st) {
  dim3 grid((d.nu + TN - 1) / TN, (d.nv + TM - 1) / TM, d.n_views);
  filter_fp32_kernel<<<grid, 256, 0, st>>>(d.nu, d.nv, proj, weights, taps_half, filtered);
  return cudaGetLastError();
}

}  // namespace monte
