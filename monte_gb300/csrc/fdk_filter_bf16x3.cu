// fdk_filter_bf16x3.cu -- cosine weighting + Ram-Lak ramp filter on the
// 5th-generation tensor cores (tcgen05, accumulators in TMEM).
//
// Reference: recon/bp3d20.cpp:36-73.  Over all detector rows of all views
// the filter is one GEMM
//     Q[(n,v)][b] = sum_c A[(n,v)][c] * T[c][b],
//     A[(n,v)][c] = P[n][c][v] * w[c][v],   T[c][b] = 0.5 * h[c-b]
// with M = n_views * nv, N = K = nu.
//
// Precision.  A and T are split into BF16 pairs (x = hi + lo) and the far
// field is accumulated as hi*hi + hi*lo + lo*hi in FP32 (three MMAs per K
// step).  A pair carries ~16 significant bits, and the ramp filter cancels
// a large DC term, so the split alone would leave ~1e-4 relative error in
// the filtered rows.  The near-diagonal band |c - b| <= 16 (17 nonzero taps,
// which carry that cancellation) is therefore removed from the tensor-core
// operand and applied exactly in FP32 in the epilogue, from the same FP32
// A values.  Result: FP32-level error (the FDK volume stays within 1e-5
// relative RMS of the FP64 oracle).
//
// Kernel shape.  One CTA computes a 128 x BN output tile (128 detector rows
// of one view, BN columns) over K = nu in chunks of 32, in 96 KB of shared
// memory and BN TMEM columns, so that two CTAs share an SM (one converts
// while the other's MMAs or epilogue run):
//  * all 8 warps load the A chunk (fp32, coalesced along v), weight it,
//    split it and store hi/lo into shared memory in the canonical K-major
//    core-matrix layout (8 rows x 16 bytes per core matrix);
//  * thread 0 brings the pre-split, pre-tiled B chunk (host-built, band
//    removed) with two cp.async.bulk copies on an mbarrier, then issues the
//    6 tcgen05.mma of the chunk (3 per 16-wide K step) and commits them to a second mbarrier;
//  * two stages alternate, so the conversion of chunk k+1 overlaps the MMAs
//    of chunk k;
//  * epilogue, per window of 64 output columns: tcgen05.ld of the
//    accumulator rows, plus the FP32 band from an fp32 copy of the window's
//    A columns (and 16 either side) staged in the (now idle) shared memory,
//    then float4 stores of the transposed output filtered[view][v][u].
// Every wait is bounded; on timeout the CTA sets *status, drains and frees
// its TMEM.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "fdk.cuh"
#include "ptx.cuh"

namespace monte {

namespace {

constexpr int KC = 32;        // K per chunk
constexpr int KBAND = 16;     // near field |c - b| <= KBAND handled in FP32
constexpr int NTHREADS = 256;

__host__ __device__ inline int bn_for(int nu) {
  return (nu % 256 == 0) ? 256 : (nu % 128 == 0) ? 128 : 64;
}

struct BandTaps {
  float t[2 * KBAND + 1];  // T at offsets -KBAND..KBAND
};

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

template <int BN>
__global__ void __launch_bounds__(NTHREADS, 2)
    filter_bf16x3_kernel(int nu, int nv, const float* __restrict__ proj,
                         const float* __restrict__ weights, const uint16_t* __restrict__ bsplit,
                         const BandTaps band, float* __restrict__ out, int* status) {
  constexpr int A_BYTES = 128 * KC * 2;        // one of hi / lo
  constexpr int B_BYTES = BN * KC * 2;         // one of hi / lo
  constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;
  constexpr uint32_t IDESC = ptx::idesc_bf16_f32(128, BN);
  constexpr int WC = 64;                           // output columns per epilogue window
  constexpr int KW = WC + 2 * KBAND;               // A columns staged per window
  constexpr int EPI = KW * 128 * 4;                // fp32 A rows for the band
  constexpr int BAR_OFF = 2 * STAGE > EPI ? 2 * STAGE : EPI;
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + BAR_OFF);  // b_full[2], mma_done[2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 4);

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int nt = blockIdx.x;  // N tile
  const int b0 = nt * BN;
  const long long row0 = (long long)blockIdx.y * 128;  // global row (n, v)
  const int n = (int)(row0 / nv);
  const int v0 = (int)(row0 - (long long)n * nv);
  const float* P = proj + (size_t)n * nu * nv;
  const int nchunks = nu / KC;

  if (tid == 0) {
    for (int i = 0; i < 4; i++) ptx::mbar_init(&bars[i], 1);
    ptx::fence_barrier_init();
  }
  if (warp == 0) {
    ptx::tmem_alloc(tmem_slot, BN);
    ptx::tmem_relinquish();
  }
  ptx::tc_fence_before();
  __syncthreads();
  ptx::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int m = tid & 127;   // A row owned during conversion
  const int khalf = tid >> 7;
  bool ok = true;

  // This thread's A elements of a chunk (row m, columns c0 + 8 j + e of its
  // KC/16 k-cores j), loaded one chunk ahead: the loads of chunk k + 1 are
  // in flight while chunk k is split, its B copy waited for and its MMAs
  // issued, instead of each chunk waiting a full L2 round trip.
  constexpr int NE = KC / 2;
  float pp[NE], pw[NE];
  const float* Pm = P + v0 + m;
  const float* Wm = weights + v0 + m;
  auto load_chunk = [&](int kc) {
#pragma unroll
    for (int jj = 0; jj < KC / 16; jj++)
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const size_t c = (size_t)(kc * KC + 8 * (khalf * (KC / 16) + jj) + e);
        pp[jj * 8 + e] = __ldg(Pm + c * nv);
        pw[jj * 8 + e] = __ldg(Wm + c * nv);
      }
  };
  load_chunk(0);

  for (int kc = 0; kc < nchunks && ok; kc++) {
    const int s = kc & 1;
    const uint32_t use = (uint32_t)(kc >> 1);
    unsigned char* st = smem + s * STAGE;
    unsigned char* a_hi = st;
    unsigned char* a_lo = st + A_BYTES;
    unsigned char* b_hi = st + 2 * A_BYTES;
    unsigned char* b_lo = st + 2 * A_BYTES + B_BYTES;
    if (kc >= 2) {  // MMAs that read this stage two chunks ago must be done
      bool w = ptx::mbar_wait(&bars[2 + s], (use - 1) & 1);
      if (!__syncthreads_and(w)) {
        ok = false;
        break;
      }
    }
    if (tid == 0) {
      const uint16_t* src = bsplit + ((size_t)kc * (nu / BN) + nt) * (2 * BN * KC);
      ptx::mbar_arrive_expect_tx(&bars[s], 2 * B_BYTES);
      ptx::bulk_load(b_hi, src, B_BYTES, &bars[s]);
      ptx::bulk_load(b_lo, src + BN * KC, B_BYTES, &bars[s]);
    }
    // ---- A chunk: weight, split, store as K-major core matrices ----------
#pragma unroll
    for (int jj = 0; jj < KC / 16; jj++) {
      const int j = khalf * (KC / 16) + jj;  // k-core within the chunk
      float a[8];
#pragma unroll
      for (int e = 0; e < 8; e++) a[e] = pp[jj * 8 + e] * pw[jj * 8 + e];
      uint32_t hi[4], lo[4];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        __nv_bfloat16 h0 = __float2bfloat16_rn(a[2 * e]);
        __nv_bfloat16 h1 = __float2bfloat16_rn(a[2 * e + 1]);
        float r0 = a[2 * e] - __bfloat162float(h0);
        float r1 = a[2 * e + 1] - __bfloat162float(h1);
        __nv_bfloat162 hh;
        hh.x = h0;
        hh.y = h1;
        hi[e] = *reinterpret_cast<uint32_t*>(&hh);
        lo[e] = pack_bf16(r0, r1);
      }
      const int off = (j * 16 + (m >> 3)) * 128 + (m & 7) * 16;
      *reinterpret_cast<uint4*>(a_hi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4*>(a_lo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
    if (kc + 1 < nchunks) load_chunk(kc + 1);
    ptx::fence_proxy_async_smem();
    bool w = ptx::mbar_wait(&bars[s], use & 1);  // B chunk landed
    if (!__syncthreads_and(w)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      ptx::tc_fence_after();
      const uint32_t ah = ptx::smem_addr(a_hi), al = ptx::smem_addr(a_lo);
      const uint32_t bh = ptx::smem_addr(b_hi), bl = ptx::smem_addr(b_lo);
#pragma unroll
      for (int ks = 0; ks < KC / 16; ks++) {
        const uint32_t ao = ks * 2 * 2048, bo = ks * 2 * (BN * 16);
        const uint64_t dah = ptx::smem_desc(ah + ao, 2048, 128);
        const uint64_t dal = ptx::smem_desc(al + ao, 2048, 128);
        const uint64_t dbh = ptx::smem_desc(bh + bo, BN * 16, 128);
        const uint64_t dbl = ptx::smem_desc(bl + bo, BN * 16, 128);
        const uint32_t acc0 = (kc > 0 || ks > 0) ? 1u : 0u;
        ptx::mma_bf16(tmem, dah, dbh, IDESC, acc0);
        ptx::mma_bf16(tmem, dah, dbl, IDESC, 1u);
        ptx::mma_bf16(tmem, dal, dbh, IDESC, 1u);
      }
      ptx::mma_commit(&bars[2 + s]);
    }
  }
  // all MMAs done (the last commit covers every earlier one)
  if (ok) {
    const int kl = nchunks - 1;
    bool w = ptx::mbar_wait(&bars[2 + (kl & 1)], (uint32_t)(kl >> 1) & 1);
    ok = __syncthreads_and(w);
  }
  ptx::tc_fence_after();
  if (ok) {
    // ---- epilogue, per window of WC output columns: stage the fp32 A
    // columns the window's band reads, As[k][m] with c = b0 + wc - KBAND + k,
    // then TMEM rows + FP32 band -> filtered[n][v][b] ----------------------
    float* As = reinterpret_cast<float*>(smem);
    const int q = warp & 3, h = warp >> 2;
    const int row = 32 * q + lane;
    float* orow = out + ((size_t)n * nv + v0 + row) * nu + b0;
#pragma unroll 1
    for (int wc = 0; wc < BN; wc += WC) {
      if (wc > 0) __syncthreads();  // every warp is done with the last window
      for (int k = khalf; k < KW; k += 2) {
        const int c = b0 + wc - KBAND + k;
        float val = 0.f;
        if (c >= 0 && c < nu) {
          const size_t idx = (size_t)c * nv + v0 + m;
          val = __ldg(P + idx) * __ldg(weights + idx);
        }
        As[k * 128 + m] = val;
      }
      __syncthreads();
      const int col0 = wc + h * 32;  // this warp's 32 output columns
      float r[32];
      ptx::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)col0, r);
      float win[32 + 2 * KBAND];
#pragma unroll
      for (int k = 0; k < 32 + 2 * KBAND; k++) win[k] = As[(h * 32 + k) * 128 + row];
#pragma unroll
      for (int i = 0; i < 32; i++) {
        float acc = r[i];
#pragma unroll
        for (int jo = -KBAND; jo <= KBAND; jo++) {
          if (jo != 0 && (jo & 1) == 0) continue;  // even taps are zero
          acc = fmaf(band.t[jo + KBAND], win[i + jo + KBAND], acc);
        }
        r[i] = acc;
      }
#pragma unroll
      for (int i = 0; i < 32; i += 4)
        *reinterpret_cast<float4*>(orow + col0 + i) = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
    }
  } else if (tid == 0) {
    atomicExch(status, 2);
    // drain: the last commit issued covers every outstanding MMA
    ptx::mbar_wait(&bars[2], 0);
    ptx::mbar_wait(&bars[3], 0);
  }
  ptx::tc_fence_before();
  __syncthreads();
  if (warp == 0) ptx::tmem_dealloc(tmem, BN);
}

size_t smem_for(int bn) {
  size_t stage = 2 * (128 * KC * 2) + 2 * ((size_t)bn * KC * 2);
  size_t epi = (size_t)(64 + 2 * KBAND) * 128 * 4;
  size_t main = 2 * stage;
  return (main > epi ? main : epi) + 64;
}

uint16_t f2bf_rne(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
float bf2f(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

}  // namespace

size_t bf16x3_bsplit_bytes(int nu) { return (size_t)nu * nu * 2 * sizeof(uint16_t); }

// B operand: for chunk kc and N tile nt, [hi | lo], each BN x 64 in K-major
// core matrices: element (k, col) at ((k/8)*(BN/8) + col/8)*64 + (col%8)*8 + k%8.
void bf16x3_build_bsplit(int nu, const float* taps_half, uint16_t* out) {
  const int bn = bn_for(nu);
  const int ntiles = nu / bn;
  for (int kc = 0; kc < nu / KC; kc++)
    for (int nt = 0; nt < ntiles; nt++) {
      uint16_t* blk = out + ((size_t)kc * ntiles + nt) * (2 * (size_t)bn * KC);
      for (int k = 0; k < KC; k++)
        for (int col = 0; col < bn; col++) {
          int c = kc * KC + k, b = nt * bn + col;
          float t = (std::abs(c - b) <= KBAND) ? 0.f : taps_half[c - b + nu - 1];
          uint16_t h = f2bf_rne(t);
          uint16_t l = f2bf_rne(t - bf2f(h));
          size_t off = ((size_t)(k / 8) * (bn / 8) + col / 8) * 64 + (col % 8) * 8 + (k % 8);
          blk[off] = h;
          blk[(size_t)bn * KC + off] = l;
        }
    }
}

bool bf16x3_supported(const FdkDev& d) {
  if (d.nu % 64 != 0 || d.nv % 128 != 0) return false;  // N tiles of 64, 128, 256 columns
  int dev = 0, major = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return major >= 10 && smem_for(bn_for(d.nu)) <= (size_t)optin;
}

cudaError_t launch_fdk_filter_bf16x3(const FdkDev& d, const float* proj, const float* weights,
                                     const uint16_t* bsplit, float* filtered, int* status,
                                     int sm_count, cudaStream_t st) {
  (void)sm_count;
  // band taps (the same float values the FP32 filter uses)
  BandTaps band;
  for (int j = -KBAND; j <= KBAND; j++) {
    float h = 0.f;
    int a = j < 0 ? -j : j;
    if (a == 0) {
      h = 0.25f;
    } else if (a % 2 == 1) {
      double x = a * M_PI;
      h = (float)(-1. / (x * x));
    }
    band.t[j + KBAND] = 0.5f * h;
  }
  const int bn = bn_for(d.nu);
  dim3 grid(d.nu / bn, (unsigned)(((long long)d.n_views * d.nv) / 128));
  size_t smem = smem_for(bn);
  cudaError_t e;
  switch (bn) {
    case 256:
      e = cudaFuncSetAttribute(filter_bf16x3_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      filter_bf16x3_kernel<256><<<grid, NTHREADS, smem, st>>>(d.nu, d.nv, proj, weights, bsplit, band, filtered, status);
      break;
    case 128:
      e = cudaFuncSetAttribute(filter_bf16x3_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      filter_bf16x3_kernel<128><<<grid, NTHREADS, smem, st>>>(d.nu, d.nv, proj, weights, bsplit, band, filtered, status);
      break;
    default:
      e = cudaFuncSetAttribute(filter_bf16x3_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      filter_bf16x3_kernel<64><<<grid, NTHREADS, smem, st>>>(d.nu, d.nv, proj, weights, bsplit, band, filtered, status);
      break;
  }
  return cudaGetLastError();
}

}  // namespace monte
