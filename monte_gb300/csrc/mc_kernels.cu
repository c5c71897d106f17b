// mc_kernels.cu -- photon-history Monte Carlo kernels for sm_103a.
//
// Reference kernel: `projection` of monte_cu/CBCT_real325im.cu:425-860 --
// one thread per detector pixel runs every view and every history of that
// pixel in sequence, so a warp waits for its longest history at every
// history boundary (a primary ends after one flight, a scattered photon
// after up to five interactions and hundreds of Woodcock steps).
//
//  * mc_plain_kernel: the same launch shape (one thread per emitting pixel,
//    views x histories in sequence), the FP32 one-instance baseline.
//  * mc_persistent_kernel: persistent warps over a global history counter.
//    A lane whose photon ends takes the next history at once: the warp
//    ballots its idle lanes, ranks them with popc and hands them
//    consecutive history ids from a per-warp chunk claimed with one atomic.
//    Flights advance a few Woodcock steps per round; lanes that reach a
//    real collision wait until enough of the warp has one (or no lane is
//    flying), so the divergent interaction code runs on a compacted set.
//    Tallies are warp-aggregated: lanes that hit the same pixel are grouped
//    with __match_any_sync and one leader adds the group's count.
//  * mc_finalize_kernel: the reference's host post-processing
//    (CBCT_real325im.cu:261-294) -- clamp, then -ln N + ln per in FP64.
//
// Every history draws from its own Philox stream (monte_rng.h) and runs the
// step functions of mc_physics.h, so both kernels produce bit-identical
// int64 tallies, equal to the CPU replay harness's.
#include <cuda_runtime.h>

#include "mc.cuh"

namespace monte {

namespace {

constexpr int kChunk = 64;          // histories claimed per warp atomic
constexpr int kStepsPerRound = 16;  // flight steps per round, single majorant
// With local majorants a flight is fewer, cheaper steps (tentative
// collisions and majorant legs), and lanes that have landed wait less for
// the warp's longest flight in shorter rounds: 8 steps measured 8.5 %
// faster than 16 on the 325^3 workload (32: 16 % slower).
constexpr int kStepsPerRoundLocal = 8;
constexpr int kCollideBatch = 2;    // interact once this many lanes wait (2: 1.6 % over 4)

// Before a flight step: a lane within one draw of the end of its random
// block (a step draws at most twice: the next exponential and the
// Woodcock test) makes every active lane without a prefetched block
// compute its next one (monte_stream_prefetch), so that the warp runs the
// Philox rounds once for many lanes, several steps apart, instead of in
// nearly every step for the lane or two whose block ran out.
__device__ __forceinline__ void prefetch_draws(mc_photon& p, const monte_philox_keys& K) {
  const unsigned act = __activemask();
  const uint32_t w = p.rng.next & 3u;
  const bool ready = (p.rng.pf & 1u) != 0u;
  if (__any_sync(act, !ready && (w == 0u || w == 3u)) && !ready) monte_stream_prefetch(&p.rng, &K);
}

// This thread's 16-byte prefetch slot in the CTA's shared array.
__device__ __forceinline__ uint32_t draw_slot(uint4* slots) {
  return (uint32_t)__cvta_generic_to_shared(slots + threadIdx.x);
}

__device__ __forceinline__ void decompose(const McDev& d, unsigned long long h, int* view,
                                          int* iu, int* iv, unsigned long long* k) {
  const unsigned long long per = d.P.per;
  const unsigned nv_roi = (unsigned)(d.P.v_end - d.P.v_begin);
  const unsigned nu_roi = (unsigned)(d.P.u_end - d.P.u_begin);
  const unsigned long long npix = (unsigned long long)nu_roi * nv_roi;
  unsigned long long vw;
  unsigned pix;
  if ((h >> 32) == 0 && (per >> 32) == 0 && (npix >> 32) == 0) {
    // 32-bit divisions (a 64-bit one is a long software routine); the
    // same quotients
    const unsigned h32 = (unsigned)h, per32 = (unsigned)per, np32 = (unsigned)npix;
    const unsigned r32 = h32 / per32;
    *k = h32 - r32 * per32;
    vw = r32 / np32;
    pix = r32 - (unsigned)vw * np32;
  } else {
    const unsigned long long rest = h / per;
    *k = h - rest * per;
    vw = rest / npix;
    pix = (unsigned)(rest - vw * npix);
  }
  *view = d.P.view_begin + (int)vw;
  *iu = d.P.u_begin + (int)(pix / nv_roi);
  *iv = d.P.v_begin + (int)(pix % nv_roi);
}

__device__ __forceinline__ void warp_stats(const McDev& d, unsigned long long v[kMcStats]) {
#pragma unroll
  for (int i = 0; i < kMcStats; i++) {
    unsigned long long x = v[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x) atomicAdd(&d.stats[i], x);
  }
}

// The kind of the interaction a collision led to (none when the history
// had used its interactions), into st[6..8]; constant indices keep st in
// registers.
__device__ __forceinline__ void count_event(const mc_photon& p, int n_before,
                                            unsigned long long (&st)[kMcStats]) {
  if (p.n_int == n_before) return;
  if (p.last == MC_EV_RAYLEIGH) st[6]++;
  else if (p.last == MC_EV_COMPTON) st[7]++;
  else st[8]++;
}

__global__ void __launch_bounds__(128) mc_plain_kernel(McDev d) {
  const int nv_roi = d.P.v_end - d.P.v_begin;
  const int nu_roi = d.P.u_end - d.P.u_begin;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long st[kMcStats] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (idx < nu_roi * nv_roi) {
    const int iu = d.P.u_begin + idx / nv_roi;
    const int iv = d.P.v_begin + idx % nv_roi;
    for (int view = d.P.view_begin; view < d.P.view_end; view++) {
      for (unsigned long long k = 0; k < d.P.per; k++) {
        mc_photon p;
        mc_start(&d.P, d.T, d.V, d.U, d.W, view, iu, iv, k, &p);
        st[0]++;
        while (true) {
          if (p.state == MC_FLY) {
            if (mc_flight_event(&d.P, d.T, d.L, d.labels, d.mclass, &p)) st[1]++; else st[9]++;
            if (p.state == MC_DEAD) st[5]++;
          } else if (p.state == MC_COLLIDED) {
            const int n0 = p.n_int;
            p.state = mc_after_collision(&d.P, d.T, &p);
            count_event(p, n0, st);
          } else if (p.state == MC_ESCAPED) {
            int kind = mc_tally_kind(&d.P, &p);
            long long cell = mc_detector_index(&d.P, d.V, &p);
            if (kind >= 0 && cell >= 0) {
              atomicAdd(kind == 0 ? &d.prim[cell] : &d.scat[cell], 1ull);
              if (kind == 0) st[3]++; else st[4]++;  // no run-time index: st stays in registers
            }
            break;
          } else {
            break;
          }
        }
        st[2] += (unsigned long long)p.n_int;
      }
    }
  }
  warp_stats(d, st);
}

// Body of the persistent kernel: SR Woodcock steps per round at most,
// collisions processed once CB lanes of the warp wait (or none flies).
template <int SR, int CB>
__device__ __forceinline__ void persistent_body(const McDev& d) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  __shared__ uint4 slots[256];
  const uint32_t slot = draw_slot(slots);
  unsigned long long st[kMcStats] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  mc_photon p;
  p.state = MC_DEAD;
  p.n_int = 0;
  bool retired = false;
  unsigned long long pool_next = 0, pool_end = 0;  // warp-uniform
  while (true) {
    // ---- refill idle lanes with the next histories ----------------------
    const unsigned need = __ballot_sync(FULL, p.state == MC_DEAD && !retired);
    if (need) {
      const unsigned cnt = __popc(need);
      const unsigned rank = __popc(need & lt_mask);
      const unsigned long long avail = pool_end - pool_next;
      unsigned long long base = 0;
      if (avail < cnt) {
        if (lane == 0) base = atomicAdd(d.counter, (unsigned long long)kChunk);
        base = __shfl_sync(FULL, base, 0);
      }
      if (need & (1u << lane)) {
        unsigned long long h = rank < avail ? pool_next + rank : base + (rank - avail);
        if (h >= d.total) {
          retired = true;
        } else {
          int view, iu, iv;
          unsigned long long k;
          decompose(d, h, &view, &iu, &iv, &k);
          st[2] += (unsigned long long)p.n_int;
          mc_start(&d.P, d.T, d.V, d.U, d.W, view, iu, iv, k, &p);
          p.rng.pf = slot;
          st[0]++;
        }
      }
      if (avail >= cnt) {
        pool_next += cnt;
      } else {
        pool_next = base + (cnt - avail);
        pool_end = base + kChunk;
        if (pool_end > d.total) pool_end = d.total;
        if (pool_next > pool_end) pool_next = pool_end;
      }
    }
    if (__all_sync(FULL, retired)) break;
    // ---- a few Woodcock steps ------------------------------------------
#pragma unroll 1
    for (int i = 0; i < SR && p.state == MC_FLY; i++) {
      prefetch_draws(p, d.P.keys);
      if (mc_flight_event(&d.P, d.T, d.L, d.labels, d.mclass, &p)) st[1]++; else st[9]++;
      if (p.state == MC_DEAD) st[5]++;
    }
    // ---- real collisions: the type at once (absorption ends the history,
    // Rayleigh flies on); Compton waits for the batch below ---------------
    if (p.state == MC_COLLIDED) {
      const int n0 = p.n_int;
      p.state = p.n_int >= d.P.max_int ? MC_DEAD : mc_interact_type(&d.P, d.T, &p);
      count_event(p, n0, st);
    }
    // ---- escaped photons: warp-aggregated tally --------------------------
    long long key = -1;
    long long cell = -1;
    int kind = 0;
    if (p.state == MC_ESCAPED) {
      kind = mc_tally_kind(&d.P, &p);
      cell = mc_detector_index(&d.P, d.V, &p);
      if (kind >= 0 && cell >= 0) key = cell * 2 + kind;
      p.state = MC_DEAD;
    }
    const unsigned tal = __ballot_sync(FULL, key >= 0);
    if (key >= 0) {
      const unsigned grp = __match_any_sync(tal, key);
      if (lane == __ffs(grp) - 1) {
        atomicAdd(kind == 0 ? &d.prim[cell] : &d.scat[cell], (unsigned long long)__popc(grp));
      }
      if (kind == 0) st[3]++; else st[4]++;  // no run-time index: st stays in registers
    }
    // ---- Compton scatterings, processed as a batch ------------------------
    const unsigned coll = __ballot_sync(FULL, p.state == MC_COMPTON);
    const unsigned fly = __ballot_sync(FULL, p.state == MC_FLY);
    if (coll && (__popc(coll) >= CB || fly == 0)) {
      if (p.state == MC_COMPTON) p.state = mc_compton(&d.P, &p);
    }
  }
  st[2] += (unsigned long long)p.n_int;
  warp_stats(d, st);
}

// CTAs per SM: with local majorants (8-step rounds) 64 registers and four
// CTAs (32 warps), with the single majorant (16-step rounds) 48 registers
// and five.  Measured on 1e8 histories of the 325^3 phantom: local 4.00e9
// histories/s at four CTAs against 3.89e9 at five and 3.80e9 at six (the
// spills of the smaller budgets), single 1.95e9 at five against 1.90e9 at
// four; 80 registers and three CTAs, and a four-step flight with the label
// reads issued together, were slower still: the kernel is bound by issue,
// not by the latency of the label gathers.
template <int SR>
struct McCtasPerSm {
  static constexpr int value = SR == kStepsPerRoundLocal ? 4 : 5;
};
template <int SR>
__global__ void __launch_bounds__(256, McCtasPerSm<SR>::value) mc_persistent_kernel(McDev d) {
  persistent_body<SR, kCollideBatch>(d);
}

// The persistent kernel over the histories of many jobs (phantoms of their
// own size, geometry and tables): the global history counter runs over the
// concatenated history ranges, and a lane that takes history h finds its
// job by binary search over the range starts.  Everything else is the
// single-job kernel's loop, reading the job's parameters through a pointer.
// Four CTAs per SM (64 registers, some spilled): 1.609 s per 64-scan batch
// against 1.635 s at three CTAs without spills.
template <int SR>
__global__ void __launch_bounds__(256, 4) mc_persistent_batch_kernel(
    const McDev* __restrict__ jobs, const unsigned long long* __restrict__ starts, int n_jobs,
    unsigned long long total, unsigned long long* counter, unsigned long long* stats) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  __shared__ unsigned long long s_starts[kMaxBatchJobs + 1];
  __shared__ uint4 slots[256];
  const uint32_t slot = draw_slot(slots);
  for (int i = threadIdx.x; i <= n_jobs; i += blockDim.x) s_starts[i] = starts[i];
  __syncthreads();
  unsigned long long st[kMcStats] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  mc_photon p;
  p.state = MC_DEAD;
  p.n_int = 0;
  const McDev* J = jobs;
  bool retired = false;
  unsigned long long pool_next = 0, pool_end = 0;
  while (true) {
    const unsigned need = __ballot_sync(FULL, p.state == MC_DEAD && !retired);
    if (need) {
      const unsigned cnt = __popc(need);
      const unsigned rank = __popc(need & lt_mask);
      const unsigned long long avail = pool_end - pool_next;
      unsigned long long base = 0;
      if (avail < cnt) {
        if (lane == 0) base = atomicAdd(counter, (unsigned long long)kChunk);
        base = __shfl_sync(FULL, base, 0);
      }
      if (need & (1u << lane)) {
        unsigned long long h = rank < avail ? pool_next + rank : base + (rank - avail);
        if (h >= total) {
          retired = true;
        } else {
          int lo = 0, hi = n_jobs - 1;  // last job whose start <= h
          while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (s_starts[mid] <= h) lo = mid; else hi = mid - 1;
          }
          J = jobs + lo;
          int view, iu, iv;
          unsigned long long k;
          decompose(*J, h - s_starts[lo], &view, &iu, &iv, &k);
          st[2] += (unsigned long long)p.n_int;
          mc_start(&J->P, J->T, J->V, J->U, J->W, view, iu, iv, k, &p);
          p.rng.pf = slot;
          st[0]++;
        }
      }
      if (avail >= cnt) {
        pool_next += cnt;
      } else {
        pool_next = base + (cnt - avail);
        pool_end = base + kChunk;
        if (pool_end > total) pool_end = total;
        if (pool_next > pool_end) pool_next = pool_end;
      }
    }
    if (__all_sync(FULL, retired)) break;
#pragma unroll 1
    for (int i = 0; i < SR && p.state == MC_FLY; i++) {
      prefetch_draws(p, J->P.keys);
      if (mc_flight_event(&J->P, J->T, J->L, J->labels, J->mclass, &p)) st[1]++; else st[9]++;
      if (p.state == MC_DEAD) st[5]++;
    }
    if (p.state == MC_COLLIDED) {
      const int n0 = p.n_int;
      p.state = p.n_int >= J->P.max_int ? MC_DEAD : mc_interact_type(&J->P, J->T, &p);
      count_event(p, n0, st);
    }
    long long cell = -1;
    int kind = 0;
    if (p.state == MC_ESCAPED) {
      kind = mc_tally_kind(&J->P, &p);
      cell = mc_detector_index(&J->P, J->V, &p);
      if (kind < 0) cell = -1;
      p.state = MC_DEAD;
    }
    // group lanes by (job, tally, pixel)
    unsigned long long* dst = nullptr;
    if (cell >= 0) dst = (kind == 0 ? J->prim : J->scat) + cell;
    const unsigned tal = __ballot_sync(FULL, dst != nullptr);
    if (dst) {
      const unsigned grp = __match_any_sync(tal, (unsigned long long)dst);
      if (lane == __ffs(grp) - 1) atomicAdd(dst, (unsigned long long)__popc(grp));
      if (kind == 0) st[3]++; else st[4]++;  // no run-time index: st stays in registers
    }
    const unsigned coll = __ballot_sync(FULL, p.state == MC_COMPTON);
    const unsigned fly = __ballot_sync(FULL, p.state == MC_FLY);
    if (coll && (__popc(coll) >= kCollideBatch || fly == 0)) {
      if (p.state == MC_COMPTON) p.state = mc_compton(&J->P, &p);
    }
  }
  st[2] += (unsigned long long)p.n_int;
#pragma unroll
  for (int i = 0; i < kMcStats; i++) {
    unsigned long long x = st[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
    if (lane == 0 && x) atomicAdd(&stats[i], x);
  }
}

// One CTA per macro cell: the cell's voxels OR their label bits into a
// shared 256-bit set, written once.
__global__ void __launch_bounds__(128) mc_macro_bits_kernel(const uint8_t* __restrict__ labels,
                                                            int nx, int ny, int nz, int shift,
                                                            int gx, int gy,
                                                            unsigned long long* __restrict__ bits) {
  __shared__ unsigned long long set[4];
  if (threadIdx.x < 4) set[threadIdx.x] = 0;
  __syncthreads();
  const int c = blockIdx.x;
  const int cx = c % gx, cy = (c / gx) % gy, cz = c / (gx * gy);
  const int m = 1 << shift;
  const int x0 = cx << shift, y0 = cy << shift, z0 = cz << shift;
  for (int i = threadIdx.x; i < m * m * m; i += blockDim.x) {
    const int x = x0 + (i & (m - 1)), y = y0 + ((i >> shift) & (m - 1)), z = z0 + (i >> (2 * shift));
    if (x < nx && y < ny && z < nz) {
      const int l = labels[((size_t)z * ny + y) * nx + x];
      atomicOr(&set[l >> 6], 1ull << (l & 63));
    }
  }
  __syncthreads();
  if (threadIdx.x < 4) bits[(size_t)c * 4 + threadIdx.x] = set[threadIdx.x];
}

__global__ void mc_energy_kernel(const mc_tables* __restrict__ T, uint64_t seed,
                                 monte_philox_keys keys, uint32_t job, unsigned long long n,
                                 float* __restrict__ out) {
  for (unsigned long long h = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; h < n;
       h += (unsigned long long)gridDim.x * blockDim.x) {
    monte_stream rng;
    monte_stream_init(&rng, seed, h, job);
    out[h] = T->n_lines > 1 ? mc_sample_energy(T, monte_uniform_keys(&rng, &keys)) : T->energy[0];
  }
}

__global__ void mc_finalize_kernel(size_t n, unsigned long long per, double log_per,
                                   const long long* __restrict__ prim,
                                   const long long* __restrict__ scat, int* __restrict__ proj0,
                                   float* __restrict__ map0, int* __restrict__ proj5,
                                   float* __restrict__ map5) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  long long a = prim ? prim[i] : 0;
  long long b = a + (scat ? scat[i] : 0);
  long long cap = (long long)per;
  if (a > cap) a = cap;
  if (a == 0) a = 1;
  if (b > cap) b = cap;
  if (b == 0) b = 1;
  if (proj0) proj0[i] = (int)a;
  if (map0) map0[i] = (float)(-log((double)a) + log_per);
  if (proj5) proj5[i] = (int)b;
  if (map5) map5[i] = (float)(-log((double)b) + log_per);
}

}  // namespace

cudaError_t launch_mc(const McDev& d, int kernel, int sm_count, cudaStream_t st) {
  if (kernel == 0) {
    const int n = (d.P.u_end - d.P.u_begin) * (d.P.v_end - d.P.v_begin);
    if (n == 0) return cudaSuccess;
    mc_plain_kernel<<<(n + 127) / 128, 128, 0, st>>>(d);
  } else {
    void (*fn)(McDev) = (d.P.flags & MC_F_LOCAL_MAJORANT) ? mc_persistent_kernel<kStepsPerRoundLocal>
                                                          : mc_persistent_kernel<kStepsPerRound>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    fn<<<sm_count * per_sm, 256, 0, st>>>(d);
  }
  return cudaGetLastError();
}

cudaError_t launch_mc_batch(const McDev* jobs, const unsigned long long* starts, int n_jobs,
                            unsigned long long total, unsigned long long* counter,
                            unsigned long long* stats, bool all_local, int sm_count,
                            cudaStream_t st) {
  if (n_jobs <= 0 || n_jobs > kMaxBatchJobs) return cudaErrorInvalidValue;
  auto fn = all_local ? mc_persistent_batch_kernel<kStepsPerRoundLocal>
                      : mc_persistent_batch_kernel<kStepsPerRound>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  fn<<<sm_count * per_sm, 256, 0, st>>>(jobs, starts, n_jobs, total, counter, stats);
  return cudaGetLastError();
}

cudaError_t launch_mc_macro_bits(const uint8_t* labels, const mc_params& P, unsigned long long* bits,
                                 cudaStream_t st) {
  const unsigned cells = (unsigned)P.mgx * P.mgy * P.mgz;
  if (cells == 0) return cudaSuccess;
  mc_macro_bits_kernel<<<cells, 128, 0, st>>>(labels, P.nx, P.ny, P.nz, P.mshift, P.mgx, P.mgy,
                                              bits);
  return cudaGetLastError();
}

namespace {
__global__ void bytes_differ_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                    size_t n, bool vec, int* __restrict__ diff) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool ne = false;
  size_t done = 0;
  if (vec) {  // both 16-byte aligned: 16 bytes per load
    const uint4* a4 = reinterpret_cast<const uint4*>(a);
    const uint4* b4 = reinterpret_cast<const uint4*>(b);
    const size_t n4 = n / 16;
    for (size_t i = i0; i < n4; i += stride) {
      const uint4 x = a4[i], y = b4[i];
      ne |= (x.x != y.x) | (x.y != y.y) | (x.z != y.z) | (x.w != y.w);
    }
    done = n4 * 16;
  }
  for (size_t i = done + i0; i < n; i += stride) ne |= a[i] != b[i];
  if (__any_sync(__activemask(), ne) && ne) *diff = 1;
}
}  // namespace

cudaError_t launch_bytes_differ(const uint8_t* a, const uint8_t* b, size_t n, int* diff,
                                int sm_count, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
  const size_t want = (n / (vec ? 16 : 1) + 255) / 256;
  const unsigned blocks = (unsigned)(want < 8ull * sm_count ? (want ? want : 1) : 8ull * sm_count);
  bytes_differ_kernel<<<blocks, 256, 0, st>>>(a, b, n, vec, diff);
  return cudaGetLastError();
}

cudaError_t launch_mc_energies(const mc_tables* T, uint64_t seed, const monte_philox_keys& keys,
                               uint32_t job, unsigned long long n, float* out, int sm_count,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const unsigned long long want = (n + 255) / 256;
  const unsigned blocks = (unsigned)(want < 8ull * sm_count ? want : 8ull * sm_count);
  mc_energy_kernel<<<blocks, 256, 0, st>>>(T, seed, keys, job, n, out);
  return cudaGetLastError();
}

cudaError_t launch_mc_finalize(size_t n, unsigned long long per, double log_per,
                               const long long* prim, const long long* scat, int* proj0,
                               float* map0, int* proj5, float* map5, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  mc_finalize_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, per, log_per, prim, scat,
                                                                   proj0, map0, proj5, map5);
  return cudaGetLastError();
}

}  // namespace monte
