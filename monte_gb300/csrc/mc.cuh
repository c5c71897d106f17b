// mc.cuh -- launch descriptor of the Monte Carlo kernels (mc_kernels.cu),
// shared with the entry points (mc_api.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/monte.h"
#include "mc_physics.h"

namespace monte {

struct McDev {
  mc_params P;
  const mc_tables* T;
  const mc_view* V;
  const mc_pixel* U;
  const mc_pixel* W;
  const uint8_t* labels;
  const mc_local_tables* L;   // local majorants (MONTE_MC_LOCAL_MAJORANT), else unused
  const uint16_t* mclass;     // class | legs << 8 per macro cell (MONTE_MC_LOCAL_MAJORANT)
  unsigned long long* prim;
  unsigned long long* scat;
  unsigned long long* stats;  // [kMcStats]: histories, steps, interactions, prim, scat,
                              // dropped, rayleigh, compton, photo, majorant legs
  unsigned long long* counter;
  unsigned long long total;   // histories in this launch
};

// Counters of a run, in monte_mc_stats order, and their copy into it.
constexpr int kMcStats = 10;
inline void mc_stats_from(const unsigned long long* h, monte_mc_stats* s) {
  s->histories = h[0];
  s->woodcock_steps = h[1];
  s->interactions = h[2];
  s->primary_counts = h[3];
  s->scatter_counts = h[4];
  s->dropped = h[5];
  s->rayleigh = h[6];
  s->compton = h[7];
  s->photoelectric = h[8];
  s->majorant_legs = h[9];
}

cudaError_t launch_mc(const McDev& d, int kernel, int sm_count, cudaStream_t st);
// *diff = 1 if the n bytes at a and b differ anywhere (*diff is not
// cleared first).
cudaError_t launch_bytes_differ(const uint8_t* a, const uint8_t* b, size_t n, int* diff,
                                int sm_count, cudaStream_t st);

// Jobs one batched persistent launch can carry.
constexpr int kMaxBatchJobs = 1024;
// One persistent launch over the histories of n_jobs jobs; starts[j] is the
// first global history of job j, starts[n_jobs] = total (device arrays).
// all_local: every job tracks with local majorants (the shorter rounds of
// that transport).
cudaError_t launch_mc_batch(const McDev* jobs, const unsigned long long* starts, int n_jobs,
                            unsigned long long total, unsigned long long* counter,
                            unsigned long long* stats, bool all_local, int sm_count,
                            cudaStream_t st);
// Labels present in each macro cell of the local majorants (mc_setup.h's
// mc_macro_bits_host, for labels in device memory): 4 words per cell.
cudaError_t launch_mc_macro_bits(const uint8_t* labels, const mc_params& P, unsigned long long* bits,
                                 cudaStream_t st);
// The local-majorant tables and class grid for P: mu per label, then the
// classes from the cells' label sets (on the host from host labels, or
// computed on the GPU for device labels).  Synchronizes the context's
// stream for device labels.  key (may be NULL) receives what the grid was
// built from; when it equals ctx->mc_macro_key, cls is left empty (the
// context's device copy is current).
int mc_build_macro(monte_ctx* ctx, const monte_mc_phantom* ph, const monte_xcom* x,
                   bool labels_on_device, const mc_params& P, mc_local_tables* L,
                   std::vector<uint16_t>* cls, std::vector<uint8_t>* key);

// Source energies of histories 0..n-1 of stream (seed, job): the first
// draw of mc_start, by the same sampler.
cudaError_t launch_mc_energies(const mc_tables* T, uint64_t seed, const monte_philox_keys& keys,
                               uint32_t job, unsigned long long n, float* out, int sm_count,
                               cudaStream_t st);
cudaError_t launch_mc_finalize(size_t n, unsigned long long per, double log_per,
                               const long long* prim, const long long* scat, int* proj0,
                               float* map0, int* proj5, float* map5, cudaStream_t st);

}  // namespace monte
