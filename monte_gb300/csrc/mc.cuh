// mc.cuh -- launch descriptor of the Monte Carlo kernels (mc_kernels.cu),
// shared with the entry points (mc_api.cu).
#pragma once

#include <cuda_runtime.h>

#include "mc_physics.h"

namespace monte {

struct McDev {
  mc_params P;
  const mc_tables* T;
  const mc_view* V;
  const mc_pixel* U;
  const mc_pixel* W;
  const uint8_t* labels;
  unsigned long long* prim;
  unsigned long long* scat;
  unsigned long long* stats;  // [histories, steps, interactions, prim, scat, dropped]
  unsigned long long* counter;
  unsigned long long total;   // histories in this launch
};

cudaError_t launch_mc(const McDev& d, int kernel, int sm_count, cudaStream_t st);

// Jobs one batched persistent launch can carry.
constexpr int kMaxBatchJobs = 1024;
// One persistent launch over the histories of n_jobs jobs; starts[j] is the
// first global history of job j, starts[n_jobs] = total (device arrays).
cudaError_t launch_mc_batch(const McDev* jobs, const unsigned long long* starts, int n_jobs,
                            unsigned long long total, unsigned long long* counter,
                            unsigned long long* stats, int sm_count, cudaStream_t st);
cudaError_t launch_mc_finalize(size_t n, unsigned long long per, double log_per,
                               const long long* prim, const long long* scat, int* proj0,
                               float* map0, int* proj5, float* map5, cudaStream_t st);

}  // namespace monte
