// fdk_filter_bf16x3.cu -- tensor-core (tcgen05) ramp filter, split 3xBF16.
// (implementation follows)
#include "fdk.cuh"

namespace monte {
size_t bf16x3_bsplit_bytes(int nu) { return (size_t)nu * nu * 2 * sizeof(uint16_t); }
void bf16x3_build_bsplit(int, const float*, uint16_t*) {}
bool bf16x3_supported(const FdkDev&) { return false; }
cudaError_t launch_fdk_filter_bf16x3(const FdkDev&, const float*, const float*, const uint16_t*,
                                     float*, int*, int, cudaStream_t) {
  return cudaErrorNotSupported;
}
}  // namespace monte
