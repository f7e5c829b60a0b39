// bf16x2 storage has no real transforms (the planner refuses them).
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_real<bf16c, float>(const FftArgs&, const Launch&, int) {
  return cudaErrorInvalidValue;
}
}  // namespace vdx
