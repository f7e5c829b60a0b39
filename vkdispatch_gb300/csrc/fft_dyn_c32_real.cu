// Runtime-plan real-transform kernels for storage c32s with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_real<c32s, float>(const FftArgs& a, const Launch& l, int op) {
  return launch_real<DynPlan<MaxE<float>::value>, c32s, float>(a, l, op, true);
}
}  // namespace vdx
