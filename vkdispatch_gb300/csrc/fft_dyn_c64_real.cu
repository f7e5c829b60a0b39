// Runtime-plan real-transform kernels for storage Cx<float> with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_real<Cx<float>, float>(const FftArgs& a, const Launch& l, int op) {
  return launch_real<DynPlan<MaxE<float>::value>, Cx<float>, float>(a, l, op, true);
}
}  // namespace vdx
