// Runtime-plan real-transform kernels for storage Cx<double> with double butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_real<Cx<double>, double>(const FftArgs& a, const Launch& l, int op) {
  return launch_real<DynPlan<MaxE<double>::value>, Cx<double>, double>(a, l, op, true);
}
}  // namespace vdx
