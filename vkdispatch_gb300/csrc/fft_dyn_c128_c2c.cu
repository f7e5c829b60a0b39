// Runtime-plan C2C kernels for storage Cx<double> with double butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_c2c<Cx<double>, double>(const FftArgs& a, const Launch& l, int op, bool strided, int variant) {
  return launch_c2c_any<DynPlan<MaxE<double>::value>, Cx<double>, double>(a, l, op, strided, variant);
}
}  // namespace vdx
