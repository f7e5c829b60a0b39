// Runtime-plan C2C kernels for storage Cx<float> with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_c2c<Cx<float>, float>(const FftArgs& a, const Launch& l, int op, bool strided, int variant) {
  return launch_c2c_any<DynPlan<MaxE<float>::value>, Cx<float>, float>(a, l, op, strided, variant);
}
}  // namespace vdx
