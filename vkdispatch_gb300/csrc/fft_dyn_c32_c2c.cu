// Runtime-plan C2C kernels for storage c32s with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_c2c<c32s, float>(const FftArgs& a, const Launch& l, int op, bool strided, int variant) {
  return launch_c2c_any<DynPlan<MaxE<float>::value>, c32s, float>(a, l, op, strided, variant);
}
}  // namespace vdx
