// Runtime-plan complex64 convolution kernels, contig axes.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_conv_layout<Cx<float>, float, false>(const FftArgs& a, const Launch& l, int kop, int variant) {
  using Plan = DynPlan<MaxE<float>::value>;
  if (kop == 0) return launch_conv_layout<Plan, 0, false, Cx<float>, float>(a, l, variant);
  return launch_conv_layout<Plan, 1, false, Cx<float>, float>(a, l, variant);
}
}  // namespace vdx
