// Runtime-plan convolution kernels for storage Cx<double> with double butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_conv<Cx<double>, double>(const FftArgs& a, const Launch& l, bool strided, int kop, int variant) {
  if (kop != 0) return cudaErrorInvalidValue;
  return launch_conv<DynPlan<MaxE<double>::value>, 0, Cx<double>, double>(a, l, strided, variant);
}
}  // namespace vdx
