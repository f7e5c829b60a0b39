// Runtime-plan convolution kernels for storage c32s with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_conv<c32s, float>(const FftArgs& a, const Launch& l, bool strided, int kop, int variant) {
  if (kop != 0) return cudaErrorInvalidValue;
  return launch_conv<DynPlan<MaxE<float>::value>, 0, c32s, float>(a, l, strided, variant);
}
}  // namespace vdx
