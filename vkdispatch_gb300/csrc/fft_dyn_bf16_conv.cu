// Runtime-plan convolution kernels for storage bf16c with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_conv<bf16c, float>(const FftArgs& a, const Launch& l, bool strided, int kop, int variant) {
  if (kop != 0) return cudaErrorInvalidValue;
  return launch_conv<DynPlan<MaxE<float>::value>, 0, bf16c, float>(a, l, strided, variant);
}
}  // namespace vdx
