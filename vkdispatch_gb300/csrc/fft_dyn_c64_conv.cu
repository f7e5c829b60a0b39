// Runtime-plan convolution kernels for complex64 storage: dispatch to the
// contiguous- and strided-axis translation units.
#include "fft_launch.cuh"

namespace vdx {
template <>
cudaError_t launch_dyn_conv<Cx<float>, float>(const FftArgs& a, const Launch& l, bool strided, int kop, int variant) {
  if (strided) return launch_dyn_conv_layout<Cx<float>, float, true>(a, l, kop, variant);
  return launch_dyn_conv_layout<Cx<float>, float, false>(a, l, kop, variant);
}
}  // namespace vdx
