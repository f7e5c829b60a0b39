// complex64 FFT kernels specialised for n = 512 (radix 16 x 16 x 2, the
// two-pass radix 32 x 16 plan, and the strided convolution with 8 points per
// thread).
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fixed_c64<512>(const FftArgs&, const Launch&, int, bool, int, int);
template cudaError_t launch_fixedpts_conv_c64<512>(int, const FftArgs&, const Launch&, int, int);
template cudaError_t launch_fixed32_c64<512>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
