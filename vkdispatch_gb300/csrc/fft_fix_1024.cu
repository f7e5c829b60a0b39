// complex64 FFT kernels specialised for n = 1024 (radix 16 x 16 x 4, and the
// two-pass radix 32 x 32 plan).
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fixed_c64<1024>(const FftArgs&, const Launch&, int, bool, int, int);
template cudaError_t launch_fixed32_c64<1024>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
