// complex64 FFT kernels specialised for n = 1024 (and the C2C transforms on the
// two-pass radix-32 x 32 plan).
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fixed_c64<1024>(const FftArgs&, const Launch&, int, bool, int, int);
template cudaError_t launch_fixedpts_c2c_c64<1024>(const FftArgs&, const Launch&, int, bool, int);
}  // namespace vdx
