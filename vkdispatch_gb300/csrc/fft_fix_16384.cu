// complex64 FFT kernels specialised for n = 16384.
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fixed_c64<16384>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
