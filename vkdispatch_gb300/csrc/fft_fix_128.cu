// complex64 FFT kernels specialised for n = 128.
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fixed_c64<128>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
