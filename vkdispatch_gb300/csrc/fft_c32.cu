// FFT kernel instantiations for storage c32s with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fft<c32s, float>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
