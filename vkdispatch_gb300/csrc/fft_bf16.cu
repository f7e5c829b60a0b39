// FFT kernel instantiations for storage bf16c with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fft<bf16c, float>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
