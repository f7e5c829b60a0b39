// FFT kernel instantiations for storage Cx<float> with float butterflies.
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fft<Cx<float>, float>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
