// FFT kernel instantiations for storage Cx<double> with double butterflies.
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fft<Cx<double>, double>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
