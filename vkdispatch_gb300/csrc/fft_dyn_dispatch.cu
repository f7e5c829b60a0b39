// Runtime-plan dispatch by operation to the per-storage-type translation units.
#include "fft_launch.cuh"

namespace vdx {
template cudaError_t launch_fft<Cx<float>, float>(const FftArgs&, const Launch&, int, bool, int, int);
template cudaError_t launch_fft<c32s, float>(const FftArgs&, const Launch&, int, bool, int, int);
template cudaError_t launch_fft<bf16c, float>(const FftArgs&, const Launch&, int, bool, int, int);
template cudaError_t launch_fft<Cx<double>, double>(const FftArgs&, const Launch&, int, bool, int, int);
}  // namespace vdx
