// FP64-built twiddle tables.
#include "vdx_internal.h"

namespace vdx {

cudaError_t launch_twiddle(void* tab, int count, int den, bool f64, cudaStream_t s) {
  const int threads = 256;
  const int blocks = (count + threads - 1) / threads;
  if (f64)
    k_twiddle<double><<<blocks, threads, 0, s>>>(reinterpret_cast<Cx<double>*>(tab), count, den);
  else
    k_twiddle<float><<<blocks, threads, 0, s>>>(reinterpret_cast<Cx<float>*>(tab), count, den);
  return cudaGetLastError();
}

}  // namespace vdx
