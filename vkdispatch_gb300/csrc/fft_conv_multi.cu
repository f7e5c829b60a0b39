// Fused multi-kernel convolutions (one signal, kernel_num kernels) on the
// runtime-plan kernels, complex64 and complex128 storage.
#include "fft_launch.cuh"

namespace vdx {

namespace {

template <class S, class Re, bool STRIDED>
cudaError_t launch_multi(const FftArgs& a, const Launch& l, int kop, int K, long long kstride, long long ostride) {
  using Plan = DynPlan<MaxE<Re>::value>;
  if (kop == 0) return enqueue(k_conv_multi<Plan, STRIDED, S, Re, 0>, l, a, K, kstride, ostride);
  return enqueue(k_conv_multi<Plan, STRIDED, S, Re, 1>, l, a, K, kstride, ostride);
}

}  // namespace

int conv_multi_points(bool f64) { return f64 ? MaxE<double>::value : MaxE<float>::value; }

cudaError_t launch_conv_multi(int store, bool strided, const FftArgs& a, const Launch& l, int kop, int K,
                              long long kstride, long long ostride) {
  switch (store) {
    case ST_C64:
      return strided ? launch_multi<Cx<float>, float, true>(a, l, kop, K, kstride, ostride)
                     : launch_multi<Cx<float>, float, false>(a, l, kop, K, kstride, ostride);
    case ST_C128:
      return strided ? launch_multi<Cx<double>, double, true>(a, l, kop, K, kstride, ostride)
                     : launch_multi<Cx<double>, double, false>(a, l, kop, K, kstride, ostride);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
