// Fused multi-kernel convolutions (one signal, kernel_num kernels) on the
// compile-time complex64 plans (radix 16, and the two-pass radix-32 plan) of power-of-two lengths 1024 to 16384.
#include "fft_launch.cuh"

namespace vdx {

namespace {

template <int N, class Plan = Pow2Plan<N>>
cudaError_t launch_fixed_multi(bool strided, const FftArgs& a, const Launch& l, int kop, int K, long long kstride,
                               long long ostride) {
  using S = Cx<float>;
  if (strided) {
    if (kop == 0) return enqueue(k_conv_multi<Plan, true, S, float, 0>, l, a, K, kstride, ostride);
    return enqueue(k_conv_multi<Plan, true, S, float, 1>, l, a, K, kstride, ostride);
  }
  if (kop == 0) return enqueue(k_conv_multi<Plan, false, S, float, 0>, l, a, K, kstride, ostride);
  return enqueue(k_conv_multi<Plan, false, S, float, 1>, l, a, K, kstride, ostride);
}

}  // namespace

cudaError_t launch_fixed_conv_multi_large(int n, int pts, bool strided, const FftArgs& a, const Launch& l, int kop,
                                     int K, long long kstride, long long ostride) {
  if (pts == 32) {
    switch (n) {
      case 1024: return launch_fixed_multi<1024, Pow2x32Plan<1024>>(strided, a, l, kop, K, kstride, ostride);
      default: return cudaErrorInvalidValue;
    }
  }
  if (pts != 16) return cudaErrorInvalidValue;
  switch (n) {
    case 1024: return launch_fixed_multi<1024>(strided, a, l, kop, K, kstride, ostride);
    case 2048: return launch_fixed_multi<2048>(strided, a, l, kop, K, kstride, ostride);
    case 4096: return launch_fixed_multi<4096>(strided, a, l, kop, K, kstride, ostride);
    case 8192: return launch_fixed_multi<8192>(strided, a, l, kop, K, kstride, ostride);
    case 16384: return launch_fixed_multi<16384>(strided, a, l, kop, K, kstride, ostride);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
