// Template launcher shared by the per-storage-type translation units.
#pragma once

#include "vdx_internal.h"

namespace vdx {

// C2C with an optional fused element-wise operation (complex64 only):
// variant 0 = none, 1 = input weight, 2 = weighted |out|^2 partials
template <class Plan, bool INV, class S, class Re>
cudaError_t launch_c2c(const FftArgs& a, const Launch& l, bool strided, int variant) {
  if constexpr (std::is_same<S, Cx<float>>::value) {
    if (variant == 1) {
      if (strided) return enqueue(k_c2c<Plan, INV, true, S, Re, 1, 0>, l, a);
      return enqueue(k_c2c<Plan, INV, false, S, Re, 1, 0>, l, a);
    }
    if (variant == 2) {
      if (strided) return enqueue(k_c2c<Plan, INV, true, S, Re, 0, 1>, l, a);
      return enqueue(k_c2c<Plan, INV, false, S, Re, 0, 1>, l, a);
    }
  }
  if (variant != 0) return cudaErrorInvalidValue;
  if (strided) return enqueue(k_c2c<Plan, INV, true, S, Re>, l, a);
  return enqueue(k_c2c<Plan, INV, false, S, Re>, l, a);
}

// convolution with optional spectrum output (complex64 only): variant 0 =
// none, 1 = write S, 2 = write aux * conj(S) * scale
template <class Plan, int KOP, class S, class Re>
cudaError_t launch_conv(const FftArgs& a, const Launch& l, bool strided, int variant) {
  if constexpr (std::is_same<S, Cx<float>>::value) {
    if (variant == 1) {
      if (strided) return enqueue(k_conv<Plan, true, S, S, Re, KOP, 1>, l, a);
      return enqueue(k_conv<Plan, false, S, S, Re, KOP, 1>, l, a);
    }
    if (variant == 2) {
      if (strided) return enqueue(k_conv<Plan, true, S, S, Re, KOP, 2>, l, a);
      return enqueue(k_conv<Plan, false, S, S, Re, KOP, 2>, l, a);
    }
  }
  if (variant != 0) return cudaErrorInvalidValue;
  if (strided) return enqueue(k_conv<Plan, true, S, S, Re, KOP>, l, a);
  return enqueue(k_conv<Plan, false, S, S, Re, KOP>, l, a);
}

// Launches `op` with plan policy Plan (DynPlan or a compile-time FixPlan).
template <class Plan, class S, class Re, bool WITH_ODD>
cudaError_t launch_with_plan(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant) {
  if (variant != 0 && op != OP_C2C_FWD && op != OP_C2C_INV && op != OP_CONV) return cudaErrorInvalidValue;
  switch (op) {
    case OP_C2C_FWD:
      return launch_c2c<Plan, false, S, Re>(a, l, strided, variant);
    case OP_C2C_INV:
      return launch_c2c<Plan, true, S, Re>(a, l, strided, variant);
    case OP_CONV:
      if (kop == 0) return launch_conv<Plan, 0, S, Re>(a, l, strided, variant);
      return launch_conv<Plan, 1, S, Re>(a, l, strided, variant);
    case OP_R2C_EVEN:
      return enqueue(k_r2c_even<Plan, S, Re>, l, a);
    case OP_C2R_EVEN:
      return enqueue(k_c2r_even<Plan, S, Re>, l, a);
    case OP_R2C_ODD:
      if constexpr (WITH_ODD) return enqueue(k_real_odd<Plan, false, S, Re>, l, a);
      return cudaErrorInvalidValue;
    case OP_C2R_ODD:
      if constexpr (WITH_ODD) return enqueue(k_real_odd<Plan, true, S, Re>, l, a);
      return cudaErrorInvalidValue;
    default:
      return cudaErrorInvalidValue;
  }
}

template <class S, class Re>
cudaError_t launch_fft(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant) {
  return launch_with_plan<DynPlan<MaxE<Re>::value>, S, Re, true>(a, l, op, strided, kop, variant);
}

template <int N>
cudaError_t launch_fixed_c64(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant) {
  return launch_with_plan<Pow2Plan<N>, Cx<float>, float, false>(a, l, op, strided, kop, variant);
}

}  // namespace vdx
