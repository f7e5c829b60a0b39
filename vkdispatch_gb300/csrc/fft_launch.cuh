// Template launcher shared by the per-storage-type translation units.
#pragma once

#include "vdx_internal.h"

namespace vdx {

// Launches `op` with plan policy Plan (DynPlan or a compile-time FixPlan).
template <class Plan, class S, class Re, bool WITH_ODD>
cudaError_t launch_with_plan(const FftArgs& a, const Launch& l, int op, bool strided, int kop) {
  switch (op) {
    case OP_C2C_FWD:
      if (strided) return enqueue(k_c2c<Plan, false, true, S, Re>, l, a);
      return enqueue(k_c2c<Plan, false, false, S, Re>, l, a);
    case OP_C2C_INV:
      if (strided) return enqueue(k_c2c<Plan, true, true, S, Re>, l, a);
      return enqueue(k_c2c<Plan, true, false, S, Re>, l, a);
    case OP_CONV:
      if (kop == 0) {
        if (strided) return enqueue(k_conv<Plan, true, S, S, Re, 0>, l, a);
        return enqueue(k_conv<Plan, false, S, S, Re, 0>, l, a);
      }
      if (strided) return enqueue(k_conv<Plan, true, S, S, Re, 1>, l, a);
      return enqueue(k_conv<Plan, false, S, S, Re, 1>, l, a);
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
cudaError_t launch_fft(const FftArgs& a, const Launch& l, int op, bool strided, int kop) {
  return launch_with_plan<DynPlan<MaxE<Re>::value>, S, Re, true>(a, l, op, strided, kop);
}

template <int N>
cudaError_t launch_fixed_c64(const FftArgs& a, const Launch& l, int op, bool strided, int kop) {
  return launch_with_plan<Pow2Plan<N>, Cx<float>, float, false>(a, l, op, strided, kop);
}

}  // namespace vdx
