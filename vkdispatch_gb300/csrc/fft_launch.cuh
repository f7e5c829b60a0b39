// Template launcher shared by the per-storage-type translation units.
#pragma once

#include "vdx_internal.h"

namespace vdx {

template <class S, class Re>
cudaError_t launch_fft(const FftArgs& a, const Launch& l, int op, bool strided, int kop) {
  constexpr int E = MaxE<Re>::value;
  switch (op) {
    case OP_C2C_FWD:
      if (strided) return enqueue(k_c2c<E, false, true, S, Re>, l, a);
      return enqueue(k_c2c<E, false, false, S, Re>, l, a);
    case OP_C2C_INV:
      if (strided) return enqueue(k_c2c<E, true, true, S, Re>, l, a);
      return enqueue(k_c2c<E, true, false, S, Re>, l, a);
    case OP_CONV:
      if (strided) return enqueue(k_conv<E, true, S, S, Re>, l, a, kop);
      return enqueue(k_conv<E, false, S, S, Re>, l, a, kop);
    case OP_R2C_EVEN:
      return enqueue(k_r2c_even<E, S, Re>, l, a);
    case OP_C2R_EVEN:
      return enqueue(k_c2r_even<E, S, Re>, l, a);
    case OP_R2C_ODD:
      return enqueue(k_real_odd<E, false, S, Re>, l, a);
    case OP_C2R_ODD:
      return enqueue(k_real_odd<E, true, S, Re>, l, a);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
