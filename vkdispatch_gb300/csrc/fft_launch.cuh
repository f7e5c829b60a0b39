// Template launcher shared by the per-storage-type translation units.
#pragma once

#include <cstdlib>

#include "vdx_internal.h"

namespace vdx {

// Strided compile-time convolutions of <= 256-thread CTAs load the kernel
// spectrum before the forward FFT (k_conv_pf) unless VDX_CONV_PREFETCH=0.
inline bool conv_prefetch() {
  static const bool on = [] {
    const char* e = std::getenv("VDX_CONV_PREFETCH");
    return !(e && e[0] == '0');
  }();
  return on;
}


// C2C with an optional fused element-wise operation (complex64 only):
// variant 0 = none, 1 = input weight, 2 = weighted |out|^2 partials
template <class Plan, bool INV, class S, class Re>
cudaError_t launch_c2c(const FftArgs& a, const Launch& l, bool strided, int variant) {
  if constexpr (std::is_same<S, Cx<float>>::value) {
    if (variant == 1) {
      if (strided) return enqueue_pdl(k_c2c<Plan, INV, true, S, Re, 1, 0>, l, a);
      return enqueue_pdl(k_c2c<Plan, INV, false, S, Re, 1, 0>, l, a);
    }
    if (variant == 2) {
      if (strided) return enqueue_pdl(k_c2c<Plan, INV, true, S, Re, 0, 1>, l, a);
      return enqueue_pdl(k_c2c<Plan, INV, false, S, Re, 0, 1>, l, a);
    }
  }
  if (variant != 0) return cudaErrorInvalidValue;
  if (strided) return enqueue_pdl(k_c2c<Plan, INV, true, S, Re>, l, a);
  return enqueue_pdl(k_c2c<Plan, INV, false, S, Re>, l, a);
}

// convolution with optional spectrum output (complex64 only): variant 0 =
// none, 1 = write S (used with the conjugate product of a forward
// convolution), 2 = write aux * conj(S) * scale (used with the plain product
// of its adjoint); the plain product (KOP 1) exists for complex64 only
template <class Plan, int KOP, bool STRIDED, class S, class Re>
cudaError_t launch_conv_layout(const FftArgs& a, const Launch& l, int variant) {
  constexpr bool C64 = std::is_same<S, Cx<float>>::value;
  if constexpr (C64 && STRIDED && IsFixPlan<Plan>::value) {
    if (variant == 0 && l.block.x <= 256 && conv_prefetch()) return enqueue_pdl(k_conv_pf<Plan, S, Re, KOP>, l, a);
  }
  if constexpr (C64 && KOP == 0) {
    if (variant == 1) return enqueue_pdl(k_conv<Plan, STRIDED, S, S, Re, 0, 1>, l, a);
  }
  if constexpr (C64 && KOP == 1) {
    if (variant == 2) return enqueue_pdl(k_conv<Plan, STRIDED, S, S, Re, 1, 2>, l, a);
  }
  if (variant != 0) return cudaErrorInvalidValue;
  if constexpr (KOP == 1 && !C64) return cudaErrorInvalidValue;
  else return enqueue_pdl(k_conv<Plan, STRIDED, S, S, Re, KOP>, l, a);
}

template <class Plan, int KOP, class S, class Re>
cudaError_t launch_conv(const FftArgs& a, const Launch& l, bool strided, int variant) {
  if (strided) return launch_conv_layout<Plan, KOP, true, S, Re>(a, l, variant);
  return launch_conv_layout<Plan, KOP, false, S, Re>(a, l, variant);
}

// Launches `op` with plan policy Plan (DynPlan or a compile-time FixPlan).
template <class Plan, class S, class Re>
cudaError_t launch_real(const FftArgs& a, const Launch& l, int op, bool with_odd) {
  switch (op) {
    case OP_R2C_EVEN:
      return enqueue_pdl(k_r2c_even<Plan, S, Re>, l, a);
    case OP_C2R_EVEN:
      return enqueue_pdl(k_c2r_even<Plan, S, Re>, l, a);
    case OP_R2C_ODD:
      if (with_odd) return enqueue_pdl(k_real_odd<Plan, false, S, Re>, l, a);
      return cudaErrorInvalidValue;
    case OP_C2R_ODD:
      if (with_odd) return enqueue_pdl(k_real_odd<Plan, true, S, Re>, l, a);
      return cudaErrorInvalidValue;
    default:
      return cudaErrorInvalidValue;
  }
}

template <class Plan, class S, class Re>
cudaError_t launch_c2c_any(const FftArgs& a, const Launch& l, int op, bool strided, int variant) {
  if (op == OP_C2C_FWD) return launch_c2c<Plan, false, S, Re>(a, l, strided, variant);
  return launch_c2c<Plan, true, S, Re>(a, l, strided, variant);
}

template <class Plan, class S, class Re>
cudaError_t launch_conv_any(const FftArgs& a, const Launch& l, bool strided, int kop, int variant) {
  if (kop == 0) return launch_conv<Plan, 0, S, Re>(a, l, strided, variant);
  return launch_conv<Plan, 1, S, Re>(a, l, strided, variant);
}

// The runtime-plan kernels of one storage type are split over three
// translation units (C2C, convolution, real) so they compile in parallel.
template <class S, class Re>
cudaError_t launch_dyn_c2c(const FftArgs& a, const Launch& l, int op, bool strided, int variant);
template <class S, class Re>
cudaError_t launch_dyn_conv(const FftArgs& a, const Launch& l, bool strided, int kop, int variant);
template <class S, class Re, bool STRIDED>
cudaError_t launch_dyn_conv_layout(const FftArgs& a, const Launch& l, int kop, int variant);
template <class S, class Re>
cudaError_t launch_dyn_real(const FftArgs& a, const Launch& l, int op);

template <class Plan, class S, class Re, bool WITH_ODD>
cudaError_t launch_with_plan(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant) {
  if (variant != 0 && op != OP_C2C_FWD && op != OP_C2C_INV && op != OP_CONV) return cudaErrorInvalidValue;
  switch (op) {
    case OP_C2C_FWD:
    case OP_C2C_INV:
      return launch_c2c_any<Plan, S, Re>(a, l, op, strided, variant);
    case OP_CONV:
      return launch_conv_any<Plan, S, Re>(a, l, strided, kop, variant);
    default:
      return launch_real<Plan, S, Re>(a, l, op, WITH_ODD);
  }
}

template <class S, class Re>
cudaError_t launch_fft(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant) {
  if (variant != 0 && op != OP_C2C_FWD && op != OP_C2C_INV && op != OP_CONV) return cudaErrorInvalidValue;
  switch (op) {
    case OP_C2C_FWD:
    case OP_C2C_INV:
      return launch_dyn_c2c<S, Re>(a, l, op, strided, variant);
    case OP_CONV:
      return launch_dyn_conv<S, Re>(a, l, strided, kop, variant);
    default:
      return launch_dyn_real<S, Re>(a, l, op);
  }
}

template <int N>
cudaError_t launch_fixed_c64(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant) {
  return launch_with_plan<Pow2Plan<N>, Cx<float>, float, false>(a, l, op, strided, kop, variant);
}

// strided complex64 convolution with the 8- or 32-points-per-thread plan
template <int N>
cudaError_t launch_fixedpts_conv_c64(int pts, const FftArgs& a, const Launch& l, int kop, int variant) {
  if (pts == 8) {
    if (kop == 0) return launch_conv_layout<Pow2x8Plan<N>, 0, true, Cx<float>, float>(a, l, variant);
    return launch_conv_layout<Pow2x8Plan<N>, 1, true, Cx<float>, float>(a, l, variant);
  }
  if (kop == 0) return launch_conv_layout<Pow2x32Plan<N>, 0, true, Cx<float>, float>(a, l, variant);
  return launch_conv_layout<Pow2x32Plan<N>, 1, true, Cx<float>, float>(a, l, variant);
}

// every complex64 operation (C2C, convolution, even-length real transforms;
// either layout) on the 32-points-per-thread plan
template <int N>
cudaError_t launch_fixed32_c64(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant) {
  return launch_with_plan<Pow2x32Plan<N>, Cx<float>, float, false>(a, l, op, strided, kop, variant);
}

}  // namespace vdx
