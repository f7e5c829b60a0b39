// FFT and fused-convolution kernels whose loads, stores and spectrum
// operation are user map hooks (the reference's input_map / output_map /
// kernel_map, vkdispatch/fft/io_manager.py:107-155, vkdispatch/shader/
// map.py:29-40).  Compiled at run time by NVRTC (jit.cu) together with a
// hooks struct that the Python tracer generates from the user's map
// functions; the passes are the same Stockham plans as the ahead-of-time
// kernels, on a compile-time radix list chosen by the planner.
//
// The hooks struct H provides, for the register type Re:
//   static Cx<Re> load(const MapArgs&, long long io, int k, int n)         input map
//   static void store(const MapArgs&, Cx<Re> v, long long io, int k, int n) output map
//   static Cx<Re> kernel(const MapArgs&, Cx<Re> v, long long io, int k, int n)  kernel map
// io is the reference's io_index (the element's flat index in the logical
// buffer shape: outer batch * N * stride + inner + k * stride), k the
// fft_index and n the fft_size.
#pragma once

#include "fft_kernels.cuh"

namespace vdx {

constexpr int kMapMaxBuffers = 8;
constexpr int kMapMaxScalars = 8;

struct MapArgs {
  void* buf[kMapMaxBuffers];
  long long count[kMapMaxBuffers];  // elements each buffer slot may be indexed with
  double fs[kMapMaxScalars];        // floating-point scalar map arguments
  long long is[kMapMaxScalars];     // integer scalar map arguments
  long long kidx;                   // mapped_kernel_index() of a multi-kernel convolution
  int* status;                      // set to 1 by an index outside its buffer (filled by the launcher)
};

// Element access of generated hooks, bounds-checked: a map's index
// expression is user code, so an index outside [0, count) of its buffer
// loads zero, skips the store and records the fault in the plan's status
// word instead of touching memory outside the buffer.
__device__ __forceinline__ bool map_in(const MapArgs& m, int slot, long long i) {
  if ((unsigned long long)i < (unsigned long long)m.count[slot]) return true;
  if (m.status) atomicOr(m.status, 1);
  return false;
}
template <class T>
__device__ __forceinline__ T map_ld(const MapArgs& m, int slot, long long i) {
  return map_in(m, slot, i) ? reinterpret_cast<const T*>(m.buf[slot])[i] : T(0);
}
template <class T>
__device__ __forceinline__ void map_st(const MapArgs& m, int slot, long long i, T v) {
  if (map_in(m, slot, i)) reinterpret_cast<T*>(m.buf[slot])[i] = v;
}
template <class S, class Re>
__device__ __forceinline__ Cx<Re> map_ldc(const MapArgs& m, int slot, long long i) {
  if (!map_in(m, slot, i)) return mk<Re>(Re(0), Re(0));
  return Conv<S, Re>::ld(reinterpret_cast<const S*>(m.buf[slot]) + i);
}
template <class S, class Re>
__device__ __forceinline__ void map_stc(const MapArgs& m, int slot, long long i, Cx<Re> v) {
  if (map_in(m, slot, i)) Conv<S, Re>::st(reinterpret_cast<S*>(m.buf[slot]) + i, v);
}

// Operations of generated hooks, with the reference's shader semantics:
// arithmetic on two complex (vec2) values is component-wise, a real operand
// applies to both components, a real value converted to complex fills both
// components (vec2(x)), and mult_complex / conj are the complex product and
// conjugate.  Generated code calls these by name (namespace mapops).
namespace mapops {

template <class R>
__device__ __forceinline__ Cx<R> splat(R v) {
  return mk<R>(v, v);
}
template <class R, class S>
__device__ __forceinline__ Cx<R> to_cx(S v) {
  return mk<R>(R(v), R(v));
}
template <class R, class Q>
__device__ __forceinline__ Cx<R> to_cx(Cx<Q> v) {
  return mk<R>(R(v.x), R(v.y));
}
template <class R, class Q>
__device__ __forceinline__ Cx<R> make(Q a, Q b) {
  return mk<R>(R(a), R(b));
}
template <class R>
__device__ __forceinline__ Cx<R> make(R a, R b) {
  return mk<R>(a, b);
}

#define VDX_MAP_BINARY(NAME, OP)                                                          \
  template <class A, class B>                                                             \
  __device__ __forceinline__ auto NAME(A a, B b) {                                        \
    return a OP b;                                                                        \
  }                                                                                       \
  template <class R>                                                                      \
  __device__ __forceinline__ Cx<R> NAME(Cx<R> a, Cx<R> b) {                               \
    return mk<R>(a.x OP b.x, a.y OP b.y);                                                 \
  }                                                                                       \
  template <class R, class B>                                                             \
  __device__ __forceinline__ Cx<R> NAME(Cx<R> a, B b) {                                   \
    return mk<R>(a.x OP R(b), a.y OP R(b));                                               \
  }                                                                                       \
  template <class A, class R>                                                             \
  __device__ __forceinline__ Cx<R> NAME(A a, Cx<R> b) {                                   \
    return mk<R>(R(a) OP b.x, R(a) OP b.y);                                               \
  }
VDX_MAP_BINARY(add, +)
VDX_MAP_BINARY(sub, -)
VDX_MAP_BINARY(mul, *)
VDX_MAP_BINARY(div, /)
#undef VDX_MAP_BINARY

template <class A>
__device__ __forceinline__ A neg(A a) {
  return -a;
}
template <class R>
__device__ __forceinline__ Cx<R> neg(Cx<R> a) {
  return mk<R>(-a.x, -a.y);
}
template <class R>
__device__ __forceinline__ Cx<R> cplx_mul(Cx<R> a, Cx<R> b) {
  return cmul(a, b);
}
template <class R>
__device__ __forceinline__ Cx<R> cplx_conj(Cx<R> a) {
  return mk<R>(a.x, -a.y);
}

// real functions, float and double, lifted component-wise to complex values
#define VDX_MAP_UNARY(NAME, FF, DF)                                                        \
  __device__ __forceinline__ float NAME(float x) { return FF(x); }                         \
  __device__ __forceinline__ double NAME(double x) { return DF(x); }                       \
  template <class R>                                                                       \
  __device__ __forceinline__ Cx<R> NAME(Cx<R> a) {                                         \
    return mk<R>(NAME(a.x), NAME(a.y));                                                    \
  }
VDX_MAP_UNARY(m_sin, sinf, sin)
VDX_MAP_UNARY(m_cos, cosf, cos)
VDX_MAP_UNARY(m_tan, tanf, tan)
VDX_MAP_UNARY(m_asin, asinf, asin)
VDX_MAP_UNARY(m_acos, acosf, acos)
VDX_MAP_UNARY(m_atan, atanf, atan)
VDX_MAP_UNARY(m_sinh, sinhf, sinh)
VDX_MAP_UNARY(m_cosh, coshf, cosh)
VDX_MAP_UNARY(m_tanh, tanhf, tanh)
VDX_MAP_UNARY(m_exp, expf, exp)
VDX_MAP_UNARY(m_exp2, exp2f, exp2)
VDX_MAP_UNARY(m_log, logf, log)
VDX_MAP_UNARY(m_log2, log2f, log2)
VDX_MAP_UNARY(m_sqrt, sqrtf, sqrt)
VDX_MAP_UNARY(m_inversesqrt, rsqrtf, rsqrt)
VDX_MAP_UNARY(m_abs, fabsf, fabs)
VDX_MAP_UNARY(m_floor, floorf, floor)
VDX_MAP_UNARY(m_ceil, ceilf, ceil)
VDX_MAP_UNARY(m_trunc, truncf, trunc)
VDX_MAP_UNARY(m_round, roundf, round)
#undef VDX_MAP_UNARY
__device__ __forceinline__ long long m_abs(long long x) { return x < 0 ? -x : x; }
template <class T>
__device__ __forceinline__ T m_fract(T x) {
  return sub(x, m_floor(x));
}
template <class T>
__device__ __forceinline__ T m_sign(T x) {
  return T(x > T(0)) - T(x < T(0));
}
template <class R>
__device__ __forceinline__ Cx<R> m_sign(Cx<R> a) {
  return mk<R>(m_sign(a.x), m_sign(a.y));
}
__device__ __forceinline__ float m_pow(float a, float b) { return powf(a, b); }
__device__ __forceinline__ double m_pow(double a, double b) { return pow(a, b); }
__device__ __forceinline__ float m_atan2(float a, float b) { return atan2f(a, b); }
__device__ __forceinline__ double m_atan2(double a, double b) { return atan2(a, b); }
__device__ __forceinline__ float m_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double m_fma(double a, double b, double c) { return fma(a, b, c); }
// GLSL mod: x - y * floor(x / y) on floats, % on integers
__device__ __forceinline__ float m_mod(float x, float y) { return x - y * floorf(x / y); }
__device__ __forceinline__ double m_mod(double x, double y) { return x - y * floor(x / y); }
__device__ __forceinline__ long long m_mod(long long x, long long y) { return x % y; }
template <class T>
__device__ __forceinline__ T m_min(T a, T b) {
  return b < a ? b : a;
}
template <class T>
__device__ __forceinline__ T m_max(T a, T b) {
  return b > a ? b : a;
}
template <class R>
__device__ __forceinline__ Cx<R> m_min(Cx<R> a, Cx<R> b) {
  return mk<R>(m_min(a.x, b.x), m_min(a.y, b.y));
}
template <class R>
__device__ __forceinline__ Cx<R> m_max(Cx<R> a, Cx<R> b) {
  return mk<R>(m_max(a.x, b.x), m_max(a.y, b.y));
}
template <class T>
__device__ __forceinline__ T m_clamp(T x, T lo, T hi) {
  return m_min(m_max(x, lo), hi);
}
template <class T, class A>
__device__ __forceinline__ T m_mix(T x, T y, A a) {
  return add(mul(x, sub(A(1), a)), mul(y, a));
}
template <class R>
__device__ __forceinline__ R m_length(Cx<R> a) {
  return m_sqrt(a.x * a.x + a.y * a.y);
}
template <class R>
__device__ __forceinline__ R m_length(R a) {
  return m_abs(a);
}

}  // namespace mapops

// MODE 0: forward FFT, 1: inverse FFT, 2: fused convolution (forward FFT,
// kernel hook, inverse FFT with the passes reversed)
template <class Plan, bool STRIDED, class Re, int MODE, class H>
__device__ __forceinline__ void mapped_body(const FftArgs& a, const MapArgs& m) {
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<STRIDED> pl(a, P.T());
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  Cx<Re> v[MAXE];
  P.assume_t(pl.t);
  const int n = P.n();
  const long long io0 = pl.in0();
  const bool ok = pl.tile_full || pl.valid;
  const int lo = a.sig_lo, hi = a.sig_hi;
  P.template first<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) {
      if (!ok || pos < lo || pos >= hi) return mk<Re>(Re(0), Re(0));
      return H::template load<Re>(m, io0 + pos * pl.ps, pos, n);
    });
  });
  P.template run<MODE == 1, false>(v, pl, sm, tw);
  constexpr bool REV = MODE == 2;
  if constexpr (MODE == 2) {
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      constexpr int B = MAXE / RR;
      const int nb = n / RR;
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int j = pl.t + b * P.T();
        if (j < nb && ok) {
#pragma unroll
          for (int r = 0; r < RR; ++r) {
            const int pos = j + r * nb;
            v[b * RR + r] = H::template kernel<Re>(m, v[b * RR + r], io0 + pos * pl.ps, pos, n);
          }
        }
      }
    });
    P.template run<true, true>(v, pl, sm, tw);
  }
  const Re s = Re(a.scale);
  P.template last<REV>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
      if (ok) H::template store<Re>(m, scale(val, s), io0 + pos * pl.ps, pos, n);
    });
  });
}

}  // namespace vdx
