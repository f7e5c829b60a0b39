// Complex arithmetic, compile-time DFT constants and register-resident radix
// butterflies shared by every FFT kernel of libvdx.
//
// The reference generates one radix-P DFT per prime group at runtime as CUDA
// source (vkdispatch/fft/cooley_tukey.py:55-92 radix_P, :132-180
// radix_composite).  Here the butterflies are C++ templates instantiated ahead
// of time: composite radices (4, 8, 16, ...) use an in-register Cooley-Tukey
// split, odd primes use the symmetric (cos/sin pair) DFT, and every constant
// twiddle is folded at compile time from a constexpr Taylor series evaluated
// in double precision.
#pragma once

#ifdef __CUDACC_RTC__
// runtime-compiled map kernels (NVRTC): no host headers
#include <cuda_fp16.h>
#include <cuda_bf16.h>
typedef unsigned short uint16_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#else
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>
#endif

namespace vdx {

// the few type traits the kernels use, here so that the same headers compile
// under NVRTC, which has no standard library
template <class T, T V>
struct IntConst {
  static constexpr T value = V;
  constexpr operator T() const { return V; }
};
using TrueT = IntConst<bool, true>;
using FalseT = IntConst<bool, false>;
template <bool B, class A, class C>
struct Cond {
  using type = A;
};
template <class A, class C>
struct Cond<false, A, C> {
  using type = C;
};
template <class A, class C>
struct Same : FalseT {};
template <class A>
struct Same<A, A> : TrueT {};

// ---------------------------------------------------------------------------
// complex value in registers
// ---------------------------------------------------------------------------
template <class R>
struct alignas(2 * sizeof(R)) Cx {
  R x, y;
};

template <class R>
__device__ __forceinline__ Cx<R> mk(R a, R b) {
  Cx<R> c;
  c.x = a;
  c.y = b;
  return c;
}
template <class R>
__device__ __forceinline__ Cx<R> operator+(Cx<R> a, Cx<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <class R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a, Cx<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <class R>
__device__ __forceinline__ Cx<R> scale(Cx<R> a, R s) { return mk<R>(a.x * s, a.y * s); }
template <class R>
__device__ __forceinline__ Cx<R> conj(Cx<R> a) { return mk<R>(a.x, -a.y); }

// a * b with one rounding per component pair (fma).
__device__ __forceinline__ Cx<float> cmul(Cx<float> a, Cx<float> b) {
  return mk<float>(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ Cx<double> cmul(Cx<double> a, Cx<double> b) {
  return mk<double>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ Cx<float> cmulc(Cx<float> a, Cx<float> b) {
  return mk<float>(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ Cx<double> cmulc(Cx<double> a, Cx<double> b) {
  return mk<double>(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}

// read-only (non-coherent cache) load of a complex table entry
__device__ __forceinline__ Cx<float> ldg(const Cx<float>* p) {
  const float2 f = __ldg(reinterpret_cast<const float2*>(p));
  return mk<float>(f.x, f.y);
}
__device__ __forceinline__ Cx<double> ldg(const Cx<double>* p) {
  const double2 f = __ldg(reinterpret_cast<const double2*>(p));
  return mk<double>(f.x, f.y);
}

// multiply by -i (forward quarter turn) or +i (inverse quarter turn)
template <bool INV, class R>
__device__ __forceinline__ Cx<R> mul_mi(Cx<R> a) {
  if (INV) return mk<R>(-a.y, a.x);  // * (+i)
  return mk<R>(a.y, -a.x);           // * (-i)
}

// ---------------------------------------------------------------------------
// compile-time cos/sin of 2*pi*num/den (double precision)
// ---------------------------------------------------------------------------
constexpr double kHalfPi = 1.57079632679489661923132169163975144;

constexpr double cx_sin_q(double x) {  // |x| <= pi/2, Taylor series
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / double((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
constexpr double cx_cos_q(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / double((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// Reduce num/den to quarter turns exactly on the integers, then evaluate the
// remaining angle in [0, pi/2) and rotate by the quarter-turn count.
constexpr double cx_cos_frac(long long num, long long den) {
  long long n = ((num % den) + den) % den;
  long long q = (4 * n) / den;
  long long r = 4 * n - q * den;
  double phi = kHalfPi * double(r) / double(den);
  double c = cx_cos_q(phi), s = cx_sin_q(phi);
  return q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}
constexpr double cx_sin_frac(long long num, long long den) {
  long long n = ((num % den) + den) % den;
  long long q = (4 * n) / den;
  long long r = 4 * n - q * den;
  double phi = kHalfPi * double(r) / double(den);
  double c = cx_cos_q(phi), s = cx_sin_q(phi);
  return q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
}

// W_R^E = exp(sign * 2*pi*i*E/R), sign = -1 forward, +1 inverse.
template <int R, int E, bool INV>
struct Wc {
  static constexpr double c = cx_cos_frac(E, R);
  static constexpr double s = (INV ? 1.0 : -1.0) * cx_sin_frac(E, R);
};

// Multiply by the compile-time twiddle W_R^E, with exact shortcuts for
// multiples of an eighth turn.
template <int R, int E, bool INV, class Re>
__device__ __forceinline__ Cx<Re> twc(Cx<Re> a) {
  constexpr int e = ((E % R) + R) % R;
  if constexpr (e == 0) {
    return a;
  } else if constexpr ((4 * e) % R == 0) {
    constexpr int q = (4 * e) / R;  // quarter turns
    if constexpr (q == 2) return mk<Re>(-a.x, -a.y);
    else if constexpr (q == 1) return mul_mi<INV>(a);
    else return mul_mi<!INV>(a);
  } else if constexpr ((8 * e) % R == 0) {
    constexpr Re h = Re(0.70710678118654752440084436210484904);
    constexpr int o = (8 * e) / R;  // odd number of eighth turns
    // (1 -+ i)/sqrt2 rotations
    Cx<Re> r = mk<Re>((a.x + (INV ? -a.y : a.y)) * h, (a.y + (INV ? a.x : -a.x)) * h);  // * W_8^1
    if constexpr (o == 1) return r;
    else if constexpr (o == 3) return mul_mi<INV>(r);
    else if constexpr (o == 5) return mk<Re>(-r.x, -r.y);
    else return mul_mi<!INV>(r);
  } else {
    constexpr Re c = Re(Wc<R, e, INV>::c);
    constexpr Re s = Re(Wc<R, e, INV>::s);
    return cmul(a, mk<Re>(c, s));
  }
}

// ---------------------------------------------------------------------------
// in-register DFTs, natural order in and out:  v[k] <- sum_n v[n] W_R^{nk}
// ---------------------------------------------------------------------------
template <int R>
struct SmallestFactor {
  static constexpr int value = (R % 4 == 0 && R > 4) ? 4 : (R % 2 == 0) ? 2 : (R % 3 == 0) ? 3 : (R % 5 == 0) ? 5 : R;
};

template <int R, bool INV, class Re>
struct Dft;

template <bool INV, class Re>
struct Dft<1, INV, Re> {
  static __device__ __forceinline__ void run(Cx<Re>*) {}
};

template <bool INV, class Re>
struct Dft<2, INV, Re> {
  static __device__ __forceinline__ void run(Cx<Re>* v) {
    Cx<Re> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  }
};

template <bool INV, class Re>
struct Dft<4, INV, Re> {
  static __device__ __forceinline__ void run(Cx<Re>* v) {
    Cx<Re> t0 = v[0] + v[2], t1 = v[0] - v[2];
    Cx<Re> t2 = v[1] + v[3], t3 = mul_mi<INV>(v[1] - v[3]);
    v[0] = t0 + t2;
    v[2] = t0 - t2;
    v[1] = t1 + t3;
    v[3] = t1 - t3;
  }
};

// Odd prime P: pair n with P-n so each constant is used on a sum and a
// difference; y_k = a_k -/+ i b_k and y_{P-k} = a_k +/- i b_k.
template <int P, bool INV, class Re>
struct DftOdd {
  static __device__ __forceinline__ void run(Cx<Re>* v) {
    constexpr int H = (P - 1) / 2;
    Cx<Re> s[H + 1], d[H + 1];
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      s[j] = v[j] + v[P - j];
      d[j] = v[j] - v[P - j];
    }
    Cx<Re> x0 = v[0];
    Cx<Re> y0 = x0;
#pragma unroll
    for (int j = 1; j <= H; ++j) y0 = y0 + s[j];
    Cx<Re> out[P];
    out[0] = y0;
    Body<1>::go(x0, s, d, out);
#pragma unroll
    for (int k = 0; k < P; ++k) v[k] = out[k];
  }
  template <int K, bool Dummy = true>
  struct Body {
    static __device__ __forceinline__ void go(Cx<Re> x0, const Cx<Re>* s, const Cx<Re>* d, Cx<Re>* out) {
      constexpr int H = (P - 1) / 2;
      Cx<Re> a = x0, b = mk<Re>(Re(0), Re(0));
      Acc<1, K>::go(a, b, s, d);
      // forward: y_k = a - i b ; inverse: y_k = a + i b
      Cx<Re> ib = mk<Re>(-b.y, b.x);
      if (INV) {
        out[K] = a + ib;
        out[P - K] = a - ib;
      } else {
        out[K] = a - ib;
        out[P - K] = a + ib;
      }
      if constexpr (K < H) Body<K + 1>::go(x0, s, d, out);
    }
  };
  template <int J, int K, bool Dummy = true>
  struct Acc {
    static __device__ __forceinline__ void go(Cx<Re>& a, Cx<Re>& b, const Cx<Re>* s, const Cx<Re>* d) {
      constexpr int H = (P - 1) / 2;
      constexpr Re c = Re(cx_cos_frac((long long)J * K, P));
      constexpr Re sn = Re(cx_sin_frac((long long)J * K, P));
      a.x = fma_(c, s[J].x, a.x);
      a.y = fma_(c, s[J].y, a.y);
      b.x = fma_(sn, d[J].x, b.x);
      b.y = fma_(sn, d[J].y, b.y);
      if constexpr (J < H) Acc<J + 1, K>::go(a, b, s, d);
    }
  };
  static __device__ __forceinline__ Re fma_(Re a, Re b, Re c) { return a * b + c; }
};

template <bool INV, class Re>
struct Dft<3, INV, Re> : DftOdd<3, INV, Re> {};
template <bool INV, class Re>
struct Dft<5, INV, Re> : DftOdd<5, INV, Re> {};
template <bool INV, class Re>
struct Dft<7, INV, Re> : DftOdd<7, INV, Re> {};
template <bool INV, class Re>
struct Dft<11, INV, Re> : DftOdd<11, INV, Re> {};
template <bool INV, class Re>
struct Dft<13, INV, Re> : DftOdd<13, INV, Re> {};

// Composite R = A*B (A = smallest factor): n = a + A*b, k = kb + B*ka.
//   y[kb + B ka] = sum_a W_A^{a ka} ( W_R^{a kb} sum_b x[a + A b] W_B^{b kb} )
template <int R, int A, bool INV, class Re>
struct DftComposite {
  static constexpr int B = R / A;
  static __device__ __forceinline__ void run(Cx<Re>* v) {
    Cx<Re> z[A][B];
#pragma unroll
    for (int a = 0; a < A; ++a)
#pragma unroll
      for (int b = 0; b < B; ++b) z[a][b] = v[a + A * b];
#pragma unroll
    for (int a = 0; a < A; ++a) Dft<B, INV, Re>::run(z[a]);
    Tw<1, 1>::go(z);
#pragma unroll
    for (int kb = 0; kb < B; ++kb) {
      Cx<Re> t[A];
#pragma unroll
      for (int a = 0; a < A; ++a) t[a] = z[a][kb];
      Dft<A, INV, Re>::run(t);
#pragma unroll
      for (int ka = 0; ka < A; ++ka) v[kb + B * ka] = t[ka];
    }
  }
  template <int a, int kb, bool Dummy = true>
  struct Tw {
    static __device__ __forceinline__ void go(Cx<Re> (&z)[A][B]) {
      z[a][kb] = twc<R, a * kb, INV>(z[a][kb]);
      if constexpr (kb + 1 < B) Tw<a, kb + 1>::go(z);
      else if constexpr (a + 1 < A) Tw<a + 1, 1>::go(z);
    }
  };
};

template <bool INV, class Re>
struct Dft<6, INV, Re> : DftComposite<6, 2, INV, Re> {};
template <bool INV, class Re>
struct Dft<8, INV, Re> : DftComposite<8, 2, INV, Re> {};
template <bool INV, class Re>
struct Dft<9, INV, Re> : DftComposite<9, 3, INV, Re> {};
template <bool INV, class Re>
struct Dft<10, INV, Re> : DftComposite<10, 2, INV, Re> {};
template <bool INV, class Re>
struct Dft<12, INV, Re> : DftComposite<12, 4, INV, Re> {};
template <bool INV, class Re>
struct Dft<16, INV, Re> : DftComposite<16, 4, INV, Re> {};
template <bool INV, class Re>
struct Dft<32, INV, Re> : DftComposite<32, 4, INV, Re> {};

// ---------------------------------------------------------------------------
// storage <-> compute conversions
// ---------------------------------------------------------------------------
struct c32s {  // complex32: (re, im) as two IEEE halves
  __half2 v;
};
struct bf16c {  // bf16 pair storage
  __nv_bfloat162 v;
};

template <class S, class Re>
struct Conv;

template <>
struct Conv<Cx<float>, float> {
  static __device__ __forceinline__ Cx<float> ld(const Cx<float>* p) { return *p; }
  static __device__ __forceinline__ void st(Cx<float>* p, Cx<float> v) { *p = v; }
};
template <>
struct Conv<Cx<double>, double> {
  static __device__ __forceinline__ Cx<double> ld(const Cx<double>* p) { return *p; }
  static __device__ __forceinline__ void st(Cx<double>* p, Cx<double> v) { *p = v; }
};
template <>
struct Conv<Cx<float>, double> {
  static __device__ __forceinline__ Cx<double> ld(const Cx<float>* p) {
    Cx<float> a = *p;
    return mk<double>(a.x, a.y);
  }
  static __device__ __forceinline__ void st(Cx<float>* p, Cx<double> v) { *p = mk<float>(float(v.x), float(v.y)); }
};
template <>
struct Conv<Cx<double>, float> {
  static __device__ __forceinline__ Cx<float> ld(const Cx<double>* p) {
    Cx<double> a = *p;
    return mk<float>(float(a.x), float(a.y));
  }
  static __device__ __forceinline__ void st(Cx<double>* p, Cx<float> v) { *p = mk<double>(v.x, v.y); }
};
template <>
struct Conv<c32s, float> {
  static __device__ __forceinline__ Cx<float> ld(const c32s* p) {
    float2 f = __half22float2(p->v);
    return mk<float>(f.x, f.y);
  }
  static __device__ __forceinline__ void st(c32s* p, Cx<float> v) { p->v = __floats2half2_rn(v.x, v.y); }
};
template <>
struct Conv<c32s, double> {
  static __device__ __forceinline__ Cx<double> ld(const c32s* p) {
    float2 f = __half22float2(p->v);
    return mk<double>(f.x, f.y);
  }
  static __device__ __forceinline__ void st(c32s* p, Cx<double> v) {
    p->v = __floats2half2_rn(float(v.x), float(v.y));
  }
};
template <>
struct Conv<bf16c, float> {
  static __device__ __forceinline__ Cx<float> ld(const bf16c* p) {
    float2 f = __bfloat1622float2(p->v);
    return mk<float>(f.x, f.y);
  }
  static __device__ __forceinline__ void st(bf16c* p, Cx<float> v) { p->v = __floats2bfloat162_rn(v.x, v.y); }
};

// scalar (real) storage of the same precision family as S
template <class S>
struct RealOf;
template <>
struct RealOf<Cx<float>> { using type = float; };
template <>
struct RealOf<Cx<double>> { using type = double; };
template <>
struct RealOf<c32s> { using type = __half; };
template <>
struct RealOf<bf16c> { using type = __nv_bfloat16; };

template <class Re>
__device__ __forceinline__ Re to_re(float a) { return Re(a); }
template <class Re>
__device__ __forceinline__ Re ld_real(const float* p) { return Re(*p); }
template <class Re>
__device__ __forceinline__ Re ld_real(const double* p) { return Re(*p); }
template <class Re>
__device__ __forceinline__ Re ld_real(const __half* p) { return Re(__half2float(*p)); }
template <class Re>
__device__ __forceinline__ Re ld_real(const __nv_bfloat16* p) { return Re(__bfloat162float(*p)); }
template <class Re>
__device__ __forceinline__ void st_real(float* p, Re v) { *p = float(v); }
template <class Re>
__device__ __forceinline__ void st_real(double* p, Re v) { *p = double(v); }
template <class Re>
__device__ __forceinline__ void st_real(__half* p, Re v) { *p = __float2half_rn(float(v)); }
template <class Re>
__device__ __forceinline__ void st_real(__nv_bfloat16* p, Re v) { *p = __float2bfloat16_rn(float(v)); }

// read-once load marked evict-first (ld.global.cs for complex64): a kernel
// spectrum read once per launch leaves room in L2 for the outputs that the
// next launch reads
template <class S, class Re>
__device__ __forceinline__ Cx<Re> ld_once(const S* p) { return Conv<S, Re>::ld(p); }
template <>
__device__ __forceinline__ Cx<float> ld_once<Cx<float>, float>(const Cx<float>* p) {
  const float2 f = __ldcs(reinterpret_cast<const float2*>(p));
  return mk<float>(f.x, f.y);
}

}  // namespace vdx
