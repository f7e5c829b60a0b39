// Map-reduce with a compiled map (the reference's vd.reduce.map_reduce /
// reduce(mapping_function=...) with an arbitrary mapping function,
// vkdispatch/reduce/stage.py:31-186).  Compiled at run time by NVRTC (jit.cu)
// with a hooks struct that the Python tracer generates from the user's map:
//   struct VdxReduceHooks {
//     template <class Re> static __device__ T map(const MapArgs& m, long long io);
//   };
// io is the reference's mapped_io_index() (the element's flat index in the
// buffer: row * n + i), and the map may read any of the call's buffers and
// scalars through m.  The two stages have the shape of the ahead-of-time
// kernels of reduce.cu: each CTA folds one contiguous chunk of a row with
// four independent maps in flight per thread, warp shuffles and one 32-slot
// shared array; stage 2 folds a row's partials in a fixed order.
#pragma once

#include "fft_mapped.cuh"

namespace vdx {

// accumulation types: float, double, int, unsigned and float2 (the
// reference's vec2, component-wise)
enum RedOp { kRedAdd = 0, kRedMul = 1, kRedMin = 2, kRedMax = 3, kRedAnd = 4, kRedOr = 5, kRedXor = 6 };

template <class T>
struct RedScalar {
  static __device__ __forceinline__ T inf_hi();
  static __device__ __forceinline__ T inf_lo();
};
template <>
struct RedScalar<float> {
  static __device__ __forceinline__ float inf_hi() { return __int_as_float(0x7f800000); }
  static __device__ __forceinline__ float inf_lo() { return __int_as_float(0xff800000); }
};
template <>
struct RedScalar<double> {
  static __device__ __forceinline__ double inf_hi() { return __longlong_as_double(0x7ff0000000000000ll); }
  static __device__ __forceinline__ double inf_lo() { return __longlong_as_double(0xfff0000000000000ll); }
};
template <>
struct RedScalar<int> {
  static __device__ __forceinline__ int inf_hi() { return 0x7fffffff; }
  static __device__ __forceinline__ int inf_lo() { return int(0x80000000u); }
};
template <>
struct RedScalar<unsigned> {
  static __device__ __forceinline__ unsigned inf_hi() { return 0xffffffffu; }
  static __device__ __forceinline__ unsigned inf_lo() { return 0u; }
};

template <class T, int OP>
__device__ __forceinline__ T red_identity1() {
  if constexpr (OP == kRedAdd || OP == kRedOr || OP == kRedXor) return T(0);
  else if constexpr (OP == kRedMul) return T(1);
  else if constexpr (OP == kRedAnd) return T(~0u);
  else if constexpr (OP == kRedMin) return RedScalar<T>::inf_hi();
  else return RedScalar<T>::inf_lo();
}

template <class T, int OP>
__device__ __forceinline__ T red_combine1(T a, T b) {
  if constexpr (OP == kRedAdd) return a + b;
  else if constexpr (OP == kRedMul) return a * b;
  else if constexpr (OP == kRedMin) return a < b ? a : b;
  else if constexpr (OP == kRedMax) return a > b ? a : b;
  else if constexpr (OP == kRedAnd) return a & b;
  else if constexpr (OP == kRedOr) return a | b;
  else return a ^ b;
}

template <class T, int OP>
struct Red {
  static __device__ __forceinline__ T identity() { return red_identity1<T, OP>(); }
  static __device__ __forceinline__ T combine(T a, T b) { return red_combine1<T, OP>(a, b); }
  static __device__ __forceinline__ T down(T v, int d) { return __shfl_down_sync(0xffffffffu, v, d); }
};
template <int OP>
struct Red<float2, OP> {
  static __device__ __forceinline__ float2 identity() {
    const float i = red_identity1<float, OP>();
    return make_float2(i, i);
  }
  static __device__ __forceinline__ float2 combine(float2 a, float2 b) {
    return make_float2(red_combine1<float, OP>(a.x, b.x), red_combine1<float, OP>(a.y, b.y));
  }
  static __device__ __forceinline__ float2 down(float2 v, int d) {
    return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
  }
};

// the map's value (of whatever type the generated expression has) as the
// accumulation type
template <class T>
struct RedCast {
  template <class V>
  static __device__ __forceinline__ T from(V v) { return T(v); }
  template <class R>
  static __device__ __forceinline__ T from(Cx<R> v) { return T(v.x); }
};
template <>
struct RedCast<float2> {
  template <class V>
  static __device__ __forceinline__ float2 from(V v) { return make_float2(float(v), float(v)); }
  template <class R>
  static __device__ __forceinline__ float2 from(Cx<R> v) { return make_float2(float(v.x), float(v.y)); }
};

template <class T, int OP>
__device__ __forceinline__ T red_block(T v, T* sh) {
  using RT = Red<T, OP>;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v = RT::combine(v, RT::down(v, d));
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  if (w == 0) {
    v = lane < nw ? sh[lane] : RT::identity();
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = RT::combine(v, RT::down(v, d));
  }
  return v;
}

constexpr int kRedThreads = 512;

// stage 1: grid (nparts, batch); CTA p of row b covers [p*chunk, min(n, (p+1)*chunk))
template <class H, class Re, class T, int OP>
__device__ __forceinline__ void reduce_mapped_partial(const MapArgs& m, long long n, long long chunk, T* part,
                                                      int nparts) {
  using RT = Red<T, OP>;
  __shared__ T sh[32];
  const long long b = blockIdx.y;
  const long long base = b * n;
  const long long lo = (long long)blockIdx.x * chunk;
  long long hi = lo + chunk;
  if (hi > n) hi = n;
  T a0 = RT::identity(), a1 = a0, a2 = a0, a3 = a0;
  long long i = lo + threadIdx.x;
  for (; i + 3 * kRedThreads < hi; i += 4 * kRedThreads) {
    a0 = RT::combine(a0, RedCast<T>::from(H::template map<Re>(m, base + i)));
    a1 = RT::combine(a1, RedCast<T>::from(H::template map<Re>(m, base + i + kRedThreads)));
    a2 = RT::combine(a2, RedCast<T>::from(H::template map<Re>(m, base + i + 2 * kRedThreads)));
    a3 = RT::combine(a3, RedCast<T>::from(H::template map<Re>(m, base + i + 3 * kRedThreads)));
  }
  for (; i < hi; i += kRedThreads) a0 = RT::combine(a0, RedCast<T>::from(H::template map<Re>(m, base + i)));
  T acc = RT::combine(RT::combine(a0, a1), RT::combine(a2, a3));
  acc = red_block<T, OP>(acc, sh);
  if (threadIdx.x == 0) part[b * nparts + blockIdx.x] = acc;
}

// stage 2: one CTA per row folds its nparts partials in a fixed order
template <class T, int OP>
__device__ __forceinline__ void reduce_mapped_final(const T* part, int nparts, T* out) {
  using RT = Red<T, OP>;
  __shared__ T sh[32];
  const long long b = blockIdx.x;
  T acc = RT::identity();
  for (int i = threadIdx.x; i < nparts; i += kRedThreads) acc = RT::combine(acc, part[b * nparts + i]);
  acc = red_block<T, OP>(acc, sh);
  if (threadIdx.x == 0) out[b] = acc;
}

}  // namespace vdx
