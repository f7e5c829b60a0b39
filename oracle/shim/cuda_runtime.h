// Host stand-in for the CUDA names used by kernels that the reference's CUDA
// code generator emits (test infrastructure only): lets a generated kernel
// compile with g++ and run one CTA at a time, one std::thread per CUDA
// thread, __syncthreads() as a std::barrier, warp shuffles through a
// per-warp exchange array.  __sinf/__cosf map to the
// host's sinf/cosf (the device intrinsics are approximations).
#pragma once

#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

struct float2 {
  float x, y;
};
struct double2 {
  double x, y;
};
struct uint3 {
  unsigned int x, y, z;
};
struct alignas(16) uint4 {
  unsigned int x, y, z, w;
};
struct alignas(16) int4 {
  int x, y, z, w;
};
struct alignas(16) float4 {
  float x, y, z, w;
};
struct int2 {
  int x, y;
};
struct uint2 {
  unsigned int x, y;
};
struct dim3 {
  unsigned int x, y, z;
};

namespace vdx_shim {
extern thread_local uint3 tid;
extern uint3 bid;
extern dim3 bdim;
extern dim3 gdim;
extern std::barrier<>* bar;
}  // namespace vdx_shim

#define threadIdx (vdx_shim::tid)
#define blockIdx (vdx_shim::bid)
#define blockDim (vdx_shim::bdim)
#define gridDim (vdx_shim::gdim)

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static

inline void __syncthreads() { vdx_shim::bar->arrive_and_wait(); }
inline float __sinf(float x) { return sinf(x); }
inline float __cosf(float x) { return cosf(x); }
inline float __expf(float x) { return expf(x); }
inline float __logf(float x) { return logf(x); }
inline float __fdividef(float a, float b) { return a / b; }

#define warpSize 32

// Warp collectives, emulated with one exchange array and one barrier per
// warp (every lane of the warp must call them, as the generated reduction
// kernels do).
namespace vdx_shim {
struct Warp {
  unsigned long long slot[32];
  std::barrier<>* bar;
};
extern thread_local int lin;  // linear thread index inside the CTA
extern Warp* warps;
}  // namespace vdx_shim

inline void __syncwarp(unsigned int = 0xffffffffu) { vdx_shim::warps[vdx_shim::lin / 32].bar->arrive_and_wait(); }

template <class T>
inline T __shfl_xor_sync(unsigned int, T value, int lane_mask) {
  static_assert(sizeof(T) <= sizeof(unsigned long long), "scalar shuffles only");
  vdx_shim::Warp& w = vdx_shim::warps[vdx_shim::lin / 32];
  const int lane = vdx_shim::lin % 32;
  std::memcpy(&w.slot[lane], &value, sizeof(T));
  w.bar->arrive_and_wait();
  T r;
  std::memcpy(&r, &w.slot[lane ^ lane_mask], sizeof(T));
  w.bar->arrive_and_wait();
  return r;
}
