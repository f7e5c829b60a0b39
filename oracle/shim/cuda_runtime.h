// Host stand-in for the CUDA names used by kernels that the reference's CUDA
// code generator emits (test infrastructure only): lets a generated kernel
// compile with g++ and run one CTA at a time, one std::thread per CUDA
// thread, __syncthreads() as a std::barrier.  __sinf/__cosf map to the
// host's sinf/cosf (the device intrinsics are approximations).
#pragma once

#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstdlib>

struct float2 {
  float x, y;
};
struct double2 {
  double x, y;
};
struct uint3 {
  unsigned int x, y, z;
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

template <class T>
inline T __shfl_xor_sync(unsigned int, T, int) {
  std::fprintf(stderr, "warp shuffles are not emulated by the host shim\n");
  std::abort();
}
