// Batched map-reduce kernels.
//
// Same two-stage shape as the reference (vkdispatch/reduce/stage.py:31-145:
// grid-stride accumulate -> shared-memory tree -> subgroup butterfly; stage 2
// folds the per-workgroup partials), re-designed: each CTA owns one
// contiguous chunk of a row and keeps four independent loads in flight per
// thread, the tree is warp shuffles plus one 32-slot shared array, partials
// go to a caller-provided workspace rather than the output buffer, and stage
// 2 folds the partials of a row in a fixed order, so results depend only on
// n and never on scheduling.
#include "vdx_internal.h"
#include "vdx.h"

#include <math_constants.h>

#include <cstdio>
#include <limits>
#include <map>
#include <mutex>
#include <utility>

namespace vdx {

namespace {

template <class T, int OP>
__device__ __forceinline__ T identity() {
  if constexpr (OP == VDX_RED_ADD || OP == VDX_RED_OR || OP == VDX_RED_XOR) return T(0);
  else if constexpr (OP == VDX_RED_MUL) return T(1);
  else if constexpr (OP == VDX_RED_AND) return T(~0ull);
  else if constexpr (std::is_floating_point<T>::value) {
    if (OP == VDX_RED_MIN) return T(CUDART_INF);
    return T(-CUDART_INF);
  } else {
    if (OP == VDX_RED_MIN) return std::numeric_limits<T>::max();
    return std::numeric_limits<T>::lowest();
  }
}

template <class T, int OP>
__device__ __forceinline__ T combine(T a, T b) {
  if constexpr (OP == VDX_RED_ADD) return a + b;
  else if constexpr (OP == VDX_RED_MUL) return a * b;
  else if constexpr (OP == VDX_RED_MIN) return a < b ? a : b;
  else if constexpr (OP == VDX_RED_MAX) return a > b ? a : b;
  else if constexpr (std::is_integral<T>::value) {
    if constexpr (OP == VDX_RED_AND) return a & b;
    else if constexpr (OP == VDX_RED_OR) return a | b;
    else return a ^ b;
  } else {
    return a;
  }
}

// map of one input element to the accumulation type
template <class In, class T, int MAP>
__device__ __forceinline__ T apply_map(In x) {
  if constexpr (std::is_same<In, Cx<float>>::value) {
    if constexpr (MAP == VDX_MAP_ABS) return T(sqrtf(x.x * x.x + x.y * x.y));
    else if constexpr (MAP == VDX_MAP_SQUARE) return T(x.x * x.x + x.y * x.y);
    else if constexpr (MAP == VDX_MAP_IMAG) return T(x.y);
    else return T(x.x);
  } else {
    if constexpr (MAP == VDX_MAP_ABS) return x < In(0) ? T(-x) : T(x);
    else if constexpr (MAP == VDX_MAP_SQUARE) return T(x) * T(x);
    else if constexpr (MAP == VDX_MAP_SIN) {
      if constexpr (std::is_same<In, double>::value) return T(sin(x));
      else return T(sinf(float(x)));
    } else return T(x);
  }
}

template <class T>
__device__ __forceinline__ T shfl_down(T v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}

template <class T, int OP>
__device__ __forceinline__ T block_reduce(T v, T* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v = combine<T, OP>(v, shfl_down(v, d));
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  if (w == 0) {
    v = lane < nw ? sh[lane] : identity<T, OP>();
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v = combine<T, OP>(v, shfl_down(v, d));
  }
  return v;
}

constexpr int kThreads = 512;

// stage 1: grid (nparts, batch); CTA p of row b covers elements
// [p*chunk, min(n, (p+1)*chunk)) with a block-stride loop.
template <class In, class T, int OP, int MAP>
__global__ void __launch_bounds__(kThreads) k_reduce_partial(const In* __restrict__ in, long long n, long long chunk,
                                                             T* __restrict__ part, int nparts) {
  __shared__ T sh[32];
  const long long b = blockIdx.y;
  const In* row = in + b * n;
  const long long lo = (long long)blockIdx.x * chunk;
  long long hi = lo + chunk;
  if (hi > n) hi = n;
  T a0 = identity<T, OP>(), a1 = a0, a2 = a0, a3 = a0;
  long long i = lo + threadIdx.x;
  for (; i + 3 * kThreads < hi; i += 4 * kThreads) {
    const In x0 = row[i], x1 = row[i + kThreads], x2 = row[i + 2 * kThreads], x3 = row[i + 3 * kThreads];
    a0 = combine<T, OP>(a0, apply_map<In, T, MAP>(x0));
    a1 = combine<T, OP>(a1, apply_map<In, T, MAP>(x1));
    a2 = combine<T, OP>(a2, apply_map<In, T, MAP>(x2));
    a3 = combine<T, OP>(a3, apply_map<In, T, MAP>(x3));
  }
  for (; i < hi; i += kThreads) a0 = combine<T, OP>(a0, apply_map<In, T, MAP>(row[i]));
  T acc = combine<T, OP>(combine<T, OP>(a0, a1), combine<T, OP>(a2, a3));
  acc = block_reduce<T, OP>(acc, sh);
  if (threadIdx.x == 0) part[b * nparts + blockIdx.x] = acc;
}

// stage 2: one CTA per row folds nparts partials
template <class T, int OP>
__global__ void __launch_bounds__(kThreads) k_reduce_final(const T* __restrict__ part, int nparts, T* __restrict__ out) {
  __shared__ T sh[32];
  const long long b = blockIdx.x;
  T acc = identity<T, OP>();
  for (int i = threadIdx.x; i < nparts; i += kThreads) acc = combine<T, OP>(acc, part[b * nparts + i]);
  acc = block_reduce<T, OP>(acc, sh);
  if (threadIdx.x == 0) out[b] = acc;
}

template <class In, class T, int OP, int MAP>
cudaError_t run(const void* in, long long n, long long batch, void* out, void* partials, int nparts, cudaStream_t s) {
  const long long chunk = (n + nparts - 1) / nparts;
  dim3 g1((unsigned)nparts, (unsigned)batch);
  k_reduce_partial<In, T, OP, MAP><<<g1, kThreads, 0, s>>>(reinterpret_cast<const In*>(in), n, chunk,
                                                          reinterpret_cast<T*>(partials), nparts);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_reduce_final<T, OP><<<(unsigned)batch, kThreads, 0, s>>>(reinterpret_cast<const T*>(partials), nparts,
                                                             reinterpret_cast<T*>(out));
  return cudaGetLastError();
}

template <class In, class T, int OP>
cudaError_t by_map(int map, const void* in, long long n, long long batch, void* out, void* partials, int nparts,
                   cudaStream_t s) {
  switch (map) {
    case VDX_MAP_IDENTITY: return run<In, T, OP, VDX_MAP_IDENTITY>(in, n, batch, out, partials, nparts, s);
    case VDX_MAP_ABS: return run<In, T, OP, VDX_MAP_ABS>(in, n, batch, out, partials, nparts, s);
    case VDX_MAP_SQUARE: return run<In, T, OP, VDX_MAP_SQUARE>(in, n, batch, out, partials, nparts, s);
    case VDX_MAP_REAL: return run<In, T, OP, VDX_MAP_REAL>(in, n, batch, out, partials, nparts, s);
    case VDX_MAP_IMAG: return run<In, T, OP, VDX_MAP_IMAG>(in, n, batch, out, partials, nparts, s);
    case VDX_MAP_SIN: return run<In, T, OP, VDX_MAP_SIN>(in, n, batch, out, partials, nparts, s);
    default: return cudaErrorInvalidValue;
  }
}

template <class In, class T>
cudaError_t by_op_arith(int op, int map, const void* in, long long n, long long batch, void* out, void* partials,
                        int nparts, cudaStream_t s) {
  switch (op) {
    case VDX_RED_ADD: return by_map<In, T, VDX_RED_ADD>(map, in, n, batch, out, partials, nparts, s);
    case VDX_RED_MUL: return by_map<In, T, VDX_RED_MUL>(map, in, n, batch, out, partials, nparts, s);
    case VDX_RED_MIN: return by_map<In, T, VDX_RED_MIN>(map, in, n, batch, out, partials, nparts, s);
    case VDX_RED_MAX: return by_map<In, T, VDX_RED_MAX>(map, in, n, batch, out, partials, nparts, s);
    default: return cudaErrorInvalidValue;
  }
}

template <class In, class T>
cudaError_t by_op_int(int op, int map, const void* in, long long n, long long batch, void* out, void* partials,
                      int nparts, cudaStream_t s) {
  switch (op) {
    case VDX_RED_AND: return run<In, T, VDX_RED_AND, VDX_MAP_IDENTITY>(in, n, batch, out, partials, nparts, s);
    case VDX_RED_OR: return run<In, T, VDX_RED_OR, VDX_MAP_IDENTITY>(in, n, batch, out, partials, nparts, s);
    case VDX_RED_XOR: return run<In, T, VDX_RED_XOR, VDX_MAP_IDENTITY>(in, n, batch, out, partials, nparts, s);
    default: return by_op_arith<In, T>(op, map, in, n, batch, out, partials, nparts, s);
  }
}

}  // namespace

cudaError_t launch_reduce(int op, int map, int in_type, const void* in, long long n, long long batch, void* out,
                          void* partials, int nparts, cudaStream_t s) {
  switch (in_type) {
    case VDX_F32: return by_op_arith<float, float>(op, map, in, n, batch, out, partials, nparts, s);
    case VDX_F64: return by_op_arith<double, double>(op, map, in, n, batch, out, partials, nparts, s);
    case VDX_C64: return by_op_arith<Cx<float>, float>(op, map, in, n, batch, out, partials, nparts, s);
    case VDX_I32: return by_op_int<int, int>(op, map, in, n, batch, out, partials, nparts, s);
    case VDX_U32: return by_op_int<unsigned, unsigned>(op, map, in, n, batch, out, partials, nparts, s);
    default: return cudaErrorInvalidValue;
  }
}

// ---------------------------------------------------------------------------
// Allocation-free reduction: the stage-1 partials live in a fixed device
// array instead of a caller-provided workspace.  Every GPU that loads libvdx
// holds VDX_REDUCE_NOALLOC_SCRATCH_BYTES of it until the process exits.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_reduce_scratch[VDX_REDUCE_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_scratch_mu;
// (device ordinal, CUDA context) -> device address of g_reduce_scratch.  The
// context is part of the key because a device reset (cudaDeviceReset, or a
// primary-context release and re-create) reloads the module, after which an
// address resolved in the old context is stale.
std::map<std::pair<int, void*>, void*> g_scratch_addr;

typedef int (*CtxGetCurrentFn)(void**);  // CUresult cuCtxGetCurrent(CUcontext*)

// cuCtxGetCurrent, fetched once from the driver without linking libcuda.
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<CtxGetCurrentFn>(p);
  });
  return fn;
}

// Host code only sees a host-side stand-in under the name g_reduce_scratch;
// its device address comes from cudaGetSymbolAddress, resolved once per
// device and context with that device current (the caller's current device).
cudaError_t scratch_for_current_device(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  // Before this thread's first runtime call no context may be current yet;
  // cudaGetSymbolAddress below makes the primary context current, and the
  // context is read again after it.
  void* ctx = nullptr;
  CtxGetCurrentFn get = ctx_get_current();
  if (get) get(&ctx);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (ctx) {
    auto it = g_scratch_addr.find({dev, ctx});
    if (it != g_scratch_addr.end()) {
      *out = it->second;
      return cudaSuccess;
    }
  }
  void* p = nullptr;
  e = cudaGetSymbolAddress(&p, g_reduce_scratch);
  if (e != cudaSuccess) return e;
  if (!ctx && get) get(&ctx);  // the lookup made the primary context current
  if (ctx) g_scratch_addr[{dev, ctx}] = p;
  *out = p;
  return cudaSuccess;
}

}  // namespace

}  // namespace vdx

extern "C" int vdx_reduce_noalloc(int op, int map, int in_type, const void* in, int64_t n, int64_t batch, void* out,
                                  void* stream) {
  using namespace vdx;
  int rc = check_reduce_args(op, map, in_type, in, n, batch, out);
  if (rc != VDX_OK) return rc;
  int64_t parts = 0;
  rc = vdx_reduce_partial_count(n, &parts);
  if (rc != VDX_OK) return rc;
  const long long need = (long long)parts * batch * reduce_out_bytes(in_type);
  if (need > (long long)VDX_REDUCE_NOALLOC_SCRATCH_BYTES) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "vdx_reduce_noalloc: %lld rows of %lld elements need %lld bytes of partials, above the %d-byte "
                  "static scratch; use vdx_reduce with a workspace",
                  (long long)batch, (long long)n, need, (int)VDX_REDUCE_NOALLOC_SCRATCH_BYTES);
    return set_error(VDX_ERR_UNSUPPORTED, msg);
  }
  void* scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) {
    char msg[256];
    std::snprintf(msg, sizeof(msg), "vdx_reduce_noalloc: cudaGetSymbolAddress of the scratch array failed: %s",
                  cudaGetErrorString(e));
    return set_error(VDX_ERR_CUDA, msg);
  }
  e = launch_reduce(op, map, in_type, in, n, batch, out, scratch, (int)parts, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    char msg[256];
    std::snprintf(msg, sizeof(msg), "vdx_reduce_noalloc launch: %s", cudaGetErrorString(e));
    return set_error(VDX_ERR_CUDA, msg);
  }
  return VDX_OK;
}
