// Element-wise storage conversion between the FFT element types: the load and
// store ends of the map-hook menu (dtype casts, real <-> complex).
#include "vdx.h"
#include "vdx_common.cuh"
#include "vdx_internal.h"

namespace vdx {

namespace {

// complex value of element i of an array of `type`; real types give (x, 0)
__device__ __forceinline__ Cx<double> load_any(const void* p, int type, long long i) {
  switch (type) {
    case VDX_C64: { const Cx<float> v = reinterpret_cast<const Cx<float>*>(p)[i]; return mk<double>(v.x, v.y); }
    case VDX_C128: return reinterpret_cast<const Cx<double>*>(p)[i];
    case VDX_C32: { const float2 f = __half22float2(reinterpret_cast<const __half2*>(p)[i]); return mk<double>(f.x, f.y); }
    case VDX_BF16X2: {
      const float2 f = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(p)[i]);
      return mk<double>(f.x, f.y);
    }
    case VDX_F32: return mk<double>(reinterpret_cast<const float*>(p)[i], 0.0);
    default: return mk<double>(reinterpret_cast<const double*>(p)[i], 0.0);
  }
}

// real types keep the real part
__device__ __forceinline__ void store_any(void* p, int type, long long i, Cx<double> v) {
  switch (type) {
    case VDX_C64: reinterpret_cast<Cx<float>*>(p)[i] = mk<float>(float(v.x), float(v.y)); break;
    case VDX_C128: reinterpret_cast<Cx<double>*>(p)[i] = v; break;
    case VDX_C32: reinterpret_cast<__half2*>(p)[i] = __floats2half2_rn(float(v.x), float(v.y)); break;
    case VDX_BF16X2: reinterpret_cast<__nv_bfloat162*>(p)[i] = __floats2bfloat162_rn(float(v.x), float(v.y)); break;
    case VDX_F32: reinterpret_cast<float*>(p)[i] = float(v.x); break;
    default: reinterpret_cast<double*>(p)[i] = v.x; break;
  }
}

__global__ void k_convert(const void* src, int st, void* dst, int dt, long long count) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    store_any(dst, dt, i, load_any(src, st, i));
}

bool known(int t) { return t == VDX_C64 || t == VDX_C128 || t == VDX_C32 || t == VDX_BF16X2 || t == VDX_F32 || t == VDX_F64; }

}  // namespace

}  // namespace vdx

extern "C" int vdx_convert(const void* src, int src_type, void* dst, int dst_type, int64_t count, void* stream) {
  using namespace vdx;
  if (!src || !dst) return set_error(VDX_ERR_INVALID, "vdx_convert: src and dst must be non-NULL device pointers");
  if (!known(src_type) || !known(dst_type)) return set_error(VDX_ERR_INVALID, "vdx_convert: unknown element type");
  if (count < 0) return set_error(VDX_ERR_INVALID, "vdx_convert: negative count");
  if (count == 0) return VDX_OK;
  long long blocks = (count + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_convert<<<(unsigned)blocks, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(src, src_type, dst, dst_type, count);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  return VDX_OK;
}
