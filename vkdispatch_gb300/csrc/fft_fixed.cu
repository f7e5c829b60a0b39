// Dispatch to the compile-time specialised complex64 kernels.
#include "vdx_internal.h"

namespace vdx {

bool has_fixed_c64(int n) {
  return n >= 16 && n <= 16384 && (n & (n - 1)) == 0;
}

cudaError_t launch_fixed_c64_any(int n, const FftArgs& a, const Launch& l, int op, bool strided, int kop,
                                 int variant) {
  switch (n) {
    case 16: return launch_fixed_c64<16>(a, l, op, strided, kop, variant);
    case 32: return launch_fixed_c64<32>(a, l, op, strided, kop, variant);
    case 64: return launch_fixed_c64<64>(a, l, op, strided, kop, variant);
    case 128: return launch_fixed_c64<128>(a, l, op, strided, kop, variant);
    case 256: return launch_fixed_c64<256>(a, l, op, strided, kop, variant);
    case 512: return launch_fixed_c64<512>(a, l, op, strided, kop, variant);
    case 1024: return launch_fixed_c64<1024>(a, l, op, strided, kop, variant);
    case 2048: return launch_fixed_c64<2048>(a, l, op, strided, kop, variant);
    case 4096: return launch_fixed_c64<4096>(a, l, op, strided, kop, variant);
    case 8192: return launch_fixed_c64<8192>(a, l, op, strided, kop, variant);
    case 16384: return launch_fixed_c64<16384>(a, l, op, strided, kop, variant);
    default: return cudaErrorInvalidValue;
  }
}

bool has_fixedpts_c64(int n, int pts, bool conv, bool strided) {
  if (pts == 8) return conv && strided && n == 512;
  return pts == 32 && (n == 512 || n == 1024);
}

cudaError_t launch_fixedpts_c64_any(int n, int pts, const FftArgs& a, const Launch& l, int op, bool strided, int kop,
                                    int variant) {
  if (pts == 8) {
    if (op == OP_CONV && strided && n == 512) return launch_fixedpts_conv_c64<512>(8, a, l, kop, variant);
    return cudaErrorInvalidValue;
  }
  if (pts != 32) return cudaErrorInvalidValue;
  switch (n) {
    case 512: return launch_fixed32_c64<512>(a, l, op, strided, kop, variant);
    case 1024: return launch_fixed32_c64<1024>(a, l, op, strided, kop, variant);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
