// Internal launch interface between the C ABI (vdx_api.cu) and the kernel
// translation units.  Each launcher picks the template instantiation for a
// (storage, compute, direction, layout) combination and enqueues it.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "fft_kernels.cuh"

struct vdx_fft_desc;  // include/vdx.h

namespace vdx {

enum Store { ST_C64 = 0, ST_C32 = 1, ST_C128 = 2, ST_BF16 = 3 };

struct Launch {
  dim3 grid;
  dim3 block;
  size_t smem;
  cudaStream_t stream;
};

// Elements per thread of the instantiated kernels: registers hold MAXE
// complex values of the current pass, and every radix used by a plan must be
// <= MAXE.  fp32 compute keeps 16 (32 registers of data under the 64-register
// cap of 1024-thread CTAs); fp64 compute keeps 8.
template <class Re>
struct MaxE;
template <>
struct MaxE<float> {
  static constexpr int value = 16;
};
template <>
struct MaxE<double> {
  static constexpr int value = 8;
};

// Supported (storage, compute) pairs: complex64/fp32, complex32/fp32,
// bf16x2/fp32, complex128/fp64.
enum Op { OP_C2C_FWD, OP_C2C_INV, OP_CONV, OP_R2C_EVEN, OP_C2R_EVEN, OP_R2C_ODD, OP_C2R_ODD, OP_CONV2D_REAL };

template <class S, class Re>
cudaError_t launch_fft(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant);
template <class S, class Re>
cudaError_t launch_dyn_c2c(const FftArgs& a, const Launch& l, int op, bool strided, int variant);
template <class S, class Re>
cudaError_t launch_dyn_conv(const FftArgs& a, const Launch& l, bool strided, int kop, int variant);
template <class S, class Re>
cudaError_t launch_dyn_real(const FftArgs& a, const Launch& l, int op);

cudaError_t launch_twiddle(void* tab, int count, int den, bool f64, cudaStream_t s);

// One pass of a four-step long-axis transform (fft_large.cu): tiles of M
// adjacent columns, one pp.n-point transform per column.  Batch b of the
// launch starts at (b / split) * bs1 + (b % split) * bs2 elements; point pos
// of column c is at c + pos * ps on input, and at c * out_cs + pos * out_ps
// on output.  Grid = batches * col_tiles, block = pp.T * pp.M.
struct FsArgs {
  PassPlan pp;
  const void* in;
  void* out;
  const void* tw;   // W_n^k of the short transform
  const void* twl;  // W_N^k of the whole axis (pass A)
  long long split;
  long long in_bs1, in_bs2, out_bs1, out_bs2;
  long long in_ps, out_ps, out_cs;
  int ncols, col_tiles;
  int tw_from_batch;  // pass A: b0 is b % split (strided axes) or the column (contiguous axes)
  float scale;
  int* status;        // TMA-staged passes: set to 1 if a tile load's completion wait gives up
  long long nbatch;   // batches of this launch (grid = nbatch * col_tiles)
};
// mode 0: plain store; 1: twiddle, unit-stride columns; 2: twiddle, transposed store (out_ps == 1).
// With tma = true the input tiles arrive by one TMA bulk-tensor copy each
// when the geometry allows it (see fourstep_tma_ok); otherwise by loads.
cudaError_t launch_fourstep_pass(const FsArgs& a, const Launch& l, int store, bool inv, int mode, bool tma = false);
// Whether a pass's input tiles can be TMA copies: short length <= 256 (one
// box), 16-byte row and batch strides, 16-byte aligned base and columns.
bool fourstep_tma_ok(const FsArgs& a, int store);
// The same pass with the 128-point short transforms on the tensor cores
// (fft_tc.cu); a.pp.n must be 128 and a.pp.M 16 or 32.  bmat = the DFT
// operand image from tc_dft_operands; *status is set to 1 if an MMA
// completion wait gives up.
cudaError_t launch_fourstep_pass_tc(const FsArgs& a, const Launch& l, int store, bool inv, int mode,
                                    const void* bmat, int* status);
cudaError_t tc_dft_operands(int dev, bool inv, const void** out);
size_t tc_pass_smem(int mt);

// Both passes of a four-step long axis in one persistent launch with an
// L2-resident ring for the intermediate (fft_fused4.cu).  Square splits
// (N0 == N1, the same compile-time short plan for both passes) only.
struct FusedLaunch {
  PassPlan ppA, ppB;  // short-transform plans; M = columns per tile, equal for both
  const void* in;
  void* out;
  void* ring;  // R slots: N * M elements each (strided axes) or N (contiguous)
  const void* twA;
  const void* twB;
  const void* twl;
  long long N, N0, N1, inner, outer;
  int M;
  float scale;
  int L, R;
  unsigned* ticket;
  int* doneA;  // R counters each
  int* doneB;
  int* status;
  long long wait_limit;  // 0 = default
  int store;
  bool inverse, strided;
  unsigned grid;
  size_t smem;
};
cudaError_t fused_fourstep_ctas_per_sm(int store, const PassPlan& pp, size_t smem, int* per_sm);
cudaError_t launch_fused_fourstep(const FusedLaunch& fl, cudaStream_t s);

// One-launch 2-D convolution of real images (fft_conv2d.cu): one image per
// thread-block cluster, the half spectrum held in the cluster's shared memory.
struct Conv2dArgs {
  Cx<float>* data;          // (images, H, W/2 + 1) packed RFFT rows, in place
  const Cx<float>* ker;     // kernel spectrum, (images or 1, H, W/2 + 1)
  long long ker_bs;         // elements between images' kernel spectra (0 = broadcast)
  const Cx<float>* tw_row;  // W_{W/2}^k, k < W/2
  const Cx<float>* tw2;     // W_W^k, k <= W/2
  const Cx<float>* tw_col;  // W_H^k, k < H
  float col_scale, row_scale;
};
// Bluestein transforms (bluestein.cu): chirp tables w (N) and b (M), the
// conj(FFT(b)) kernel slab replicated over `inner` columns, and the
// chirp-in (zero-padded, to the (outer, M, inner) workspace) / chirp-out
// (cropped, scaled) element-wise launches.
cudaError_t launch_chirp_tables(void* w, void* b, int N, int M, int sign, bool f64, cudaStream_t s);
cudaError_t launch_conj_slab(void* K, const void* B, int M, long long inner, bool f64, cudaStream_t s);
cudaError_t launch_bluestein_mul(void* ws, const void* K, long long outer, int M, long long inner, bool f64,
                                 cudaStream_t s);
cudaError_t launch_bluestein_io(bool in_phase, int store, const void* x, void* ws, const void* w, long long outer,
                                int N, int M, long long inner, double scale, cudaStream_t s);

bool conv2d_real_supported(int H, int W);
cudaError_t conv2d_real_max_clusters(int H, int W, int* count);
cudaError_t launch_conv2d_real(const Conv2dArgs& a, int H, int W, long long images, int kop, cudaStream_t s);

// complex64 kernels specialised at compile time for power-of-two n in
// [16, 16384] (radix-16 passes, n/16 threads per transform)
template <int N>
cudaError_t launch_fixed_c64(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant);
bool has_fixed_c64(int n);
cudaError_t launch_fixed_c64_any(int n, const FftArgs& a, const Launch& l, int op, bool strided, int kop,
                                 int variant);
// complex64 kernels on the alternative compile-time plans: pts = 32 (two
// passes: radix 32 x 16 for n = 512, 32 x 32 for n = 1024; n/32 threads per
// transform) for every operation, and pts = 8 (radix-8 passes, n/8 threads)
// for strided convolutions of n = 512
template <int N>
cudaError_t launch_fixedpts_conv_c64(int pts, const FftArgs& a, const Launch& l, int kop, int variant);
template <int N>
cudaError_t launch_fixed32_c64(const FftArgs& a, const Launch& l, int op, bool strided, int kop, int variant);
bool has_fixedpts_c64(int n, int pts, bool conv, bool strided);

// fused multi-kernel convolution on the runtime-plan kernels (ST_C64 or
// ST_C128 storage); conv_multi_points = the kernel's points per thread
cudaError_t launch_conv_multi(int store, bool strided, const FftArgs& a, const Launch& l, int kop, int K,
                              long long kstride, long long ostride);
int conv_multi_points(bool f64);
// the same on the compile-time complex64 plans (n = 16 .. 512 and 1024 ..
// 16384 in two translation units)
// pts = 16 (Pow2Plan) or 32 (the two-pass plans of 512 and 1024 points)
cudaError_t launch_fixed_conv_multi_small(int n, int pts, bool strided, const FftArgs& a, const Launch& l, int kop,
                                          int K, long long kstride, long long ostride);
cudaError_t launch_fixed_conv_multi_large(int n, int pts, bool strided, const FftArgs& a, const Launch& l, int kop,
                                          int K, long long kstride, long long ostride);
cudaError_t launch_fixedpts_c64_any(int n, int pts, const FftArgs& a, const Launch& l, int op, bool strided, int kop,
                                    int variant);

// Opt a kernel into more than 48 KB of dynamic shared memory once.
template <class K>
inline cudaError_t prepare_smem(K kernel, size_t smem) {
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <class K, class... Args>
inline cudaError_t enqueue(K kernel, const Launch& l, Args... args) {
  cudaError_t e = prepare_smem(kernel, l.smem);
  if (e != cudaSuccess) return e;
  kernel<<<l.grid, l.block, l.smem, l.stream>>>(args...);
  return cudaGetLastError();
}

// Programmatic dependent launch for the kernels that open with pdl_enter()
// (fft_kernels.cuh): on unless VDX_PDL=0.
bool pdl_enabled();

template <class... KArgs, class... Args>
inline cudaError_t enqueue_pdl(void (*kernel)(KArgs...), const Launch& l, Args... args) {
  if (!pdl_enabled()) return enqueue(kernel, l, args...);
  cudaError_t e = prepare_smem(kernel, l.smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = l.grid;
  cfg.blockDim = l.block;
  cfg.dynamicSmemBytes = l.smem;
  cfg.stream = l.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Geometry of a single-CTA-per-transform plan (no four-step, no Bluestein)
// for the run-time compiled map kernels of jit.cu: the planner's pass plan,
// launch shape and twiddle table for the descriptor's axis.
struct MapGeometry {
  FftArgs args;
  Launch launch;
  std::vector<int> radices;
  bool strided;
  bool f64;
  int N;
  int dev;
};
int map_plan_geometry(const ::vdx_fft_desc& d, MapGeometry* g);

// error reporting and argument checks shared by the C entry points
int set_error(int code, const char* msg);
int check_reduce_args(int op, int map, int in_type, const void* in, long long n, long long batch, const void* out);
int reduce_out_bytes(int in_type);

// reductions
cudaError_t launch_reduce(int op, int map, int in_type, const void* in, long long n, long long batch, void* out,
                          void* partials, int nparts, cudaStream_t s);

}  // namespace vdx
