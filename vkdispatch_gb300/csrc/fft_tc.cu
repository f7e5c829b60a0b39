// Four-step passes whose 128-point short transforms run on the tensor cores.
//
// A tile is 128 points x MT adjacent columns (the geometry of k_fs in
// fft_large.cu).  With n = 8p + q and k = k1 + 16 k2:
//   stage 1: for every (q, column), the DFT-16 over p, times W_128^{q k1};
//   stage 2: for every (k1, column), the DFT-8 over q, giving X[k1 + 16 k2].
// Each stage is one real GEMM per 128 DFT vectors: a vector of P complex
// points is a row of 2P reals (re, im interleaved), and the DFT matrix is the
// 2P x 2P real matrix [[Fr, Fi], [-Fi, Fr]] (interleaved the same way).  The
// operands are BF16; accuracy is recovered with the three-product split
//   A B ~= A_hi B_hi + A_lo B_hi + A_hi B_lo,   X_hi = bf16(X), X_lo = bf16(X - X_hi),
// accumulated in FP32 in tensor memory.  The DFT matrices are split on the
// host from FP64 values; the twiddles W_128 and W_N come from FP64-built
// tables.  One elected thread issues the tcgen05.mma instructions; the whole
// CTA reads the accumulators back with tcgen05.ld.
//
// The reference has no tensor-core path (its FFT stages are scalar code
// generated per radix, vkdispatch/fft/cooley_tukey.py:55-180).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>

#include "fft_kernels.cuh"
#include "tc_ptx.cuh"
#include "vdx_internal.h"

namespace vdx {

namespace {

constexpr int kTcThreads = 128;
constexpr long long kTcWait = 1ll << 24;  // polls before an MMA completion wait gives up

// byte image of the four DFT operand matrices (K-major core-matrix layout)
constexpr int kB1 = 32 * 32 * 2;  // stage 1: N = 32 outputs x K = 32 inputs, bf16
constexpr int kB2 = 16 * 16 * 2;  // stage 2: N = 16 x K = 16
constexpr int kBBytes = 2 * kB1 + 2 * kB2;

// hi/lo split of a complex value into two packed bf16 pairs
__device__ __forceinline__ void split2(float re, float im, uint32_t& hi, uint32_t& lo) {
  __nv_bfloat162 h = __floats2bfloat162_rn(re, im);
  const float2 hf = __bfloat1622float2(h);
  __nv_bfloat162 l = __floats2bfloat162_rn(re - hf.x, im - hf.y);
  hi = *reinterpret_cast<uint32_t*>(&h);
  lo = *reinterpret_cast<uint32_t*>(&l);
}

constexpr int cmax(int a, int b) { return a > b ? a : b; }

template <int MT>
struct TcLayout {
  static constexpr int V1 = 8 * MT;     // stage-1 vectors (q, column)
  static constexpr int V2 = 16 * MT;    // stage-2 vectors (k1, column)
  static constexpr int T1 = V1 / 128;   // stage-1 M tiles
  static constexpr int T2 = V2 / 128;   // stage-2 M tiles
  static constexpr int A1 = V1 * 32 * 2;  // one stage-1 operand (hi or lo): V1 rows x 32 bf16
  static constexpr int A2 = V2 * 16 * 2;  // one stage-2 operand: V2 rows x 16 bf16
  static constexpr int STAGE = 129 * MT * 8;  // transposed-store staging (n + 1 slots per column)
  static constexpr int AREG = cmax(cmax(2 * A1, 2 * A2), STAGE);
  static constexpr int B_OFF = (AREG + 1023) / 1024 * 1024;
  static constexpr int BAR_OFF = B_OFF + kBBytes;
  static constexpr int SMEM = BAR_OFF + 16;
  static constexpr int TMEM_COLS = cmax(32, cmax(T1 * 32, T2 * 16));
};

// Stage-1 DFT vector of GEMM row v: (q, column).  For 32-column tiles of
// 4-byte storage the low 3 bits of v pick the column within a group of 8 and
// the next 2 bits the low bits of q, so a warp's 32 rows cover 8 columns x 4
// values of q: its stage-2 operand writes (row k1 * MT + column, K position
// 2q) fall in 32 distinct banks (row-major rows: 4-way conflicts, 13.1 M per
// launch -> 0.58 M) and its tile loads are 4 rows x 8 columns, whole 32-byte
// sectors.  16-column tiles (the default) keep the row-major order, which
// measured faster there (2-way conflicts, longer row segments).
template <int MT, int ES>
__device__ __forceinline__ void vec_qc(int v, int& q, int& c) {
  if constexpr (ES == 4 && MT == 32) {
    constexpr int CH = MT / 8;  // column groups of 8
    const int hi = v >> 5;
    q = ((v >> 3) & 3) + 4 * (hi / CH);
    c = (v & 7) + 8 * (hi % CH);
  } else {
    q = v / MT;
    c = v % MT;
  }
}

template <bool INV, class S, int MODE, int MT>
__global__ void __launch_bounds__(kTcThreads) k_fs_tc(FsArgs a, const unsigned char* __restrict__ bmat,
                                                     int* __restrict__ status) {
  using Lay = TcLayout<MT>;
  static_assert(Lay::T1 >= 1 && Lay::T2 >= 1, "MT must be 16 or 32");
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;
  unsigned char* sB = smem + Lay::B_OFF;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + Lay::BAR_OFF);
  uint32_t* slot = reinterpret_cast<uint32_t*>(smem + Lay::BAR_OFF + 8);
  const int tid = threadIdx.x, warp = tid >> 5;

  if (warp == 0) tc::tmem_alloc(slot, Lay::TMEM_COLS);
  if (tid == 0) tc::mbar_init(bar, 1);
  // DFT operand matrices: 5 KB, 16 bytes per thread per step
  for (int i = tid; i < kBBytes / 16; i += kTcThreads)
    reinterpret_cast<uint4*>(sB)[i] = __ldg(reinterpret_cast<const uint4*>(bmat) + i);

  const int tile = blockIdx.x % a.col_tiles;
  const long long b = blockIdx.x / a.col_tiles;
  const long long bq = b / a.split, br = b - bq * a.split;
  const S* in = reinterpret_cast<const S*>(a.in) + bq * a.in_bs1 + br * a.in_bs2;
  const long long ips = a.in_ps;

  // ---- stage-1 operands: vector v = 128 t + tid = (q, column), points x[8p + q]
#pragma unroll
  for (int t = 0; t < Lay::T1; ++t) {
    const int v = t * 128 + tid;
    int q, c;
    vec_qc<MT, (int)sizeof(S)>(v, q, c);
    const int col = tile * MT + c;
    const bool valid = col < a.ncols;
    uint32_t hi[16], lo[16];
#pragma unroll
    for (int p = 0; p < 16; ++p) {
      Cx<float> x = valid ? Conv<S, float>::ld(in + col + (8 * p + q) * ips) : mk<float>(0.f, 0.f);
      split2(x.x, x.y, hi[p], lo[p]);
    }
#pragma unroll
    for (int g = 0; g < 4; ++g) {  // K positions 8g .. 8g+7 = points p = 4g .. 4g+3
      const int off = tc::kmajor_off(v, 8 * g, 32);
      *reinterpret_cast<uint4*>(sA + off) = make_uint4(hi[4 * g], hi[4 * g + 1], hi[4 * g + 2], hi[4 * g + 3]);
      *reinterpret_cast<uint4*>(sA + Lay::A1 + off) =
          make_uint4(lo[4 * g], lo[4 * g + 1], lo[4 * g + 2], lo[4 * g + 3]);
    }
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *slot;
  const uint32_t sa = tc::smem_u32(sA), sb = tc::smem_u32(sB);
  if (tid == 0) {
    const uint32_t id1 = tc::idesc_bf16_f32(128, 32);
#pragma unroll
    for (int t = 0; t < Lay::T1; ++t) {
      const uint32_t ah = sa + t * 128 * 64, al = ah + Lay::A1;
      const uint32_t bh = sb, bl = sb + kB1;
      const uint32_t as[3] = {ah, al, ah}, bs[3] = {bh, bh, bl};
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
          tc::mma_bf16(taddr + 32 * t, tc::make_desc(as[j] + ks * 256, 128, 512),
                       tc::make_desc(bs[j] + ks * 256, 128, 512), id1, (j | ks) != 0);
    }
    tc::mma_commit(bar);
  }
  bool ok = tc::mbar_wait(bar, 0, kTcWait);
  int pending = ok ? -1 : 0;  // phase of an MMA batch whose completion wait gave up
  tc::fence_after_sync();

  // ---- stage-1 results -> twiddle W_128^{q k1} -> stage-2 operands
  const Cx<float>* tw128 = reinterpret_cast<const Cx<float>*>(a.tw);
  const uint32_t lane_base = taddr + ((uint32_t)(warp * 32) << 16);
  if (ok) {
#pragma unroll
    for (int t = 0; t < Lay::T1; ++t) {
      const int v = t * 128 + tid;
      int q, c;
      vec_qc<MT, (int)sizeof(S)>(v, q, c);
      float y[32];
      tc::tmem_ld16(lane_base + 32 * t, y);
      tc::tmem_ld16(lane_base + 32 * t + 16, y + 16);
#pragma unroll
      for (int k1 = 0; k1 < 16; ++k1) {
        Cx<float> val = mk<float>(y[2 * k1], y[2 * k1 + 1]);
        if (k1 > 0 && q > 0) {
          const Cx<float> w = ldg(tw128 + q * k1);
          val = INV ? cmulc(val, w) : cmul(val, w);
        }
        uint32_t h, l;
        split2(val.x, val.y, h, l);
        const int off = tc::kmajor_off(k1 * MT + c, 2 * q, 16);
        *reinterpret_cast<uint32_t*>(sA + off) = h;
        *reinterpret_cast<uint32_t*>(sA + Lay::A2 + off) = l;
      }
    }
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (tid == 0 && ok) {
    const uint32_t id2 = tc::idesc_bf16_f32(128, 16);
#pragma unroll
    for (int t = 0; t < Lay::T2; ++t) {
      const uint32_t ah = sa + t * 128 * 32, al = ah + Lay::A2;
      const uint32_t bh = sb + 2 * kB1, bl = bh + kB2;
      tc::mma_bf16(taddr + 16 * t, tc::make_desc(ah, 128, 256), tc::make_desc(bh, 128, 256), id2, 0);
      tc::mma_bf16(taddr + 16 * t, tc::make_desc(al, 128, 256), tc::make_desc(bh, 128, 256), id2, 1);
      tc::mma_bf16(taddr + 16 * t, tc::make_desc(ah, 128, 256), tc::make_desc(bl, 128, 256), id2, 1);
    }
    tc::mma_commit(bar);
  }
  if (ok) {
    ok = tc::mbar_wait(bar, 1, kTcWait);
    if (!ok) pending = 1;
  }
  tc::fence_after_sync();

  // ---- stage-2 results: vector u = (k1, column) holds X[k1 + 16 k2], k2 = 0..7
  S* out = reinterpret_cast<S*>(a.out) + bq * a.out_bs1 + br * a.out_bs2;
  const float s = a.scale;
  const Cx<float>* twl = reinterpret_cast<const Cx<float>*>(a.twl);
  if (ok) {
#pragma unroll
    for (int t = 0; t < Lay::T2; ++t) {
      const int u = t * 128 + tid;
      const int k1 = u / MT, c = u % MT;
      const int col = tile * MT + c;
      const bool valid = col < a.ncols;
      float x[16];
      tc::tmem_ld16(lane_base + 16 * t, x);
      // W_N^{b0 k}: b0 < N0 and k = pos < N1, so the exponent is below N
      const int b0 = a.tw_from_batch ? (int)br : (valid ? col : 0);  // no table index past N for absent columns
#pragma unroll
      for (int k2 = 0; k2 < 8; ++k2) {
        const int pos = k1 + 16 * k2;
        Cx<float> val = mk<float>(x[2 * k2], x[2 * k2 + 1]);
        if (MODE != 0) {
          const Cx<float> w = ldg(twl + b0 * pos);
          val = INV ? cmulc(val, w) : cmul(val, w);
        }
        val = scale(val, s);
        if (MODE == 2) {
          // the operand area is free: both MMA batches have completed
          reinterpret_cast<Cx<float>*>(sA)[c * 129 + pos] = val;
        } else if (valid) {
          Conv<S, float>::st(out + col + pos * a.out_ps, val);
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(status, 1);
  }
  if (MODE == 2) {
    __syncthreads();
    const long long ocs = a.out_cs;
    for (int idx = tid; idx < 128 * MT; idx += kTcThreads) {
      const int mm = idx >> 7, pos = idx & 127;
      const int c = tile * MT + mm;
      if (c < a.ncols && ok) Conv<S, float>::st(out + c * ocs + pos, reinterpret_cast<Cx<float>*>(sA)[mm * 129 + pos]);
    }
  }
  if (pending >= 0) tc::mbar_wait(bar, pending, kTcWait);  // let an overdue MMA finish before TMEM is released
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(taddr, Lay::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// host: DFT operand matrices, split into bf16 hi/lo from FP64
// ---------------------------------------------------------------------------
uint16_t bf16_bits(float f) {  // round to nearest even
  uint32_t u;
  std::memcpy(&u, &f, 4);
  const uint32_t r = 0x7FFFu + ((u >> 16) & 1u);
  return uint16_t((u + r) >> 16);
}
float bf16_value(uint16_t h) {
  const uint32_t u = uint32_t(h) << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
int kmajor_off_host(int row, int k, int K) {
  return (((row >> 3) * (K >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
}

// Bt[j][i] (N = 2P rows, K = 2P columns) of the P-point DFT, j = 2k + d and
// i = 2p + c interleaving (re, im): re-in/re-out Fr, re-in/im-out Fi,
// im-in/re-out -Fi, im-in/im-out Fr, with F = exp(-+2 pi i p k / P).
void dft_operands(int P, bool inv, unsigned char* hi, unsigned char* lo) {
  const int K = 2 * P;
  const double sgn = inv ? 1.0 : -1.0;
  for (int p = 0; p < P; ++p)
    for (int k = 0; k < P; ++k) {
      const long long e = (long long)p * k % P;
      const double fr = std::cos(2.0 * M_PI * double(e) / P), fi = sgn * std::sin(2.0 * M_PI * double(e) / P);
      const double vals[2][2] = {{fr, fi}, {-fi, fr}};  // [c][d]
      for (int c = 0; c < 2; ++c)
        for (int d = 0; d < 2; ++d) {
          const double x = vals[c][d];
          const uint16_t h = bf16_bits(float(x));
          const uint16_t l = bf16_bits(float(x - double(bf16_value(h))));
          const int off = kmajor_off_host(2 * k + d, 2 * p + c, K);
          std::memcpy(hi + off, &h, 2);
          std::memcpy(lo + off, &l, 2);
        }
    }
}

std::mutex g_bmu;
std::map<std::pair<int, bool>, void*> g_bmats;

template <int MT, class S>
cudaError_t launch_mt(const FsArgs& a, const Launch& l0, bool inv, int mode, const unsigned char* bm, int* status) {
  Launch l = l0;
  l.block = dim3(kTcThreads);
  l.smem = TcLayout<MT>::SMEM;
  switch (mode * 2 + (inv ? 1 : 0)) {
    case 0: return enqueue(k_fs_tc<false, S, 0, MT>, l, a, bm, status);
    case 1: return enqueue(k_fs_tc<true, S, 0, MT>, l, a, bm, status);
    case 2: return enqueue(k_fs_tc<false, S, 1, MT>, l, a, bm, status);
    case 3: return enqueue(k_fs_tc<true, S, 1, MT>, l, a, bm, status);
    case 4: return enqueue(k_fs_tc<false, S, 2, MT>, l, a, bm, status);
    default: return enqueue(k_fs_tc<true, S, 2, MT>, l, a, bm, status);
  }
}

}  // namespace

cudaError_t tc_dft_operands(int dev, bool inv, const void** out) {
  std::lock_guard<std::mutex> lock(g_bmu);
  auto key = std::make_pair(dev, inv);
  auto it = g_bmats.find(key);
  if (it != g_bmats.end()) {
    *out = it->second;
    return cudaSuccess;
  }
  unsigned char img[kBBytes];
  std::memset(img, 0, sizeof(img));
  dft_operands(16, inv, img, img + kB1);
  dft_operands(8, inv, img + 2 * kB1, img + 2 * kB1 + kB2);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, kBBytes);
  if (e != cudaSuccess) return e;
  e = cudaMemcpy(p, img, kBBytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p);
    return e;
  }
  g_bmats[key] = p;
  *out = p;
  return cudaSuccess;
}

size_t tc_pass_smem(int mt) { return mt == 16 ? TcLayout<16>::SMEM : TcLayout<32>::SMEM; }

cudaError_t launch_fourstep_pass_tc(const FsArgs& a, const Launch& l, int store, bool inv, int mode,
                                    const void* bmat, int* status) {
  const unsigned char* bm = static_cast<const unsigned char*>(bmat);
  const int mt = a.pp.M;
  if (a.pp.n != 128 || (mt != 16 && mt != 32)) return cudaErrorInvalidValue;
  switch (store) {
    case ST_C64: return mt == 16 ? launch_mt<16, Cx<float>>(a, l, inv, mode, bm, status)
                                 : launch_mt<32, Cx<float>>(a, l, inv, mode, bm, status);
    case ST_C32: return mt == 16 ? launch_mt<16, c32s>(a, l, inv, mode, bm, status)
                                 : launch_mt<32, c32s>(a, l, inv, mode, bm, status);
    case ST_BF16: return mt == 16 ? launch_mt<16, bf16c>(a, l, inv, mode, bm, status)
                                  : launch_mt<32, bf16c>(a, l, inv, mode, bm, status);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
