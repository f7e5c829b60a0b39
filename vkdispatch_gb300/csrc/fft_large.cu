// Long axes as a four-step pair of launches (complex-to-complex, fp32 compute).
//
// An axis of length N = N1 * N0 is indexed n = b1 * N0 + b0 and k = k1 + N1 * k2.
//   pass A: for every b0, the N1-point transform over b1, times W_N^{b0 k1},
//           into a workspace;
//   pass B: for every k1, the N0-point transform over b0, written to
//           X[k1 + N1 k2].
// Both passes are tiles of M adjacent columns and one short transform per
// column (n = N1 or N0, a few hundred points at most), so each CTA is small,
// several run on an SM at once and their loads overlap the other CTAs'
// butterflies -- which a single CTA holding a whole 16384-point transform
// (one per SM, all 64K registers) cannot do.  The price is a second trip
// through HBM for the intermediate; the host can walk the array in chunks
// whose workspace fits in L2 instead (VDX_FOURSTEP_WS_MB).
//
// The reference has no multi-kernel transform: its planner rejects axes
// above 16384 points (vkdispatch/fft/config.py:185-190) and runs every axis
// inside one workgroup (vkdispatch/fft/shader_factories.py:11-60).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "fft_kernels.cuh"
#include "tc_ptx.cuh"
#include "vdx_internal.h"

namespace vdx {

namespace {

// thread placement inside a column tile: m = column, t = thread of the column
// (the interface run_passes / FixPlan::run use)
struct FsPlace {
  int t, m, M;
  __device__ __forceinline__ int sidx(const PassPlan&, int i) const { return i * M + m; }
};

// MODE 0: plain store (pass B).  MODE 1: four-step twiddle, then a store
// whose columns are unit-stride (strided axes).  MODE 2: four-step twiddle,
// then a transposed store through shared memory so that each column's points
// land contiguously (out_ps == 1; contiguous axes).
// TMA tile copies: dims (columns, then the other axes by increasing stride),
// coordinates in that order; the box is M columns x n rows.
struct TmaTile {
  int rank;
  int row_dim, br_dim, bq_dim;  // position of each in the map (-1: not a dimension)
};
constexpr long long kTmaWait = 1ll << 24;  // polls before a tile-load wait gives up

template <int RANK>
__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap* map, const int* c, uint64_t* bar) {
  const uint64_t m = reinterpret_cast<uint64_t>(map);
  const uint32_t b = tc::smem_u32(bar);
  if constexpr (RANK == 2) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(m), "r"(c[0]), "r"(c[1]), "r"(b)
        : "memory");
  } else if constexpr (RANK == 3) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            dst),
        "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(b)
        : "memory");
  } else {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(b)
        : "memory");
  }
}

// TMA > 0: the input tile arrives by one bulk-tensor copy of rank TMA into
// shared memory behind the exchange area, and the first pass gathers from it.
template <class Plan, bool INV, class S, int MODE, int TMA>
__global__ void __launch_bounds__(512) k_fs(const __grid_constant__ CUtensorMap tmap, FsArgs a, TmaTile tt) {
  using Re = float;
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const int M = a.pp.M;
  FsPlace pl;
  pl.M = M;
  pl.m = threadIdx.x % M;
  pl.t = threadIdx.x / M;
  P.assume_t(pl.t);
  const int n = P.n();
  const int tile = blockIdx.x % a.col_tiles;
  const long long b = blockIdx.x / a.col_tiles;
  const long long bq = b / a.split, br = b - bq * a.split;
  const int col = tile * M + pl.m;
  const bool valid = col < a.ncols;
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  Cx<Re> v[MAXE];
  if constexpr (TMA > 0) {
    // staging after the exchange area ((n + 1) * M complex slots), on the
    // 128-byte boundary a tensor copy's destination needs
    const uint32_t stg_addr = (tc::smem_u32(sm + (n + 1) * M) + 127u) & ~127u;
    const S* stg = reinterpret_cast<const S*>(reinterpret_cast<const unsigned char*>(sm) +
                                              (stg_addr - tc::smem_u32(sm)));
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
      tc::mbar_init(&bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t bytes = uint32_t(n) * uint32_t(M) * uint32_t(sizeof(S));
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(&bar)), "r"(bytes)
                   : "memory");
      int c[4] = {0, 0, 0, 0};
      c[0] = tile * M;
      if (tt.br_dim >= 0) c[tt.br_dim] = (int)br;
      if (tt.bq_dim >= 0) c[tt.bq_dim] = (int)bq;
      tma_load<TMA>(stg_addr, &tmap, c, &bar);
    }
    if (!__syncthreads_and(tc::mbar_wait(&bar, 0, kTmaWait))) {
      if (threadIdx.x == 0 && a.status) atomicExch(a.status, 1);
      tc::mbar_wait(&bar, 0, kTmaWait);  // the copy is still in flight: let it land before leaving
      return;
    }
    P.template first<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) { return Conv<S, Re>::ld(stg + pos * M + pl.m); });
    });
  } else {
    const S* in = reinterpret_cast<const S*>(a.in) + bq * a.in_bs1 + br * a.in_bs2 + col;
    const long long ips = a.in_ps;
    P.template first<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) {
        return valid ? Conv<S, Re>::ld(in + pos * ips) : mk<Re>(0.f, 0.f);
      });
    });
  }
  P.template run<INV, false>(v, pl, sm, tw);
  S* out = reinterpret_cast<S*>(a.out) + bq * a.out_bs1 + br * a.out_bs2;
  const Re s = a.scale;
  if constexpr (MODE == 0) {
    const long long ops = a.out_ps;
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
        if (valid) Conv<S, Re>::st(out + col + pos * ops, scale(val, s));
      });
    });
  } else {
    // W_N^{b0 k1}: b0 < N0 and k1 = pos < N1, so the exponent is below N.
    // Columns past the last one of a partial tile (col >= ncols) take b0 = 0:
    // their products would index past the table's N entries
    const Cx<Re>* twl = reinterpret_cast<const Cx<Re>*>(a.twl);
    const int b0 = a.tw_from_batch ? (int)br : (valid ? col : 0);
    if constexpr (MODE == 1) {
      const long long ops = a.out_ps;
      P.template last<false>([&](auto rc) {
        constexpr int RR = decltype(rc)::value;
        each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
          const Cx<Re> w = ldg(twl + b0 * pos);
          if (valid) Conv<S, Re>::st(out + col + pos * ops, scale(INV ? cmulc(val, w) : cmul(val, w), s));
        });
      });
    } else {
      const int ld = n + 1;  // odd row pitch: the column-major writes below spread over the banks
      __syncthreads();       // every exchange of the passes is finished with sm
      P.template last<false>([&](auto rc) {
        constexpr int RR = decltype(rc)::value;
        each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
          const Cx<Re> w = ldg(twl + b0 * pos);
          sm[pl.m * ld + pos] = scale(INV ? cmulc(val, w) : cmul(val, w), s);
        });
      });
      __syncthreads();
      const long long ocs = a.out_cs;
      const int total = n * M;
      for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int mm = idx / n, pos = idx - mm * n;
        const int c = tile * M + mm;
        if (c < a.ncols) Conv<S, Re>::st(out + c * ocs + pos, sm[mm * ld + pos]);
      }
    }
  }
}

template <class Plan, class S, int TMA>
cudaError_t launch_mode(const CUtensorMap& m, const FsArgs& a, const TmaTile& tt, const Launch& l, bool inv,
                        int mode) {
  switch (mode * 2 + (inv ? 1 : 0)) {
    case 0: return enqueue(k_fs<Plan, false, S, 0, TMA>, l, m, a, tt);
    case 1: return enqueue(k_fs<Plan, true, S, 0, TMA>, l, m, a, tt);
    case 2: return enqueue(k_fs<Plan, false, S, 1, TMA>, l, m, a, tt);
    case 3: return enqueue(k_fs<Plan, true, S, 1, TMA>, l, m, a, tt);
    case 4: return enqueue(k_fs<Plan, false, S, 2, TMA>, l, m, a, tt);
    default: return enqueue(k_fs<Plan, true, S, 2, TMA>, l, m, a, tt);
  }
}

template <class S, int TMA>
cudaError_t launch_store(const CUtensorMap& m, const FsArgs& a, const TmaTile& tt, const Launch& l, bool inv,
                         int mode) {
  const int n = a.pp.n, T = a.pp.T;
  if constexpr (TMA > 0) {  // staged passes exist for the 128-point short transforms only
    if (n == 128 && T == 8) return launch_mode<FixPlan<128, 8, RList<16, 8>>, S, TMA>(m, a, tt, l, inv, mode);
    return cudaErrorInvalidValue;
  } else {
    if (n == 128 && T == 8) return launch_mode<FixPlan<128, 8, RList<16, 8>>, S, 0>(m, a, tt, l, inv, mode);
    if (n == 256 && T == 16) return launch_mode<FixPlan<256, 16, RList<16, 16>>, S, 0>(m, a, tt, l, inv, mode);
    if (n == 64 && T == 4) return launch_mode<FixPlan<64, 4, RList<16, 4>>, S, 0>(m, a, tt, l, inv, mode);
    return launch_mode<DynPlan<16>, S, 0>(m, a, tt, l, inv, mode);
  }
}

template <class S>
cudaError_t launch_any(const CUtensorMap& m, const FsArgs& a, const TmaTile& tt, const Launch& l, bool inv,
                       int mode) {
  if constexpr (sizeof(S) == 4) {
    switch (tt.rank) {
      case 2: return launch_store<S, 2>(m, a, tt, l, inv, mode);
      case 3: return launch_store<S, 3>(m, a, tt, l, inv, mode);
      case 4: return launch_store<S, 4>(m, a, tt, l, inv, mode);
      default: break;
    }
  }
  return launch_store<S, 0>(m, a, tt, l, inv, mode);
}

// cuTensorMapEncodeTiled, fetched once from the driver without linking libcuda
PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  });
  return fn;
}

size_t store_size(int store) { return store == ST_C64 ? 8 : 4; }

// The pass input as a tensor: element (c, pos, br, bq) at
// base + bq * in_bs1 + br * in_bs2 + pos * in_ps + c; dimensions of extent 1
// are dropped and the rest ordered by stride.
bool encode_tile_map(const FsArgs& a, int store, CUtensorMap* map, TmaTile* tt) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc) return false;
  const long long es = (long long)store_size(store);
  const int M = a.pp.M, n = a.pp.n;
  struct D {
    long long extent, stride;
    int which;  // 0 = pos, 1 = br, 2 = bq
  };
  D d[3];
  int k = 0;
  d[k++] = D{n, a.in_ps, 0};
  if (a.split > 1) d[k++] = D{a.split, a.in_bs2, 1};
  const long long bq_count = (a.nbatch + a.split - 1) / a.split;
  if (bq_count > 1) d[k++] = D{bq_count, a.in_bs1, 2};
  std::sort(d, d + k, [](const D& x, const D& y) { return x.stride < y.stride; });
  cuuint64_t dims[5], strides[4];
  cuuint32_t box[5], estr[5];
  dims[0] = (cuuint64_t)a.ncols;
  box[0] = (cuuint32_t)M;
  estr[0] = 1;
  tt->rank = 1 + k;
  tt->row_dim = tt->br_dim = tt->bq_dim = -1;
  for (int i = 0; i < k; ++i) {
    dims[i + 1] = (cuuint64_t)d[i].extent;
    strides[i] = (cuuint64_t)(d[i].stride * es);
    box[i + 1] = d[i].which == 0 ? (cuuint32_t)n : 1;
    estr[i + 1] = 1;
    if (d[i].which == 0) tt->row_dim = i + 1;
    if (d[i].which == 1) tt->br_dim = i + 1;
    if (d[i].which == 2) tt->bq_dim = i + 1;
    if (strides[i] % 16 != 0 || strides[i] >= (1ull << 40)) return false;
  }
  // box extents of 1 add no stride, so the staged tile is [row][column] wherever the rows sit
  if (tt->rank < 2 || tt->rank > 4 || tt->row_dim < 1) return false;
  const CUtensorMapDataType ty = store == ST_C64 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT32;
  const CUresult r = enc(map, ty, (cuuint32_t)tt->rank, const_cast<void*>(a.in), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace

// Staged passes are used where they measured faster: 4-byte storage (bf16 or
// fp16 pairs) on strided axes, whose rows are 128-byte segments far apart
// (16384^2 bf16 strided axis: 1.295 -> 1.131 ms).  For complex64 and for the
// contiguous-axis passes the staging tile's shared memory costs more
// occupancy than the bulk copy saves (1.40 -> 1.53 ms, 1.56 -> 2.04 ms).
bool fourstep_tma_ok(const FsArgs& a, int store) {
  const long long es = (long long)store_size(store);
  const int n = a.pp.n, M = a.pp.M;
  if (store != ST_C32 && store != ST_BF16) return false;
  if (n != 128) return false;  // one box of 128 rows, the compile-time 128-point plan
  if ((M * es) % 16 != 0) return false;
  if (reinterpret_cast<uintptr_t>(a.in) % 16 != 0) return false;
  return encoder() != nullptr;
}

cudaError_t launch_fourstep_pass(const FsArgs& a, const Launch& l, int store, bool inv, int mode, bool tma) {
  CUtensorMap map;
  std::memset(&map, 0, sizeof(map));
  TmaTile tt{0, -1, -1, -1};
  Launch lt = l;
  if (tma && fourstep_tma_ok(a, store) && encode_tile_map(a, store, &map, &tt)) {
    lt.smem = std::max(l.smem, size_t(a.pp.n + 1) * a.pp.M * 8) + size_t(a.pp.n) * a.pp.M * store_size(store) + 128;
  } else {
    tt.rank = 0;
  }
  switch (store) {
    case ST_C64: return launch_any<Cx<float>>(map, a, tt, lt, inv, mode);
    case ST_C32: return launch_any<c32s>(map, a, tt, lt, inv, mode);
    case ST_BF16: return launch_any<bf16c>(map, a, tt, lt, inv, mode);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
