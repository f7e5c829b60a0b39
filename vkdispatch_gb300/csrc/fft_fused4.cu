// Long axes as ONE persistent launch of both four-step passes, with the
// intermediate held in an L2-resident ring instead of a full-size workspace.
//
// The two-launch form (fft_large.cu) writes the whole intermediate to HBM in
// pass A and reads it back in pass B: each axis costs two read+write trips
// over the array.  Here the array is cut into groups whose passes depend on
// each other only inside the group:
//   strided axis (outer, N, inner): group = (outer batch, tile of M columns),
//     N0 pass-A units (one per b0) and N1 pass-B units (one per k1);
//   contiguous rows: group = one row, N0/M pass-A units and N1/M pass-B units.
// A work queue (atomic ticket) interleaves pass A of group s with pass B of
// group s - L, and the intermediate of group g lives in ring slot g mod R
// (R = L + 1 slots of one group each, a few MB), so it is written and read
// back while still in L2.  Per-slot counters order the units: a pass-B unit
// waits until every pass-A unit of its group is done, a pass-A unit until
// the group that last used its slot has been read.  Units are claimed in
// queue order by running CTAs and each waits only on units queued before
// it, so every wait ends; it is still bounded (a poll limit, then the plan's
// status word is set and the unit is skipped).  Ring reads bypass L1
// (ld.global.cg): the ring's lines are rewritten by other SMs.
//
// The reference has no multi-pass transform at all: its planner rejects
// axes above 16384 points (vkdispatch/fft/config.py:185-190).
#include <cuda_runtime.h>

#include <algorithm>

#include "fft_kernels.cuh"
#include "vdx_internal.h"

namespace vdx {

namespace {

constexpr long long kFusedWait = 1ll << 22;  // polls of ~100 ns before a dependency wait gives up

// loads of the ring (L2 only) and streaming (evict-first) accesses of the array
template <class S>
struct Raw;
template <>
struct Raw<Cx<float>> {
  static __device__ __forceinline__ Cx<float> ld_cg(const Cx<float>* p) {
    const float2 f = __ldcg(reinterpret_cast<const float2*>(p));
    return mk<float>(f.x, f.y);
  }
  static __device__ __forceinline__ Cx<float> ld_cs(const Cx<float>* p) {
    const float2 f = __ldcs(reinterpret_cast<const float2*>(p));
    return mk<float>(f.x, f.y);
  }
  static __device__ __forceinline__ void st_cs(Cx<float>* p, Cx<float> v) {
    __stcs(reinterpret_cast<float2*>(p), make_float2(v.x, v.y));
  }
};
template <class S>
struct Raw4 {  // 4-byte pair storage (bf16 or fp16 pairs), converted by Conv
  static __device__ __forceinline__ Cx<float> ld_cg(const S* p) {
    const unsigned u = __ldcg(reinterpret_cast<const unsigned*>(p));
    return Conv<S, float>::ld(reinterpret_cast<const S*>(&u));
  }
  static __device__ __forceinline__ Cx<float> ld_cs(const S* p) {
    const unsigned u = __ldcs(reinterpret_cast<const unsigned*>(p));
    return Conv<S, float>::ld(reinterpret_cast<const S*>(&u));
  }
  static __device__ __forceinline__ void st_cs(S* p, Cx<float> v) {
    S t;
    Conv<S, float>::st(&t, v);
    __stcs(reinterpret_cast<unsigned*>(p), *reinterpret_cast<const unsigned*>(&t));
  }
};
template <>
struct Raw<c32s> : Raw4<c32s> {};
template <>
struct Raw<bf16c> : Raw4<bf16c> {};

struct FusedArgs {
  PassPlan ppA, ppB;
  const void* in;
  void* out;
  void* ring;             // R slots of `slot` elements each
  const void* twA;        // W_N1^k
  const void* twB;        // W_N0^k
  const void* twl;        // W_N^k
  long long N, N0, N1, inner, outer;
  long long slot;         // elements per ring slot
  int M;                  // columns per tile (both passes)
  int col_tiles;          // strided: tiles per outer batch
  long long groups;       // G
  int nA, nB;             // units per group
  int L, R;               // queue lag (stages) and ring slots (R > L)
  long long nunits;
  float scale;            // pass B's output scale
  unsigned* ticket;
  int* doneA;             // per ring slot: pass-A units finished (monotone over the launch)
  int* doneB;
  int* status;
  long long wait_limit;
};

struct TilePlace {
  int t, m, M;
  __device__ __forceinline__ int sidx(const PassPlan&, int i) const { return i * M + m; }
};

// One tile: M columns x n points.  Point pos of column m is read at
// in[m + pos * ips] and written at out[m * ocs + pos * ops].
//   MODE 0: scale, store.
//   MODE 1: twiddle W_N^{b0 pos} (b0 fixed for the tile), store.
//   MODE 2: twiddle W_N^{(col0 + m) pos}, store transposed through shared
//           memory (ops == 1: each column's points land contiguously).
// IN_RING: the input side is the ring (read from L2) rather than the array.
template <class Plan, bool INV, class S, int MODE, bool IN_RING>
__device__ __forceinline__ void fused_tile(const Plan& P, const TilePlace& pl, const S* in, long long ips, S* out,
                                           long long ops, long long ocs, int ncols, const Cx<float>* tw,
                                           const Cx<float>* twl, int b0, int col0, float sc, Cx<float>* sm) {
  constexpr int MAXE = Plan::MAXE;
  const int n = P.n();
  const bool valid = pl.m < ncols;
  Cx<float> v[MAXE];
  P.template first<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    gather<RR, MAXE, float>(v, n / RR, P.T(), pl.t, [&](int pos) {
      if (!valid) return mk<float>(0.f, 0.f);
      const S* p = in + pl.m + pos * ips;
      return IN_RING ? Raw<S>::ld_cg(p) : Raw<S>::ld_cs(p);
    });
  });
  P.template run<INV, false>(v, pl, sm, tw);
  if constexpr (MODE == 0) {
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      each_natural<RR, MAXE, float>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<float> val) {
        if (valid) Raw<S>::st_cs(out + pl.m + pos * ops, scale(val, sc));
      });
    });
  } else if constexpr (MODE == 1) {
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      each_natural<RR, MAXE, float>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<float> val) {
        const Cx<float> w = ldg(twl + (long long)b0 * pos);
        if (valid) Conv<S, float>::st(out + pl.m + pos * ops, INV ? cmulc(val, w) : cmul(val, w));
      });
    });
  } else {
    const int ld = n + 1;
    __syncthreads();  // the passes' exchanges are finished with sm
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      each_natural<RR, MAXE, float>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<float> val) {
        // columns past ncols take exponent 0 (their products would index past the table)
        const Cx<float> w = ldg(twl + (valid ? (long long)(col0 + pl.m) * pos : 0ll));
        sm[pl.m * ld + pos] = INV ? cmulc(val, w) : cmul(val, w);
      });
    });
    __syncthreads();
    const int total = n * pl.M;
    for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
      const int mm = idx / n, pos = idx - mm * n;
      if (mm < ncols) Conv<S, float>::st(out + mm * ocs + pos, sm[mm * ld + pos]);
    }
  }
}

// queue position -> (pass A?, group, unit index inside the group's pass).
// Stages 0 .. L'-1 hold pass A of groups 0 .. L'-1; stage s in [L', G) holds
// pass A of group s then pass B of group s - L'; the last L' stages hold
// pass B only (L' = min(L, G)).
__device__ __forceinline__ void decode(const FusedArgs& f, long long u, bool& isA, long long& g, int& i) {
  const long long Lp = f.L < f.groups ? f.L : f.groups;
  const long long head = Lp * f.nA;
  if (u < head) {
    isA = true;
    g = u / f.nA;
    i = int(u - g * f.nA);
    return;
  }
  const long long v = u - head, per = f.nA + f.nB, mid = (f.groups - Lp) * per;
  if (v < mid) {
    const long long s = Lp + v / per;
    const int r = int(v % per);
    isA = r < f.nA;
    g = isA ? s : s - Lp;
    i = isA ? r : r - f.nA;
    return;
  }
  const long long w = v - mid;
  isA = false;
  g = (f.groups - Lp) + w / f.nB;
  i = int(w % f.nB);
}

__device__ __forceinline__ bool wait_at_least(const int* ctr, int target, long long limit) {
  long long polls = 0;
  while (*reinterpret_cast<const volatile int*>(ctr) < target) {
    if (++polls > limit) return false;
    __nanosleep(100);
  }
  return true;
}

// Both pass plans are the same compile-time plan (square splits).  The
// launch bound keeps 80 registers per thread (three 256-thread or six
// 128-thread CTAs per SM).
template <class Plan, bool INV, class S, bool STRIDED>
__global__ void __launch_bounds__(256, 3) k_fs_fused(FusedArgs f) {
  __shared__ long long s_unit;
  __shared__ int s_ok;
  Cx<float>* sm = smem_base<float>();
  const Plan PA(f.ppA);
  const Plan PB(f.ppB);
  TilePlace pl;
  pl.M = f.M;
  pl.m = threadIdx.x % f.M;
  pl.t = threadIdx.x / f.M;
  const S* in = reinterpret_cast<const S*>(f.in);
  S* out = reinterpret_cast<S*>(f.out);
  S* ring = reinterpret_cast<S*>(f.ring);
  const Cx<float>* twA = reinterpret_cast<const Cx<float>*>(f.twA);
  const Cx<float>* twB = reinterpret_cast<const Cx<float>*>(f.twB);
  const Cx<float>* twl = reinterpret_cast<const Cx<float>*>(f.twl);
  // a unit is claimed only when its CTA is ready to run it: a claimed unit
  // that waits behind another in the same CTA would stall the units that
  // depend on it
  for (;;) {
    if (threadIdx.x == 0) s_unit = (long long)atomicAdd(f.ticket, 1u);
    __syncthreads();
    const long long u = s_unit;
    if (u >= f.nunits) return;
    bool isA;
    long long g;
    int i;
    decode(f, u, isA, g, i);
    const int slot = int(g % f.R);
    const int epoch = int(g / f.R);
    if (threadIdx.x == 0) {
      bool ok = true;
      if (isA && g >= f.R) ok = wait_at_least(f.doneB + slot, f.nB * epoch, f.wait_limit);
      if (!isA) ok = wait_at_least(f.doneA + slot, f.nA * (epoch + 1), f.wait_limit);
      if (!ok) atomicExch(f.status, 1);
      __threadfence();
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) {
      S* rs = ring + (long long)slot * f.slot;
      if constexpr (STRIDED) {
        const long long o = g / f.col_tiles;
        const int tile = int(g - o * f.col_tiles);
        const int ncols = int(min((long long)f.M, f.inner - (long long)tile * f.M));
        const long long base = o * f.N * f.inner + (long long)tile * f.M;
        if (isA) {  // b0 = i: points b1 * N0 + b0 -> ring rows (k1, b0)
          fused_tile<Plan, INV, S, 1, false>(PA, pl, in + base + (long long)i * f.inner, f.N0 * f.inner,
                                             rs + (long long)i * f.M, f.N0 * f.M, 1, ncols, twA, twl, i, 0, 1.f, sm);
        } else {  // k1 = i: ring rows (k1, b0 = 0 .. N0 - 1) -> X[k1 + N1 k2]
          fused_tile<Plan, INV, S, 0, true>(PB, pl, rs + (long long)i * f.N0 * f.M, f.M,
                                            out + base + (long long)i * f.inner, f.N1 * f.inner, 1, ncols, twB, twl,
                                            0, 0, f.scale, sm);
        }
      } else {
        const long long base = g * f.N;
        const int c0 = i * f.M;
        if (isA) {  // columns b0 = c0 .. c0 + M - 1 of the row -> ring[b0 * N1 + k1]
          const int ncols = int(min((long long)f.M, f.N0 - c0));
          fused_tile<Plan, INV, S, 2, false>(PA, pl, in + base + c0, f.N0, rs + (long long)c0 * f.N1, 1, f.N1,
                                             ncols, twA, twl, 0, c0, 1.f, sm);
        } else {  // k1 = c0 .. c0 + M - 1: ring[b0 * N1 + k1] -> X[k1 + N1 k2]
          const int ncols = int(min((long long)f.M, f.N1 - c0));
          fused_tile<Plan, INV, S, 0, true>(PB, pl, rs + c0, f.N1, out + base + c0, f.N1, 1, ncols, twB, twl, 0,
                                            0, f.scale, sm);
        }
      }
    }
    // every thread's stores of the unit precede the barrier; thread 0's
    // fence then releases them at device scope before the count moves (the
    // barrier also keeps the next unit's exchanges clear of this unit's
    // shared-memory reads)
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(isA ? f.doneA + slot : f.doneB + slot, 1);
    }
  }
}

template <class Plan, class S>
cudaError_t launch_plan(const FusedArgs& f, const Launch& l, bool inv, bool strided, int* max_ctas) {
  if (max_ctas) {  // occupancy query: opt every instantiation into the shared memory first
    cudaError_t e = prepare_smem(k_fs_fused<Plan, false, S, true>, l.smem);
    if (e == cudaSuccess) e = prepare_smem(k_fs_fused<Plan, true, S, true>, l.smem);
    if (e == cudaSuccess) e = prepare_smem(k_fs_fused<Plan, false, S, false>, l.smem);
    if (e == cudaSuccess) e = prepare_smem(k_fs_fused<Plan, true, S, false>, l.smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(max_ctas, k_fs_fused<Plan, false, S, true>, (int)l.block.x,
                                                        l.smem);
    return e;
  }
  if (strided) return inv ? enqueue(k_fs_fused<Plan, true, S, true>, l, f) : enqueue(k_fs_fused<Plan, false, S, true>, l, f);
  return inv ? enqueue(k_fs_fused<Plan, true, S, false>, l, f) : enqueue(k_fs_fused<Plan, false, S, false>, l, f);
}

// both passes on the same compile-time plan (square splits N = n * n)
template <class S>
cudaError_t launch_store(const FusedArgs& f, const Launch& l, bool inv, bool strided, int* max_ctas) {
  const int n = f.ppA.n, T = f.ppA.T;
  if (n != f.ppB.n || T != f.ppB.T) return cudaErrorInvalidValue;
  if (n == 128 && T == 8) return launch_plan<FixPlan<128, 8, RList<16, 8>>, S>(f, l, inv, strided, max_ctas);
  if (n == 256 && T == 16) return launch_plan<FixPlan<256, 16, RList<16, 16>>, S>(f, l, inv, strided, max_ctas);
  if (n == 64 && T == 4) return launch_plan<FixPlan<64, 4, RList<16, 4>>, S>(f, l, inv, strided, max_ctas);
  return cudaErrorInvalidValue;
}

}  // namespace

// Occupancy (CTAs per SM) of the fused kernel for a pass geometry; fails for
// geometries without a fused instantiation.
cudaError_t fused_fourstep_ctas_per_sm(int store, const PassPlan& pp, size_t smem, int* per_sm) {
  FusedArgs f{};
  f.ppA = f.ppB = pp;
  Launch l{dim3(1), dim3(pp.T * pp.M), smem, nullptr};
  switch (store) {
    case ST_C64: return launch_store<Cx<float>>(f, l, false, true, per_sm);
    case ST_C32: return launch_store<c32s>(f, l, false, true, per_sm);
    case ST_BF16: return launch_store<bf16c>(f, l, false, true, per_sm);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_fused_fourstep(const FusedLaunch& fl, cudaStream_t s) {
  FusedArgs f{};
  f.ppA = fl.ppA;
  f.ppB = fl.ppB;
  f.in = fl.in;
  f.out = fl.out;
  f.ring = fl.ring;
  f.twA = fl.twA;
  f.twB = fl.twB;
  f.twl = fl.twl;
  f.N = fl.N;
  f.N0 = fl.N0;
  f.N1 = fl.N1;
  f.inner = fl.inner;
  f.outer = fl.outer;
  f.M = fl.M;
  f.scale = fl.scale;
  f.L = fl.L;
  f.R = fl.R;
  f.ticket = fl.ticket;
  f.doneA = fl.doneA;
  f.doneB = fl.doneB;
  f.status = fl.status;
  f.wait_limit = fl.wait_limit > 0 ? fl.wait_limit : kFusedWait;
  if (fl.strided) {
    f.col_tiles = int((fl.inner + fl.M - 1) / fl.M);
    f.groups = fl.outer * f.col_tiles;
    f.nA = int(fl.N0);
    f.nB = int(fl.N1);
    f.slot = fl.N * fl.M;
  } else {
    f.col_tiles = 1;
    f.groups = fl.outer;
    f.nA = int((fl.N0 + fl.M - 1) / fl.M);
    f.nB = int((fl.N1 + fl.M - 1) / fl.M);
    f.slot = fl.N;
  }
  f.nunits = f.groups * (f.nA + f.nB);
  cudaError_t e = cudaMemsetAsync(fl.ticket, 0, sizeof(unsigned), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(fl.doneA, 0, sizeof(int) * size_t(fl.R), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(fl.doneB, 0, sizeof(int) * size_t(fl.R), s);
  if (e != cudaSuccess) return e;
  Launch l{dim3(fl.grid), dim3(fl.ppA.T * fl.M), fl.smem, s};
  switch (fl.store) {
    case ST_C64: return launch_store<Cx<float>>(f, l, fl.inverse, fl.strided, nullptr);
    case ST_C32: return launch_store<c32s>(f, l, fl.inverse, fl.strided, nullptr);
    case ST_BF16: return launch_store<bf16c>(f, l, fl.inverse, fl.strided, nullptr);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
