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
#include <cuda_runtime.h>

#include "fft_kernels.cuh"
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
template <class Plan, bool INV, class S, int MODE>
__global__ void __launch_bounds__(512) k_fs(FsArgs a) {
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
  const S* in = reinterpret_cast<const S*>(a.in) + bq * a.in_bs1 + br * a.in_bs2 + col;
  const long long ips = a.in_ps;
  Cx<Re> v[MAXE];
  P.template first<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) {
      return valid ? Conv<S, Re>::ld(in + pos * ips) : mk<Re>(0.f, 0.f);
    });
  });
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
    // W_N^{b0 k1}: b0 < N0 and k1 = pos < N1, so the exponent is below N
    const Cx<Re>* twl = reinterpret_cast<const Cx<Re>*>(a.twl);
    const int b0 = a.tw_from_batch ? (int)br : col;
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

template <class Plan, class S>
cudaError_t launch_mode(const FsArgs& a, const Launch& l, bool inv, int mode) {
  switch (mode * 2 + (inv ? 1 : 0)) {
    case 0: return enqueue(k_fs<Plan, false, S, 0>, l, a);
    case 1: return enqueue(k_fs<Plan, true, S, 0>, l, a);
    case 2: return enqueue(k_fs<Plan, false, S, 1>, l, a);
    case 3: return enqueue(k_fs<Plan, true, S, 1>, l, a);
    case 4: return enqueue(k_fs<Plan, false, S, 2>, l, a);
    default: return enqueue(k_fs<Plan, true, S, 2>, l, a);
  }
}

template <class S>
cudaError_t launch_store(const FsArgs& a, const Launch& l, bool inv, int mode) {
  const int n = a.pp.n, T = a.pp.T;
  if (n == 128 && T == 8) return launch_mode<FixPlan<128, 8, RList<16, 8>>, S>(a, l, inv, mode);
  if (n == 256 && T == 16) return launch_mode<FixPlan<256, 16, RList<16, 16>>, S>(a, l, inv, mode);
  if (n == 64 && T == 4) return launch_mode<FixPlan<64, 4, RList<16, 4>>, S>(a, l, inv, mode);
  return launch_mode<DynPlan<16>, S>(a, l, inv, mode);
}

}  // namespace

cudaError_t launch_fourstep_pass(const FsArgs& a, const Launch& l, int store, bool inv, int mode) {
  switch (store) {
    case ST_C64: return launch_store<Cx<float>>(a, l, inv, mode);
    case ST_C32: return launch_store<c32s>(a, l, inv, mode);
    case ST_BF16: return launch_store<bf16c>(a, l, inv, mode);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
