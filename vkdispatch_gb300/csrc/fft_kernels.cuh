// Batched 1-D FFT kernels along one axis of a C-order array, viewed as
// (outer, N, inner): contiguous axes (inner == 1) and strided axes
// (inner > 1, "columns").
//
// Algorithm: Stockham autosort with a runtime list of radix passes.  Pass p
// with radix R and Ns = product of the radices before it maps butterfly j to
//   inputs  j + r*(n/R)                     (r = 0..R-1)
//   twiddle W_{Ns*R}^{(j mod Ns) * r}
//   outputs (j - j mod Ns)*R + (j mod Ns) + r*Ns
// The inputs of the first pass and the outputs of the last pass both sit at
// j + r*(n/R), so the first pass loads straight from HBM into registers and
// the last pass stores straight to HBM, both coalesced across threads; only
// the exchanges between passes go through shared memory.  A fused
// convolution runs the inverse with the pass order reversed, so the spectrum
// never leaves registers between the forward and the inverse transform.
//
// The reference decomposes the same transforms into per-stage prime groups
// executed by generated code (vkdispatch/fft/context.py:152-179,
// vkdispatch/fft/stages.py:104-172); this file is an independent design.
#pragma once

#include "vdx_common.cuh"

namespace vdx {

constexpr int kMaxPasses = 12;

struct PassPlan {
  int n;      // complex points per transform
  int npass;  // number of radix passes
  int radix[kMaxPasses];
  int T;     // threads per transform
  int M;     // transforms (rows or columns) per CTA
  int npad;  // shared-memory slots per transform (contiguous layout)
  // per-pass index constants of the runtime passes in forward order, set by
  // set_pass_tables (0 = not set: the kernels derive them): the twiddle
  // stride n / (ns R) and inv_magic(ns), ns = product of the earlier radices
  int tws[kMaxPasses];
  unsigned nsm[kMaxPasses];
  unsigned tmag, mmag;  // inv_magic(T), inv_magic(M) where a kernel splits thread indices with them
};

// m = ceil(2^32 / d) for d >= 2 (0 for d < 2), the multiplier of mod_inv
__host__ __device__ __forceinline__ unsigned inv_magic(int d) { return d > 1 ? 0xFFFFFFFFu / unsigned(d) + 1u : 0u; }

// Fills the per-pass constants of a pass plan whose n and radix list are set.
inline void set_pass_tables(PassPlan& pp) {
  int ns = 1;
  for (int q = 0; q < pp.npass; ++q) {
    const int R = pp.radix[q];
    pp.tws[q] = pp.n / (ns * R);
    pp.nsm[q] = inv_magic(ns);
    ns *= R;
  }
  pp.tmag = inv_magic(pp.T);
  pp.mmag = inv_magic(pp.M);
}

struct FftArgs {
  PassPlan pp;
  const void* in;
  void* out;
  const void* ker;        // convolution: kernel spectrum
  const void* tw;         // W_n^k, k in [0, n), compute precision
  const void* tw2;        // real transforms: W_{2n}^k, k in [0, n]
  long long ntrans;       // contiguous: number of transforms
  long long inner;        // strided: number of columns (axis stride in elements)
  long long outer;        // strided: number of outer batches
  long long in_bs;        // elements between transforms (contiguous) / outer batches (strided)
  long long out_bs;
  long long ker_bs;       // kernel batch stride (0 = one spectrum broadcast to all batches)
  int col_tiles;          // strided: ceil(inner / M)
  int sig_lo, sig_hi;     // input positions outside [lo, hi) read as zero
  double scale;           // applied at the final store
  int nreal;              // real transforms: logical real length N
  // fused element-wise operations (complex64 kernels; see vdx_exec_ops)
  const float* in_weight;  // C2C: input point *= in_weight[element] * in_weight_scale on load
  const float* in_weight_scale_ptr;  // optional device scalar multiplied into in_weight_scale
  float in_weight_scale;
  float spec_scale;        // CONV: spec_out = spec_aux * conj(S) * spec_scale (mode 2)
  void* spec_out;          // CONV: receives the forward spectrum S (mode 1) or the product (mode 2)
  const void* spec_aux;
  const float* loss_weight;  // C2C: per-CTA partial of sum(loss_weight * |out|^2)
  float* loss_partials;
};

// ---------------------------------------------------------------------------
// thread placement
// ---------------------------------------------------------------------------
template <bool STRIDED>
struct Place {
  int t, m;
  bool valid;
  bool tile_full;  // every transform slot of this CTA exists (uniform per CTA)
  long long ps;    // point stride in elements
  const FftArgs& a;
  __device__ __forceinline__ Place(const FftArgs& args, int T) : a(args) {
    const int tid = threadIdx.x;
    if (STRIDED) {
      m = tid % a.pp.M;
      t = tid / a.pp.M;
      const long long c = col();
      valid = c < a.inner;
      tile_full = (long long)(blockIdx.x % a.col_tiles + 1) * a.pp.M <= a.inner;
      ps = a.inner;
    } else {
      t = tid % T;
      m = tid / T;
      valid = row() < a.ntrans;
      tile_full = (long long)(blockIdx.x + 1) * a.pp.M <= a.ntrans;
      ps = 1;
    }
  }
  // transform coordinates, recomputed where needed so that 64-bit offsets do
  // not stay live across the passes
  __device__ __forceinline__ long long col() const { return (long long)(blockIdx.x % a.col_tiles) * a.pp.M + m; }
  __device__ __forceinline__ long long row() const { return (long long)blockIdx.x * a.pp.M + m; }
  __device__ __forceinline__ long long off(long long bs) const {
    if (STRIDED) return (long long)(blockIdx.x / a.col_tiles) * bs + col();
    return row() * bs;
  }
  __device__ __forceinline__ long long in0() const { return off(a.in_bs); }
  __device__ __forceinline__ long long out0() const { return off(a.out_bs); }
  __device__ __forceinline__ long long ker0() const { return off(a.ker_bs); }
  // shared-memory slot of point i of this thread's transform; padded by one
  // slot every 16 so the stride-R scatters of the passes do not bank-conflict
  __device__ __forceinline__ int sidx(const PassPlan& pp, int i) const {
    if (STRIDED) return i * pp.M + m;
    return m * pp.npad + i + (i >> 4);
  }
  // unpadded slot, for exchanges whose accesses are unit-stride in either
  // direction (the mirrored k / n-k accesses of the real transforms)
  __device__ __forceinline__ int sidx_plain(const PassPlan& pp, int i) const {
    if (STRIDED) return i * pp.M + m;
    return m * pp.npad + i;
  }
};

// A placement whose transforms each occupy consecutive threads (t fastest)
// keeps every transform of T | 32 threads inside one warp, with shared-memory
// slots of its own: its exchanges between passes need only warp
// synchronisation.  Strided column tiles spread a transform over warps.
template <class PL>
struct WarpLocal : FalseT {};
template <>
struct WarpLocal<Place<false>> : TrueT {};

__host__ __device__ constexpr bool warp_sized(int T) { return T >= 1 && T <= 32 && 32 % T == 0; }

template <bool WARP>
__device__ __forceinline__ void xsync() {
  if constexpr (WARP) __syncwarp();
  else __syncthreads();
}
// runtime scope; `warp` must be the same for the whole CTA
__device__ __forceinline__ void xsync(bool warp) {
  if (warp) __syncwarp();
  else __syncthreads();
}

template <int V>
using IC = IntConst<int, V>;

// Runtime radix -> compile-time radix.
template <class F>
__device__ __forceinline__ void radix_dispatch(int R, F&& f) {
  switch (R) {
    case 1: f(IC<1>{}); break;
    case 2: f(IC<2>{}); break;
    case 3: f(IC<3>{}); break;
    case 4: f(IC<4>{}); break;
    case 5: f(IC<5>{}); break;
    case 7: f(IC<7>{}); break;
    case 8: f(IC<8>{}); break;
    case 9: f(IC<9>{}); break;
    case 11: f(IC<11>{}); break;
    case 13: f(IC<13>{}); break;
    case 16: f(IC<16>{}); break;
    default: break;
  }
}

// v[b*R + r] <- f(j + r*nb) for the thread's butterflies j = t + b*T < nb
template <int R, int MAXE, class Re, class F>
__device__ __forceinline__ void gather(Cx<Re>* v, int nb, int T, int t, F&& f) {
  constexpr int B = MAXE / R;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int j = t + b * T;
    if (j < nb) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[b * R + r] = f(j + r * nb);
    }
  }
}

// f(j + r*nb, v[b*R + r]) : natural-order positions (last pass outputs)
template <int R, int MAXE, class Re, class F>
__device__ __forceinline__ void each_natural(Cx<Re>* v, int nb, int T, int t, F&& f) {
  constexpr int B = MAXE / R;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int j = t + b * T;
    if (j < nb) {
#pragma unroll
      for (int r = 0; r < R; ++r) f(j + r * nb, v[b * R + r]);
    }
  }
}

// j mod d for d >= 2 and j * d < 2^32, given m = ceil(2^32 / d): one
// multiply-high and a multiply-subtract instead of an integer division by a
// runtime value (division by invariant integers, Granlund & Montgomery,
// PLDI 1994: with m = (2^32 + e) / d, 0 <= e < d, the floor of j m / 2^32 is
// floor(j / d) while j e < 2^32).  Transform indices stay below 2^15, so
// j * d < 2^30 for every pass of every supported length.
__device__ __forceinline__ int mod_inv(int j, int d, unsigned m) {
  return j - int(__umulhi(unsigned(j), m)) * d;
}

// RT: ns is a runtime value with nsm = inv_magic(ns) and tws = n / (ns R);
// otherwise ns is a compile-time constant and j % ns folds
template <int R, int MAXE, bool INV, class Re, bool RT = false>
__device__ __forceinline__ void butterflies(Cx<Re>* v, int nb, int T, int t, int ns, int n, const Cx<Re>* tw,
                                            unsigned nsm = 0, int tws = 0) {
  constexpr int B = MAXE / R;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int j = t + b * T;
    if (j < nb) {
      if (ns > 1) {
        const int k = RT ? mod_inv(j, ns, nsm) : j % ns;
        const int step = k * (RT ? tws : n / (ns * R));
#pragma unroll
        for (int r = 1; r < R; ++r) {
          const Cx<Re> w = ldg(&tw[r * step]);
          v[b * R + r] = INV ? cmulc(v[b * R + r], w) : cmul(v[b * R + r], w);
        }
      }
      Dft<R, INV, Re>::run(&v[b * R]);
    }
  }
}

template <int R, int MAXE, class Re, bool RT = false, class G>
__device__ __forceinline__ void scatter(const Cx<Re>* v, int nb, int T, int t, int ns, G&& g, unsigned nsm = 0) {
  constexpr int B = MAXE / R;
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int j = t + b * T;
    if (j < nb) {
      const int k = RT ? (ns > 1 ? mod_inv(j, ns, nsm) : 0) : j % ns;
      const int base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) g(base + r * ns, v[b * R + r]);
    }
  }
}

// Runs every pass on v, which must already hold the inputs of the first
// executed pass.  reversed = run radices last-to-first.  Returns with v
// holding natural-order outputs laid out for the last executed radix.
template <int MAXE, bool INV, class PL, class Re>
__device__ __forceinline__ void run_passes(Cx<Re>* v, const PassPlan& pp, bool reversed, const PL& pl,
                                           Cx<Re>* sm, const Cx<Re>* tw, bool warp = false) {
  const int n = pp.n, P = pp.npass, T = pp.T, t = pl.t;
  int ns = 1;
  for (int q = 0; q < P; ++q) {
    const int p = reversed ? P - 1 - q : q;
    const int R = pp.radix[p];
    const bool more = q + 1 < P;
    // per-pass constants: from the plan's tables when it has them (forward
    // order), else one division each per pass
    const bool tab = !reversed && pp.tws[p] > 0;
    const unsigned nsm = tab ? pp.nsm[p] : inv_magic(ns);
    const int tws = tab ? pp.tws[p] : n / (ns * R);
    // one radix dispatch per pass covers the butterflies and the scatter
    radix_dispatch(R, [&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      butterflies<RR, MAXE, INV, Re, true>(v, n / RR, T, t, ns, n, tw, nsm, tws);
      if (more) {
        xsync(warp);
        scatter<RR, MAXE, Re, true>(
            v, n / RR, T, t, ns, [&](int pos, Cx<Re> val) { sm[pl.sidx(pp, pos)] = val; }, nsm);
      }
    });
    if (more) {
      xsync(warp);
      const int R2 = pp.radix[reversed ? P - 2 - q : q + 1];
      radix_dispatch(R2, [&](auto rc) {
        constexpr int RR = decltype(rc)::value;
        gather<RR, MAXE, Re>(v, n / RR, T, t, [&](int pos) { return sm[pl.sidx(pp, pos)]; });
      });
    }
    ns *= R;
  }
}

// ---------------------------------------------------------------------------
// plan policies: how the kernels below learn n, T and the radix passes.
//   DynPlan   - runtime pass list (any 13-smooth length), radix by switch
//   FixPlan   - compile-time length, threads per transform and radix list;
//               every index, division and twiddle stride folds at compile time
// ---------------------------------------------------------------------------
template <int... Rs>
struct RList {};

template <class L>
struct RFirst;
template <int R0, int... Rs>
struct RFirst<RList<R0, Rs...>> {
  static constexpr int value = R0;
};
template <class L>
struct RLast;
template <int R0>
struct RLast<RList<R0>> {
  static constexpr int value = R0;
};
template <int R0, int R1, int... Rs>
struct RLast<RList<R0, R1, Rs...>> {
  static constexpr int value = RLast<RList<R1, Rs...>>::value;
};
template <class In, class Out = RList<>>
struct RRev;
template <int R0, int... Rs, int... Os>
struct RRev<RList<R0, Rs...>, RList<Os...>> : RRev<RList<Rs...>, RList<R0, Os...>> {};
template <int... Os>
struct RRev<RList<>, RList<Os...>> {
  using type = RList<Os...>;
};

template <int MAXE_>
struct DynPlan {
  static constexpr int MAXE = MAXE_;
  __device__ __forceinline__ void assume_t(int) const {}
  const PassPlan& pp;
  __device__ __forceinline__ explicit DynPlan(const PassPlan& p) : pp(p) {}
  __device__ __forceinline__ int n() const { return pp.n; }
  __device__ __forceinline__ int T() const { return pp.T; }
  // radix of the first executed pass (REV: passes run last-to-first)
  template <bool REV, class F>
  __device__ __forceinline__ void first(F&& f) const {
    radix_dispatch(pp.radix[REV ? pp.npass - 1 : 0], f);
  }
  template <bool REV, class F>
  __device__ __forceinline__ void last(F&& f) const {
    radix_dispatch(pp.radix[REV ? 0 : pp.npass - 1], f);
  }
  template <bool INV, bool REV, class PL, class Re>
  __device__ __forceinline__ void run(Cx<Re>* v, const PL& pl, Cx<Re>* sm, const Cx<Re>* tw) const {
    run_passes<MAXE, INV>(v, pp, REV, pl, sm, tw, WarpLocal<PL>::value && warp_sized(pp.T));
  }
};

template <int N, int T, int MAXE, bool INV, class Re, class PL, int NS, int R, int... Rest>
__device__ __forceinline__ void chain(Cx<Re>* v, const PassPlan& pp, const PL& pl, Cx<Re>* sm, const Cx<Re>* tw) {
  constexpr bool W = WarpLocal<PL>::value && warp_sized(T);
  butterflies<R, MAXE, INV, Re>(v, N / R, T, pl.t, NS, N, tw);
  if constexpr (sizeof...(Rest) > 0) {
    xsync<W>();
    scatter<R, MAXE, Re>(v, N / R, T, pl.t, NS, [&](int pos, Cx<Re> val) { sm[pl.sidx(pp, pos)] = val; });
    xsync<W>();
    constexpr int R2 = RFirst<RList<Rest...>>::value;
    gather<R2, MAXE, Re>(v, N / R2, T, pl.t, [&](int pos) { return sm[pl.sidx(pp, pos)]; });
    chain<N, T, MAXE, INV, Re, PL, NS * R, Rest...>(v, pp, pl, sm, tw);
  }
}

template <int N, int T, int MAXE, bool INV, class Re, class PL, int... Rs>
__device__ __forceinline__ void chain_list(RList<Rs...>, Cx<Re>* v, const PassPlan& pp, const PL& pl, Cx<Re>* sm,
                                           const Cx<Re>* tw) {
  chain<N, T, MAXE, INV, Re, PL, 1, Rs...>(v, pp, pl, sm, tw);
}

template <int N_, int T_, class L, int MAXE_ = 16>
struct FixPlan {
  static constexpr int MAXE = MAXE_;
  // the thread's index inside its transform is below T (lets the compiler
  // drop the j < n/R guards of exact plans)
  __device__ __forceinline__ void assume_t(int t) const { __builtin_assume(t >= 0 && t < T_); }
  const PassPlan& pp;
  __device__ __forceinline__ explicit FixPlan(const PassPlan& p) : pp(p) {}
  __device__ __forceinline__ static constexpr int n() { return N_; }
  __device__ __forceinline__ static constexpr int T() { return T_; }
  template <bool REV, class F>
  __device__ __forceinline__ void first(F&& f) const {
    f(IC<REV ? RLast<L>::value : RFirst<L>::value>{});
  }
  template <bool REV, class F>
  __device__ __forceinline__ void last(F&& f) const {
    f(IC<REV ? RFirst<L>::value : RLast<L>::value>{});
  }
  // PL: a thread placement (Place<STRIDED> or any type with t and sidx(pp, i))
  template <bool INV, bool REV, class PL, class Re>
  __device__ __forceinline__ void run(Cx<Re>* v, const PL& pl, Cx<Re>* sm, const Cx<Re>* tw) const {
    using Order = typename Cond<REV, typename RRev<L>::type, L>::type;
    chain_list<N_, T_, MAXE, INV, Re, PL>(Order{}, v, pp, pl, sm, tw);
  }
};

template <class P>
struct IsFixPlan : FalseT {};
template <int N_, int T_, class L, int MAXE_>
struct IsFixPlan<FixPlan<N_, T_, L, MAXE_>> : TrueT {};

// Programmatic dependent launch.  These kernels are launched with
// programmatic stream serialisation (enqueue_pdl): the next kernel of the
// stream may be scheduled while this one's last CTAs still run, and this one
// may have been scheduled before the previous kernel finished.  So every CTA
// first lets its successor launch, then waits until the previous kernel of
// the stream has completed and its writes are visible -- before any global
// memory access.  Launched without the attribute, both are no-ops.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <class Re>
__device__ __forceinline__ Cx<Re>* smem_base() {
  extern __shared__ __align__(16) unsigned char vdx_smem_raw[];
  return reinterpret_cast<Cx<Re>*>(vdx_smem_raw);
}

// First-pass gather of a complex input (signal-range masked).  CTAs whose
// slots all exist and whose range is the whole axis take the unpredicated
// path.
template <class Plan, class S, class Re, bool STRIDED>
__device__ __forceinline__ void gather_input(const Plan& P, const Place<STRIDED>& pl, const FftArgs& a, Cx<Re>* v,
                                             const S* in) {
  constexpr int MAXE = Plan::MAXE;
  const int n = P.n();
  const int lo = a.sig_lo, hi = a.sig_hi;
  if (pl.tile_full && lo <= 0 && hi >= n) {
    P.template first<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) { return Conv<S, Re>::ld(in + pos * pl.ps); });
    });
  } else {
    P.template first<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) {
        if (!pl.valid || pos < lo || pos >= hi) return mk<Re>(Re(0), Re(0));
        return Conv<S, Re>::ld(in + pos * pl.ps);
      });
    });
  }
}

// Natural-order store of the last executed pass, scaled, to `base` (a.out
// unless given) at the thread's transform offset.
template <class Plan, bool REV, class S, class Re, bool STRIDED>
__device__ __forceinline__ void store_output(const Plan& P, const Place<STRIDED>& pl, const FftArgs& a, Cx<Re>* v,
                                             S* base = nullptr) {
  constexpr int MAXE = Plan::MAXE;
  S* out = (base ? base : reinterpret_cast<S*>(a.out)) + pl.out0();
  const int n = P.n();
  const Re s = Re(a.scale);
  const bool all = pl.tile_full;
  P.template last<REV>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
      if (all || pl.valid) Conv<S, Re>::st(out + pos * pl.ps, scale(val, s));
    });
  });
}

// ---------------------------------------------------------------------------
// complex-to-complex
// ---------------------------------------------------------------------------
// IW: multiply each input point by in_weight[element] * in_weight_scale as it
// is loaded (the 2 w y of a weighted |y|^2 loss's gradient).
// LOSS: write one partial of sum(loss_weight[element] * |output|^2) per CTA.
// Plans of 32 points per thread run CTAs of at most 256 threads with up to
// 128 registers per thread.
template <class Plan, bool INV, bool STRIDED, class S, class Re, int IW = 0, int LOSS = 0>
__global__ void __launch_bounds__(Plan::MAXE >= 32 ? 256 : 1024, Plan::MAXE >= 32 ? 2 : 1) k_c2c(FftArgs a) {
  pdl_enter();
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<STRIDED> pl(a, P.T());
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  const S* in = reinterpret_cast<const S*>(a.in) + pl.in0();
  Cx<Re> v[MAXE];
  P.assume_t(pl.t);
  const int n = P.n();
  gather_input<Plan, S, Re>(P, pl, a, v, in);
  if constexpr (IW) {
    const float* w = a.in_weight + pl.in0();
    const Re f = Re(a.in_weight_scale) * (a.in_weight_scale_ptr ? Re(__ldg(a.in_weight_scale_ptr)) : Re(1));
    const bool ok = pl.tile_full || pl.valid;
    P.template first<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      constexpr int B = MAXE / RR;
      const int nb = n / RR;
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int j = pl.t + b * P.T();
        if (j < nb) {
#pragma unroll
          for (int r = 0; r < RR; ++r) {
            const Re wv = ok ? Re(__ldg(w + (j + r * nb) * pl.ps)) * f : Re(0);
            v[b * RR + r] = scale(v[b * RR + r], wv);
          }
        }
      }
    });
  }
  P.template run<INV, false>(v, pl, sm, tw);
  store_output<Plan, false, S, Re>(P, pl, a, v);
  if constexpr (LOSS) {
    const float* lw = a.loss_weight + pl.out0();
    const Re s = Re(a.scale);
    const bool ok = pl.tile_full || pl.valid;
    float acc = 0.f;
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
        if (ok) {
          const Cx<Re> y = scale(val, s);
          acc += __ldg(lw + pos * pl.ps) * float(y.x * y.x + y.y * y.y);
        }
      });
    });
    // block sum in a fixed order through shared memory (any CTA size; the
    // plan reserves blockDim floats of dynamic shared memory)
    float* red = reinterpret_cast<float*>(sm);
    const int nt = blockDim.x, tid = threadIdx.x;
    __syncthreads();
    red[tid] = acc;
    __syncthreads();
    int span = 1;
    while (span < nt) span <<= 1;
    for (int h = span >> 1; h > 0; h >>= 1) {
      if (tid < h && tid + h < nt) red[tid] += red[tid + h];
      __syncthreads();
    }
    if (tid == 0) a.loss_partials[blockIdx.x] = red[0];
  }
}

// ---------------------------------------------------------------------------
// fused convolution: forward FFT -> spectrum * op(kernel) -> inverse FFT
// kop: 0 = multiply by conj(kernel) (reference default,
// vkdispatch/fft/shader_factories.py:136-145), 1 = multiply by kernel.
// ---------------------------------------------------------------------------
// SPEC 1: also write the forward spectrum S to spec_out (kept for a backward
// pass).  SPEC 2: write spec_aux * conj(S) * spec_scale to spec_out instead
// (the kernel-spectrum gradient X conj(G) / N of an FFT convolution).
template <class Plan, bool STRIDED, class S, class K, class Re, int KOP, int SPEC = 0>
__global__ void __launch_bounds__(Plan::MAXE >= 32 ? 256 : 1024, Plan::MAXE >= 32 ? 2 : 1) k_conv(FftArgs a) {
  pdl_enter();
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<STRIDED> pl(a, P.T());
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  const S* in = reinterpret_cast<const S*>(a.in) + pl.in0();
  Cx<Re> v[MAXE];
  P.assume_t(pl.t);
  const int n = P.n();
  gather_input<Plan, S, Re>(P, pl, a, v, in);
  const bool kvalid = pl.tile_full || pl.valid;
  P.template run<false, false>(v, pl, sm, tw);
  if constexpr (SPEC != 0) {
    S* so = reinterpret_cast<S*>(a.spec_out) + pl.out0();
    const S* sa = reinterpret_cast<const S*>(a.spec_aux) + pl.out0();
    const Re ss = Re(a.spec_scale);
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
        if (!kvalid) return;
        if (SPEC == 1) {
          Conv<S, Re>::st(so + pos * pl.ps, val);
        } else {
          const Cx<Re> x = Conv<S, Re>::ld(sa + pos * pl.ps);
          Conv<S, Re>::st(so + pos * pl.ps, scale(cmulc(x, val), ss));
        }
      });
    });
  }
  const K* ker = reinterpret_cast<const K*>(a.ker) + pl.ker0();
  P.template last<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    constexpr int B = MAXE / RR;
    const int nb = n / RR;
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int j = pl.t + b * P.T();
      if (j < nb) {
#pragma unroll
        for (int r = 0; r < RR; ++r) {
          const int pos = j + r * nb;
          Cx<Re> kv = kvalid ? Conv<K, Re>::ld(ker + pos * pl.ps) : mk<Re>(Re(0), Re(0));
          v[b * RR + r] = KOP == 0 ? cmulc(v[b * RR + r], kv) : cmul(v[b * RR + r], kv);
        }
      }
    }
  });
  P.template run<true, true>(v, pl, sm, tw);
  store_output<Plan, true, S, Re>(P, pl, a, v);
}

// Strided fused convolution for CTAs of at most 256 threads, complex64.  The
// launch bound allows 128 registers per thread (80 for plans of 8 points
// per thread).  Plans of up to 16 points per thread load the kernel
// spectrum into registers right after issuing the signal loads, so its HBM
// latency overlaps the forward passes instead of following them; with 32
// points per thread the registers are full and it is loaded after the
// forward FFT.  The kernel spectrum is read once, with evict-first loads.
template <class Plan, class S, class Re, int KOP>
__global__ void __launch_bounds__(256, Plan::MAXE <= 8 ? 3 : 2) k_conv_pf(FftArgs a) {
  pdl_enter();
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<true> pl(a, P.T());
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  const S* in = reinterpret_cast<const S*>(a.in) + pl.in0();
  const S* ker = reinterpret_cast<const S*>(a.ker) + pl.ker0();
  P.assume_t(pl.t);
  const int n = P.n();
  const bool kvalid = pl.tile_full || pl.valid;
  constexpr bool PF = MAXE <= 16;
  Cx<Re> v[MAXE];
  gather_input<Plan, S, Re>(P, pl, a, v, in);
  Cx<Re> kr[PF ? MAXE : 1];
  if constexpr (PF) P.template last<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    constexpr int B = MAXE / RR;
    const int nb = n / RR;
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int j = pl.t + b * P.T();
#pragma unroll
      for (int r = 0; r < RR; ++r)
        kr[b * RR + r] = (j < nb && kvalid) ? ld_once<S, Re>(ker + (j + r * nb) * pl.ps) : mk<Re>(Re(0), Re(0));
    }
  });
  P.template run<false, false>(v, pl, sm, tw);
  P.template last<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    constexpr int B = MAXE / RR;
    const int nb = n / RR;
#pragma unroll
    for (int b = 0; b < B; ++b)
#pragma unroll
      for (int r = 0; r < RR; ++r) {
        Cx<Re> k;
        if constexpr (PF) {
          k = kr[b * RR + r];
        } else {
          const int j = pl.t + b * P.T();
          k = (j < nb && kvalid) ? ld_once<S, Re>(ker + (j + r * nb) * pl.ps) : mk<Re>(Re(0), Re(0));
        }
        v[b * RR + r] = KOP == 0 ? cmulc(v[b * RR + r], k) : cmul(v[b * RR + r], k);
      }
  });
  P.template run<true, true>(v, pl, sm, tw);
  store_output<Plan, true, S, Re>(P, pl, a, v);
}

// Fused multi-kernel convolution (the reference's kernel_num > 1 shader,
// vkdispatch/fft/shader_factories.py:166-193): the signal is read and
// transformed once, then for each kernel k: * K_k (conjugate or plain
// product) -> inverse FFT -> output slice k.  Kernel k is read at
// a.ker + k * kstride and output slice k written at a.out + k * ostride
// (elements).  The forward spectrum waits in a thread-private region at the
// end of the dynamic shared memory (slot i * blockDim.x + threadIdx.x, MAXE
// slots per thread), so only the exchange region is shared between threads.
template <class Plan, bool STRIDED, class S, class Re, int KOP>
__global__ void __launch_bounds__(Plan::MAXE >= 32 ? 256 : 1024, Plan::MAXE >= 32 ? 2 : 1)
    k_conv_multi(FftArgs a, int K, long long kstride, long long ostride) {
  pdl_enter();
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<STRIDED> pl(a, P.T());
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  unsigned dyn;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
  Cx<Re>* keep = sm + (dyn / sizeof(Cx<Re>) - unsigned(MAXE) * blockDim.x);
  const S* in = reinterpret_cast<const S*>(a.in) + pl.in0();
  Cx<Re> v[MAXE];
  P.assume_t(pl.t);
  const int n = P.n();
  gather_input<Plan, S, Re>(P, pl, a, v, in);
  const bool kvalid = pl.tile_full || pl.valid;
  P.template run<false, false>(v, pl, sm, tw);
#pragma unroll
  for (int i = 0; i < MAXE; ++i) keep[i * blockDim.x + threadIdx.x] = v[i];
  for (int k = 0; k < K; ++k) {
    if (k > 0) {
#pragma unroll
      for (int i = 0; i < MAXE; ++i) v[i] = keep[i * blockDim.x + threadIdx.x];
    }
    const S* ker = reinterpret_cast<const S*>(a.ker) + k * kstride + pl.ker0();
    P.template last<false>([&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      constexpr int B = MAXE / RR;
      const int nb = n / RR;
#pragma unroll
      for (int b = 0; b < B; ++b) {
        const int j = pl.t + b * P.T();
        if (j < nb) {
#pragma unroll
          for (int r = 0; r < RR; ++r) {
            const int pos = j + r * nb;
            const Cx<Re> kv = kvalid ? Conv<S, Re>::ld(ker + pos * pl.ps) : mk<Re>(Re(0), Re(0));
            v[b * RR + r] = KOP == 0 ? cmulc(v[b * RR + r], kv) : cmul(v[b * RR + r], kv);
          }
        }
      }
    });
    P.template run<true, true>(v, pl, sm, tw);
    store_output<Plan, true, S, Re>(P, pl, a, v, reinterpret_cast<S*>(a.out) + k * ostride);
  }
}

// ---------------------------------------------------------------------------
// real-to-complex, even N = 2n, rows of the packed RFFT layout: row pitch
// n+1 complex elements = 2n+2 reals (vkdispatch/base/buffer.py:377-448).
// z[m] = x[2m] + i x[2m+1] -> Z = FFT_n(z) ->
// X[k] = (Z[k] + conj Z[n-k])/2 - i W_2n^k (Z[k] - conj Z[n-k])/2, k = 0..n
// ---------------------------------------------------------------------------
template <class Plan, class S, class Re>
__global__ void __launch_bounds__(Plan::MAXE >= 32 ? 256 : 1024, Plan::MAXE >= 32 ? 2 : 1) k_r2c_even(FftArgs a) {
  pdl_enter();
  using SR = typename RealOf<S>::type;
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<false> pl(a, P.T());
  const PassPlan& pp = a.pp;
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  const Cx<Re>* tw2 = reinterpret_cast<const Cx<Re>*>(a.tw2);
  const S* in = reinterpret_cast<const S*>(a.in) + pl.in0();
  const SR* inr = reinterpret_cast<const SR*>(in);
  S* out = reinterpret_cast<S*>(a.out) + pl.out0();
  Cx<Re> v[MAXE];
  P.assume_t(pl.t);
  const int n = P.n();
  const int lo = a.sig_lo, hi = a.sig_hi;
  const bool full = lo <= 0 && hi >= 2 * n && pl.tile_full;
  P.template first<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    if (full) {
      gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) { return Conv<S, Re>::ld(in + pos); });
      return;
    }
    gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) {
      if (!pl.valid) return mk<Re>(Re(0), Re(0));
      const int e = 2 * pos, o = 2 * pos + 1;
      Re xr = (e >= lo && e < hi) ? ld_real<Re>(inr + e) : Re(0);
      Re xi = (o >= lo && o < hi) ? ld_real<Re>(inr + o) : Re(0);
      return mk<Re>(xr, xi);
    });
  });
  P.template run<false, false>(v, pl, sm, tw);
  const bool wsync = warp_sized(P.T());  // rows: the exchange below stays inside the row's warp
  xsync(wsync);
  P.template last<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t,
                               [&](int pos, Cx<Re> val) { sm[pl.sidx_plain(pp, pos)] = val; });
  });
  xsync(wsync);
  const Re half = Re(0.5);
  const bool wr = pl.tile_full || pl.valid;
  P.template last<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int k, Cx<Re> zk) {
      const int kc = k == 0 ? 0 : n - k;
      const Cx<Re> zc = conj(sm[pl.sidx_plain(pp, kc)]);
      const Cx<Re> e = scale(zk + zc, half);
      const Cx<Re> d = scale(zk - zc, half);
      const Cx<Re> o = mk<Re>(d.y, -d.x);  // d / i
      const Cx<Re> x = e + cmul(ldg(&tw2[k]), o);
      if (wr) Conv<S, Re>::st(out + k, x);
    });
  });
  if (pl.t == 0 && pl.valid) {
    const Cx<Re> z0 = sm[pl.sidx_plain(pp, 0)];
    Conv<S, Re>::st(out + n, mk<Re>(z0.x - z0.y, Re(0)));
  }
}

// ---------------------------------------------------------------------------
// complex-to-real, even N = 2n (Hermitian half X[0..n] -> N reals).
// Z[k] = (X[k] + conj X[n-k]) + i W_2n^{-k} (X[k] - conj X[n-k]), with the
// imaginary parts of X[0] and X[n] dropped (the real part of the full-length
// inverse does not depend on them) -> z = IFFT_n(Z) -> x[2m] + i x[2m+1] = z[m]
// ---------------------------------------------------------------------------
template <class Plan, class S, class Re>
__global__ void __launch_bounds__(Plan::MAXE >= 32 ? 256 : 1024, Plan::MAXE >= 32 ? 2 : 1) k_c2r_even(FftArgs a) {
  pdl_enter();
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<false> pl(a, P.T());
  const PassPlan& pp = a.pp;
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  const Cx<Re>* tw2 = reinterpret_cast<const Cx<Re>*>(a.tw2);
  const S* in = reinterpret_cast<const S*>(a.in) + pl.in0();
  Cx<Re> v[MAXE];
  P.assume_t(pl.t);
  const int n = P.n();
  // X[0..n-1] through registers with every load in flight before the first
  // shared-memory store (n <= T * MAXE for every plan); X[n] by thread 0
  const bool ld_ok = pl.tile_full || pl.valid;
#pragma unroll
  for (int u = 0; u < MAXE; ++u) {
    const int i = pl.t + u * P.T();
    if (i < n) v[u] = ld_ok ? Conv<S, Re>::ld(in + i) : mk<Re>(Re(0), Re(0));
  }
#pragma unroll
  for (int u = 0; u < MAXE; ++u) {
    const int i = pl.t + u * P.T();
    if (i < n) {
      Cx<Re> x = v[u];
      if (i == 0) x.y = Re(0);
      sm[pl.sidx_plain(pp, i)] = x;
    }
  }
  if (pl.t == 0) {
    Cx<Re> x = ld_ok ? Conv<S, Re>::ld(in + n) : mk<Re>(Re(0), Re(0));
    x.y = Re(0);
    sm[pl.sidx_plain(pp, n)] = x;
  }
  xsync(warp_sized(P.T()));  // rows: the exchange stays inside the row's warp
  P.template first<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int k) {
      const Cx<Re> xk = sm[pl.sidx_plain(pp, k)];
      const Cx<Re> xc = conj(sm[pl.sidx_plain(pp, n - k)]);
      const Cx<Re> s = xk + xc;
      const Cx<Re> d = xk - xc;
      const Cx<Re> wd = cmulc(d, ldg(&tw2[k]));  // d * W^{-k}
      return mk<Re>(s.x - wd.y, s.y + wd.x);     // s + i*wd
    });
  });
  P.template run<true, false>(v, pl, sm, tw);
  store_output<Plan, false, S, Re>(P, pl, a, v);
}

// ---------------------------------------------------------------------------
// real transforms of odd length N: full-length complex FFT of the real row
// (imaginary part zero), keeping bins 0..N/2 (forward), or of the
// Hermitian-extended half spectrum, keeping real parts (inverse) -- the
// reference's own R2C I/O rules (vkdispatch/fft/global_memory_iterators.py:
// 85-92, 214-226).  Row pitch N+1 reals = N/2+1 complex.
// ---------------------------------------------------------------------------
template <class Plan, bool INV, class S, class Re>
__global__ void __launch_bounds__(1024) k_real_odd(FftArgs a) {
  pdl_enter();
  using SR = typename RealOf<S>::type;
  const Plan P(a.pp);
  constexpr int MAXE = Plan::MAXE;
  const Place<false> pl(a, P.T());
  Cx<Re>* sm = smem_base<Re>();
  const Cx<Re>* tw = reinterpret_cast<const Cx<Re>*>(a.tw);
  const S* in = reinterpret_cast<const S*>(a.in) + pl.in0();
  S* out = reinterpret_cast<S*>(a.out) + pl.out0();
  Cx<Re> v[MAXE];
  const int n = P.n();
  const int h = n / 2;
  const int lo = a.sig_lo, hi = a.sig_hi;
  P.template first<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    gather<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos) {
      if (!pl.valid) return mk<Re>(Re(0), Re(0));
      if (!INV) {
        if (pos < lo || pos >= hi) return mk<Re>(Re(0), Re(0));
        return mk<Re>(ld_real<Re>(reinterpret_cast<const SR*>(in) + pos), Re(0));
      }
      if (pos <= h) return Conv<S, Re>::ld(in + pos);
      return conj(Conv<S, Re>::ld(in + (n - pos)));
    });
  });
  P.template run<INV, false>(v, pl, sm, tw);
  const Re s = Re(a.scale);
  P.template last<false>([&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    each_natural<RR, MAXE, Re>(v, n / RR, P.T(), pl.t, [&](int pos, Cx<Re> val) {
      if (!pl.valid) return;
      if (!INV) {
        if (pos <= h) Conv<S, Re>::st(out + pos, val);
      } else {
        st_real<Re>(reinterpret_cast<SR*>(out) + pos, val.x * s);
      }
    });
  });
}

// ---------------------------------------------------------------------------
// twiddle tables, built in FP64: tab[k] = exp(-2 pi i k / den), k < count
// ---------------------------------------------------------------------------
template <class Re>
__global__ void k_twiddle(Cx<Re>* tab, int count, int den) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  double s, c;
  // 2k/den carries one double rounding (relative 2^-53); no range reduction is
  // needed because k < den
  sincospi(2.0 * double(k) / double(den), &s, &c);
  tab[k] = mk<Re>(Re(c), Re(-s));
}

// ---------------------------------------------------------------------------
// compile-time plans for power-of-two lengths (radix 16 passes, then the
// leftover power of two); threads per transform = n / 16
// ---------------------------------------------------------------------------
template <int N>
struct Pow2;
template <> struct Pow2<16> { using L = RList<16>; static constexpr int T = 1; };
template <> struct Pow2<32> { using L = RList<16, 2>; static constexpr int T = 2; };
template <> struct Pow2<64> { using L = RList<16, 4>; static constexpr int T = 4; };
template <> struct Pow2<128> { using L = RList<16, 8>; static constexpr int T = 8; };
template <> struct Pow2<256> { using L = RList<16, 16>; static constexpr int T = 16; };
template <> struct Pow2<512> { using L = RList<16, 16, 2>; static constexpr int T = 32; };
template <> struct Pow2<1024> { using L = RList<16, 16, 4>; static constexpr int T = 64; };
template <> struct Pow2<2048> { using L = RList<16, 16, 8>; static constexpr int T = 128; };
template <> struct Pow2<4096> { using L = RList<16, 16, 16>; static constexpr int T = 256; };
template <> struct Pow2<8192> { using L = RList<16, 16, 16, 2>; static constexpr int T = 512; };
template <> struct Pow2<16384> { using L = RList<16, 16, 16, 4>; static constexpr int T = 1024; };

template <int N>
using Pow2Plan = FixPlan<N, Pow2<N>::T, typename Pow2<N>::L>;

// compile-time plans of radix-8 passes, 8 points per thread (n/8 threads per
// transform): half the registers of the radix-16 plans, for the strided
// fused convolution that also holds the kernel spectrum in registers
template <int N>
struct Pow2x8;
template <> struct Pow2x8<512> { using L = RList<8, 8, 8>; static constexpr int T = 64; };

template <int N>
using Pow2x8Plan = FixPlan<N, Pow2x8<N>::T, typename Pow2x8<N>::L, 8>;

// two-pass compile-time plans, 32 points per thread (n/32 threads per
// transform): one shared-memory exchange per FFT instead of two
template <int N>
struct Pow2x32;
template <> struct Pow2x32<512> { using L = RList<32, 16>; static constexpr int T = 16; };
template <> struct Pow2x32<1024> { using L = RList<32, 32>; static constexpr int T = 32; };

template <int N>
using Pow2x32Plan = FixPlan<N, Pow2x32<N>::T, typename Pow2x32<N>::L, 32>;


}  // namespace vdx
