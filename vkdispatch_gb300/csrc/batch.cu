// Batched FFTs of uneven lengths in one persistent launch.
//
// The host turns a list of items (offset, length, count) into a table of
// work units; one CTA per SM claims units with an atomic ticket and runs the
// runtime-plan Stockham passes on each.  Lengths up to 16384 (with at most
// 1024 threads per transform) are tiles of whole transforms (UK_ROWS).
// Longer lengths L = L1 * L2 run as a four-step pair: UK_COLS units transform
// the L1-point columns (stride L2) and multiply by W_L^{n2 k1} into a
// workspace, then UK_ROWS2 units transform the L2-point rows and write
// X[k1 + L1 k2] back.  All UK_COLS units are queued before everything else,
// so by the time a UK_ROWS2 unit is claimed every unit it waits for has been
// claimed by a running CTA; the wait is still bounded (kWaitLimit polls),
// after which the kernel records an error in the status word and skips the
// unit instead of hanging.
//
// The reference runs one generated kernel per length and batch
// (vkdispatch/fft/shader_factories.py:11-60), each launched separately, and
// its planner rejects lengths above 16384 (vkdispatch/fft/config.py:185-190).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "fft_kernels.cuh"
#include "vdx.h"
#include "vdx_internal.h"

namespace vdx {

namespace {

constexpr int kMaxBatchThreads = 1024;
constexpr long long kWaitLimit = 1ll << 22;  // default polls of ~100 ns before a dependency wait gives up

enum UnitKind { UK_ROWS = 0, UK_COLS = 1, UK_ROWS2 = 2 };

// How a row unit moves its tile between global and shared memory.
//   UF_STAGE_IN:  the tile's rows are contiguous; one coalesced copy fills
//                 the padded row slots and the first pass gathers from them.
//                 Used for rows held by one thread each, where every warp
//                 load would touch 32 rows (2^25 points of length 16: 291 ->
//                 218 us); for rows of 2-8 threads the copy and its barrier
//                 cost more than they save (length 21: 247 -> 356 us).
//   UF_STAGE_OUT: the same for the store of contiguous rows.
//   UF_STAGE_OUT_T: the four-step second pass writes point k of row r at
//                 dst + r + k * dst_pt; the results go through shared memory
//                 and leave with adjacent rows in adjacent lanes, so each
//                 store covers a run of rows instead of one point per row
//                 (2^25 points of length 32768: 444 -> 363 us; 65536: 450 -> 370 us).
enum UnitFlags { UF_STAGE_IN = 1, UF_STAGE_OUT = 2, UF_STAGE_OUT_T = 4 };

struct UnitPlan {
  PassPlan pp;
  const Cx<float>* tw;  // W_n^k for this transform length
};

struct WorkUnit {
  PassPlan pp;                  // the unit's pass plan (a copy, so one table read fetches everything)
  const Cx<float>* tw;          // W_n^k for the unit's transform length
  long long src, dst;           // element offset of point 0 of slot 0 (data or workspace)
  long long src_slot, dst_slot;  // elements between slots
  long long src_pt, dst_pt;     // elements between points
  const Cx<float>* twl;         // UK_COLS: W_L table of the full length
  int kind;
  int plan;
  int nslots;  // slots (transforms, columns or rows) of this tile that exist
  int item;    // counter of a four-step item (UK_COLS signals it, UK_ROWS2 waits on it)
  int wait;    // UK_ROWS2: number of UK_COLS units of the item
  int c0;      // UK_COLS: first column of the tile
  int flags;   // UnitFlags
  unsigned nmag, smag;  // inv_magic(n), inv_magic(nslots): row and slot of a staged element
  float scale;
};

struct BatchArgs {
  const UnitPlan* plans;
  const WorkUnit* units;
  int nunits;
  int inverse;
  Cx<float>* data;
  Cx<float>* ws;
  unsigned* ticket;
  int* counters;
  int* status;
  long long wait_limit;  // polls before a dependency wait gives up
  int extra_wait;        // added to every dependency count (0 unless a test injects an unmet dependency)
};

// placement of a thread inside the current unit (the interface run_passes
// uses).  The shared-memory slot is i*ci + m*cm + (i >> 4)*cp: (M, 1, 0) for
// strided column tiles, (1, npad, 1) for contiguous rows -- one branch-free
// code path for every unit kind.
struct UnitPlace {
  int t, m;
  int ci, cmo, cp;  // cmo = m * cm, precomputed
  __device__ __forceinline__ int sidx(const PassPlan&, int i) const { return i * ci + cmo + (i >> 4) * cp; }
};

// Copies a tile of contiguous rows into the padded row slots of shared
// memory: element e is point e % n of row e / n (e < M n <= 16 * 1024, so
// the multiply-high quotient is exact).
__device__ __forceinline__ void stage_rows_in(const Cx<float>* __restrict__ s0, Cx<float>* __restrict__ sm, int total,
                                           int n, int npad, unsigned nmag) {
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int r = int(__umulhi(unsigned(e), nmag));
    const int i = e - r * n;
    sm[r * npad + i + (i >> 4)] = s0[e];
  }
}

// One code path for every unit kind (separate inlined copies per kind exhaust
// the 64 registers a thread has): the store multiplies by a per-point factor
// that is the four-step twiddle W_L^{n2 k1} for UK_COLS and the output scale
// otherwise.  UK_ROWS2 reads workspace that other CTAs wrote in this launch
// with ordinary (L1-cached) loads: the SM has not cached those lines before,
// because each workspace element is read by exactly one UK_ROWS2 unit, only
// after all UK_COLS units of its item completed, and every item's workspace
// region starts on its own 256-byte boundary, so no cache line is shared
// between items.
template <bool INV>
__device__ __forceinline__ void run_unit(const BatchArgs& a, const WorkUnit* __restrict__ pu, int kind,
                                         Cx<float>* sm) {
  constexpr int MAXE = 16;
  // fields are read from the (L1-cached, CTA-uniform) unit table: read-only
  // global loads the compiler may repeat instead of holding them in registers
  const WorkUnit& wu = *pu;
  const PassPlan& pp = wu.pp;
  const Cx<float>* tw = wu.tw;
  const int n = pp.n, T = pp.T, M = pp.M;
  const bool cols = kind == UK_COLS;
  UnitPlace pl;
  const int tid = threadIdx.x;
  // thread index split by the plan's multiply-high reciprocals (tid < 1024)
  if (cols) {
    pl.t = M > 1 ? int(__umulhi(unsigned(tid), pp.mmag)) : tid;
    pl.m = tid - pl.t * M;
    pl.ci = M;
    pl.cmo = pl.m;
    pl.cp = 0;
  } else {
    pl.m = T > 1 ? int(__umulhi(unsigned(tid), pp.tmag)) : tid;
    pl.t = tid - pl.m * T;
    pl.ci = 1;
    pl.cmo = pl.m * pp.npad;
    pl.cp = 1;
  }
  const bool active = pl.t < T && pl.m < M;
  if (!active) pl.t = 1 << 20;  // every butterfly index of an idle thread is out of range
  const bool valid = active && pl.m < wu.nslots;
  const int flags = wu.flags;
  // the first pass gathers point pos of slot m from src + pos * pt +
  // (pos >> 4) * pad: the tile in global memory, or the copy the kernel loop
  // staged into the padded row slots of shared memory (UF_STAGE_IN).  One
  // generic-address load path: a branch between two gathers here, or a
  // barrier inside this function, costs the kernel 400 more bytes of spills.
  const bool stg = (flags & UF_STAGE_IN) != 0;
  const Cx<float>* src = stg ? sm + pl.m * pp.npad : (kind == UK_ROWS2 ? a.ws : a.data) + wu.src + pl.m * wu.src_slot;
  // point offsets inside a unit stay below 2^28 (n, L1, L2 <= 16384): 32-bit
  const int src_pt = stg ? 1 : int(wu.src_pt);
  const int pad = stg ? 1 : 0;
  Cx<float> v[MAXE];
  radix_dispatch(pp.radix[0], [&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    gather<RR, MAXE, float>(v, n / RR, T, pl.t, [&](int pos) {
      if (!valid) return mk<float>(0.f, 0.f);
      return src[pos * src_pt + (pos >> 4) * pad];
    });
  });
  // row units keep each transform inside one warp when T divides 32
  run_passes<MAXE, INV>(v, pp, false, pl, sm, tw, !cols && warp_sized(T));
  const float sc = wu.scale;
  if (flags & (UF_STAGE_OUT | UF_STAGE_OUT_T)) {
    __syncthreads();  // every thread's last gather from sm is done
    radix_dispatch(pp.radix[pp.npass - 1], [&](auto rc) {
      constexpr int RR = decltype(rc)::value;
      each_natural<RR, MAXE, float>(v, n / RR, T, pl.t,
                                    [&](int pos, Cx<float> val) { sm[pl.sidx(pp, pos)] = scale(val, sc); });
    });
    __syncthreads();
    Cx<float>* d0 = a.data + wu.dst;
    const int ns = wu.nslots, total = ns * n, npad = pp.npad;
    if (flags & UF_STAGE_OUT) {
      const unsigned nmag = wu.nmag;
      for (int e = tid; e < total; e += blockDim.x) {
        const int r = int(__umulhi(unsigned(e), nmag));
        const int i = e - r * n;
        d0[e] = sm[r * npad + i + (i >> 4)];
      }
    } else {
      // point k of row r goes to d0[r + k * dst_pt]; rows fastest across lanes
      const unsigned smag = wu.smag;
      const int dpt = int(wu.dst_pt);
      for (int e = tid; e < total; e += blockDim.x) {
        const int k = ns > 1 ? int(__umulhi(unsigned(e), smag)) : e;
        const int r = e - k * ns;
        d0[r + k * dpt] = sm[r * npad + k + (k >> 4)];
      }
    }
    return;
  }
  Cx<float>* dst = (kind == UK_COLS ? a.ws : a.data) + wu.dst + pl.m * wu.dst_slot;
  const int dst_pt = int(wu.dst_pt);
  const bool twiddle = cols;
  const Cx<float>* twl = wu.twl;
  const int twstep = twiddle ? wu.c0 + pl.m : 0;  // n2; n2 * k1 < L <= 2^24
  radix_dispatch(pp.radix[pp.npass - 1], [&](auto rc) {
    constexpr int RR = decltype(rc)::value;
    each_natural<RR, MAXE, float>(v, n / RR, T, pl.t, [&](int pos, Cx<float> val) {
      if (!valid) return;
      if (twiddle) {
        // W_L^{n2 k1} with n2 = column, k1 = pos (n2 k1 < L)
        const Cx<float> w = ldg(twl + twstep * pos);
        val = INV ? cmulc(val, w) : cmul(val, w);
      } else {
        val = scale(val, sc);
      }
      dst[pos * dst_pt] = val;
    });
  });
}

// THREADS per CTA, MINB resident CTAs per SM (64 registers per thread).
//
// Claiming runs two units ahead: while a CTA works on unit u it already
// knows the next unit, whose descriptor (pass plan included) is prefetched
// into L1 at the start of u, and thread 0 holds the ticket of the one after,
// whose atomic was issued a whole unit earlier.  No ticket or pass-plan
// round trip to L2 lies between two units.  A CTA may hold two claimed
// units, but a claimed UK_COLS unit only ever follows another UK_COLS unit
// of the same CTA, which does not wait, so every claimed UK_COLS unit runs.
constexpr int kUnitLines = int((sizeof(WorkUnit) + 127) / 128) + 1;  // 128-byte lines a descriptor touches

template <bool INV, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_batch(BatchArgs a) {
  // (current, next) unit indices, double-buffered by iteration parity so
  // that one barrier per unit separates their reads from the next writes
  __shared__ int s_cur[2], s_next[2];
  __shared__ int s_ok;
  Cx<float>* sm = smem_base<float>();
  const int tid = threadIdx.x;
  int claim = 0;  // thread 0: the ticket two units ahead
  if (tid == 0) {
    s_cur[0] = (int)atomicAdd(a.ticket, 1u);
    s_next[0] = (int)atomicAdd(a.ticket, 1u);
    claim = s_next[0] < a.nunits ? (int)atomicAdd(a.ticket, 1u) : a.nunits;
  }
  __syncthreads();
  for (int par = 0;; par ^= 1) {
    const int u = s_cur[par];
    if (u >= a.nunits) return;
    const int un = s_next[par];
    if (tid < kUnitLines && un < a.nunits) {
      const char* line = reinterpret_cast<const char*>(&a.units[un]) + 128 * tid;
      asm volatile("prefetch.global.L1 [%0];" ::"l"(line));
    }
    const WorkUnit* pu = &a.units[u];
    const WorkUnit& wu = *pu;
    const int kind = wu.kind;
    bool run = true;
    if (kind == UK_ROWS2) {
      if (tid == 0) {
        int ok = 1;
        long long polls = 0;
        const int item = wu.item, wait = wu.wait + a.extra_wait;
        while (atomicAdd(&a.counters[item], 0) < wait) {
          if (++polls > a.wait_limit) {
            atomicExch(a.status, 1);
            ok = 0;
            break;
          }
          __nanosleep(100);
        }
        __threadfence();
        s_ok = ok;
      }
      __syncthreads();
      run = s_ok != 0;
    }
    if (run && (wu.flags & UF_STAGE_IN)) {
      stage_rows_in((kind == UK_ROWS2 ? a.ws : a.data) + wu.src, sm, wu.nslots * wu.pp.n, wu.pp.n, wu.pp.npad,
                    wu.nmag);
      __syncthreads();
    }
    if (run) run_unit<INV>(a, pu, kind, sm);
    if (kind == UK_COLS) {
      __threadfence();
      __syncthreads();
      if (tid == 0) atomicAdd(&a.counters[wu.item], 1);
    }
    // move the ticket pipeline on by one; the barrier also keeps the next
    // unit's shared-memory exchanges clear of this unit's last reads
    if (tid == 0) {
      s_cur[par ^ 1] = un;
      s_next[par ^ 1] = claim;
      if (claim < a.nunits) claim = (int)atomicAdd(a.ticket, 1u);
    }
    __syncthreads();
  }
}

// -------------------------------------------------------------------------
// host side
// -------------------------------------------------------------------------
int threads_for(const std::vector<int>& radices, int n) {
  int T = 1;
  for (int r : radices) {
    const int nb = n / r;
    const int per = std::max(1, 16 / r);
    T = std::max(T, (nb + per - 1) / per);
  }
  return T;
}

int npad_of(int n) { return n + 1 + ((n + 1) >> 4) + 1; }

}  // namespace

bool factor_radices(int n, int maxe, std::vector<int>& radices, std::string& why);
int get_twiddle_table(int dev, int count, int den, bool f64, void** out);

}  // namespace vdx

struct vdx_batch_plan {
  int dev;
  int cta;
  int inverse;
  int nunits;
  int nitems_large;
  size_t ws_bytes;
  size_t smem;
  int grid;
  vdx::UnitPlan* d_plans;
  vdx::WorkUnit* d_units;
  unsigned* d_ticket;
  int* d_counters;
  int* d_status;
  long long wait_limit = vdx::kWaitLimit;
  int extra_wait = 0;
  std::string desc;
};

namespace {

using namespace vdx;

struct PlanKey {
  int n;
  bool cols;
  bool operator<(const PlanKey& o) const { return n != o.n ? n < o.n : cols < o.cols; }
};

// Splits a long length into L1 * L2 with both factors transformable by one
// CTA, L1 as close to sqrt(L) as the divisors allow.
bool split_long(int L, int cta, int& L1, int& L2) {
  int best = -1;
  for (int d = 2; d <= 16384 && d < L; ++d) {
    if (L % d) continue;
    const int e = L / d;
    if (e > 16384) continue;
    std::vector<int> r;
    std::string why;
    if (!factor_radices(d, 16, r, why) || threads_for(r, d) > cta) continue;
    if (!factor_radices(e, 16, r, why) || threads_for(r, e) > cta) continue;
    if (best < 0 || std::abs(std::log((double)d) - 0.5 * std::log((double)L)) <
                        std::abs(std::log((double)best) - 0.5 * std::log((double)L)))
      best = d;
  }
  if (best < 0) return false;
  L1 = best;
  L2 = L / best;
  return true;
}

}  // namespace

extern "C" {

int vdx_batch_plan_create(const vdx_batch_item* items, int nitems, int inverse, int normalize,
                          vdx_batch_plan** out) {
  if (!items || !out || nitems < 1) return set_error(VDX_ERR_INVALID, "items, out and nitems >= 1 are required");
  *out = nullptr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  int smem_optin = 0, nsm = 0, smem_sm = 0;
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // CTA size: 512 threads (2 per SM, 64 registers each) by default;
  // VDX_BATCH_THREADS = 256 | 512 | 1024
  int cta = 512;
  if (const char* ev = std::getenv("VDX_BATCH_THREADS")) cta = std::atoi(ev);
  if (cta != 256 && cta != 512 && cta != 1024) return set_error(VDX_ERR_INVALID, "VDX_BATCH_THREADS must be 256, 512 or 1024");
  // row tiles staged through shared memory (UnitFlags).  VDX_BATCH_STAGE is a
  // mask: 1 = rows of fewer than VDX_BATCH_STAGE_T threads (whole-length
  // items), 2 = the transposed store of four-step second passes, 4 = their
  // input rows of fewer than VDX_BATCH_STAGE_T threads
  int stage = 3, stage_t = 2;
  if (const char* ev = std::getenv("VDX_BATCH_STAGE")) stage = std::atoi(ev);
  if (const char* ev = std::getenv("VDX_BATCH_STAGE_T")) stage_t = std::atoi(ev);
  const int per_sm = 1024 / cta;  // 64 registers per thread at any of the three sizes
  // shared memory per CTA so that per_sm CTAs fit on one SM
  const int smem_cap = std::min(smem_optin, smem_sm / per_sm - 1024);

  std::map<PlanKey, int> plan_index;
  std::vector<UnitPlan> plans;
  size_t smem = 64;
  std::string why;

  auto get_plan = [&](int n, bool cols, int slots_max) -> int {
    PlanKey key{n, cols};
    auto it = plan_index.find(key);
    if (it != plan_index.end()) return it->second;
    std::vector<int> radices;
    if (!factor_radices(n, 16, radices, why)) return -1;
    const int T = threads_for(radices, n);
    if (T > cta) return -2;
    int M = std::max(1, cta / T);
    if (cols) M = std::min(M, 64);  // column tiles: up to 64 columns (256-byte row segments per warp)
    M = std::min(M, std::max(1, slots_max));
    const int npad = npad_of(n);
    // leave room for the kernel's static shared variables
    auto need = [&](int m) { return size_t(cols ? n : npad) * size_t(m) * 8; };
    while (M > 1 && need(M) + 1024 > size_t(smem_cap)) --M;
    if (need(M) + 1024 > size_t(smem_cap)) return -3;
    UnitPlan up{};
    up.pp.n = n;
    up.pp.npass = (int)radices.size();
    for (int i = 0; i < up.pp.npass; ++i) up.pp.radix[i] = radices[i];
    up.pp.T = T;
    up.pp.M = M;
    up.pp.npad = npad;
    set_pass_tables(up.pp);
    void* tw = nullptr;
    if (get_twiddle_table(dev, n, n, false, &tw) != VDX_OK) return -4;
    up.tw = reinterpret_cast<const Cx<float>*>(tw);
    smem = std::max(smem, need(M));
    plans.push_back(up);
    plan_index[key] = (int)plans.size() - 1;
    return (int)plans.size() - 1;
  };

  std::vector<WorkUnit> cols_units, rows_units, rows2_units;
  long long ws_elems = 0;
  long long long_points = 0;
  int nlarge = 0;
  std::vector<int> large_wait;
  for (int i = 0; i < nitems; ++i) {
    const vdx_batch_item& it = items[i];
    if (it.length < 1 || it.count < 1 || it.offset < 0)
      return set_error(VDX_ERR_INVALID, "every item needs length >= 1, count >= 1 and offset >= 0");
    const int L = it.length;
    const float scale = (inverse && normalize) ? 1.0f / float(L) : 1.0f;
    std::vector<int> r;
    bool single = L <= 16384 && factor_radices(L, 16, r, why) && threads_for(r, L) <= cta &&
                  size_t(npad_of(L)) * 8 + 1024 <= size_t(smem_cap);
    if (single) {
      const int p = get_plan(L, false, it.count);
      if (p < 0) return set_error(VDX_ERR_UNSUPPORTED, ("length " + std::to_string(L) + ": " + why).c_str());
      const int M = plans[p].pp.M;
      for (long long t0 = 0; t0 < it.count; t0 += M) {
        WorkUnit w{};
        w.kind = UK_ROWS;
        w.plan = p;
        w.pp = plans[p].pp;
        w.tw = plans[p].tw;
        w.src = w.dst = it.offset + t0 * L;
        w.src_slot = w.dst_slot = L;
        w.src_pt = w.dst_pt = 1;
        w.nslots = (int)std::min<long long>(M, it.count - t0);
        w.item = -1;
        w.scale = scale;
        // narrow rows (fewer than 16 threads each) move through shared memory
        if ((stage & 1) && L >= 2 && plans[p].pp.T < stage_t) w.flags = UF_STAGE_IN | UF_STAGE_OUT;
        w.nmag = inv_magic(L);
        w.smag = inv_magic(w.nslots);
        w.twl = plans[p].tw;  // valid pointer; only column units read it
        rows_units.push_back(w);
      }
      continue;
    }
    int L1 = 0, L2 = 0;
    if (!split_long(L, cta, L1, L2))
      return set_error(VDX_ERR_UNSUPPORTED,
                       ("length " + std::to_string(L) + " has no split into two single-CTA factors").c_str());
    const int pc = get_plan(L1, true, L2);
    const int pr = get_plan(L2, false, L1);
    if (pc < 0 || pr < 0) return set_error(VDX_ERR_UNSUPPORTED, ("length " + std::to_string(L) + ": " + why).c_str());
    void* twl = nullptr;
    if (get_twiddle_table(dev, L, L, false, &twl) != VDX_OK) return VDX_ERR_NOMEM;
    const int item = nlarge++;
    const long long wsoff = (ws_elems + 31) & ~31ll;  // 256-byte aligned region per item
    ws_elems = wsoff + (long long)L * it.count;
    long_points += (long long)L * it.count;
    const int Mc = plans[pc].pp.M, Mr = plans[pr].pp.M;
    int ncols = 0;
    for (long long bt = 0; bt < it.count; ++bt) {
      for (int c0 = 0; c0 < L2; c0 += Mc) {
        WorkUnit w{};
        w.kind = UK_COLS;
        w.plan = pc;
        w.pp = plans[pc].pp;
        w.tw = plans[pc].tw;
        w.src = it.offset + bt * L + c0;
        w.dst = wsoff + bt * L + c0;
        w.src_slot = w.dst_slot = 1;
        w.src_pt = w.dst_pt = L2;
        w.twl = reinterpret_cast<const Cx<float>*>(twl);
        w.c0 = c0;
        w.nslots = std::min(Mc, L2 - c0);
        w.item = item;
        w.scale = 1.0f;
        cols_units.push_back(w);
        ++ncols;
      }
    }
    for (long long bt = 0; bt < it.count; ++bt) {
      for (int r0 = 0; r0 < L1; r0 += Mr) {
        WorkUnit w{};
        w.kind = UK_ROWS2;
        w.plan = pr;
        w.pp = plans[pr].pp;
        w.tw = plans[pr].tw;
        w.src = wsoff + bt * L + (long long)r0 * L2;
        w.dst = it.offset + bt * L + r0;
        w.src_slot = L2;
        w.dst_slot = 1;
        w.src_pt = 1;
        w.dst_pt = L1;
        w.nslots = std::min(Mr, L1 - r0);
        w.item = item;
        w.scale = scale;
        // the transposed store goes through shared memory wherever a unit holds several rows
        if (L2 >= 2) {
          if ((stage & 2) && w.nslots > 1) w.flags |= UF_STAGE_OUT_T;
          if ((stage & 4) && plans[pr].pp.T < stage_t) w.flags |= UF_STAGE_IN;
        }
        w.nmag = inv_magic(L2);
        w.smag = inv_magic(w.nslots);
        w.twl = plans[pr].tw;  // valid pointer; only column units read it
        rows2_units.push_back(w);
      }
    }
    large_wait.push_back(ncols);
  }
  // all waits of an item's row units equal its column-unit count
  for (auto& w : rows2_units) w.wait = large_wait[w.item];
  std::vector<WorkUnit> units;
  units.reserve(cols_units.size() + rows_units.size() + rows2_units.size());
  units.insert(units.end(), cols_units.begin(), cols_units.end());
  units.insert(units.end(), rows_units.begin(), rows_units.end());
  units.insert(units.end(), rows2_units.begin(), rows2_units.end());
  if (units.size() > 0x7fffffffu) return set_error(VDX_ERR_UNSUPPORTED, "too many work units");

  auto* p = new vdx_batch_plan();
  p->dev = dev;
  p->inverse = inverse ? 1 : 0;
  p->nunits = (int)units.size();
  p->nitems_large = nlarge;
  p->ws_bytes = size_t(ws_elems) * 8;
  p->smem = smem;
  p->grid = (nsm > 0 ? nsm : 148) * per_sm;
  p->cta = cta;
  e = cudaMalloc(&p->d_plans, sizeof(UnitPlan) * plans.size());
  if (e == cudaSuccess) e = cudaMalloc(&p->d_units, sizeof(WorkUnit) * units.size());
  if (e == cudaSuccess) e = cudaMalloc(&p->d_ticket, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_counters, sizeof(int) * std::max(1, nlarge));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_status, sizeof(int));
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_plans, plans.data(), sizeof(UnitPlan) * plans.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_units, units.data(), sizeof(WorkUnit) * units.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e != cudaSuccess) {
    cudaFree(p->d_plans);
    cudaFree(p->d_units);
    cudaFree(p->d_ticket);
    cudaFree(p->d_counters);
    cudaFree(p->d_status);
    delete p;
    return set_error(VDX_ERR_NOMEM, cudaGetErrorString(e));
  }
  p->desc = "{\"units\": " + std::to_string(units.size()) + ", \"column_units\": " +
            std::to_string(cols_units.size()) + ", \"row_units\": " + std::to_string(rows_units.size()) +
            ", \"second_row_units\": " + std::to_string(rows2_units.size()) + ", \"plans\": " +
            std::to_string(plans.size()) + ", \"long_items\": " + std::to_string(nlarge) +
            ", \"long_points\": " + std::to_string(long_points) +
            ", \"workspace_bytes\": " + std::to_string(p->ws_bytes) + ", \"smem\": " + std::to_string(smem) +
            ", \"grid\": " + std::to_string(p->grid) + ", \"cta_threads\": " + std::to_string(cta) + "}";
  *out = p;
  return VDX_OK;
}

int vdx_batch_plan_destroy(vdx_batch_plan* p) {
  if (!p) return VDX_OK;
  cudaFree(p->d_plans);
  cudaFree(p->d_units);
  cudaFree(p->d_ticket);
  cudaFree(p->d_counters);
  cudaFree(p->d_status);
  delete p;
  return VDX_OK;
}

int vdx_batch_workspace_bytes(const vdx_batch_plan* p, size_t* bytes) {
  if (!p || !bytes) return set_error(VDX_ERR_INVALID, "plan and bytes must be non-NULL");
  *bytes = p->ws_bytes;
  return VDX_OK;
}

int vdx_batch_plan_describe(const vdx_batch_plan* p, char* buf, size_t n) {
  if (!p || !buf || n == 0) return set_error(VDX_ERR_INVALID, "plan and buf must be non-NULL");
  std::snprintf(buf, n, "%s", p->desc.c_str());
  return VDX_OK;
}

int vdx_batch_exec(const vdx_batch_plan* p, void* data, void* workspace, void* stream) {
  if (!p || !data) return set_error(VDX_ERR_INVALID, "plan and data must be non-NULL");
  if (p->ws_bytes > 0 && !workspace) return set_error(VDX_ERR_INVALID, "this batch needs a workspace");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->dev) return set_error(VDX_ERR_INVALID, "batch plan was created on another device");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(p->d_ticket, 0, sizeof(unsigned), s);
  if (e == cudaSuccess && p->nitems_large > 0)
    e = cudaMemsetAsync(p->d_counters, 0, sizeof(int) * p->nitems_large, s);
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  BatchArgs a{};
  a.plans = p->d_plans;
  a.units = p->d_units;
  a.nunits = p->nunits;
  a.inverse = p->inverse;
  a.data = reinterpret_cast<Cx<float>*>(data);
  a.ws = reinterpret_cast<Cx<float>*>(workspace);
  a.ticket = p->d_ticket;
  a.counters = p->d_counters;
  a.status = p->d_status;
  a.wait_limit = p->wait_limit;
  a.extra_wait = p->extra_wait;
  Launch l;
  l.grid = dim3(p->grid);
  l.block = dim3(p->cta);
  l.smem = p->smem;
  l.stream = s;
  switch (p->cta) {
    case 256: e = p->inverse ? enqueue(k_batch<true, 256, 4>, l, a) : enqueue(k_batch<false, 256, 4>, l, a); break;
    case 512: e = p->inverse ? enqueue(k_batch<true, 512, 2>, l, a) : enqueue(k_batch<false, 512, 2>, l, a); break;
    default: e = p->inverse ? enqueue(k_batch<true, 1024, 1>, l, a) : enqueue(k_batch<false, 1024, 1>, l, a); break;
  }
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  return VDX_OK;
}

int vdx_batch_plan_set_wait(vdx_batch_plan* p, int64_t wait_limit, int32_t extra_dependency) {
  if (!p) return set_error(VDX_ERR_INVALID, "plan must be non-NULL");
  if (wait_limit < 1 || extra_dependency < 0)
    return set_error(VDX_ERR_INVALID, "wait_limit must be >= 1 and extra_dependency >= 0");
  cudaError_t e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  p->wait_limit = wait_limit;
  p->extra_wait = extra_dependency;
  return VDX_OK;
}

int vdx_batch_status(const vdx_batch_plan* p, int* status) {
  if (!p || !status) return set_error(VDX_ERR_INVALID, "plan and status must be non-NULL");
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, p->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  *status = h;
  return VDX_OK;
}

}  // extern "C"
