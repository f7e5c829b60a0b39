// C ABI of libvdx: argument validation, the FFT plan builder, twiddle-table
// cache and kernel dispatch.  See include/vdx.h for the contract.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "vdx.h"
#include "vdx_internal.h"

using namespace vdx;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(VDX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

// ---------------------------------------------------------------------------
// twiddle tables: one per (device, count, denominator, precision), built once
// and kept for the life of the process (a few KB each)
// ---------------------------------------------------------------------------
std::mutex g_tab_mu;
std::map<std::tuple<int, int, int, bool>, void*> g_tabs;

int get_table(int dev, int count, int den, bool f64, void** out) {
  std::lock_guard<std::mutex> lock(g_tab_mu);
  auto key = std::make_tuple(dev, count, den, f64);
  auto it = g_tabs.find(key);
  if (it != g_tabs.end()) {
    *out = it->second;
    return VDX_OK;
  }
  void* p = nullptr;
  const size_t bytes = size_t(count) * (f64 ? 16 : 8);
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return fail(VDX_ERR_NOMEM, std::string("twiddle table allocation: ") + cudaGetErrorString(e));
  cudaStream_t s;
  e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "twiddle stream");
  e = launch_twiddle(p, count, den, f64, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    cudaFree(p);
    return cuda_fail(e, "twiddle table build");
  }
  g_tabs[key] = p;
  *out = p;
  return VDX_OK;
}

int store_of(int t) {
  switch (t) {
    case VDX_C64: return ST_C64;
    case VDX_C32: return ST_C32;
    case VDX_C128: return ST_C128;
    case VDX_BF16X2: return ST_BF16;
    default: return -1;
  }
}

size_t store_bytes(int st) { return st == ST_C128 ? 16 : st == ST_C64 ? 8 : 4; }

// desc.normalize: 0 = none, 1 = 1/N, 2 = 1/sqrt(N) (orthonormal)
double norm_scale(int normalize, int N) {
  if (normalize == 2) return 1.0 / std::sqrt(double(N));
  return normalize ? 1.0 / N : 1.0;
}

}  // namespace

namespace vdx {

// ---------------------------------------------------------------------------
// radix factorisation
// ---------------------------------------------------------------------------
// Splits n into passes: radix 16 for each 2^4, the leftover power of two
// (2, 4 or 8), 9 for pairs of 3s, then 3, 5, 7, 11, 13.  Fails for primes above 13, the reference's largest
// supported prime (vkdispatch/fft/prime_utils.py:9-10).
bool factor_radices(int n, int maxe, std::vector<int>& radices, std::string& why) {
  radices.clear();
  if (n == 1) {
    radices.push_back(1);
    return true;
  }
  int m = n, a = 0, cnt[14] = {0};
  while (m % 2 == 0) {
    m /= 2;
    ++a;
  }
  for (int p : {3, 5, 7, 11, 13})
    while (m % p == 0) {
      m /= p;
      ++cnt[p];
    }
  if (m != 1) {
    why = "FFT length " + std::to_string(n) + " has a prime factor " + std::to_string(m) +
          " larger than 13 (supported radices: 2, 3, 5, 7, 11, 13)";
    return false;
  }
  const int big2 = maxe >= 16 ? 16 : 8;
  const int big2log = big2 == 16 ? 4 : 3;
  while (a >= big2log) {
    radices.push_back(big2);
    a -= big2log;
  }
  int rem2 = 1 << a;  // 1, 2, 4 or 8
  while (cnt[3] >= 2 && maxe >= 9) {
    radices.push_back(9);
    cnt[3] -= 2;
  }
  while (cnt[3] > 0) {
    radices.push_back(3);
    --cnt[3];
  }
  for (int i = 0; i < cnt[5]; ++i) radices.push_back(5);
  for (int p : {7, 11, 13})
    for (int i = 0; i < cnt[p]; ++i) radices.push_back(p);
  if (rem2 > 1) radices.push_back(rem2);
  for (int r : radices)
    if (r > maxe) {
      why = "radix " + std::to_string(r) + " exceeds the per-thread register budget";
      return false;
    }
  if ((int)radices.size() > kMaxPasses) {
    why = "too many radix passes";
    return false;
  }
  std::sort(radices.begin(), radices.end(), [](int x, int y) { return x > y; });
  return true;
}

int get_twiddle_table(int dev, int count, int den, bool f64, void** out) { return get_table(dev, count, den, f64, out); }

int set_error(int code, const char* msg) { return fail(code, msg); }

int reduce_out_bytes(int in_type) { return in_type == VDX_F64 ? 8 : 4; }

int check_reduce_args(int op, int map, int in_type, const void* in, long long n, long long batch, const void* out) {
  if (!in || !out) return fail(VDX_ERR_INVALID, "in and out must be non-NULL device pointers");
  if (n < 1 || batch < 1) return fail(VDX_ERR_INVALID, "n and batch must be >= 1");
  if (batch > 65535) return fail(VDX_ERR_UNSUPPORTED, "batch above 65535 rows");
  if (op < VDX_RED_ADD || op > VDX_RED_XOR) return fail(VDX_ERR_INVALID, "unknown reduction op");
  if (map < VDX_MAP_IDENTITY || map > VDX_MAP_SIN) return fail(VDX_ERR_INVALID, "unknown map");
  const bool integer = in_type == VDX_I32 || in_type == VDX_U32;
  if (!integer && in_type != VDX_F32 && in_type != VDX_F64 && in_type != VDX_C64)
    return fail(VDX_ERR_INVALID, "in_type must be F32, F64, C64, I32 or U32");
  if (op >= VDX_RED_AND && !integer) return fail(VDX_ERR_INVALID, "bitwise reductions need integer input");
  if (op >= VDX_RED_AND && map != VDX_MAP_IDENTITY) return fail(VDX_ERR_INVALID, "bitwise reductions take no map");
  if (in_type == VDX_C64 && (map == VDX_MAP_IDENTITY || map == VDX_MAP_SIN))
    return fail(VDX_ERR_INVALID, "complex input needs a map to a real value (abs, square, real, imag)");
  if (in_type != VDX_C64 && (map == VDX_MAP_REAL || map == VDX_MAP_IMAG))
    return fail(VDX_ERR_INVALID, "real/imag maps need complex input");
  if (integer && map == VDX_MAP_SIN) return fail(VDX_ERR_INVALID, "sin map needs floating-point input");
  return VDX_OK;
}

}  // namespace vdx

namespace vdx {
// Plan choices the autotuner varies (-1 / 0 = the planner's default).
struct Tune {
  int width = -1;     // contiguous axes: threads per CTA; strided axes: columns per tile
  int order = 0;      // radix passes: 0 = largest radix first, 1 = smallest first
  int fixed = -1;     // compile-time kernels where available: -1 = yes, 0 = no
  int fourstep = -1;  // long C2C axes: -1 = from 8192 points (VDX_FOURSTEP_MIN), 0 = only above one CTA, 1 = always
  int maxe = 0;       // points per thread: 0 = the plan's default, or 16 / 8 / 32 (compile-time plans where they exist)
};
}  // namespace vdx

struct vdx_plan {
  vdx_fft_desc d;
  int dev;
  int op;  // vdx::Op
  bool strided;
  bool f64;
  int store;
  int N;  // axis length (real length for R2C/C2R)
  bool fixed;  // compile-time specialised kernels (complex64, power-of-two n)
  FftArgs args;
  Launch launch;
  std::vector<int> radices;
  // four-step long axis (fft_large.cu): N = N1 * N0, processed in chunks of
  // `chunk_cols` columns x `chunk_outer` outer batches (strided axes) or
  // `chunk_outer` rows (contiguous axes); `ws` holds one chunk
  bool fourstep = false;
  int fixed_pts = 0;  // 8 or 32: strided convolution on that points-per-thread compile-time plan
  int N1 = 0, N0 = 0;
  long long inner = 1, outer = 1;
  long long chunk_cols = 0, chunk_outer = 0;
  FsArgs fsA{}, fsB{};  // pass plans, twiddles and scale; geometry is set per chunk
  dim3 blockA, blockB;
  size_t smemA = 0, smemB = 0;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  // both passes in one persistent launch with an L2-resident ring (fft_fused4.cu)
  bool fused = false;
  FusedLaunch fl{};
  unsigned* d_ticket = nullptr;
  int* d_done = nullptr;  // 2 R counters
  // tensor-core short transforms (VDX_FFT_FLAG_TENSOR_CORE)
  bool tensor_core = false;
  const void* tc_bmat = nullptr;  // DFT operand image, shared per (device, direction)
  int* d_status = nullptr;        // bounded-wait status word
  // autotuned choices (VDX_FFT_FLAG_AUTOTUNE)
  bool tuned = false;
  Tune tune;
  float tuned_ms = 0.f;
  int tuned_candidates = 0;
  // Bluestein (bluestein.cu): chirp w, kernel slab conj(FFT_M(b)), workspace, conv plan
  bool bluestein = false;
  int bs_M = 0;
  void* bs_w = nullptr;
  void* bs_K = nullptr;
  void* bs_ws = nullptr;
  vdx_plan* bs_conv = nullptr;  // fused convolution (M fits one CTA), else:
  vdx_plan* bs_fwd = nullptr;   // four-step forward transform of length M
  vdx_plan* bs_inv = nullptr;   // and its normalised inverse
  // one-launch convolve2DR (fft_conv2d.cu)
  int c2_H = 0, c2_W = 0;
  long long c2_images = 0;
  Conv2dArgs c2{};
  ~vdx_plan() {
    if (ws) cudaFree(ws);
    if (d_status) cudaFree(d_status);
    if (d_ticket) cudaFree(d_ticket);
    if (d_done) cudaFree(d_done);
    if (bs_w) cudaFree(bs_w);
    if (bs_K) cudaFree(bs_K);
    if (bs_ws) cudaFree(bs_ws);
    delete bs_conv;
    delete bs_fwd;
    delete bs_inv;
  }
};

namespace {

int sub_pass_plan(int n, int M, PassPlan& pp, std::string& why) {
  std::vector<int> r;
  if (!factor_radices(n, 16, r, why)) return VDX_ERR_UNSUPPORTED;
  std::memset(&pp, 0, sizeof(pp));
  pp.n = n;
  pp.npass = (int)r.size();
  int T = 1;
  for (int i = 0; i < pp.npass; ++i) {
    pp.radix[i] = r[i];
    const int nb = n / r[i];
    const int per = std::max(1, 16 / r[i]);
    T = std::max(T, (nb + per - 1) / per);
  }
  pp.T = T;
  pp.M = M;
  pp.npad = n + 1 + ((n + 1) >> 4) + 1;
  set_pass_tables(pp);
  return VDX_OK;
}

// The fused form of a square four-step split (fft_fused4.cu): tile width,
// persistent grid from the kernel's occupancy, queue lag L and ring of
// R = L + 1 group slots sized so that the ring stays far below L2.
int plan_fused_fourstep(vdx_plan* p, int N1, int N0, long long inner, long long outer, PassPlan pp, size_t sb) {
  const int N = p->N;
  const bool strided = inner > 1;
  int M = strided ? 32 : 16;
  if (const char* e = std::getenv("VDX_FUSED_COLUMNS")) M = std::max(8, std::min(32, std::atoi(e)));
  if (strided) M = (int)std::min<long long>(M, inner);
  M = std::max(1, std::min(M, 256 / pp.T));
  pp.M = M;
  pp.mmag = inv_magic(M);
  const size_t smem = size_t(N1 + 1) * M * 8;
  int per_sm = 0;
  cudaError_t e = fused_fourstep_ctas_per_sm(p->store, pp, smem, &per_sm);
  if (e != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return fail(VDX_ERR_UNSUPPORTED, "no fused four-step kernel for this split");
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->dev);
  const long long grid = (long long)per_sm * std::max(1, sms);
  const long long nA = strided ? N0 : (N0 + M - 1) / M, nB = strided ? N1 : (N1 + M - 1) / M;
  const long long slot = strided ? (long long)N * M : (long long)N;
  const long long slot_bytes = slot * (long long)sb;
  // span = queue stages the resident CTAs cover at once.  Pass B of group g
  // is queued L = 2 spans after its pass A, so its inputs are done when it
  // runs; a ring slot is reused R = L + span + 2 groups later, so the pass B
  // that last read it has finished too (with R = L + 1 the reuse wait falls
  // inside the window of running units and stalls most pass-A units).
  const long long span = std::max(1ll, (grid + nA + nB - 1) / (nA + nB));
  long long L = 2 * span;
  if (const char* e2 = std::getenv("VDX_FUSED_LAG")) L = std::max(1ll, std::atoll(e2));
  long long extra = span + 2;
  const long long ring_cap = 64ll << 20;  // half the 126 MB L2
  while (L > 1 && (L + extra) * slot_bytes > ring_cap) {
    --L;
    if (extra > 2 && (L + extra) * slot_bytes > ring_cap) --extra;
  }
  const long long groups = strided ? outer * ((inner + M - 1) / M) : outer;
  L = std::min(L, std::max(1ll, groups));
  const int R = int(L + extra);
  p->fused = true;
  p->fourstep = true;
  p->N1 = N1;
  p->N0 = N0;
  p->inner = inner;
  p->outer = outer;
  p->ws_bytes = size_t(R) * size_t(slot_bytes);
  FusedLaunch& fl = p->fl;
  fl.ppA = fl.ppB = pp;
  fl.N = N;
  fl.N0 = N0;
  fl.N1 = N1;
  fl.inner = inner;
  fl.outer = outer;
  fl.M = M;
  fl.scale = float(p->args.scale);
  fl.L = int(L);
  fl.R = R;
  fl.store = p->store;
  fl.inverse = p->op == OP_C2C_INV;
  fl.strided = strided;
  fl.grid = (unsigned)grid;
  fl.smem = smem;
  int rc = get_table(p->dev, N1, N1, false, const_cast<void**>(&fl.twA));
  if (rc == VDX_OK) rc = get_table(p->dev, N0, N0, false, const_cast<void**>(&fl.twB));
  if (rc == VDX_OK) rc = get_table(p->dev, N, N, false, const_cast<void**>(&fl.twl));
  if (rc != VDX_OK) return rc;
  e = cudaMalloc(&p->ws, p->ws_bytes);
  if (e != cudaSuccess) {
    p->ws = nullptr;
    return fail(VDX_ERR_NOMEM, std::string("four-step ring: ") + cudaGetErrorString(e));
  }
  e = cudaMalloc(reinterpret_cast<void**>(&p->d_status), sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->d_ticket), sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->d_done), sizeof(int) * 2 * size_t(R));
  if (e != cudaSuccess) return cuda_fail(e, "fused four-step counters");
  fl.ring = p->ws;
  fl.ticket = p->d_ticket;
  fl.doneA = p->d_done;
  fl.doneB = p->d_done + R;
  fl.status = p->d_status;
  p->fsA.pp = p->fsB.pp = pp;
  p->blockA = p->blockB = dim3(pp.T * M);
  p->smemA = p->smemB = smem;
  p->chunk_cols = inner;
  p->chunk_outer = outer;
  return VDX_OK;
}

// Plans an axis as the four-step pair (fft_large.cu).  N0 is the largest
// divisor of N not above sqrt(N); both short lengths must be 13-smooth (they
// are, as divisors of a 13-smooth N) and at most 4096.
int plan_fourstep(vdx_plan* p, long long inner, long long outer, int smem_optin) {
  const int N = p->N;
  int N0 = 1;
  for (int c = 1; (long long)c * c <= N; ++c)
    if (N % c == 0) N0 = c;
  const int N1 = N / N0;
  if (N0 < 8 || N1 > 4096)
    return fail(VDX_ERR_UNSUPPORTED, "FFT length " + std::to_string(N) + " has no four-step split into two lengths "
                                     "in [8, 4096]");
  const size_t sb = store_bytes(p->store);
  // columns per tile: 32 on strided axes and 16 on contiguous ones, for every
  // storage type (16384^2: strided c64 1.40 / 1.36 / 1.40 ms and bf16 1.20 /
  // 1.13 / 1.19 ms at 16 / 32 / 64 columns; contiguous c64 1.56 / 1.70 / 1.70
  // and bf16 1.41 / 1.49 / 1.60 ms); VDX_FS_COLUMNS overrides
  int mw = inner > 1 ? 32 : 16;
  if (const char* e = std::getenv("VDX_FS_COLUMNS")) mw = std::max(8, std::min(64, std::atoi(e)));
  // tensor-core passes: 16 columns for every storage type (half the operand and
  // staging shared memory of 32, so more CTAs per SM: 16384^2 bf16 3.68 ->
  // 3.59 ms, fp16 3.76 -> 3.55 ms); VDX_TC_COLUMNS=32 restores 32 for 4-byte types
  if (p->tensor_core) {
    mw = 16;
    if (const char* e = std::getenv("VDX_TC_COLUMNS")) mw = std::atoi(e) == 32 && sb == 4 ? 32 : 16;
  }
  std::string why;
  auto tile_m = [&](int n, long long cols, int T) {
    int M = (int)std::min<long long>(mw, cols);
    M = std::max(1, std::min(M, 512 / T));
    while (M > 1 && size_t(n + 1) * M * 8 > size_t(smem_optin)) M /= 2;
    return M;
  };
  PassPlan ppA, ppB;
  if (sub_pass_plan(N1, 1, ppA, why) != VDX_OK || sub_pass_plan(N0, 1, ppB, why) != VDX_OK)
    return fail(VDX_ERR_UNSUPPORTED, why);
  const bool strided = inner > 1;
  ppA.M = tile_m(N1, strided ? inner : N0, ppA.T);
  ppB.M = tile_m(N0, strided ? inner : N1, ppB.T);
  ppA.mmag = inv_magic(ppA.M);
  ppB.mmag = inv_magic(ppB.M);
  if (ppA.T * ppA.M > 512 || ppB.T * ppB.M > 512)
    return fail(VDX_ERR_UNSUPPORTED, "four-step sub-transform needs more than 512 threads");

  // Square splits (the same compile-time short plan for both passes) can run
  // as one persistent launch whose intermediate stays in an L2-resident ring
  // (fft_fused4.cu) with VDX_FOURSTEP_FUSED=1.  It halves the HBM traffic but
  // measured slower on GB300 (16384^2 complex64: 2.16-2.25 ms per axis
  // against 1.37-1.56 ms for the two launches, bf16 the same): each unit's
  // claim, dependency check and load -> compute -> store run in series, and
  // three to six resident CTAs per SM do not hide that, while the two-launch
  // passes already move their traffic at about 0.9 of the measured HBM peak.
  if (!p->tensor_core && N1 == N0 && (p->store == ST_C64 || p->store == ST_C32 || p->store == ST_BF16)) {
    const char* fe = std::getenv("VDX_FOURSTEP_FUSED");
    if (fe && std::atoi(fe) == 1) {
      const int rc = plan_fused_fourstep(p, N1, N0, inner, outer, ppA, sb);
      if (rc == VDX_OK) return VDX_OK;
      if (rc != VDX_ERR_UNSUPPORTED) return rc;
    }
  }

  // workspace bytes per chunk; 0 = the whole array in one pair of launches.
  // Chunks small enough to stay in L2 save HBM traffic but each launch is
  // then a single partial wave, and on GB300 the ramp and drain of those
  // waves cost more than the traffic saved (16384^2 complex64, strided axis:
  // 1.39 ms whole-array vs 1.64-2.53 ms for 96-16 MB chunks).
  long long budget = 0;
  if (const char* e = std::getenv("VDX_FOURSTEP_WS_MB")) budget = std::atoll(e) << 20;
  const long long col_bytes = (long long)N * (long long)sb;  // one column (strided) or row (contiguous)
  if (strided) {
    long long C = inner;
    long long O = 1;
    if (budget > 0) {
      const long long fit = std::max(1ll, budget / col_bytes);
      if (fit >= inner) {
        O = std::max(1ll, std::min(outer, fit / inner));
      } else {
        C = std::max<long long>(ppA.M, fit / ppA.M * ppA.M);
        C = std::min(C, inner);
      }
    } else {
      O = outer;
    }
    p->chunk_cols = C;
    p->chunk_outer = O;
    p->ws_bytes = size_t(O) * size_t(C) * size_t(col_bytes);
  } else {
    long long R = outer;
    if (budget > 0) R = std::max(1ll, std::min(outer, budget / col_bytes));
    p->chunk_cols = 1;
    p->chunk_outer = R;
    p->ws_bytes = size_t(R) * size_t(col_bytes);
  }
  p->fourstep = true;
  p->N1 = N1;
  p->N0 = N0;
  p->inner = inner;
  p->outer = outer;
  p->fsA.pp = ppA;
  p->fsB.pp = ppB;
  p->blockA = dim3(ppA.T * ppA.M);
  p->blockB = dim3(ppB.T * ppB.M);
  p->smemA = size_t(std::max(N1 * ppA.M, (N1 + 1) * ppA.M)) * 8;
  p->smemB = size_t(N0) * ppB.M * 8;
  int rc = get_table(p->dev, N1, N1, false, const_cast<void**>(&p->fsA.tw));
  if (rc == VDX_OK) rc = get_table(p->dev, N0, N0, false, const_cast<void**>(&p->fsB.tw));
  if (rc == VDX_OK) rc = get_table(p->dev, N, N, false, const_cast<void**>(&p->fsA.twl));
  if (rc != VDX_OK) return rc;
  p->fsA.scale = 1.f;
  p->fsB.scale = float(p->args.scale);
  cudaError_t e = cudaMalloc(&p->ws, p->ws_bytes);
  if (e != cudaSuccess) {
    p->ws = nullptr;
    return fail(VDX_ERR_NOMEM, std::string("four-step workspace: ") + cudaGetErrorString(e));
  }
  e = cudaMalloc(reinterpret_cast<void**>(&p->d_status), sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e != cudaSuccess) {
    p->d_status = nullptr;
    return cuda_fail(e, "four-step status word");
  }
  if (p->tensor_core) {
    // 128-point tiles of 16 (8-byte) or 32 (4-byte) columns, 128 threads
    if (N1 != 128 || N0 != 128 || ppA.M != ppB.M || (ppA.M != 16 && ppA.M != 32))
      return fail(VDX_ERR_UNSUPPORTED, "tensor-core stages need 128 x 128 tiles of 16 or 32 columns");
    e = tc_dft_operands(p->dev, p->op == OP_C2C_INV, &p->tc_bmat);
    if (e != cudaSuccess) return cuda_fail(e, "tensor-core plan set-up");
    p->blockA = p->blockB = dim3(128);
    p->smemA = p->smemB = tc_pass_smem(ppA.M);
  }
  return VDX_OK;
}

int plan_conv2d_real(const vdx_fft_desc& d, vdx_plan** plan) {
  if (d.ndim != 2 && d.ndim != 3) return fail(VDX_ERR_INVALID, "the fused 2-D convolution takes 2 or 3 dimensions");
  if (d.axis != d.ndim - 2) return fail(VDX_ERR_INVALID, "the fused 2-D convolution convolves along axis ndim-2");
  if (d.io_type != VDX_C64 || d.compute_type != VDX_C64 || d.kernel_type != VDX_C64)
    return fail(VDX_ERR_UNSUPPORTED, "the fused 2-D convolution runs on complex64 only");
  if (d.kernel_op != VDX_KOP_MUL_CONJ && d.kernel_op != VDX_KOP_MUL) return fail(VDX_ERR_INVALID, "unknown kernel_op");
  if (d.normalize != 0 && d.normalize != 1) return fail(VDX_ERR_INVALID, "normalize must be 0 or 1 here");
  if (d.flags != 0) return fail(VDX_ERR_INVALID, "the fused 2-D convolution takes no flags");
  if (!(d.signal_lo < 0 && d.signal_hi < 0) && !(d.signal_lo == 0 && d.signal_hi <= 0))
    return fail(VDX_ERR_UNSUPPORTED, "the fused 2-D convolution takes no signal range");
  const long long Hl = d.shape[d.ndim - 2], Wl = d.shape[d.ndim - 1];
  if (Hl > 65536 || Wl > 65536 || !conv2d_real_supported((int)Hl, (int)Wl))
    return fail(VDX_ERR_UNSUPPORTED, "no fused 2-D convolution kernel for " + std::to_string(Hl) + " x " +
                                         std::to_string(Wl) + " images (available: 512 x 512)");
  const int H = (int)Hl, W = (int)Wl;
  const long long images = d.ndim == 3 ? d.shape[0] : 1;
  auto* p = new vdx_plan();
  p->d = d;
  p->op = OP_CONV2D_REAL;
  p->store = ST_C64;
  p->N = W;
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "cudaGetDevice");
  }
  int clusters = 0;
  e = conv2d_real_max_clusters(H, W, &clusters);
  if (e != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    delete p;
    return fail(VDX_ERR_UNSUPPORTED, "this device cannot schedule the 8-CTA clusters of the fused 2-D convolution");
  }
  p->c2_H = H;
  p->c2_W = W;
  p->c2_images = images;
  Conv2dArgs& c = p->c2;
  c.ker_bs = d.kernel_broadcast ? 0 : (long long)H * (W / 2 + 1);
  c.col_scale = d.normalize ? 1.f / float(H) : 1.f;
  c.row_scale = d.normalize ? 1.f / float(W) : 1.f;
  void* t = nullptr;
  int rc = get_table(p->dev, W / 2, W / 2, false, &t);
  c.tw_row = static_cast<const Cx<float>*>(t);
  if (rc == VDX_OK) rc = get_table(p->dev, W / 2 + 1, W, false, &t);
  c.tw2 = static_cast<const Cx<float>*>(t);
  if (rc == VDX_OK) rc = get_table(p->dev, H, H, false, &t);
  c.tw_col = static_cast<const Cx<float>*>(t);
  if (rc != VDX_OK) {
    delete p;
    return rc;
  }
  p->launch.grid = dim3((unsigned)(images * 8));
  *plan = p;
  return VDX_OK;
}

// Four-step passes of strided axes stage their input tiles with TMA tensor
// copies where fourstep_tma_ok allows it, unless VDX_FOURSTEP_TMA=0.
bool fourstep_tma() {
  static const bool on = [] {
    const char* e = std::getenv("VDX_FOURSTEP_TMA");
    return !(e && e[0] == '0');
  }();
  return on;
}

cudaError_t exec_fourstep(const vdx_plan* p, const void* in, void* out, cudaStream_t s) {
  if (p->fused) {
    FusedLaunch fl = p->fl;
    fl.in = in;
    fl.out = out;
    return launch_fused_fourstep(fl, s);
  }
  const long long N = p->N, N0 = p->N0, N1 = p->N1, inner = p->inner, outer = p->outer;
  const size_t sb = store_bytes(p->store);
  const bool inv = p->op == OP_C2C_INV;
  const char* src = static_cast<const char*>(in);
  char* dst = static_cast<char*>(out);
  Launch la{dim3(1), p->blockA, p->smemA, s}, lb{dim3(1), p->blockB, p->smemB, s};
  const int MA = p->fsA.pp.M, MB = p->fsB.pp.M;
  cudaError_t e = cudaSuccess;
  if (inner > 1) {
    for (long long o0 = 0; o0 < outer; o0 += p->chunk_outer) {
      const long long Oc = std::min(p->chunk_outer, outer - o0);
      for (long long i0 = 0; i0 < inner; i0 += p->chunk_cols) {
        const long long Cc = std::min(p->chunk_cols, inner - i0);
        const size_t off = size_t(o0 * N * inner + i0) * sb;
        FsArgs A = p->fsA;
        A.in = src + off;
        A.out = p->ws;
        A.split = N0;
        A.in_bs1 = N * inner;
        A.in_bs2 = inner;
        A.in_ps = N0 * inner;
        A.out_bs1 = N * Cc;
        A.out_bs2 = Cc;
        A.out_ps = N0 * Cc;
        A.out_cs = 1;
        A.ncols = (int)Cc;
        A.col_tiles = (int)((Cc + MA - 1) / MA);
        A.tw_from_batch = 1;
        A.nbatch = Oc * N0;
        A.status = p->d_status;
        la.grid = dim3((unsigned)(Oc * N0 * A.col_tiles));
        e = p->tensor_core ? launch_fourstep_pass_tc(A, la, p->store, inv, 1, p->tc_bmat, p->d_status)
                           : launch_fourstep_pass(A, la, p->store, inv, 1, fourstep_tma());
        if (e != cudaSuccess) return e;
        FsArgs B = p->fsB;
        B.in = p->ws;
        B.out = dst + off;
        B.split = N1;
        B.in_bs1 = N * Cc;
        B.in_bs2 = N0 * Cc;
        B.in_ps = Cc;
        B.out_bs1 = N * inner;
        B.out_bs2 = inner;
        B.out_ps = N1 * inner;
        B.out_cs = 1;
        B.ncols = (int)Cc;
        B.col_tiles = (int)((Cc + MB - 1) / MB);
        B.nbatch = Oc * N1;
        B.status = p->d_status;
        lb.grid = dim3((unsigned)(Oc * N1 * B.col_tiles));
        e = p->tensor_core ? launch_fourstep_pass_tc(B, lb, p->store, inv, 0, p->tc_bmat, p->d_status)
                           : launch_fourstep_pass(B, lb, p->store, inv, 0, fourstep_tma());
        if (e != cudaSuccess) return e;
      }
    }
    return e;
  }
  for (long long r0 = 0; r0 < outer; r0 += p->chunk_outer) {
    const long long Rr = std::min(p->chunk_outer, outer - r0);
    const size_t off = size_t(r0 * N) * sb;
    FsArgs A = p->fsA;
    A.in = src + off;
    A.out = p->ws;
    A.split = 1;
    A.in_bs1 = N;
    A.in_bs2 = 0;
    A.in_ps = N0;
    A.out_bs1 = N;
    A.out_bs2 = 0;
    A.out_ps = 1;
    A.out_cs = N1;
    A.ncols = (int)N0;
    A.col_tiles = (int)((N0 + MA - 1) / MA);
    A.tw_from_batch = 0;
    A.nbatch = Rr;
    A.status = p->d_status;
    la.grid = dim3((unsigned)(Rr * A.col_tiles));
    e = p->tensor_core ? launch_fourstep_pass_tc(A, la, p->store, inv, 2, p->tc_bmat, p->d_status)
                       : launch_fourstep_pass(A, la, p->store, inv, 2, false);
    if (e != cudaSuccess) return e;
    FsArgs B = p->fsB;
    B.in = p->ws;
    B.out = dst + off;
    B.split = 1;
    B.in_bs1 = N;
    B.in_bs2 = 0;
    B.in_ps = N1;
    B.out_bs1 = N;
    B.out_bs2 = 0;
    B.out_ps = N1;
    B.out_cs = 1;
    B.ncols = (int)N1;
    B.col_tiles = (int)((N1 + MB - 1) / MB);
    B.nbatch = Rr;
    B.status = p->d_status;
    lb.grid = dim3((unsigned)(Rr * B.col_tiles));
    e = p->tensor_core ? launch_fourstep_pass_tc(B, lb, p->store, inv, 0, p->tc_bmat, p->d_status)
                       : launch_fourstep_pass(B, lb, p->store, inv, 0, false);
    if (e != cudaSuccess) return e;
  }
  return e;
}

}  // namespace

namespace {

int create_plan(const vdx_fft_desc* desc, const Tune& tune, vdx_plan** plan);

// Bluestein plan (bluestein.cu): three launches per execution.
int plan_bluestein(const vdx_fft_desc& d, long long inner, long long outer, int N, int st, bool f64,
                   vdx_plan** plan) {
  int M = 1;
  while (M < 2 * N - 1) M <<= 1;
  // fp32: up to 2^24 (longer than one CTA: four-step transforms); fp64: the
  // single-CTA convolution only
  const int mmax = f64 ? 8192 : (1 << 24);
  if (M > mmax)
    return fail(VDX_ERR_UNSUPPORTED, "Bluestein length " + std::to_string(N) + " needs a " + std::to_string(M) +
                                         "-point convolution (limit " + std::to_string(mmax) + ")");
  const bool split = M > 16384;
  auto* p = new vdx_plan();
  p->d = d;
  p->op = d.inverse ? OP_C2C_INV : OP_C2C_FWD;
  p->store = st;
  p->f64 = f64;
  p->N = N;
  p->bluestein = true;
  p->bs_M = M;
  p->inner = inner;
  p->outer = outer;
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "cudaGetDevice");
  }
  const int cx = f64 ? VDX_C128 : VDX_C64;
  vdx_fft_desc dc;
  std::memset(&dc, 0, sizeof(dc));
  dc.ndim = 3;
  dc.shape[0] = outer;
  dc.shape[1] = M;
  dc.shape[2] = inner;
  dc.axis = 1;
  dc.kind = VDX_KIND_CONV;
  dc.normalize = 1;
  dc.io_type = dc.compute_type = dc.kernel_type = cx;
  dc.signal_lo = dc.signal_hi = -1;
  dc.kernel_op = VDX_KOP_MUL_CONJ;
  dc.kernel_broadcast = 1;
  int rc = VDX_OK;
  if (!split) {
    rc = create_plan(&dc, Tune{}, &p->bs_conv);
  } else {
    dc.kind = VDX_KIND_C2C;
    dc.normalize = 0;
    rc = create_plan(&dc, Tune{}, &p->bs_fwd);
    if (rc == VDX_OK) {
      dc.inverse = 1;
      dc.normalize = 1;
      rc = create_plan(&dc, Tune{}, &p->bs_inv);
    }
  }
  if (rc != VDX_OK) {
    delete p;
    return rc;
  }
  const size_t es = f64 ? 16 : 8;
  void* b = nullptr;
  vdx_plan* tmp = nullptr;
  cudaStream_t s = nullptr;
  e = cudaMalloc(&p->bs_w, size_t(N) * es);
  if (e == cudaSuccess) e = cudaMalloc(&b, size_t(M) * es);
  if (e == cudaSuccess) e = cudaMalloc(&p->bs_K, size_t(M) * size_t(inner) * es);
  if (e == cudaSuccess) e = cudaMalloc(&p->bs_ws, size_t(outer) * size_t(M) * size_t(inner) * es);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = launch_chirp_tables(p->bs_w, b, N, M, d.inverse ? 1 : -1, f64, s);
  if (e == cudaSuccess) {
    vdx_fft_desc df;
    std::memset(&df, 0, sizeof(df));
    df.ndim = 2;
    df.shape[0] = 1;
    df.shape[1] = M;
    df.axis = 1;
    df.kind = VDX_KIND_C2C;
    df.io_type = df.compute_type = cx;
    df.signal_lo = df.signal_hi = -1;
    rc = create_plan(&df, Tune{}, &tmp);
    if (rc == VDX_OK) rc = vdx_fft_exec(tmp, b, b, nullptr, s);  // B = FFT_M(b)
    if (rc == VDX_OK) e = launch_conj_slab(p->bs_K, b, M, inner, f64, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  delete tmp;
  if (s) cudaStreamDestroy(s);
  if (b) cudaFree(b);
  if (rc != VDX_OK) {
    delete p;
    return rc;
  }
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "Bluestein plan set-up");
  }
  *plan = p;
  return VDX_OK;
}

int create_plan(const vdx_fft_desc* desc, const Tune& tune, vdx_plan** plan) {
  if (!desc || !plan) return fail(VDX_ERR_INVALID, "desc and plan must be non-NULL");
  *plan = nullptr;
  const vdx_fft_desc& d = *desc;
  if (d.ndim < 1 || d.ndim > 4) return fail(VDX_ERR_INVALID, "ndim must be 1..4");
  for (int i = 0; i < d.ndim; ++i)
    if (d.shape[i] < 1) return fail(VDX_ERR_INVALID, "every dimension must be >= 1");
  if (d.axis < 0 || d.axis >= d.ndim) return fail(VDX_ERR_INVALID, "axis out of range");
  if (d.kind < VDX_KIND_C2C || d.kind > VDX_KIND_CONV2D_REAL) return fail(VDX_ERR_INVALID, "unknown transform kind");
  if (d.kind == VDX_KIND_CONV2D_REAL) return plan_conv2d_real(d, plan);
  const bool real = d.kind == VDX_KIND_R2C || d.kind == VDX_KIND_C2R;
  if (real && d.axis != d.ndim - 1)
    return fail(VDX_ERR_INVALID, "R2C/C2R transforms run on the last (contiguous) axis only");

  const int st = store_of(d.io_type);
  if (st < 0) return fail(VDX_ERR_INVALID, "io_type must be VDX_C64, VDX_C32, VDX_C128 or VDX_BF16X2");
  if (d.compute_type != VDX_C64 && d.compute_type != VDX_C128)
    return fail(VDX_ERR_INVALID, "compute_type must be VDX_C64 or VDX_C128");
  const bool f64 = d.compute_type == VDX_C128;
  if (f64 != (st == ST_C128))
    return fail(VDX_ERR_UNSUPPORTED,
                "supported (io, compute) pairs: complex64/complex64, complex32/complex64, bf16x2/complex64, "
                "complex128/complex128");
  if (d.kind == VDX_KIND_CONV) {
    if (d.kernel_type != d.io_type) return fail(VDX_ERR_UNSUPPORTED, "kernel_type must equal io_type");
    if (d.kernel_op != VDX_KOP_MUL_CONJ && d.kernel_op != VDX_KOP_MUL)
      return fail(VDX_ERR_INVALID, "unknown kernel_op");
    if (d.kernel_op == VDX_KOP_MUL && st != ST_C64)
      return fail(VDX_ERR_UNSUPPORTED, "VDX_KOP_MUL convolutions need complex64 storage");
  }
  if (real && (st == ST_BF16)) return fail(VDX_ERR_UNSUPPORTED, "real transforms support complex64/complex32/complex128");
  if (d.flags & ~(VDX_FFT_FLAG_TENSOR_CORE | VDX_FFT_FLAG_AUTOTUNE | VDX_FFT_FLAG_BLUESTEIN))
    return fail(VDX_ERR_INVALID, "unknown bits in desc.flags");
  if (d.normalize < 0 || d.normalize > 2) return fail(VDX_ERR_INVALID, "normalize must be 0, 1 or 2");

  long long inner = 1, outer = 1;
  for (int i = d.axis + 1; i < d.ndim; ++i) inner *= d.shape[i];
  for (int i = 0; i < d.axis; ++i) outer *= d.shape[i];
  const long long N64 = d.shape[d.axis];
  if (N64 > (1 << 24)) return fail(VDX_ERR_UNSUPPORTED, "axis length above 2^24");
  const int N = (int)N64;

  int lo = 0, hi = N;
  if (!(d.signal_lo == 0 && (d.signal_hi <= 0 || d.signal_hi == N)) && !(d.signal_lo < 0 && d.signal_hi < 0)) {
    if (d.signal_lo < 0 || d.signal_hi <= d.signal_lo || d.signal_hi > N)
      return fail(VDX_ERR_INVALID, "signal range must satisfy 0 <= lo < hi <= N");
    if (d.kind == VDX_KIND_C2R) return fail(VDX_ERR_UNSUPPORTED, "signal range is defined for forward inputs only");
    lo = (int)d.signal_lo;
    hi = (int)d.signal_hi;
  }

  auto* p = new vdx_plan();
  p->d = d;
  p->f64 = f64;
  p->store = st;
  p->N = N;
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) {
    delete p;
    return cuda_fail(e, "cudaGetDevice");
  }

  const bool even_real = real && (N % 2 == 0);
  const int n = even_real ? N / 2 : N;  // complex points per transform
  // 8 or 32 points per thread: complex64 compile-time plans of two radix-32
  // passes for 512 and 1024 complex points (any operation) and of radix-8
  // passes for strided 512-point convolutions, chosen by the autotuner or
  // by VDX_POINTS_PER_THREAD=8|32
  const bool canpts = st == ST_C64 && !f64 && (!real || even_real) && tune.order == 0 && tune.fixed != 0 &&
                      std::getenv("VDX_NO_FIXED") == nullptr;
  const bool is_conv = d.kind == VDX_KIND_CONV;
  int pmaxe = (tune.maxe == 8 || tune.maxe == 32) ? tune.maxe : 16;
  // default for strided complex64 convolutions of 512 or 1024 points: the
  // two-pass radix-32 plan (64 x 512 x 257 along axis 1: 58.0 us against
  // 70.3 us for radix 16 x 16 x 2, each launch alone from a cold L2)
  if (tune.maxe == 0 && is_conv && inner > 1 && canpts && has_fixedpts_c64(n, 32, true, true)) pmaxe = 32;
  if (const char* e = std::getenv("VDX_POINTS_PER_THREAD")) {
    const int v = std::atoi(e);
    if (v == 16) pmaxe = 16;
    if ((v == 8 || v == 32) && canpts && has_fixedpts_c64(n, v, is_conv, inner > 1)) pmaxe = v;
  }
  if (pmaxe != 16 && !(canpts && has_fixedpts_c64(n, pmaxe, is_conv, inner > 1))) {
    delete p;
    return fail(VDX_ERR_UNSUPPORTED,
                "32 points per thread exist for complex64 transforms of 512 or 1024 complex points, 8 for strided "
                "complex64 convolutions of 512 points");
  }
  const int maxe = f64 ? MaxE<double>::value : (pmaxe == 8 ? 8 : MaxE<float>::value);
  std::string why;
  if (!factor_radices(n, maxe, p->radices, why)) {
    delete p;
    if ((d.flags & VDX_FFT_FLAG_BLUESTEIN) && d.kind == VDX_KIND_C2C && lo == 0 && hi == N)
      return plan_bluestein(d, inner, outer, N, st, f64, plan);
    return fail(VDX_ERR_UNSUPPORTED, why + " (VDX_FFT_FLAG_BLUESTEIN plans such lengths)");
  }
  if (tune.order == 1) std::reverse(p->radices.begin(), p->radices.end());
  if (pmaxe == 32) p->radices = {32, n / 32};  // the two-pass compile-time plan

  // threads per transform: enough that every pass fits in MAXE registers
  int T = 1;
  for (int r : p->radices) {
    const int nb = n / r;
    const int per = std::max(1, (pmaxe == 32 ? 32 : maxe) / r);
    T = std::max(T, (nb + per - 1) / per);
  }
  int smem_optin = 0;
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->dev);
  if (smem_optin <= 0) smem_optin = 48 * 1024;

  // long C2C axes run as a four-step pair of launches: always above the
  // single-CTA limit, and from VDX_FOURSTEP_MIN points (default 8192) where
  // one CTA per transform leaves a single CTA per SM
  {
    int fs_min = 8192;
    if (const char* e = std::getenv("VDX_FOURSTEP_MIN")) fs_min = std::atoi(e);
    if (tune.fourstep == 0) fs_min = 0;  // only where one CTA cannot hold the transform
    if (tune.fourstep == 1) fs_min = 1;  // wherever the split exists
    const bool fs_allowed = d.kind == VDX_KIND_C2C && !f64 && lo == 0 && hi == N;
    const bool tcore = (d.flags & VDX_FFT_FLAG_TENSOR_CORE) != 0;
    if (tcore && !(fs_allowed && N == 16384)) {
      delete p;
      return fail(VDX_ERR_UNSUPPORTED, "tensor-core DFT stages need a C2C axis of 16384 points (128 x 128 four-step) "
                                       "with complex64, complex32 or bf16x2 storage and no signal range");
    }
    if (fs_allowed && (tcore || T > 1024 || (fs_min > 0 && N >= fs_min))) {
      p->tensor_core = tcore;
      p->args.scale = norm_scale(d.normalize, N);
      p->op = d.inverse ? OP_C2C_INV : OP_C2C_FWD;
      const int rc = plan_fourstep(p, inner, outer, smem_optin);
      if (rc == VDX_OK) {
        *plan = p;
        return VDX_OK;
      }
      if (T > 1024 || tcore) {
        delete p;
        return rc;
      }
      if (p->ws) cudaFree(p->ws);
      p->ws = nullptr;
      p->fourstep = false;
    }
  }
  if (T > 1024) {
    delete p;
    return fail(VDX_ERR_UNSUPPORTED, "FFT length " + std::to_string(n) + " needs more than 1024 threads per transform");
  }
  const size_t cbytes = f64 ? 16 : 8;
  const bool strided = inner > 1;
  p->strided = strided;
  const bool need_smem = p->radices.size() > 1 || even_real;
  const int npad = n + 1 + ((n + 1) >> 4) + 1;

  int M = 1;
  size_t smem = 0;
  if (strided) {
    int mcols = 8;
    if (const char* e = std::getenv("VDX_STRIDED_COLUMNS")) mcols = std::max(1, std::min(32, std::atoi(e)));
    if (tune.width > 0) mcols = std::min(32, tune.width);
    M = (int)std::min<long long>(mcols, inner);
    M = std::max(1, std::min(M, (pmaxe == 32 ? 256 : 1024) / T));  // 32-point plans: CTAs of <= 256 threads
    while (M > 1 && need_smem && size_t(n) * M * cbytes > size_t(smem_optin)) M /= 2;
    smem = need_smem ? size_t(n) * M * cbytes : 0;
  } else {
    const long long ntrans = outer;
    int cta_threads = 128;
    if (const char* e = std::getenv("VDX_CTA_THREADS")) cta_threads = std::max(32, std::min(1024, std::atoi(e)));
    if (tune.width > 0) cta_threads = std::max(32, std::min(1024, tune.width));
    M = std::max(1, cta_threads / T);
    M = (int)std::min<long long>(M, ntrans);
    M = std::max(1, std::min(M, (pmaxe == 32 ? 256 : 1024) / T));  // 32-point plans: CTAs of <= 256 threads
    while (M > 1 && need_smem && size_t(npad) * M * cbytes > size_t(smem_optin) / 2) M /= 2;
    smem = need_smem ? size_t(npad) * M * cbytes : 0;
  }
  // the fused loss epilogue of C2C launches reduces one float per thread
  // through shared memory, so every C2C plan reserves at least that much
  if (d.kind == VDX_KIND_C2C) smem = std::max(smem, size_t(T) * size_t(M) * sizeof(float));
  if (smem > size_t(smem_optin)) {
    delete p;
    return fail(VDX_ERR_UNSUPPORTED, "FFT length " + std::to_string(n) + " does not fit in shared memory");
  }
  FftArgs& a = p->args;
  std::memset(&a, 0, sizeof(a));
  a.pp.n = n;
  a.pp.npass = (int)p->radices.size();
  for (int i = 0; i < a.pp.npass; ++i) a.pp.radix[i] = p->radices[i];
  a.pp.T = T;
  a.pp.M = M;
  a.pp.npad = npad;
  set_pass_tables(a.pp);
  a.sig_lo = lo;
  a.sig_hi = hi;
  a.nreal = N;

  switch (d.kind) {
    case VDX_KIND_C2C:
      p->op = d.inverse ? OP_C2C_INV : OP_C2C_FWD;
      a.scale = norm_scale(d.normalize, N);
      break;
    case VDX_KIND_CONV:
      p->op = OP_CONV;
      a.scale = norm_scale(d.normalize, N);
      break;
    case VDX_KIND_R2C:
      p->op = even_real ? OP_R2C_EVEN : OP_R2C_ODD;
      a.scale = 1.0;
      break;
    default:
      p->op = even_real ? OP_C2R_EVEN : OP_C2R_ODD;
      a.scale = norm_scale(d.normalize, N);
      break;
  }

  const long long row = real ? (N / 2 + 1) : N;  // complex elements per row of the buffer
  if (strided) {
    a.inner = inner;
    a.outer = outer;
    a.in_bs = a.out_bs = (long long)N * inner;
    a.ker_bs = d.kernel_broadcast ? 0 : (long long)N * inner;
    a.col_tiles = (int)((inner + M - 1) / M);
    const long long blocks = outer * a.col_tiles;
    if (blocks > 0x7fffffffLL) {
      delete p;
      return fail(VDX_ERR_UNSUPPORTED, "too many transforms for one launch");
    }
    p->launch.grid = dim3((unsigned)blocks);
  } else {
    a.ntrans = outer;
    a.inner = 1;
    a.in_bs = a.out_bs = row;
    a.ker_bs = d.kernel_broadcast ? 0 : row;
    const long long blocks = (outer + M - 1) / M;
    if (blocks > 0x7fffffffLL) {
      delete p;
      return fail(VDX_ERR_UNSUPPORTED, "too many transforms for one launch");
    }
    p->launch.grid = dim3((unsigned)blocks);
  }
  p->launch.block = dim3(T * M);
  p->launch.smem = smem;
  p->fixed = st == ST_C64 && !f64 && has_fixed_c64(n) && p->op != OP_R2C_ODD &&
             p->op != OP_C2R_ODD && T == n / 16 && std::getenv("VDX_NO_FIXED") == nullptr && tune.order == 0 &&
             tune.fixed != 0;
  p->fixed_pts = (pmaxe != 16 && T == n / pmaxe && p->op != OP_R2C_ODD && p->op != OP_C2R_ODD &&
                  (pmaxe == 32 || (p->op == OP_CONV && strided)))
                     ? pmaxe
                     : 0;
  if (pmaxe != 16 && !p->fixed_pts) {
    delete p;
    return fail(VDX_ERR_UNSUPPORTED, "no compile-time plan of 8 points per thread for this convolution");
  }

  void* tw = nullptr;
  int rc = get_table(p->dev, n, n, f64, &tw);
  if (rc != VDX_OK) {
    delete p;
    return rc;
  }
  a.tw = tw;
  if (even_real) {
    void* tw2 = nullptr;
    rc = get_table(p->dev, n + 1, 2 * n, f64, &tw2);
    if (rc != VDX_OK) {
      delete p;
      return rc;
    }
    a.tw2 = tw2;
  }
  *plan = p;
  return VDX_OK;
}

}  // namespace

namespace {

// ---------------------------------------------------------------------------
// autotuner: times the candidate plan choices for a (kind, N, stride class,
// batch class, dtype, direction) on scratch buffers and caches the fastest
// ---------------------------------------------------------------------------
using TuneKey = std::array<int, 12>;
std::mutex g_tune_mu;
std::map<TuneKey, Tune> g_tuned;
long long g_tunings = 0;  // candidate searches run (cache misses)

int floor_log2(long long v) {
  int b = 0;
  while (b < 40 && (1ll << (b + 1)) <= v) ++b;
  return b;
}

TuneKey tune_key(int dev, const vdx_fft_desc& d, long long inner, long long outer) {
  const int N = (int)d.shape[d.axis];
  const int ib = inner == 1 ? 0 : 1 + std::min(floor_log2(inner), 20);
  return TuneKey{dev, d.kind, N, ib, std::min(floor_log2(outer), 24), d.io_type, d.compute_type, d.inverse,
                 d.kernel_op, d.kernel_broadcast, d.flags & VDX_FFT_FLAG_TENSOR_CORE,
                 d.signal_lo < 0 && d.signal_hi < 0 ? 0 : 1};
}

// Median of 7 timed executions.  With `flush` (problems larger than a
// quarter of L2) every execution starts from a cold L2, as it does when the
// data streams through a long pipeline; smaller problems are timed warm.
float time_plan(const vdx_plan* p, void* sig, const void* ker, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1,
                void* flush, size_t flush_bytes) {
  for (int w = 0; w < 2; ++w)
    if (vdx_fft_exec(p, sig, sig, ker, s) != VDX_OK) return -1.f;
  constexpr int reps = 7;
  float t[reps];
  for (int r = 0; r < reps; ++r) {
    if (flush) cudaMemsetAsync(flush, r, flush_bytes, s);
    cudaEventRecord(e0, s);
    vdx_fft_exec(p, sig, sig, ker, s);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
    cudaEventElapsedTime(&t[r], e0, e1);
  }
  std::sort(t, t + reps);
  return t[reps / 2];
}

// Autotuned plan creation.  The search runs on a copy of the problem with the
// same axis length and stride class, shrunk to at most VDX_AUTOTUNE_MB
// (default 256) MB of data, on a private stream; it allocates and
// synchronises, so autotuned plans must be created outside stream capture.
int autotune_plan(const vdx_fft_desc& d0, vdx_plan** plan) {
  vdx_fft_desc d = d0;
  d.flags &= ~VDX_FFT_FLAG_AUTOTUNE;
  if (d.kind == VDX_KIND_CONV2D_REAL) return create_plan(&d, Tune{}, plan);
  if (d.ndim < 1 || d.ndim > 4 || d.axis < 0 || d.axis >= d.ndim) return create_plan(&d, Tune{}, plan);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  long long inner = 1, outer = 1;
  for (int i = d.axis + 1; i < d.ndim; ++i) inner *= d.shape[i];
  for (int i = 0; i < d.axis; ++i) outer *= d.shape[i];
  const TuneKey key = tune_key(dev, d, inner, outer);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      const int rc = create_plan(&d, it->second, plan);
      if (rc == VDX_OK) {
        (*plan)->tuned = true;
        (*plan)->tune = it->second;
      }
      return rc;
    }
  }
  // validate the request (and keep the default choice) before searching
  vdx_plan* base = nullptr;
  int rc = create_plan(&d, Tune{}, &base);
  if (rc != VDX_OK) return rc;

  const long long N = d.shape[d.axis];
  const bool real = d.kind == VDX_KIND_R2C || d.kind == VDX_KIND_C2R;
  const long long row = real ? N / 2 + 1 : N;
  const size_t es = store_bytes(store_of(d.io_type));
  long long cap = 256ll << 20;
  if (const char* ev = std::getenv("VDX_AUTOTUNE_MB")) cap = std::max(1ll, (long long)std::atoll(ev)) << 20;
  long long inner_t = inner;
  if (inner > 1 && (long long)(row * inner * es) > cap) {
    inner_t = std::max(1ll, cap / (long long)(row * es));
    if (inner_t >= 32) inner_t = inner_t / 32 * 32;
  }
  const long long outer_t = std::min(outer, std::max(1ll, cap / (long long)(row * inner_t * es)));
  vdx_fft_desc dt = d;
  if (inner_t > 1) {
    dt.ndim = 3;
    dt.shape[0] = outer_t;
    dt.shape[1] = N;
    dt.shape[2] = inner_t;
  } else {
    dt.ndim = 2;
    dt.shape[0] = outer_t;
    dt.shape[1] = N;
  }
  dt.axis = 1;
  const size_t sig_bytes = size_t(outer_t) * size_t(row) * size_t(inner_t) * es;
  const size_t ker_bytes = d.kind == VDX_KIND_CONV ? (d.kernel_broadcast ? size_t(row) * size_t(inner_t) * es : sig_bytes)
                                                    : 0;
  void* sig = nullptr;
  void* ker = nullptr;
  void* flush = nullptr;
  int l2 = 0;
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
  const size_t flush_bytes = size_t(std::max(l2, 1 << 20)) * 2;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaMalloc(&sig, sig_bytes);
  if (e == cudaSuccess && ker_bytes) e = cudaMalloc(&ker, ker_bytes);
  if (e == cudaSuccess) e = cudaMemset(sig, 0, sig_bytes);
  if (e == cudaSuccess && ker_bytes) e = cudaMemset(ker, 0, ker_bytes);
  if (e == cudaSuccess && 2 * sig_bytes + ker_bytes > size_t(l2) / 4) e = cudaMalloc(&flush, flush_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  Tune best{};
  float best_ms = -1.f;
  int tried = 0;
  if (e == cudaSuccess) {
    std::vector<int> widths = inner_t > 1 ? std::vector<int>{2, 4, 8, 16, 32}
                                          : std::vector<int>{64, 128, 256, 512, 1024};
    const bool fs_opt = d.kind == VDX_KIND_C2C && d.compute_type == VDX_C64 && N >= 2048 &&
                        (d.signal_lo < 0 && d.signal_hi < 0) && !(d.flags & VDX_FFT_FLAG_TENSOR_CORE);
    std::vector<Tune> cands{Tune{}};  // the default choice first: others must beat it by 3 %
    for (int fsv : fs_opt ? std::vector<int>{0, 1} : std::vector<int>{-1})
      for (int order : {0, 1})
        for (int fixed : {-1, 0})
          for (int w : widths) {
            if (order == 1 && fixed == -1) continue;  // compile-time kernels exist for one order only
            Tune t;
            t.width = w;
            t.order = order;
            t.fixed = fixed;
            t.fourstep = fsv;
            cands.push_back(t);
          }
    // the 8-, 16- and 32-points-per-thread plans (16 differs from the
    // default only where the default is 32: strided convolutions of 512 or
    // 1024 points; create_plan refuses the combinations that have none)
    if (d.io_type == VDX_C64 && d.compute_type == VDX_C64)
      for (int pts : {8, 16, 32})
        for (int w : widths) {
          Tune t;
          t.width = w;
          t.maxe = pts;
          cands.push_back(t);
        }
    std::vector<std::string> seen;
    for (const Tune& t : cands) {
      vdx_plan* c = nullptr;
      if (create_plan(&dt, t, &c) != VDX_OK) continue;
      char sig_desc[1024];
      vdx_fft_plan_describe(c, sig_desc, sizeof(sig_desc));
      if (std::find(seen.begin(), seen.end(), std::string(sig_desc)) != seen.end()) {
        delete c;
        continue;
      }
      seen.emplace_back(sig_desc);
      const float ms = time_plan(c, sig, ker, s, e0, e1, flush, flush_bytes);
      ++tried;
      delete c;
      if (ms > 0.f && (best_ms < 0.f || ms < 0.97f * best_ms)) {
        best_ms = ms;
        best = t;
      }
    }
  }
  if (e1) cudaEventDestroy(e1);
  if (e0) cudaEventDestroy(e0);
  if (s) cudaStreamDestroy(s);
  if (ker) cudaFree(ker);
  if (sig) cudaFree(sig);
  if (flush) cudaFree(flush);
  cudaGetLastError();
  if (best_ms < 0.f) {  // nothing could be timed: keep the default choice
    *plan = base;
    return VDX_OK;
  }
  delete base;
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[key] = best;
    ++g_tunings;
  }
  rc = create_plan(&d, best, plan);
  if (rc == VDX_OK) {
    (*plan)->tuned = true;
    (*plan)->tune = best;
    (*plan)->tuned_ms = best_ms;
    (*plan)->tuned_candidates = tried;
  }
  return rc;
}

}  // namespace

namespace vdx {

bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("VDX_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

int map_plan_geometry(const vdx_fft_desc& d, MapGeometry* g) {
  Tune t;
  t.fourstep = 0;  // one CTA per transform wherever it fits
  t.fixed = 0;
  vdx_plan* p = nullptr;
  const int rc = create_plan(&d, t, &p);
  if (rc != VDX_OK) return rc;
  if (p->fourstep || p->bluestein || p->radices.empty()) {
    delete p;
    return fail(VDX_ERR_UNSUPPORTED, "map hooks run on axes of at most 16384 points whose transform fits one CTA");
  }
  g->args = p->args;
  g->launch = p->launch;
  g->radices = p->radices;
  g->strided = p->strided;
  g->f64 = p->f64;
  g->N = p->N;
  g->dev = p->dev;
  delete p;
  return VDX_OK;
}

}  // namespace vdx

extern "C" {

int vdx_version(void) { return 100; }

int vdx_last_error(char* buf, size_t n) {
  if (!buf || n == 0) return VDX_ERR_INVALID;
  std::snprintf(buf, n, "%s", g_last_error.c_str());
  return VDX_OK;
}

int vdx_device_count(int* count) {
  if (!count) return fail(VDX_ERR_INVALID, "count is NULL");
  cudaError_t e = cudaGetDeviceCount(count);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  return VDX_OK;
}

int vdx_fft_plan_create(const vdx_fft_desc* desc, vdx_plan** plan) {
  if (!desc || !plan) return fail(VDX_ERR_INVALID, "desc and plan must be non-NULL");
  *plan = nullptr;
  if (desc->flags & VDX_FFT_FLAG_AUTOTUNE) return autotune_plan(*desc, plan);
  return create_plan(desc, Tune{}, plan);
}

int vdx_autotune_entries(int64_t* entries, int64_t* searches) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (entries) *entries = (int64_t)g_tuned.size();
  if (searches) *searches = (int64_t)g_tunings;
  return VDX_OK;
}

int vdx_autotune_save(const char* path) {
  if (!path) return fail(VDX_ERR_INVALID, "path is NULL");
  std::lock_guard<std::mutex> lock(g_tune_mu);
  FILE* f = std::fopen(path, "w");
  if (!f) return fail(VDX_ERR_INVALID, std::string("cannot write ") + path);
  std::fprintf(f, "# libvdx autotune cache: 12 key fields, then width order fixed fourstep points-per-thread\n");
  for (const auto& kv : g_tuned) {
    for (int v : kv.first) std::fprintf(f, "%d ", v);
    std::fprintf(f, "%d %d %d %d %d\n", kv.second.width, kv.second.order, kv.second.fixed, kv.second.fourstep,
                 kv.second.maxe);
  }
  std::fclose(f);
  return VDX_OK;
}

int vdx_autotune_load(const char* path) {
  if (!path) return fail(VDX_ERR_INVALID, "path is NULL");
  FILE* f = std::fopen(path, "r");
  if (!f) return fail(VDX_ERR_INVALID, std::string("cannot read ") + path);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  char line[512];
  int loaded = 0;
  while (std::fgets(line, sizeof(line), f)) {
    if (line[0] == '#') continue;
    TuneKey k{};
    Tune t;
    int v[17];
    v[16] = 16;  // caches written before the points-per-thread field hold 16
    int cnt = std::sscanf(line, "%d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d", &v[0], &v[1], &v[2], &v[3],
                          &v[4], &v[5], &v[6], &v[7], &v[8], &v[9], &v[10], &v[11], &v[12], &v[13], &v[14], &v[15],
                          &v[16]);
    if (cnt != 16 && cnt != 17) continue;
    for (int i = 0; i < 12; ++i) k[i] = v[i];
    t.width = v[12];
    t.order = v[13];
    t.fixed = v[14];
    t.fourstep = v[15];
    t.maxe = (v[16] == 8 || v[16] == 16 || v[16] == 32) ? v[16] : 0;
    g_tuned[k] = t;
    ++loaded;
  }
  std::fclose(f);
  return loaded >= 0 ? VDX_OK : VDX_ERR_INVALID;
}

int vdx_fft_plan_destroy(vdx_plan* plan) {
  delete plan;
  return VDX_OK;
}

int vdx_fft_plan_describe(const vdx_plan* p, char* buf, size_t n) {
  if (!p || !buf || n == 0) return fail(VDX_ERR_INVALID, "plan and buf must be non-NULL");
  std::string r;
  for (size_t i = 0; i < p->radices.size(); ++i) r += (i ? "x" : "") + std::to_string(p->radices[i]);
  if (p->bluestein) {
    std::snprintf(buf, n,
                  "{\"op\": \"%s\", \"N\": %d, \"bluestein\": %d, \"strided\": %s, \"autotuned\": false}",
                  p->op == OP_C2C_INV ? "c2c_inv" : "c2c_fwd", p->N, p->bs_M, p->inner > 1 ? "true" : "false");
    return VDX_OK;
  }
  if (p->fourstep) {
    std::snprintf(buf, n,
                  "{\"op\": \"%s\", \"N\": %d, \"fourstep\": [%d, %d], \"strided\": %s, "
                  "\"columns_per_tile\": [%d, %d], \"chunk_columns\": %lld, \"chunk_outer\": %lld, "
                  "\"workspace_bytes\": %zu, \"block\": [%u, %u], \"smem\": [%zu, %zu], \"tensor_core\": %s, "
                  "\"autotuned\": %s, \"tune_candidates\": %d, \"fused\": %s, \"ring_slots\": %d, "
                  "\"grid\": %u}",
                  p->op == OP_C2C_INV ? "c2c_inv" : "c2c_fwd", p->N, p->N1, p->N0, p->inner > 1 ? "true" : "false",
                  p->fsA.pp.M, p->fsB.pp.M, p->chunk_cols, p->chunk_outer, p->ws_bytes, p->blockA.x, p->blockB.x,
                  p->smemA, p->smemB, p->tensor_core ? "true" : "false", p->tuned ? "true" : "false",
                  p->tuned_candidates, p->fused ? "true" : "false", p->fused ? p->fl.R : 0, p->fused ? p->fl.grid : 0);
    return VDX_OK;
  }
  if (p->op == OP_CONV2D_REAL) {
    std::snprintf(buf, n,
                  "{\"op\": \"conv2d_real\", \"H\": %d, \"W\": %d, \"images\": %lld, \"cluster\": 8, "
                  "\"kernel_broadcast\": %s}",
                  p->c2_H, p->c2_W, p->c2_images, p->c2.ker_bs ? "false" : "true");
    return VDX_OK;
  }
  static const char* ops[] = {"c2c_fwd", "c2c_inv", "conv", "r2c_even", "c2r_even", "r2c_odd", "c2r_odd"};
  std::snprintf(buf, n,
                "{\"op\": \"%s\", \"N\": %d, \"n\": %d, \"radices\": \"%s\", \"threads_per_transform\": %d, "
                "\"transforms_per_cta\": %d, \"strided\": %s, \"fixed\": %s, \"grid\": %u, \"block\": %u, "
                "\"smem\": %zu, \"autotuned\": %s, \"tune\": [%d, %d, %d, %d, %d], \"tune_candidates\": %d}",
                ops[p->op], p->N, p->args.pp.n, r.c_str(), p->args.pp.T, p->args.pp.M, p->strided ? "true" : "false",
                (p->fixed || p->fixed_pts) ? "true" : "false", p->launch.grid.x, p->launch.block.x, p->launch.smem,
                p->tuned ? "true" : "false", p->tune.width, p->tune.order, p->tune.fixed, p->tune.fourstep,
                p->tune.maxe, p->tuned_candidates);
  return VDX_OK;
}

namespace {

int exec_plan(const vdx_plan* p, const void* in, void* out, const void* kernel, const vdx_exec_ops* ops,
              void* stream) {
  if (!p) return fail(VDX_ERR_INVALID, "plan is NULL");
  if (!in || !out) return fail(VDX_ERR_INVALID, "in and out must be non-NULL device pointers");
  if (p->op == OP_CONV2D_REAL) {
    if (in != out) return fail(VDX_ERR_INVALID, "the fused 2-D convolution runs in place (in == out)");
    if (!kernel) return fail(VDX_ERR_INVALID, "convolution needs a kernel spectrum");
    if (ops && (ops->in_weight || ops->spec_out || ops->loss_weight))
      return fail(VDX_ERR_UNSUPPORTED, "fused operations are not available on the fused 2-D convolution");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev != p->dev) return fail(VDX_ERR_INVALID, "plan was created on another device");
    Conv2dArgs c = p->c2;
    c.data = static_cast<Cx<float>*>(out);
    c.ker = static_cast<const Cx<float>*>(kernel);
    e = launch_conv2d_real(c, p->c2_H, p->c2_W, p->c2_images, p->d.kernel_op, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "fused 2-D convolution launch");
    return VDX_OK;
  }
  if (p->op == OP_CONV && !kernel) return fail(VDX_ERR_INVALID, "convolution needs a kernel spectrum");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != p->dev) return fail(VDX_ERR_INVALID, "plan was created on another device");
  if (p->bluestein) {
    if (ops && (ops->in_weight || ops->spec_out || ops->loss_weight))
      return fail(VDX_ERR_UNSUPPORTED, "fused operations are not available on Bluestein plans");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    e = launch_bluestein_io(true, p->store, in, p->bs_ws, p->bs_w, p->outer, p->N, p->bs_M, p->inner, 1.0, s);
    if (e != cudaSuccess) return cuda_fail(e, "Bluestein chirp-in launch");
    if (p->bs_conv) {
      const int rc = exec_plan(p->bs_conv, p->bs_ws, p->bs_ws, p->bs_K, nullptr, stream);
      if (rc != VDX_OK) return rc;
    } else {
      int rc = exec_plan(p->bs_fwd, p->bs_ws, p->bs_ws, nullptr, nullptr, stream);
      if (rc != VDX_OK) return rc;
      e = launch_bluestein_mul(p->bs_ws, p->bs_K, p->outer, p->bs_M, p->inner, p->f64, s);
      if (e != cudaSuccess) return cuda_fail(e, "Bluestein spectrum product launch");
      rc = exec_plan(p->bs_inv, p->bs_ws, p->bs_ws, nullptr, nullptr, stream);
      if (rc != VDX_OK) return rc;
    }
    e = launch_bluestein_io(false, p->store, out, p->bs_ws, p->bs_w, p->outer, p->N, p->bs_M, p->inner,
                            norm_scale(p->d.normalize, p->N), s);
    if (e != cudaSuccess) return cuda_fail(e, "Bluestein chirp-out launch");
    return VDX_OK;
  }
  if (p->fourstep) {
    if (ops && (ops->in_weight || ops->spec_out || ops->loss_weight))
      return fail(VDX_ERR_UNSUPPORTED, "fused operations are not available on four-step (long-axis) plans");
    e = exec_fourstep(p, in, out, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "four-step FFT launch");
    return VDX_OK;
  }
  FftArgs a = p->args;
  a.in = in;
  a.out = out;
  a.ker = kernel;
  int variant = 0;
  if (ops) {
    const int nops = (ops->in_weight != nullptr) + (ops->spec_out != nullptr) + (ops->loss_weight != nullptr);
    if (nops > 1) return fail(VDX_ERR_INVALID, "at most one fused operation per launch");
    if (nops == 1 && p->store != ST_C64) return fail(VDX_ERR_UNSUPPORTED, "fused operations need complex64 plans");
    const bool c2c = p->op == OP_C2C_FWD || p->op == OP_C2C_INV;
    if (ops->in_weight) {
      if (!c2c) return fail(VDX_ERR_INVALID, "in_weight applies to C2C plans");
      variant = 1;
      a.in_weight = ops->in_weight;
      a.in_weight_scale_ptr = ops->in_weight_scale_ptr;
      a.in_weight_scale = ops->in_weight_scale;
    } else if (ops->loss_weight) {
      if (!c2c) return fail(VDX_ERR_INVALID, "loss_weight applies to C2C plans");
      if (!ops->loss_partials) return fail(VDX_ERR_INVALID, "loss_weight needs loss_partials");
      variant = 2;
      a.loss_weight = ops->loss_weight;
      a.loss_partials = ops->loss_partials;
    } else if (ops->spec_out) {
      if (p->op != OP_CONV) return fail(VDX_ERR_INVALID, "spec_out applies to convolution plans");
      variant = ops->spec_aux ? 2 : 1;
      a.spec_out = ops->spec_out;
      a.spec_aux = ops->spec_aux;
      a.spec_scale = ops->spec_scale;
    }
  }
  Launch l = p->launch;
  l.stream = reinterpret_cast<cudaStream_t>(stream);
  if (p->fixed_pts) {
    e = launch_fixedpts_c64_any(p->args.pp.n, p->fixed_pts, a, l, p->op, p->strided, p->d.kernel_op, variant);
    if (e != cudaSuccess) return cuda_fail(e, "FFT launch");
    return VDX_OK;
  }
  if (p->fixed) {
    e = launch_fixed_c64_any(p->args.pp.n, a, l, p->op, p->strided, p->d.kernel_op, variant);
    if (e != cudaSuccess) return cuda_fail(e, "FFT launch");
    return VDX_OK;
  }
  switch (p->store) {
    case ST_C64: e = launch_fft<Cx<float>, float>(a, l, p->op, p->strided, p->d.kernel_op, variant); break;
    case ST_C32: e = launch_fft<c32s, float>(a, l, p->op, p->strided, p->d.kernel_op, variant); break;
    case ST_BF16: e = launch_fft<bf16c, float>(a, l, p->op, p->strided, p->d.kernel_op, variant); break;
    case ST_C128: e = launch_fft<Cx<double>, double>(a, l, p->op, p->strided, p->d.kernel_op, variant); break;
    default: return fail(VDX_ERR_INVALID, "bad plan storage type");
  }
  if (e != cudaSuccess) return cuda_fail(e, "FFT launch");
  return VDX_OK;
}

}  // namespace

int vdx_fft_exec(const vdx_plan* p, const void* in, void* out, const void* kernel, void* stream) {
  return exec_plan(p, in, out, kernel, nullptr, stream);
}

int vdx_fft_exec_ops(const vdx_plan* p, const void* in, void* out, const void* kernel, const vdx_exec_ops* ops,
                     void* stream) {
  return exec_plan(p, in, out, kernel, ops, stream);
}

int vdx_conv_exec_multi(const vdx_plan* p, const void* in, void* out, const void* kernel, int kernel_num,
                        int64_t kernel_stride, int64_t out_stride, void* stream) {
  if (!p) return fail(VDX_ERR_INVALID, "plan is NULL");
  if (!in || !out || !kernel) return fail(VDX_ERR_INVALID, "in, out and kernel must be non-NULL device pointers");
  if (kernel_num < 1 || kernel_stride < 0 || out_stride < 0)
    return fail(VDX_ERR_INVALID, "kernel_num must be >= 1 and the strides >= 0");
  if (p->op != OP_CONV) return fail(VDX_ERR_INVALID, "vdx_conv_exec_multi needs a convolution plan");
  if (p->fourstep || p->bluestein || p->fixed_pts == 8 || (p->store != ST_C64 && p->store != ST_C128))
    return fail(VDX_ERR_UNSUPPORTED, "no fused multi-kernel kernel for this plan (run one convolution per kernel)");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != p->dev) return fail(VDX_ERR_INVALID, "plan was created on another device");
  FftArgs a = p->args;
  a.in = in;
  a.out = out;
  a.ker = kernel;
  Launch l = p->launch;
  l.stream = reinterpret_cast<cudaStream_t>(stream);
  // the exchange region, then MAXE complex slots per thread for the spectrum
  const size_t cbytes = p->f64 ? 16 : 8;
  const int pts = p->fixed_pts ? p->fixed_pts : conv_multi_points(p->f64);
  l.smem = ((l.smem + 15) & ~size_t(15)) + size_t(pts) * l.block.x * cbytes;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (l.smem > size_t(optin))
    return fail(VDX_ERR_UNSUPPORTED, "the multi-kernel spectrum does not fit in shared memory (run one convolution "
                                     "per kernel)");
  if (p->fixed || p->fixed_pts) {
    const int n = p->args.pp.n;
    e = n <= 512 ? launch_fixed_conv_multi_small(n, pts, p->strided, a, l, p->d.kernel_op, kernel_num,
                                                 (long long)kernel_stride, (long long)out_stride)
                 : launch_fixed_conv_multi_large(n, pts, p->strided, a, l, p->d.kernel_op, kernel_num,
                                                 (long long)kernel_stride, (long long)out_stride);
  } else {
    e = launch_conv_multi(p->store, p->strided, a, l, p->d.kernel_op, kernel_num, (long long)kernel_stride,
                          (long long)out_stride);
  }
  if (e != cudaSuccess) return cuda_fail(e, "multi-kernel convolution launch");
  return VDX_OK;
}

int vdx_fft_plan_ctas(const vdx_plan* p, int64_t* ctas) {
  if (!p || !ctas) return fail(VDX_ERR_INVALID, "plan and ctas must be non-NULL");
  *ctas = (int64_t)p->launch.grid.x;
  return VDX_OK;
}

int vdx_fft_plan_status(const vdx_plan* p, int* status) {
  if (!p || !status) return fail(VDX_ERR_INVALID, "plan and status must be non-NULL");
  *status = 0;
  if (!p->d_status) return VDX_OK;
  cudaError_t e = cudaMemcpy(status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "plan status read");
  return VDX_OK;
}

int vdx_reduce_partial_count(int64_t n, int64_t* partial_count) {
  if (!partial_count || n < 1) return fail(VDX_ERR_INVALID, "n must be >= 1 and partial_count non-NULL");
  long long parts = (n + 4095) / 4096;
  if (parts > 1024) parts = 1024;
  *partial_count = parts;
  return VDX_OK;
}

int vdx_reduce(int op, int map, int in_type, const void* in, int64_t n, int64_t batch, void* out, void* workspace,
               void* stream) {
  int rc = check_reduce_args(op, map, in_type, in, n, batch, out);
  if (rc != VDX_OK) return rc;
  if (!workspace) return fail(VDX_ERR_INVALID, "workspace must be a non-NULL device pointer");
  int64_t parts = 0;
  vdx_reduce_partial_count(n, &parts);
  cudaError_t e = launch_reduce(op, map, in_type, in, n, batch, out, workspace, (int)parts,
                                reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "reduce launch");
  return VDX_OK;
}

}  // extern "C"
