// Bluestein (chirp-z) transforms for axis lengths with prime factors above 13,
// which the reference's planner rejects (vkdispatch/fft/prime_utils.py:6-10).
//
// With nk = (n^2 + k^2 - (k - n)^2) / 2 and w[n] = exp(s i pi n^2 / N)
// (s = -1 forward, +1 inverse):
//   X[k] = w[k] * sum_n (x[n] w[n]) conj(w[k - n]),
// a linear convolution, computed as a circular one of length M >= 2N - 1:
//   a[m] = x[m] w[m] (m < N), 0 otherwise;
//   b[m] = conj(w[m]) for m < N, b[M - m] = conj(w[m]) for 0 < m < N, 0 otherwise;
//   X[k] = w[k] * IFFT_M(FFT_M(a) * FFT_M(b))[k].
// The middle step is one fused convolution launch (k_conv multiplies by the
// conjugate of its kernel, so the kernel passed is conj(FFT_M(b))) while M
// fits one CTA per transform; longer M run it as a four-step forward
// transform, a spectrum product (k_bs_mul) and a four-step inverse.  The chirp
// is built in FP64 from the exact integer n^2 mod 2N, so no angle grows with n.
#include <cuda_runtime.h>

#include <algorithm>

#include "fft_kernels.cuh"
#include "vdx_internal.h"

namespace vdx {

namespace {

// w[n] = exp(s i pi (n^2 mod 2N) / N), n < N
template <class Re>
__global__ void k_chirp(Cx<Re>* w, int N, int sign) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const long long r = ((long long)n * n) % (2ll * N);
  double sv, cv;
  sincospi(double(sign) * double(r) / double(N), &sv, &cv);
  w[n] = mk<Re>(Re(cv), Re(sv));
}

// b[m] of length M (see the file comment), from the chirp w
template <class Re>
__global__ void k_chirp_b(Cx<Re>* b, const Cx<Re>* w, int N, int M) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  Cx<Re> v = mk<Re>(Re(0), Re(0));
  if (m < N) v = conj(w[m]);
  else if (m > M - N) v = conj(w[M - m]);
  b[m] = v;
}

// kernel slab K[m][i] = conj(B[m]) for every column i of a strided layout
template <class Re>
__global__ void k_conj_slab(Cx<Re>* K, const Cx<Re>* B, int M, long long inner) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)M * inner) return;
  K[e] = conj(B[e / inner]);
}

// ws (outer, M, inner) <- x (outer, N, inner) * w, zero-padded
template <class S, class Re>
__global__ void k_bs_in(const S* __restrict__ x, Cx<Re>* __restrict__ ws, const Cx<Re>* __restrict__ w,
                        long long outer, int N, int M, long long inner) {
  const long long total = outer * M * inner;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % inner;
    const long long om = e / inner;
    const int m = int(om % M);
    const long long o = om / M;
    Cx<Re> v = mk<Re>(Re(0), Re(0));
    if (m < N) v = cmul(Conv<S, Re>::ld(x + (o * N + m) * inner + i), ldg(w + m));
    ws[e] = v;
  }
}

// y (outer, N, inner) <- ws[:, :N, :] * w * scale
template <class S, class Re>
__global__ void k_bs_out(const Cx<Re>* __restrict__ ws, S* __restrict__ y, const Cx<Re>* __restrict__ w,
                         long long outer, int N, int M, long long inner, Re sc) {
  const long long total = outer * N * inner;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long i = e % inner;
    const long long ok = e / inner;
    const int k = int(ok % N);
    const long long o = ok / N;
    const Cx<Re> v = ws[(o * M + k) * inner + i];
    Conv<S, Re>::st(y + e, scale(cmul(v, ldg(w + k)), sc));
  }
}

// ws (outer, M, inner) *= conj(K[m][i]): the spectrum product of the long
// (four-step) form, where the convolution is two separate transforms
template <class Re>
__global__ void k_bs_mul(Cx<Re>* __restrict__ ws, const Cx<Re>* __restrict__ K, long long outer, long long slab) {
  const long long total = outer * slab;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x)
    ws[e] = cmulc(ws[e], K[e % slab]);
}

unsigned grid_for(long long total, int threads) {
  long long g = (total + threads - 1) / threads;
  return (unsigned)std::min<long long>(std::max<long long>(g, 1), 152 * 32);
}

template <class S, class Re>
cudaError_t launch_io(bool in_phase, const void* x, void* ws, const void* w, long long outer, int N, int M,
                      long long inner, double scale, cudaStream_t s) {
  constexpr int TH = 256;
  if (in_phase) {
    k_bs_in<S, Re><<<grid_for(outer * M * inner, TH), TH, 0, s>>>(
        static_cast<const S*>(x), static_cast<Cx<Re>*>(ws), static_cast<const Cx<Re>*>(w), outer, N, M, inner);
  } else {
    k_bs_out<S, Re><<<grid_for(outer * N * inner, TH), TH, 0, s>>>(
        static_cast<const Cx<Re>*>(ws), static_cast<S*>(const_cast<void*>(x)), static_cast<const Cx<Re>*>(w), outer,
        N, M, inner, Re(scale));
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_chirp_tables(void* w, void* b, int N, int M, int sign, bool f64, cudaStream_t s) {
  constexpr int TH = 256;
  if (f64) {
    k_chirp<double><<<(N + TH - 1) / TH, TH, 0, s>>>(static_cast<Cx<double>*>(w), N, sign);
    k_chirp_b<double><<<(M + TH - 1) / TH, TH, 0, s>>>(static_cast<Cx<double>*>(b), static_cast<Cx<double>*>(w), N, M);
  } else {
    k_chirp<float><<<(N + TH - 1) / TH, TH, 0, s>>>(static_cast<Cx<float>*>(w), N, sign);
    k_chirp_b<float><<<(M + TH - 1) / TH, TH, 0, s>>>(static_cast<Cx<float>*>(b), static_cast<Cx<float>*>(w), N, M);
  }
  return cudaGetLastError();
}

cudaError_t launch_conj_slab(void* K, const void* B, int M, long long inner, bool f64, cudaStream_t s) {
  constexpr int TH = 256;
  const long long total = (long long)M * inner;
  const unsigned g = (unsigned)((total + TH - 1) / TH);
  if (f64) k_conj_slab<double><<<g, TH, 0, s>>>(static_cast<Cx<double>*>(K), static_cast<const Cx<double>*>(B), M, inner);
  else k_conj_slab<float><<<g, TH, 0, s>>>(static_cast<Cx<float>*>(K), static_cast<const Cx<float>*>(B), M, inner);
  return cudaGetLastError();
}

cudaError_t launch_bluestein_mul(void* ws, const void* K, long long outer, int M, long long inner, bool f64,
                                 cudaStream_t s) {
  constexpr int TH = 256;
  const long long slab = (long long)M * inner;
  const unsigned g = grid_for(outer * slab, TH);
  if (f64) k_bs_mul<double><<<g, TH, 0, s>>>(static_cast<Cx<double>*>(ws), static_cast<const Cx<double>*>(K), outer, slab);
  else k_bs_mul<float><<<g, TH, 0, s>>>(static_cast<Cx<float>*>(ws), static_cast<const Cx<float>*>(K), outer, slab);
  return cudaGetLastError();
}

cudaError_t launch_bluestein_io(bool in_phase, int store, const void* x, void* ws, const void* w, long long outer,
                                int N, int M, long long inner, double scale, cudaStream_t s) {
  switch (store) {
    case ST_C64: return launch_io<Cx<float>, float>(in_phase, x, ws, w, outer, N, M, inner, scale, s);
    case ST_C32: return launch_io<c32s, float>(in_phase, x, ws, w, outer, N, M, inner, scale, s);
    case ST_BF16: return launch_io<bf16c, float>(in_phase, x, ws, w, outer, N, M, inner, scale, s);
    case ST_C128: return launch_io<Cx<double>, double>(in_phase, x, ws, w, outer, N, M, inner, scale, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace vdx
