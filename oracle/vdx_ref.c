/*
 * CPU restatement of the reference's (sharhar/vkdispatch) FFT, FFT
 * convolution and reduction algorithms -- TEST INFRASTRUCTURE ONLY: used by
 * tests/ as a second oracle beside FP64 numpy.fft, and by bench.py as the
 * timed CPU baseline.  Never linked into libvdx.
 *
 * Follows, step for step, in fp32:
 *   - the plan builder: vkdispatch/fft/prime_utils.py:12-45 (prime_factors,
 *     group_primes), vkdispatch/fft/stages.py:67-198 (FFTRegisterStageConfig,
 *     input/output formats), vkdispatch/fft/config.py:12-190 (plan
 *     candidates, transfer counting, select_fft_plan_candidate), with the
 *     CUDA backend's GB300 limits (1024 threads per block);
 *   - stage execution: vkdispatch/fft/context.py:152-179 (stages over
 *     invocations), vkdispatch/fft/memory_iterators.py:21-99 (read offsets
 *     o + i*N/L, write offsets (o-k)*L + k + j*S),
 *     vkdispatch/fft/cooley_tukey.py:11-180 (runtime twiddle
 *     fp32(angle*i/N)*fp32(k) through cos/sin, constant twiddles with
 *     right-angle shortcuts, radix-P DFT accumulation order, composite
 *     permutation); complex products as in
 *     vkdispatch/codegen/functions/complex_numbers.py:41-60 (fma form);
 *     1/N normalisation by division, vkdispatch/fft/registers.py:55-58;
 *   - real I/O: vkdispatch/fft/global_memory_iterators.py:17-49, 71-92,
 *     197-229 (packed real rows, bins 0..N/2, Hermitian reconstruction);
 *   - convolution: vkdispatch/fft/shader_factories.py:107-195 (forward FFT,
 *     multiply by conj(kernel) at the same index, inverse FFT, 1/N);
 *   - reductions: vkdispatch/reduce/stage.py:31-145 and
 *     reduce_function.py:73-162 (grid-stride order over 1024-thread groups,
 *     shared-memory tree, xor-butterfly subgroup op, second stage).
 * The only deliberate difference: runtime twiddles use the host's cosf/sinf
 * where the generated CUDA uses the fast-math __cosf/__sinf intrinsics.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXP 32
#define MAXSTAGES 16

typedef struct {
  float re, im;
} cf;

static const double kPi = 3.14159265358979323846;

/* ------------------------------------------------------------------------ */
/* plan builder restatement                                                  */
/* ------------------------------------------------------------------------ */
static int prime_factors(int n, int* out) {
  int c = 0;
  while (n % 2 == 0) {
    out[c++] = 2;
    n /= 2;
  }
  for (int f = 3; f * f <= n; f += 2)
    while (n % f == 0) {
      out[c++] = f;
      n /= f;
    }
  if (n > 1) out[c++] = n;
  return c;
}

typedef struct {
  int L; /* fft_length */
  int np;
  int primes[MAXP];
  int input_stride;
  int instance_count;
  int registers_used;
  int thread_count;
} stage_t;

typedef struct {
  int nstages;
  stage_t st[MAXSTAGES];
  int register_count;
  int batch_threads;
  int transfer_count;
  int valid;
} cand_t;

static void stage_init(stage_t* s, const int* primes, int np, int max_reg, int N, int input_stride) {
  s->np = np;
  s->L = 1;
  for (int i = 0; i < np; ++i) {
    s->primes[i] = primes[i];
    s->L *= primes[i];
  }
  s->input_stride = input_stride;
  int ip[MAXP];
  int nip = prime_factors(N / s->L, ip);
  s->instance_count = 1;
  for (int i = 0; i < nip; ++i) {
    if (s->instance_count * s->L * ip[i] > max_reg) break;
    s->instance_count *= ip[i];
  }
  s->registers_used = s->L * s->instance_count;
  int rem = N % s->registers_used;
  s->thread_count = N / s->registers_used + (rem != 0);
}

/* keys of get_input_format / get_output_format as sorted sets */
static int cmp_int(const void* a, const void* b) { return (*(const int*)a > *(const int*)b) - (*(const int*)a < *(const int*)b); }

static int input_keys(const stage_t* s, int N, int* keys) {
  int c = 0, stride = N / s->L;
  int iis = N / (s->L * s->instance_count);
  for (int ii = 0; ii < s->instance_count; ++ii) {
    int id0 = iis * ii;
    for (int i = 0; i < s->L; ++i) keys[c++] = id0 + stride * i;
  }
  qsort(keys, c, sizeof(int), cmp_int);
  return c;
}

static int output_keys(const stage_t* s, int N, int* keys) {
  int c = 0;
  int iis = N / (s->L * s->instance_count);
  for (int jj = 0; jj < s->L; ++jj)
    for (int ii = 0; ii < s->instance_count; ++ii) {
      int id0 = iis * ii;
      int ibo = id0 % s->input_stride;
      int sso = id0 * s->L - ibo * (s->L - 1);
      keys[c++] = sso + jj * s->input_stride;
    }
  qsort(keys, c, sizeof(int), cmp_int);
  /* dictionary keys: duplicates collapse */
  int u = 0;
  for (int i = 0; i < c; ++i)
    if (i == 0 || keys[i] != keys[i - 1]) keys[u++] = keys[i];
  return u;
}

static void make_candidate(int N, int max_reg, cand_t* c) {
  int pf[MAXP];
  int npf = prime_factors(N, pf);
  /* group_primes */
  int groups[MAXSTAGES][MAXP], gn[MAXSTAGES], ng = 0;
  for (int i = 0; i < npf; ++i) {
    if (ng > 0) {
      int prod = 1;
      for (int k = 0; k < gn[ng - 1]; ++k) prod *= groups[ng - 1][k];
      if (prod * pf[i] <= max_reg) {
        groups[ng - 1][gn[ng - 1]++] = pf[i];
        continue;
      }
    }
    gn[ng] = 0;
    groups[ng][gn[ng]++] = pf[i];
    ++ng;
  }
  int stride = 1;
  c->nstages = ng;
  c->register_count = 0;
  c->batch_threads = 0;
  for (int g = 0; g < ng; ++g) {
    stage_init(&c->st[g], groups[g], gn[g], max_reg, N, stride);
    stride *= c->st[g].L;
    if (c->st[g].registers_used > c->register_count) c->register_count = c->st[g].registers_used;
    if (c->st[g].thread_count > c->batch_threads) c->batch_threads = c->st[g].thread_count;
  }
  c->valid = c->register_count <= max_reg;
  c->transfer_count = 0;
  if (!c->valid) return;
  int* ka = (int*)malloc(sizeof(int) * (size_t)N * 2);
  int* kb = (int*)malloc(sizeof(int) * (size_t)N * 2);
  for (int g = 0; g + 1 < ng; ++g) {
    int na = output_keys(&c->st[g], N, ka);
    int nb = input_keys(&c->st[g + 1], N, kb);
    int same = na == nb;
    for (int i = 0; same && i < na; ++i) same = ka[i] == kb[i];
    if (!same) c->transfer_count++;
  }
  free(ka);
  free(kb);
}

/* select_fft_plan_candidate with max_register_count=None and the GB300 CUDA
 * limits (1024 threads in x and y).  Returns 0, or -1 when the reference
 * raises "Unable to build an FFT plan". */
int vdxref_plan(int N, cand_t* out) {
  const int limit = 1024;
  int max_registers = 16;
  if (N == 16 || N == 8 || N == 4 || N == 2) max_registers = (N / 2 > 2) ? N / 2 : 2;
  int baseline = N < 8 ? N : 8;
  /* candidates: baseline, then divisors of max_registers in (baseline, max_registers] */
  int cands[16], nc = 0;
  cands[nc++] = baseline;
  for (int d = 1; d <= max_registers; ++d)
    if (max_registers % d == 0 && d > baseline) cands[nc++] = d;
  cand_t base;
  make_candidate(N, baseline, &base);
  if (base.valid && base.batch_threads <= limit) {
    for (int i = 1; i < nc; ++i) {
      cand_t c;
      make_candidate(N, cands[i], &c);
      if (!c.valid) continue;
      if (c.batch_threads > limit) continue;
      if (c.transfer_count < base.transfer_count) {
        *out = c;
        return 0;
      }
    }
    *out = base;
    return 0;
  }
  for (int i = 1; i < nc; ++i) {
    cand_t c;
    make_candidate(N, cands[i], &c);
    if (!c.valid) continue;
    if (c.batch_threads <= limit) {
      *out = c;
      return 0;
    }
  }
  return -1;
}

/* Flat description for Python: [nstages, register_count, batch_threads,
 * (np, primes...) per stage].  Returns the number of ints written or -1. */
int vdxref_plan_describe(int N, int* buf, int cap) {
  cand_t c;
  if (vdxref_plan(N, &c) != 0) return -1;
  int k = 0;
  if (cap < 3) return -1;
  buf[k++] = c.nstages;
  buf[k++] = c.register_count;
  buf[k++] = c.batch_threads;
  for (int s = 0; s < c.nstages; ++s) {
    if (k + 1 + c.st[s].np > cap) return -1;
    buf[k++] = c.st[s].np;
    for (int i = 0; i < c.st[s].np; ++i) buf[k++] = c.st[s].primes[i];
  }
  return k;
}

/* ------------------------------------------------------------------------ */
/* arithmetic                                                                */
/* ------------------------------------------------------------------------ */
static inline cf cmul(cf a, cf b) {
  cf r;
  r.re = fmaf(a.re, b.re, -(a.im * b.im));
  r.im = fmaf(a.re, b.im, a.im * b.re);
  return r;
}
static inline cf cadd(cf a, cf b) {
  cf r = {a.re + b.re, a.im + b.im};
  return r;
}
static inline cf csub(cf a, cf b) {
  cf r = {a.re - b.re, a.im - b.im};
  return r;
}

/* constant twiddle exp(i*af*num/den) applied as the reference does */
static inline cf const_twiddle(cf v, double af, double num, double den) {
  double ang = af * num / den;
  double c = cos(ang), s = sin(ang);
  double a = atan2(s, c); /* numpy.angle of exp(i ang) */
  double scaled = 2.0 * a / kPi;
  double rounded = nearbyint(scaled);
  if (fabs(scaled - rounded) < 1e-8) {
    int ai = (int)rounded;
    if (ai == 0) return v;
    if (ai == 1) {
      cf r = {-v.im, v.re};
      return r;
    }
    if (ai == -1) {
      cf r = {v.im, -v.re};
      return r;
    }
    if (ai == 2 || ai == -2) {
      cf r = {-v.re, -v.im};
      return r;
    }
  }
  cf w = {(float)c, (float)s};
  return cmul(v, w);
}

static void radix_p(cf* x, int P, double af) {
  if (P == 1) return;
  if (P == 2) {
    cf r0 = x[1];
    x[1] = csub(x[0], r0);
    x[0] = cadd(x[0], r0);
    return;
  }
  cf rr[MAXP];
  for (int i = 0; i < P; ++i) {
    for (int j = 0; j < P; ++j) {
      if (j == 0) {
        rr[i] = x[0];
        continue;
      }
      if (i == 0) {
        rr[i] = cadd(rr[i], x[j]);
        continue;
      }
      if (i * j == P / 2 && P % 2 == 0) {
        rr[i] = csub(rr[i], x[j]);
        continue;
      }
      double ang = af * (double)i * (double)j / (double)P;
      cf w = {(float)cos(ang), (float)sin(ang)};
      rr[i] = cadd(rr[i], cmul(x[j], w));
    }
  }
  for (int i = 0; i < P; ++i) x[i] = rr[i];
}

/* radix_composite on L registers; runtime twiddle index k (k < 0: none) */
static void radix_composite(cf* regs, const stage_t* s, int k, int twN, double af) {
  const int L = s->L;
  if (L == 1) return;
  if (k >= 0) {
    float tscale = (float)k;
    for (int i = 1; i < L; ++i) {
      float ascale = (float)(af * (double)i / (double)twN);
      float ang = ascale * tscale;
      cf w = {cosf(ang), sinf(ang)};
      regs[i] = cmul(regs[i], w);
    }
  }
  int ostride = 1;
  cf out[MAXP * 16], tmp[MAXP];
  for (int pi = 0; pi < s->np; ++pi) {
    const int p = s->primes[pi];
    const int nsub = L / p;
    const int bw = ostride * p;
    for (int i = 0; i < nsub; ++i) {
      const int inner = i % ostride;
      const int bidx = (i * p) / bw;
      for (int j = 0; j < p; ++j) tmp[j] = regs[i + j * nsub];
      if (inner != 0)
        for (int j = 1; j < p; ++j) tmp[j] = const_twiddle(tmp[j], af, (double)j * inner, (double)bw);
      radix_p(tmp, p, af);
      const int sso = bidx * bw + inner;
      for (int j = 0; j < p; ++j) out[sso + j * ostride] = tmp[j];
    }
    memcpy(regs, out, sizeof(cf) * (size_t)L);
    ostride *= p;
  }
}

/* One full transform of x[0..N) (natural order in and out), work buffer y. */
static void ref_transform(cf* x, cf* y, int N, const cand_t* plan, int inverse) {
  const double af = 2.0 * kPi * (inverse ? 1.0 : -1.0);
  int S = 1;
  cf regs[MAXP * 16];
  for (int g = 0; g < plan->nstages; ++g) {
    const stage_t* s = &plan->st[g];
    const int L = s->L, nb = N / L;
    for (int o = 0; o < nb; ++o) {
      for (int i = 0; i < L; ++i) regs[i] = x[o + i * nb];
      int k;
      if (S == 1)
        k = -1; /* stage input stride 1: twiddle index is the constant 0 */
      else
        k = o % S;
      radix_composite(regs, s, k, S * L, af);
      const int kk = (S == 1) ? 0 : o % S;
      const int base = (o - kk) * L + kk;
      for (int j = 0; j < L; ++j) y[base + j * S] = regs[j];
    }
    memcpy(x, y, sizeof(cf) * (size_t)N);
    S *= L;
  }
}

/* ------------------------------------------------------------------------ */
/* array-level entry points (data = interleaved complex64 unless noted)      */
/* ------------------------------------------------------------------------ */

/* C2C along `axis` of a C-order (outer, N, inner) array, in place. */
int vdxref_fft_c2c(float* data, long long outer, int N, long long inner, int inverse, int normalize,
                   int sig_lo, int sig_hi) {
  cand_t plan;
  if (vdxref_plan(N, &plan) != 0) return -1;
  cf* d = (cf*)data;
  const long long nt = outer * inner;
#pragma omp parallel
  {
    cf* x = (cf*)malloc(sizeof(cf) * (size_t)N);
    cf* y = (cf*)malloc(sizeof(cf) * (size_t)N);
#pragma omp for schedule(static)
    for (long long t = 0; t < nt; ++t) {
      const long long o = t / inner, c = t % inner;
      cf* base = d + o * (long long)N * inner + c;
      for (int n = 0; n < N; ++n) {
        if (n < sig_lo || n >= sig_hi) {
          x[n].re = 0.f;
          x[n].im = 0.f;
        } else
          x[n] = base[(long long)n * inner];
      }
      ref_transform(x, y, N, &plan, inverse);
      for (int n = 0; n < N; ++n) {
        cf v = x[n];
        if (inverse && normalize) {
          v.re = v.re / (float)N;
          v.im = v.im / (float)N;
        }
        base[(long long)n * inner] = v;
      }
    }
    free(x);
    free(y);
  }
  return 0;
}

/* R2C (forward) or C2R (inverse) of rows of the packed layout: rows of
 * N/2+1 complex; reals at float offsets row*2*(N/2+1) + n. */
int vdxref_fft_real(float* data, long long rows, int N, int inverse, int normalize, int sig_lo, int sig_hi) {
  cand_t plan;
  if (vdxref_plan(N, &plan) != 0) return -1;
  const int H = N / 2 + 1;
#pragma omp parallel
  {
    cf* x = (cf*)malloc(sizeof(cf) * (size_t)N);
    cf* y = (cf*)malloc(sizeof(cf) * (size_t)N);
#pragma omp for schedule(static)
    for (long long r = 0; r < rows; ++r) {
      float* row = data + r * 2LL * H;
      cf* crow = (cf*)row;
      if (!inverse) {
        for (int n = 0; n < N; ++n) {
          x[n].re = (n < sig_lo || n >= sig_hi) ? 0.f : row[n];
          x[n].im = 0.f;
        }
        ref_transform(x, y, N, &plan, 0);
        for (int k = 0; k < H; ++k) crow[k] = x[k];
      } else {
        for (int k = 0; k < N; ++k) {
          if (k >= H) {
            cf v = crow[N - k];
            v.im = -v.im;
            x[k] = v;
          } else
            x[k] = crow[k];
        }
        ref_transform(x, y, N, &plan, 1);
        for (int n = 0; n < N; ++n) row[n] = normalize ? x[n].re / (float)N : x[n].re;
      }
    }
    free(x);
    free(y);
  }
  return 0;
}

/* fused convolution along `axis`: kernel read at the signal's index, or with
 * kernel_outer_stride = 0 from one slab for all outer batches. */
int vdxref_convolve(float* data, const float* kernel, long long outer, int N, long long inner,
                    long long kernel_outer_stride, int normalize) {
  cand_t plan;
  if (vdxref_plan(N, &plan) != 0) return -1;
  cf* d = (cf*)data;
  const cf* kd = (const cf*)kernel;
  const long long nt = outer * inner;
#pragma omp parallel
  {
    cf* x = (cf*)malloc(sizeof(cf) * (size_t)N);
    cf* y = (cf*)malloc(sizeof(cf) * (size_t)N);
#pragma omp for schedule(static)
    for (long long t = 0; t < nt; ++t) {
      const long long o = t / inner, c = t % inner;
      cf* base = d + o * (long long)N * inner + c;
      const cf* kb = kd + o * kernel_outer_stride + c;
      for (int n = 0; n < N; ++n) x[n] = base[(long long)n * inner];
      ref_transform(x, y, N, &plan, 0);
      for (int n = 0; n < N; ++n) {
        cf kv = kb[(long long)n * inner];
        kv.im = -kv.im;
        x[n] = cmul(x[n], kv);
      }
      ref_transform(x, y, N, &plan, 1);
      for (int n = 0; n < N; ++n) {
        cf v = x[n];
        if (normalize) {
          v.re = v.re / (float)N;
          v.im = v.im / (float)N;
        }
        base[(long long)n * inner] = v;
      }
    }
    free(x);
    free(y);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* reductions in the reference's order                                       */
/* ------------------------------------------------------------------------ */
enum { R_ADD, R_MUL, R_MIN, R_MAX, R_AND, R_OR, R_XOR };
enum { M_ID, M_ABS, M_SQUARE, M_REAL, M_IMAG, M_SIN };
enum { T_F32 = 4, T_F64 = 5, T_I32 = 6, T_U32 = 7, T_C64 = 0 };

#define DEFINE_REDUCE(NAME, T)                                                                        \
  static T NAME##_op(T a, T b, int op) {                                                              \
    switch (op) {                                                                                     \
      case R_ADD: return a + b;                                                                       \
      case R_MUL: return a * b;                                                                       \
      case R_MIN: return b < a ? b : a;                                                               \
      default: return b > a ? b : a;                                                                  \
    }                                                                                                 \
  }                                                                                                   \
  static T NAME##_group(const T* vals, long long count, long long stride_total, long long offset,     \
                        T ident, int op, T* sdata) {                                                  \
    (void)stride_total;                                                                               \
    (void)offset;                                                                                     \
    (void)count;                                                                                      \
    for (int cur = 512; cur > 32; cur /= 2)                                                           \
      for (int t = 0; t < cur; ++t) sdata[t] = NAME##_op(sdata[t], sdata[t + cur], op);               \
    for (int t = 0; t < 32; ++t) sdata[t] = NAME##_op(sdata[t], sdata[t + 32], op);                   \
    T lane[32], nxt[32];                                                                              \
    for (int l = 0; l < 32; ++l) lane[l] = sdata[l];                                                  \
    for (int off = 16; off > 0; off /= 2) {                                                           \
      for (int l = 0; l < 32; ++l) nxt[l] = NAME##_op(lane[l], lane[l ^ off], op);                    \
      for (int l = 0; l < 32; ++l) lane[l] = nxt[l];                                                  \
    }                                                                                                 \
    (void)vals;                                                                                       \
    (void)ident;                                                                                      \
    return lane[0];                                                                                   \
  }

DEFINE_REDUCE(rf32, float)
DEFINE_REDUCE(rf64, double)

static float map_f32(const void* in, int type, long long i, int map) {
  if (type == T_C64) {
    const float* p = (const float*)in + 2 * i;
    float re = p[0], im = p[1];
    switch (map) {
      case M_ABS: return sqrtf(re * re + im * im);
      case M_SQUARE: return re * re + im * im;
      case M_IMAG: return im;
      default: return re;
    }
  }
  float v = ((const float*)in)[i];
  switch (map) {
    case M_ABS: return fabsf(v);
    case M_SQUARE: return v * v;
    case M_SIN: return sinf(v);
    default: return v;
  }
}

/* Float reductions (f32 or complex64 mapped to f32) of `batch` rows of n. */
int vdxref_reduce_f32(const void* in, int type, long long n, long long batch, int op, int map, float* out) {
  long long wg = (n + 1023) / 1024;
  if (wg > 1024) wg = 1024;
  const long long G = wg * 1024;
  float ident = op == R_ADD ? 0.f : op == R_MUL ? 1.f : op == R_MIN ? INFINITY : -INFINITY;
  float* part = (float*)malloc(sizeof(float) * (size_t)wg);
  float sdata[1024];
  for (long long b = 0; b < batch; ++b) {
    for (long long w = 0; w < wg; ++w) {
      for (int t = 0; t < 1024; ++t) {
        float agg = ident;
        for (long long idx = w * 1024 + t; idx < n; idx += G) agg = rf32_op(agg, map_f32(in, type, b * n + idx, map), op);
        sdata[t] = agg;
      }
      part[w] = rf32_group(NULL, 0, 0, 0, ident, op, sdata);
    }
    for (int t = 0; t < 1024; ++t) {
      float agg = ident;
      for (long long idx = t; idx < wg; idx += 1024) agg = rf32_op(agg, part[idx], op);
      sdata[t] = agg;
    }
    out[b] = rf32_group(NULL, 0, 0, 0, ident, op, sdata);
  }
  free(part);
  return 0;
}

int vdxref_reduce_f64(const double* in, long long n, long long batch, int op, double* out) {
  long long wg = (n + 1023) / 1024;
  if (wg > 1024) wg = 1024;
  const long long G = wg * 1024;
  double ident = op == R_ADD ? 0.0 : op == R_MUL ? 1.0 : op == R_MIN ? INFINITY : -INFINITY;
  double* part = (double*)malloc(sizeof(double) * (size_t)wg);
  double sdata[1024];
  for (long long b = 0; b < batch; ++b) {
    for (long long w = 0; w < wg; ++w) {
      for (int t = 0; t < 1024; ++t) {
        double agg = ident;
        for (long long idx = w * 1024 + t; idx < n; idx += G) agg = rf64_op(agg, in[b * n + idx], op);
        sdata[t] = agg;
      }
      part[w] = rf64_group(NULL, 0, 0, 0, ident, op, sdata);
    }
    for (int t = 0; t < 1024; ++t) {
      double agg = ident;
      for (long long idx = t; idx < wg; idx += 1024) agg = rf64_op(agg, part[idx], op);
      sdata[t] = agg;
    }
    out[b] = rf64_group(NULL, 0, 0, 0, ident, op, sdata);
  }
  free(part);
  return 0;
}
