/*
 * A plain C consumer of include/vdx.h: no Python, no torch.  It is the shape
 * of what a non-Python binding (cgo, JNI, N-API, a C++ host) does with
 * libvdx: cudaMalloc'd buffers, plans created once, enqueue-only calls on a
 * stream, status codes and vdx_last_error().
 *
 *   vdx_c_consumer validate   argument checks only; needs no GPU
 *   vdx_c_consumer run        transforms on the GPU (C2C, convolve2DR image
 *                             groups, a reduction, a batch of uneven
 *                             lengths), checked against double-precision
 *                             DFTs computed here
 *
 * Exit status 0 when every check passes.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "vdx.h"

static int failures = 0;

static void expect(int cond, const char* what) {
  if (!cond) {
    char msg[512];
    vdx_last_error(msg, sizeof msg);
    fprintf(stderr, "FAILED: %s (last error: %s)\n", what, msg);
    ++failures;
  }
}

static vdx_fft_desc desc3(int64_t b, int64_t h, int64_t w, int axis, int kind) {
  vdx_fft_desc d;
  memset(&d, 0, sizeof d);
  d.ndim = 3;
  d.shape[0] = b;
  d.shape[1] = h;
  d.shape[2] = w;
  d.axis = axis;
  d.kind = kind;
  d.io_type = VDX_C64;
  d.compute_type = VDX_C64;
  d.signal_lo = d.signal_hi = -1;
  d.kernel_op = VDX_KOP_MUL_CONJ;
  d.kernel_type = VDX_C64;
  return d;
}

static int validate(void) {
  vdx_plan* p = NULL;
  vdx_group_plan* g = NULL;
  vdx_conv2d_groups_plan* c = NULL;
  char msg[256];
  expect(vdx_version() >= 100, "vdx_version");
  expect(vdx_fft_plan_create(NULL, &p) == VDX_ERR_INVALID && p == NULL, "NULL descriptor refused");
  vdx_last_error(msg, sizeof msg);
  expect(strlen(msg) > 0, "last error message set");
  vdx_fft_desc d = desc3(4, 8, 64, 2, VDX_KIND_C2C);
  d.ndim = 0;
  expect(vdx_fft_plan_create(&d, &p) == VDX_ERR_INVALID && p == NULL, "ndim 0 refused");
  expect(vdx_group_plan_create(NULL, 0, 2, &g) == VDX_ERR_INVALID && g == NULL, "empty chain refused");
  d = desc3(8, 64, 64, 1, VDX_KIND_C2C);
  expect(vdx_conv2d_groups_plan_create(&d, 2, &c) == VDX_ERR_INVALID && c == NULL, "conv2d groups need kind 4");
  expect(vdx_reduce(99, VDX_MAP_IDENTITY, VDX_F32, (const void*)16, 10, 1, (void*)16, (void*)16, NULL) ==
             VDX_ERR_INVALID,
         "unknown reduce op refused");
  expect(vdx_group_exec(NULL, NULL, NULL, NULL) == VDX_ERR_INVALID, "NULL group plan refused");
  return failures;
}

/* ---- double-precision references ---------------------------------------- */

typedef struct {
  double re, im;
} cd;

/* out[k] = sum_n in[n] e^{sign 2 pi i n k / N}, strided in/out */
static void dft(const cd* in, long istride, cd* out, long ostride, int n, int sign) {
  for (int k = 0; k < n; ++k) {
    double sr = 0, si = 0;
    for (int t = 0; t < n; ++t) {
      const double a = sign * 2.0 * M_PI * (double)((long)t * k % n) / n;
      const double c = cos(a), s = sin(a);
      sr += in[t * istride].re * c - in[t * istride].im * s;
      si += in[t * istride].re * s + in[t * istride].im * c;
    }
    out[k * ostride].re = sr;
    out[k * ostride].im = si;
  }
}

static double rel_l2(const double* got, const double* ref, long n) {
  double num = 0, den = 0;
  for (long i = 0; i < n; ++i) {
    num += (got[i] - ref[i]) * (got[i] - ref[i]);
    den += ref[i] * ref[i];
  }
  return sqrt(num / (den > 0 ? den : 1));
}

/* C2C along the last axis of (16, 1000): a runtime-radix length (2^3 5^3) */
static double check_c2c(void) {
  const int B = 16, N = 1000;
  const long total = (long)B * N;
  float* h = malloc(sizeof(float) * 2 * total);
  cd* in = malloc(sizeof(cd) * total);
  cd* ref = malloc(sizeof(cd) * total);
  double* got = malloc(sizeof(double) * 2 * total);
  for (long i = 0; i < total; ++i) {
    const long b = i / N, t = i % N;
    h[2 * i] = (float)cos(0.37 * t + 0.5 * b);
    h[2 * i + 1] = (float)sin(0.011 * t * (b + 1));
    in[i].re = h[2 * i];
    in[i].im = h[2 * i + 1];
  }
  for (int b = 0; b < B; ++b) dft(in + (long)b * N, 1, ref + (long)b * N, 1, N, -1);
  void* dev = NULL;
  vdx_plan* p = NULL;
  vdx_fft_desc d = desc3(1, B, N, 2, VDX_KIND_C2C);
  expect(cudaMalloc(&dev, sizeof(float) * 2 * total) == cudaSuccess, "cudaMalloc");
  expect(cudaMemcpy(dev, h, sizeof(float) * 2 * total, cudaMemcpyHostToDevice) == cudaSuccess, "upload");
  expect(vdx_fft_plan_create(&d, &p) == VDX_OK, "C2C plan");
  expect(vdx_fft_exec(p, dev, dev, NULL, NULL) == VDX_OK, "C2C exec");
  expect(cudaMemcpy(h, dev, sizeof(float) * 2 * total, cudaMemcpyDeviceToHost) == cudaSuccess, "download");
  for (long i = 0; i < 2 * total; ++i) got[i] = h[i];
  const double err = rel_l2(got, (const double*)ref, 2 * total);
  vdx_fft_plan_destroy(p);
  cudaFree(dev);
  free(h);
  free(in);
  free(ref);
  free(got);
  return err;
}

/* convolve2DR of (B, H, W) real images with a per-image spectrum K (B, H,
 * W/2+1): rfft rows -> columns * conj(K) -> irfft rows, normalised by 1/H
 * and 1/W; the half spectrum's DC and Nyquist columns contribute their real
 * parts to the real output, as irfft does. */
static void conv2d_ref(const float* x, const cd* K, int B, int H, int W, double* out) {
  const int C = W / 2 + 1;
  cd* row = malloc(sizeof(cd) * W);
  cd* spec = malloc(sizeof(cd) * H * C);
  cd* col = malloc(sizeof(cd) * H);
  for (int b = 0; b < B; ++b) {
    for (int r = 0; r < H; ++r) {
      for (int t = 0; t < W; ++t) {
        row[t].re = x[((long)b * H + r) * W + t];
        row[t].im = 0;
      }
      cd* full = malloc(sizeof(cd) * W);
      dft(row, 1, full, 1, W, -1);
      memcpy(spec + (long)r * C, full, sizeof(cd) * C);
      free(full);
    }
    for (int c = 0; c < C; ++c) {
      dft(spec + c, C, col, 1, H, -1);
      for (int r = 0; r < H; ++r) {
        const cd k = K[((long)b * H + r) * C + c];
        const cd v = col[r];
        col[r].re = v.re * k.re + v.im * k.im; /* v * conj(k) */
        col[r].im = v.im * k.re - v.re * k.im;
      }
      dft(col, 1, spec + c, C, H, +1);
      for (int r = 0; r < H; ++r) {
        spec[(long)r * C + c].re /= H;
        spec[(long)r * C + c].im /= H;
      }
    }
    for (int r = 0; r < H; ++r) {
      const cd* s = spec + (long)r * C;
      for (int t = 0; t < W; ++t) {
        double acc = s[0].re + ((t & 1) ? -s[W / 2].re : s[W / 2].re);
        for (int k = 1; k < W / 2; ++k) {
          const double a = 2.0 * M_PI * (double)((long)k * t % W) / W;
          acc += 2.0 * (s[k].re * cos(a) - s[k].im * sin(a));
        }
        out[((long)b * H + r) * W + t] = acc / W;
      }
    }
  }
  free(row);
  free(spec);
  free(col);
}

static void conv2d_check(double* err_groups, int* chain_equal) {
  const int B = 8, H = 64, W = 64, C = W / 2 + 1;
  const long nreal = (long)B * H * W, ncx = (long)B * H * C;
  float* x = malloc(sizeof(float) * nreal);
  cd* K = malloc(sizeof(cd) * ncx);
  float* packed = calloc(2 * ncx, sizeof(float));
  float* kf = malloc(sizeof(float) * 2 * ncx);
  double* ref = malloc(sizeof(double) * nreal);
  double* got = malloc(sizeof(double) * nreal);
  unsigned s = 12345u;
  for (long i = 0; i < nreal; ++i) {
    s = s * 1664525u + 1013904223u;
    x[i] = (float)((s >> 8) * (1.0 / 16777216.0) * 2.0 - 1.0);
  }
  for (long i = 0; i < ncx; ++i) {
    s = s * 1664525u + 1013904223u;
    K[i].re = (float)(((s >> 8) * (1.0 / 16777216.0)) - 0.5);
    s = s * 1664525u + 1013904223u;
    K[i].im = (float)(((s >> 8) * (1.0 / 16777216.0)) - 0.5);
    kf[2 * i] = (float)K[i].re;
    kf[2 * i + 1] = (float)K[i].im;
  }
  for (long r = 0; r < (long)B * H; ++r) memcpy(packed + r * (W + 2), x + r * W, sizeof(float) * W);
  conv2d_ref(x, K, B, H, W, ref);

  const size_t bytes = sizeof(float) * 2 * ncx;
  void *dev = NULL, *dev2 = NULL, *ker = NULL;
  expect(cudaMalloc(&dev, bytes) == cudaSuccess && cudaMalloc(&dev2, bytes) == cudaSuccess &&
             cudaMalloc(&ker, bytes) == cudaSuccess,
         "cudaMalloc");
  cudaMemcpy(dev, packed, bytes, cudaMemcpyHostToDevice);
  cudaMemcpy(dev2, packed, bytes, cudaMemcpyHostToDevice);
  cudaMemcpy(ker, kf, bytes, cudaMemcpyHostToDevice);
  cudaStream_t st;
  cudaStreamCreate(&st);

  /* the convolve2DR entry point: two image groups */
  vdx_fft_desc d = desc3(B, H, W, 1, VDX_KIND_CONV2D_REAL);
  d.normalize = 1;
  vdx_conv2d_groups_plan* cp = NULL;
  expect(vdx_conv2d_groups_plan_create(&d, 2, &cp) == VDX_OK, "conv2d groups plan");
  expect(vdx_conv2d_groups_exec(cp, dev, ker, st) == VDX_OK, "conv2d groups exec");

  /* the same chain spelled out as a group plan of three steps */
  vdx_fft_desc steps[3] = {desc3(B, H, W, 2, VDX_KIND_R2C), desc3(B, H, C, 1, VDX_KIND_CONV),
                           desc3(B, H, W, 2, VDX_KIND_C2R)};
  steps[1].normalize = 1;
  steps[2].inverse = 1;
  steps[2].normalize = 1;
  vdx_group_plan* gp = NULL;
  expect(vdx_group_plan_create(steps, 3, 2, &gp) == VDX_OK, "group plan");
  expect(vdx_group_exec(gp, dev2, ker, st) == VDX_OK, "group exec");
  expect(cudaStreamSynchronize(st) == cudaSuccess, "stream sync");

  cudaMemcpy(packed, dev, bytes, cudaMemcpyDeviceToHost);
  for (long r = 0; r < (long)B * H; ++r)
    for (int t = 0; t < W; ++t) got[r * W + t] = packed[r * (W + 2) + t];
  *err_groups = rel_l2(got, ref, nreal);
  float* packed2 = malloc(bytes);
  cudaMemcpy(packed2, dev2, bytes, cudaMemcpyDeviceToHost);
  *chain_equal = 1;
  for (long r = 0; r < (long)B * H; ++r)
    if (memcmp(packed + r * (W + 2), packed2 + r * (W + 2), sizeof(float) * W) != 0) *chain_equal = 0;

  vdx_conv2d_groups_plan_destroy(cp);
  vdx_group_plan_destroy(gp);
  cudaStreamDestroy(st);
  cudaFree(dev);
  cudaFree(dev2);
  cudaFree(ker);
  free(x);
  free(K);
  free(packed);
  free(packed2);
  free(kf);
  free(ref);
  free(got);
}

/* uneven lengths in one persistent launch: (length, count) items packed back
 * to back in one buffer */
static double check_batch(int* status) {
  const int lens[4] = {12, 100, 1024, 4096}, counts[4] = {5, 3, 2, 1};
  vdx_batch_item items[4];
  long total = 0;
  for (int i = 0; i < 4; ++i) {
    items[i].offset = total;
    items[i].length = lens[i];
    items[i].count = counts[i];
    total += (long)lens[i] * counts[i];
  }
  float* h = malloc(sizeof(float) * 2 * total);
  cd* in = malloc(sizeof(cd) * total);
  cd* ref = malloc(sizeof(cd) * total);
  double* got = malloc(sizeof(double) * 2 * total);
  for (long i = 0; i < total; ++i) {
    h[2 * i] = (float)sin(0.013 * i + 0.3);
    h[2 * i + 1] = (float)cos(0.007 * (double)(i * i % 977));
    in[i].re = h[2 * i];
    in[i].im = h[2 * i + 1];
  }
  for (int i = 0; i < 4; ++i)
    for (int c = 0; c < counts[i]; ++c) {
      const long o = items[i].offset + (long)c * lens[i];
      dft(in + o, 1, ref + o, 1, lens[i], -1);
    }
  vdx_batch_plan* bp = NULL;
  size_t ws_bytes = 0;
  void *dev = NULL, *ws = NULL;
  expect(vdx_batch_plan_create(items, 4, 0, 0, &bp) == VDX_OK, "batch plan");
  expect(vdx_batch_workspace_bytes(bp, &ws_bytes) == VDX_OK, "batch workspace size");
  expect(cudaMalloc(&dev, sizeof(float) * 2 * total) == cudaSuccess, "cudaMalloc");
  if (ws_bytes) expect(cudaMalloc(&ws, ws_bytes) == cudaSuccess, "cudaMalloc workspace");
  cudaMemcpy(dev, h, sizeof(float) * 2 * total, cudaMemcpyHostToDevice);
  expect(vdx_batch_exec(bp, dev, ws, NULL) == VDX_OK, "batch exec");
  expect(vdx_batch_status(bp, status) == VDX_OK, "batch status");
  cudaMemcpy(h, dev, sizeof(float) * 2 * total, cudaMemcpyDeviceToHost);
  for (long i = 0; i < 2 * total; ++i) got[i] = h[i];
  const double err = rel_l2(got, (const double*)ref, 2 * total);
  vdx_batch_plan_destroy(bp);
  cudaFree(dev);
  if (ws) cudaFree(ws);
  free(h);
  free(in);
  free(ref);
  free(got);
  return err;
}

/* sum over rows of (3, 100000) float32 */
static double check_reduce(void) {
  const int B = 3;
  const int64_t n = 100000;
  float* h = malloc(sizeof(float) * B * n);
  double want[3] = {0, 0, 0};
  for (long i = 0; i < B * n; ++i) {
    h[i] = (float)sin(0.001 * i);
    want[i / n] += h[i];
  }
  int64_t parts = 0;
  expect(vdx_reduce_partial_count(n, &parts) == VDX_OK, "partial count");
  void *in = NULL, *out = NULL, *ws = NULL;
  cudaMalloc(&in, sizeof(float) * B * n);
  cudaMalloc(&out, sizeof(float) * B);
  cudaMalloc(&ws, sizeof(float) * B * (parts > 0 ? parts : 1));
  cudaMemcpy(in, h, sizeof(float) * B * n, cudaMemcpyHostToDevice);
  expect(vdx_reduce(VDX_RED_ADD, VDX_MAP_IDENTITY, VDX_F32, in, n, B, out, ws, NULL) == VDX_OK, "reduce");
  float got[3];
  cudaMemcpy(got, out, sizeof got, cudaMemcpyDeviceToHost);
  double g[3] = {got[0], got[1], got[2]};
  cudaFree(in);
  cudaFree(out);
  cudaFree(ws);
  free(h);
  return rel_l2(g, want, B);
}

int main(int argc, char** argv) {
  if (argc < 2 || (strcmp(argv[1], "validate") && strcmp(argv[1], "run"))) {
    fprintf(stderr, "usage: %s validate|run\n", argv[0]);
    return 2;
  }
  validate();
  if (!strcmp(argv[1], "validate")) {
    printf("validate: %s\n", failures ? "FAILED" : "ok");
    return failures ? 1 : 0;
  }
  int count = 0;
  expect(vdx_device_count(&count) == VDX_OK && count > 0, "a CUDA device");
  if (failures) return 1;
  const double e_fft = check_c2c();
  double e_conv = 1;
  int same = 0;
  conv2d_check(&e_conv, &same);
  const double e_red = check_reduce();
  int bstatus = -1;
  const double e_batch = check_batch(&bstatus);
  expect(e_fft < 1e-5, "C2C against the double DFT");
  expect(e_conv < 1e-5, "conv2d groups against the double reference");
  expect(same, "group chain equals the conv2d groups plan bit for bit");
  expect(e_red < 1e-5, "reduce against the double sum");
  expect(e_batch < 1e-5 && bstatus == 0, "batched uneven lengths against the double DFT");
  printf("run: %s c2c_rel_l2=%.3g conv2d_rel_l2=%.3g chain_bit_equal=%d reduce_rel=%.3g batch_rel_l2=%.3g\n",
         failures ? "FAILED" : "ok", e_fft, e_conv, same, e_red, e_batch);
  return failures ? 1 : 0;
}
