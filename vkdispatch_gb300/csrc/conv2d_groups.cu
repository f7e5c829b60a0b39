// convolve2DR of a batch of images as image groups on plan-owned streams.
//
// The reference runs convolve2DR as three launches over the whole batch
// (vkdispatch/fft/functions.py:614-646).  Each of those kernels is
// latency-bound at partial occupancy on GB300, so here the batch is cut into
// `groups` runs of images, and each run's rfft -> column convolution -> irfft
// chain goes on its own stream, forked from the caller's stream with an event
// and joined back with one: while one group's kernel drains, the other
// groups' kernels take the idle SMs (64 x 512^2: 0.0954 ms for two groups
// against 0.1019 ms for one).  Every image goes through the same plans'
// arithmetic, so the results are those of one group.  Built on the public
// plan API only (vdx_fft_plan_create / vdx_fft_exec).
#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <vector>

#include "vdx.h"
#include "vdx_internal.h"

struct vdx_conv2d_groups_plan {
  int dev = 0;
  int groups = 0;
  long long image_elems = 0;  // complex elements of one image's packed half spectrum
  bool broadcast = false;
  std::vector<long long> first;  // first image of each group
  std::vector<vdx_plan*> r2c, conv, c2r;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  std::string desc;

  ~vdx_conv2d_groups_plan() {
    for (auto* p : r2c) vdx_fft_plan_destroy(p);
    for (auto* p : conv) vdx_fft_plan_destroy(p);
    for (auto* p : c2r) vdx_fft_plan_destroy(p);
    for (auto s : side)
      if (s) cudaStreamDestroy(s);
    for (auto e : join)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
  }
};

namespace {

vdx_fft_desc sub_desc(const vdx_fft_desc& d, long long nb, int kind) {
  vdx_fft_desc s = d;
  s.ndim = 3;
  s.shape[0] = nb;
  s.shape[1] = d.shape[1];
  s.shape[2] = kind == VDX_KIND_CONV ? d.shape[2] / 2 + 1 : d.shape[2];
  s.axis = kind == VDX_KIND_CONV ? 1 : 2;
  s.kind = kind;
  s.inverse = kind == VDX_KIND_C2R ? 1 : 0;
  s.normalize = kind == VDX_KIND_R2C ? 0 : d.normalize;
  s.signal_lo = s.signal_hi = -1;
  s.kernel_op = VDX_KOP_MUL_CONJ;
  s.kernel_type = VDX_C64;
  s.kernel_broadcast = kind == VDX_KIND_CONV ? d.kernel_broadcast : 0;
  return s;
}

}  // namespace

extern "C" {

int vdx_conv2d_groups_plan_create(const vdx_fft_desc* desc, int groups, vdx_conv2d_groups_plan** plan) {
  if (!desc || !plan) return vdx::set_error(VDX_ERR_INVALID, "desc and plan must be non-NULL");
  *plan = nullptr;
  const vdx_fft_desc& d = *desc;
  if (d.kind != VDX_KIND_CONV2D_REAL || d.ndim != 3 || d.axis != 1)
    return vdx::set_error(VDX_ERR_INVALID,
                          "image groups take a VDX_KIND_CONV2D_REAL descriptor of a (batch, H, W) real shape, axis 1");
  if (d.io_type != VDX_C64 || d.compute_type != VDX_C64)
    return vdx::set_error(VDX_ERR_UNSUPPORTED, "image groups run complex64 storage and compute");
  if (d.flags & ~VDX_FFT_FLAG_AUTOTUNE) return vdx::set_error(VDX_ERR_INVALID, "image groups take only the autotune flag");
  if (d.shape[0] < 1 || d.shape[1] < 1 || d.shape[2] < 2 || d.shape[2] % 2)
    return vdx::set_error(VDX_ERR_INVALID, "image groups need at least one image of even width");
  if (groups < 1 || groups > 8) return vdx::set_error(VDX_ERR_INVALID, "groups must be in [1, 8]");
  const long long nimg = d.shape[0];
  if (groups > nimg) groups = (int)nimg;
  auto* p = new vdx_conv2d_groups_plan();
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) {
    delete p;
    return vdx::set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  }
  p->groups = groups;
  p->image_elems = d.shape[1] * (d.shape[2] / 2 + 1);
  p->broadcast = d.kernel_broadcast != 0;
  std::string sizes;
  for (int g = 0; g < groups; ++g) {
    const long long b0 = nimg * g / groups, b1 = nimg * (g + 1) / groups;
    p->first.push_back(b0);
    vdx_plan *a = nullptr, *c = nullptr, *i = nullptr;
    vdx_fft_desc da = sub_desc(d, b1 - b0, VDX_KIND_R2C), dc = sub_desc(d, b1 - b0, VDX_KIND_CONV),
                 di = sub_desc(d, b1 - b0, VDX_KIND_C2R);
    int rc = vdx_fft_plan_create(&da, &a);
    if (rc == VDX_OK) rc = vdx_fft_plan_create(&dc, &c);
    if (rc == VDX_OK) rc = vdx_fft_plan_create(&di, &i);
    p->r2c.push_back(a);
    p->conv.push_back(c);
    p->c2r.push_back(i);
    if (rc != VDX_OK) {
      delete p;
      return rc;  // the sub-plan's error message stays in vdx_last_error
    }
    sizes += (g ? ", " : "") + std::to_string(b1 - b0);
  }
  if (groups > 1) {
    e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    for (int g = 0; g < groups && e == cudaSuccess; ++g) {
      cudaStream_t s = nullptr;
      cudaEvent_t j = nullptr;
      e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
      p->side.push_back(s);
      p->join.push_back(j);
    }
    if (e != cudaSuccess) {
      delete p;
      return vdx::set_error(VDX_ERR_CUDA, (std::string("image-group streams: ") + cudaGetErrorString(e)).c_str());
    }
  }
  p->desc = "{\"op\": \"conv2d_groups\", \"images\": " + std::to_string(nimg) + ", \"H\": " +
            std::to_string(d.shape[1]) + ", \"W\": " + std::to_string(d.shape[2]) + ", \"groups\": " +
            std::to_string(groups) + ", \"group_images\": [" + sizes + "], \"kernel_broadcast\": " +
            (p->broadcast ? "true" : "false") + "}";
  *plan = p;
  return VDX_OK;
}

int vdx_conv2d_groups_plan_destroy(vdx_conv2d_groups_plan* plan) {
  delete plan;
  return VDX_OK;
}

int vdx_conv2d_groups_plan_describe(const vdx_conv2d_groups_plan* p, char* buf, size_t n) {
  if (!p || !buf || n == 0) return vdx::set_error(VDX_ERR_INVALID, "plan and buf must be non-NULL");
  std::snprintf(buf, n, "%s", p->desc.c_str());
  return VDX_OK;
}

int vdx_conv2d_groups_exec(const vdx_conv2d_groups_plan* p, void* data, const void* kernel, void* stream) {
  if (!p || !data || !kernel) return vdx::set_error(VDX_ERR_INVALID, "plan, data and kernel must be non-NULL");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->dev) return vdx::set_error(VDX_ERR_INVALID, "image-group plan was created on another device");
  cudaStream_t caller = reinterpret_cast<cudaStream_t>(stream);
  auto run = [&](int g, cudaStream_t s) {
    const long long off = p->first[g] * p->image_elems * 8;
    char* ptr = static_cast<char*>(data) + off;
    const char* kptr = static_cast<const char*>(kernel) + (p->broadcast ? 0 : off);
    int rc = vdx_fft_exec(p->r2c[g], ptr, ptr, nullptr, s);
    if (rc == VDX_OK) rc = vdx_fft_exec(p->conv[g], ptr, ptr, kptr, s);
    if (rc == VDX_OK) rc = vdx_fft_exec(p->c2r[g], ptr, ptr, nullptr, s);
    return rc;
  };
  if (p->groups == 1) return run(0, caller);
  cudaError_t e = cudaEventRecord(p->fork, caller);
  for (int g = 0; g < p->groups && e == cudaSuccess; ++g) {
    e = cudaStreamWaitEvent(p->side[g], p->fork, 0);
    if (e != cudaSuccess) break;
    const int rc = run(g, p->side[g]);
    if (rc != VDX_OK) return rc;
    e = cudaEventRecord(p->join[g], p->side[g]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(caller, p->join[g], 0);
  }
  if (e != cudaSuccess) return vdx::set_error(VDX_ERR_CUDA, (std::string("image groups: ") + cudaGetErrorString(e)).c_str());
  return VDX_OK;
}

}  // extern "C"
