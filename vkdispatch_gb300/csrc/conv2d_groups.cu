// Chains of per-image transforms of a batch of images as image groups on
// plan-owned streams (convolve2DR, convolve2D, rfft2, irfft2, fft2, ifft2).
//
// The reference runs each of these as one launch per transform over the whole
// batch (vkdispatch/fft/functions.py:164-300, 373-448, 549-646).  Each such kernel is
// latency-bound at partial occupancy on GB300, so here the batch is cut into
// `groups` runs of images, and each run's chain of transforms goes on its own
// stream, forked from the caller's stream with an event and joined back with
// one: while one group's kernel drains, the other groups' kernels take the
// idle SMs (convolve2DR of 64 x 512^2: 0.0944 ms for two groups against
// 0.1019 ms for one).  Every image goes through the same arithmetic, so the
// results are those of one group.  Each group owns its plans (made with
// vdx_fft_plan_create), so plans with a workspace (four-step, Bluestein) may
// split too.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <vector>

#include "vdx.h"
#include "vdx_internal.h"

struct vdx_group_plan {
  int dev = 0;
  int groups = 0;
  int nsteps = 0;
  long long image_bytes = 0;
  std::vector<int> conv_step;         // per step: 1 = reads the kernel
  std::vector<int> broadcast;         // per step: 1 = one kernel for every image
  std::vector<long long> first;       // first image of each group
  std::vector<vdx_plan*> plans;       // groups x nsteps
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  std::string desc;

  virtual ~vdx_group_plan() {
    for (auto* p : plans) vdx_fft_plan_destroy(p);
    for (auto s : side)
      if (s) cudaStreamDestroy(s);
    for (auto e : join)
      if (e) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
  }
};

// convolve2DR's plan is a group plan of three steps
struct vdx_conv2d_groups_plan : vdx_group_plan {};

namespace {

// complex64 elements of one image's data for step d (R2C / C2R take the real
// shape and use the packed layout of rows of W/2 + 1 complex elements)
long long image_elems(const vdx_fft_desc& d) {
  long long e = 1;
  for (int i = 1; i < d.ndim; ++i) {
    const long long n = (i == d.ndim - 1 && (d.kind == VDX_KIND_R2C || d.kind == VDX_KIND_C2R)) ? d.shape[i] / 2 + 1
                                                                                              : d.shape[i];
    e *= n;
  }
  return e;
}

int build(vdx_group_plan* p, const vdx_fft_desc* steps, int nsteps, int groups, const char* op) {
  const vdx_fft_desc& d0 = steps[0];
  const long long nimg = d0.shape[0];
  if (groups > nimg) groups = (int)nimg;
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) return vdx::set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  p->groups = groups;
  p->nsteps = nsteps;
  p->image_bytes = image_elems(d0) * 8;
  for (int s = 0; s < nsteps; ++s) {
    p->conv_step.push_back(steps[s].kind == VDX_KIND_CONV);
    p->broadcast.push_back(steps[s].kind == VDX_KIND_CONV && steps[s].kernel_broadcast);
  }
  std::string sizes;
  for (int g = 0; g < groups; ++g) {
    const long long b0 = nimg * g / groups, b1 = nimg * (g + 1) / groups;
    p->first.push_back(b0);
    for (int s = 0; s < nsteps; ++s) {
      vdx_fft_desc d = steps[s];
      d.shape[0] = b1 - b0;
      vdx_plan* h = nullptr;
      const int rc = vdx_fft_plan_create(&d, &h);
      if (rc != VDX_OK) return rc;  // the sub-plan's message stays in vdx_last_error
      p->plans.push_back(h);
    }
    sizes += (g ? ", " : "") + std::to_string(b1 - b0);
  }
  if (groups > 1) {
    e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    for (int g = 0; g < groups && e == cudaSuccess; ++g) {
      cudaStream_t st = nullptr;
      cudaEvent_t j = nullptr;
      e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
      p->side.push_back(st);
      p->join.push_back(j);
    }
    if (e != cudaSuccess)
      return vdx::set_error(VDX_ERR_CUDA, (std::string("image-group streams: ") + cudaGetErrorString(e)).c_str());
  }
  std::string shape;
  for (int i = 0; i < d0.ndim; ++i) shape += (i ? ", " : "") + std::to_string(d0.shape[i]);
  p->desc = std::string("{\"op\": \"") + op + "\", \"images\": " + std::to_string(nimg) + ", \"shape\": [" + shape +
            "], \"steps\": " + std::to_string(nsteps) + ", \"groups\": " + std::to_string(groups) +
            ", \"group_images\": [" + sizes + "]}";
  return VDX_OK;
}

int check_steps(const vdx_fft_desc* steps, int nsteps, int groups) {
  if (!steps) return vdx::set_error(VDX_ERR_INVALID, "steps must be non-NULL");
  if (nsteps < 1 || nsteps > 4) return vdx::set_error(VDX_ERR_INVALID, "an image-group chain has 1 to 4 steps");
  if (groups < 1 || groups > 8) return vdx::set_error(VDX_ERR_INVALID, "groups must be in [1, 8]");
  long long bytes = -1;
  for (int s = 0; s < nsteps; ++s) {
    const vdx_fft_desc& d = steps[s];
    if (d.kind < VDX_KIND_C2C || d.kind > VDX_KIND_CONV)
      return vdx::set_error(VDX_ERR_INVALID, "image-group steps are C2C, R2C, C2R or CONV transforms");
    if (d.ndim != 3 || d.axis < 1 || d.axis > 2)
      return vdx::set_error(VDX_ERR_INVALID, "image-group steps take a (batch, H, W) shape and axis 1 or 2");
    if (d.io_type != VDX_C64 || d.compute_type != VDX_C64)
      return vdx::set_error(VDX_ERR_UNSUPPORTED, "image groups run complex64 storage and compute");
    if (d.shape[0] < 1 || d.shape[0] != steps[0].shape[0])
      return vdx::set_error(VDX_ERR_INVALID, "every step of an image-group chain has the same image count");
    if ((d.kind == VDX_KIND_R2C || d.kind == VDX_KIND_C2R) && (d.shape[2] < 2 || d.shape[2] % 2))
      return vdx::set_error(VDX_ERR_INVALID, "real steps of an image-group chain need an even width");
    for (int i = 1; i < 3; ++i)
      if (d.shape[i] < 1) return vdx::set_error(VDX_ERR_INVALID, "image dimensions must be positive");
    const long long b = image_elems(d) * 8;
    if (bytes >= 0 && b != bytes)
      return vdx::set_error(VDX_ERR_INVALID, "the steps of an image-group chain disagree on the bytes of one image");
    bytes = b;
  }
  return VDX_OK;
}

int exec_groups(const vdx_group_plan* p, void* data, const void* kernel, void* stream) {
  if (!p || !data) return vdx::set_error(VDX_ERR_INVALID, "plan and data must be non-NULL");
  for (int s = 0; s < p->nsteps; ++s)
    if (p->conv_step[s] && !kernel) return vdx::set_error(VDX_ERR_INVALID, "a convolution step needs a kernel");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->dev) return vdx::set_error(VDX_ERR_INVALID, "image-group plan was created on another device");
  cudaStream_t caller = reinterpret_cast<cudaStream_t>(stream);
  auto run = [&](int g, cudaStream_t st) {
    const long long off = p->first[g] * p->image_bytes;
    char* ptr = static_cast<char*>(data) + off;
    int rc = VDX_OK;
    for (int s = 0; s < p->nsteps && rc == VDX_OK; ++s) {
      const void* k = p->conv_step[s] ? static_cast<const char*>(kernel) + (p->broadcast[s] ? 0 : off) : nullptr;
      rc = vdx_fft_exec(p->plans[(size_t)g * p->nsteps + s], ptr, ptr, k, st);
    }
    return rc;
  };
  if (p->groups == 1) return run(0, caller);
  cudaError_t e = cudaEventRecord(p->fork, caller);
  int rc = VDX_OK;
  for (int g = 0; g < p->groups && e == cudaSuccess; ++g) {
    e = cudaStreamWaitEvent(p->side[g], p->fork, 0);
    if (e != cudaSuccess) break;
    rc = run(g, p->side[g]);
    // a group that has started is joined back even when one of its launches
    // failed, so work the caller queues next never races with it
    e = cudaEventRecord(p->join[g], p->side[g]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(caller, p->join[g], 0);
    if (rc != VDX_OK) break;
  }
  if (rc != VDX_OK) return rc;  // the failing launch's message stays in vdx_last_error
  if (e != cudaSuccess)
    return vdx::set_error(VDX_ERR_CUDA, (std::string("image groups: ") + cudaGetErrorString(e)).c_str());
  return VDX_OK;
}

}  // namespace

extern "C" {

int vdx_group_plan_create(const vdx_fft_desc* steps, int nsteps, int groups, vdx_group_plan** plan) {
  if (!plan) return vdx::set_error(VDX_ERR_INVALID, "plan must be non-NULL");
  *plan = nullptr;
  const int rc = check_steps(steps, nsteps, groups);
  if (rc != VDX_OK) return rc;
  auto* p = new vdx_group_plan();
  const int rb = build(p, steps, nsteps, groups, "image_groups");
  if (rb != VDX_OK) {
    delete p;
    return rb;
  }
  *plan = p;
  return VDX_OK;
}

int vdx_group_plan_destroy(vdx_group_plan* plan) {
  delete plan;
  return VDX_OK;
}

int vdx_group_plan_describe(const vdx_group_plan* p, char* buf, size_t n) {
  if (!p || !buf || n == 0) return vdx::set_error(VDX_ERR_INVALID, "plan and buf must be non-NULL");
  std::snprintf(buf, n, "%s", p->desc.c_str());
  return VDX_OK;
}

int vdx_group_exec(const vdx_group_plan* p, void* data, const void* kernel, void* stream) {
  return exec_groups(p, data, kernel, stream);
}

int vdx_conv2d_groups_plan_create(const vdx_fft_desc* desc, int groups, vdx_conv2d_groups_plan** plan) {
  if (!desc || !plan) return vdx::set_error(VDX_ERR_INVALID, "desc and plan must be non-NULL");
  *plan = nullptr;
  const vdx_fft_desc& d = *desc;
  if (d.kind != VDX_KIND_CONV2D_REAL || d.ndim != 3 || d.axis != 1)
    return vdx::set_error(VDX_ERR_INVALID,
                          "image groups take a VDX_KIND_CONV2D_REAL descriptor of a (batch, H, W) real shape, axis 1");
  if (d.flags & ~VDX_FFT_FLAG_AUTOTUNE) return vdx::set_error(VDX_ERR_INVALID, "image groups take only the autotune flag");
  // rfft of the rows -> convolution along the columns -> irfft of the rows
  vdx_fft_desc steps[3];
  const int kinds[3] = {VDX_KIND_R2C, VDX_KIND_CONV, VDX_KIND_C2R};
  for (int s = 0; s < 3; ++s) {
    vdx_fft_desc& t = steps[s];
    t = d;
    t.kind = kinds[s];
    t.shape[2] = t.kind == VDX_KIND_CONV ? d.shape[2] / 2 + 1 : d.shape[2];
    t.axis = t.kind == VDX_KIND_CONV ? 1 : 2;
    t.inverse = t.kind == VDX_KIND_C2R;
    t.normalize = t.kind == VDX_KIND_R2C ? 0 : d.normalize;
    t.signal_lo = t.signal_hi = -1;
    t.kernel_op = VDX_KOP_MUL_CONJ;
    t.kernel_type = VDX_C64;
    t.kernel_broadcast = t.kind == VDX_KIND_CONV ? d.kernel_broadcast : 0;
  }
  if (d.shape[2] < 2 || d.shape[2] % 2)
    return vdx::set_error(VDX_ERR_INVALID, "image groups need at least one image of even width");
  const int rc = check_steps(steps, 3, groups);
  if (rc != VDX_OK) return rc;
  auto* p = new vdx_conv2d_groups_plan();
  const int rb = build(p, steps, 3, groups, "conv2d_groups");
  if (rb != VDX_OK) {
    delete p;
    return rb;
  }
  *plan = p;
  return VDX_OK;
}

int vdx_conv2d_groups_plan_destroy(vdx_conv2d_groups_plan* plan) {
  delete plan;
  return VDX_OK;
}

int vdx_conv2d_groups_plan_describe(const vdx_conv2d_groups_plan* p, char* buf, size_t n) {
  return vdx_group_plan_describe(p, buf, n);
}

int vdx_conv2d_groups_exec(const vdx_conv2d_groups_plan* p, void* data, const void* kernel, void* stream) {
  if (!kernel) return vdx::set_error(VDX_ERR_INVALID, "plan, data and kernel must be non-NULL");
  return exec_groups(p, data, kernel, stream);
}

}  // extern "C"
