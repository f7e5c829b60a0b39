// Map hooks compiled at run time (vdx_map_*).
//
// The reference turns every input_map / output_map / kernel_map into code
// inside the FFT shader it generates and compiles per call
// (vkdispatch/fft/io_manager.py:107-155, vkdispatch/backends/cuda_backend/
// api_compute.py:30-70).  Here the FFT kernel stays hand-written
// (fft_mapped.cuh on the Stockham passes of fft_kernels.cuh); only the hooks
// struct is user code.  This file compiles the hooks with that template by
// NVRTC, specialised to the planner's compile-time radix list, and launches
// the result.  NVRTC is opened with dlopen so that libvdx itself does not
// depend on it; the kernel headers are embedded at build time.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>
#include <unistd.h>

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fft_mapped.cuh"
#include "reduce_mapped.cuh"
#include "jit_headers.inc"  // kJitHeaderCount, kJitHeaderNames[], kJitHeaderSources[] (written by the build)
#include "vdx.h"
#include "vdx_internal.h"

static_assert(offsetof(vdx::MapArgs, status) == sizeof(vdx_map_args), "vdx::MapArgs must extend vdx_map_args");
static_assert(VDX_MAP_MAX_BUFFERS == vdx::kMapMaxBuffers && VDX_MAP_MAX_SCALARS == vdx::kMapMaxScalars,
              "map argument limits");

namespace {

using namespace vdx;

// ---------------------------------------------------------------------------
// NVRTC, resolved at first use
// ---------------------------------------------------------------------------
struct Nvrtc {
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  decltype(&nvrtcGetErrorString) error_string = nullptr;
  std::string where;  // library path, or why it could not be opened
  bool ok = false;
};

std::string env(const char* name) {
  const char* v = std::getenv(name);
  return v ? std::string(v) : std::string();
}

const Nvrtc& nvrtc() {
  static Nvrtc n;
  static std::once_flag once;
  std::call_once(once, [] {
    std::vector<std::string> cands;
    if (!env("VDX_NVRTC").empty()) cands.push_back(env("VDX_NVRTC"));
    cands.push_back("libnvrtc.so.13");
    cands.push_back("libnvrtc.so");
    for (const char* root : {"CUDA_HOME", "CUDA_PATH"})
      if (!env(root).empty()) cands.push_back(env(root) + "/lib64/libnvrtc.so");
    cands.push_back("/usr/local/cuda/lib64/libnvrtc.so");
    void* h = nullptr;
    for (const auto& c : cands) {
      h = dlopen(c.c_str(), RTLD_NOW | RTLD_LOCAL);
      if (h) {
        n.where = c;
        break;
      }
    }
    if (!h) {
      n.where = "NVRTC not found (set VDX_NVRTC to libnvrtc.so)";
      return;
    }
    n.create = reinterpret_cast<decltype(n.create)>(dlsym(h, "nvrtcCreateProgram"));
    n.compile = reinterpret_cast<decltype(n.compile)>(dlsym(h, "nvrtcCompileProgram"));
    n.log_size = reinterpret_cast<decltype(n.log_size)>(dlsym(h, "nvrtcGetProgramLogSize"));
    n.log = reinterpret_cast<decltype(n.log)>(dlsym(h, "nvrtcGetProgramLog"));
    n.cubin_size = reinterpret_cast<decltype(n.cubin_size)>(dlsym(h, "nvrtcGetCUBINSize"));
    n.cubin = reinterpret_cast<decltype(n.cubin)>(dlsym(h, "nvrtcGetCUBIN"));
    n.destroy = reinterpret_cast<decltype(n.destroy)>(dlsym(h, "nvrtcDestroyProgram"));
    n.error_string = reinterpret_cast<decltype(n.error_string)>(dlsym(h, "nvrtcGetErrorString"));
    n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy && n.error_string;
    if (!n.ok) n.where += ": missing NVRTC entry points";
  });
  return n;
}

// directory holding cuda_fp16.h (the kernel headers include it)
std::string cuda_include_dir() {
  std::vector<std::string> cands;
  if (!env("VDX_CUDA_INCLUDE").empty()) cands.push_back(env("VDX_CUDA_INCLUDE"));
  for (const char* root : {"CUDA_HOME", "CUDA_PATH"})
    if (!env(root).empty()) cands.push_back(env(root) + "/include");
  cands.push_back("/usr/local/cuda/include");
  for (const auto& c : cands)
    if (access((c + "/cuda_fp16.h").c_str(), R_OK) == 0) return c;
  return std::string();
}

// ---------------------------------------------------------------------------
// compiled modules: one per (source, device), kept for the process
// ---------------------------------------------------------------------------
struct Module {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
};
std::mutex g_mu;
std::map<std::pair<std::string, int>, Module> g_modules;

int compile(const std::string& src, int dev, Module* out) {
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_modules.find({src, dev});
    if (it != g_modules.end()) {
      *out = it->second;
      return VDX_OK;
    }
  }
  const Nvrtc& n = nvrtc();
  if (!n.ok) return set_error(VDX_ERR_UNSUPPORTED, ("map hooks: " + n.where).c_str());
  const std::string inc = cuda_include_dir();
  if (inc.empty())
    return set_error(VDX_ERR_UNSUPPORTED, "map hooks: CUDA headers (cuda_fp16.h) not found; set VDX_CUDA_INCLUDE");
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  const std::string arch = "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor) + "a";
  const std::string incopt = "-I" + inc;
  const char* opts[] = {arch.c_str(), "-std=c++17", "-default-device", "-lineinfo", incopt.c_str()};
  nvrtcProgram prog = nullptr;
  nvrtcResult r = n.create(&prog, src.c_str(), "vdx_mapped.cu", kJitHeaderCount, kJitHeaderSources, kJitHeaderNames);
  if (r != NVRTC_SUCCESS) return set_error(VDX_ERR_CUDA, (std::string("nvrtcCreateProgram: ") + n.error_string(r)).c_str());
  r = n.compile(prog, int(sizeof(opts) / sizeof(opts[0])), opts);
  if (r != NVRTC_SUCCESS) {
    size_t ls = 0;
    n.log_size(prog, &ls);
    std::string log(ls, '\0');
    if (ls) n.log(prog, &log[0]);
    n.destroy(&prog);
    if (log.size() > 3000) log.resize(3000);
    return set_error(VDX_ERR_INVALID, ("map hooks do not compile: " + log).c_str());
  }
  size_t cs = 0;
  n.cubin_size(prog, &cs);
  std::vector<char> cubin(cs);
  n.cubin(prog, cubin.data());
  n.destroy(&prog);
  Module m;
  cudaError_t e = cudaLibraryLoadData(&m.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&m.kernel, m.lib, "vdx_mapped");
  if (e != cudaSuccess) {
    if (m.lib) cudaLibraryUnload(m.lib);
    return set_error(VDX_ERR_CUDA, (std::string("loading the map kernel: ") + cudaGetErrorString(e)).c_str());
  }
  std::lock_guard<std::mutex> lock(g_mu);
  auto ins = g_modules.emplace(std::make_pair(src, dev), m);
  if (!ins.second) cudaLibraryUnload(m.lib);  // compiled concurrently by another thread
  *out = ins.first->second;
  return VDX_OK;
}

}  // namespace

struct vdx_map_plan {
  MapGeometry g;
  Module mod;
  std::string source;
  int* d_status = nullptr;  // out-of-range map index flag
  ~vdx_map_plan() {
    if (d_status) cudaFree(d_status);
  }
};

extern "C" {

int vdx_map_plan_create(const vdx_fft_desc* desc, const char* hooks_source, vdx_map_plan** plan) {
  if (!desc || !hooks_source || !plan) return set_error(VDX_ERR_INVALID, "desc, hooks_source and plan must be non-NULL");
  *plan = nullptr;
  if (desc->kind != VDX_KIND_C2C && desc->kind != VDX_KIND_CONV)
    return set_error(VDX_ERR_INVALID, "map hooks run on C2C or CONV descriptors");
  if (desc->io_type != desc->compute_type)
    return set_error(VDX_ERR_INVALID, "map plans: io_type must equal compute_type (the hooks do the I/O)");
  if (desc->flags != 0) return set_error(VDX_ERR_UNSUPPORTED, "map plans take no desc.flags");
  vdx_fft_desc d = *desc;
  d.kernel_type = d.io_type;
  d.kernel_op = VDX_KOP_MUL_CONJ;
  auto* p = new vdx_map_plan();
  int rc = map_plan_geometry(d, &p->g);
  if (rc != VDX_OK) {
    delete p;
    return rc;
  }
  const MapGeometry& g = p->g;
  const int mode = desc->kind == VDX_KIND_CONV ? 2 : (desc->inverse ? 1 : 0);
  const int maxe = g.f64 ? MaxE<double>::value : MaxE<float>::value;
  std::string radices;
  for (size_t i = 0; i < g.radices.size(); ++i) radices += (i ? ", " : "") + std::to_string(g.radices[i]);
  p->source = std::string("#include \"fft_mapped.cuh\"\n\n") + hooks_source +
              "\n\nextern \"C\" __global__ void __launch_bounds__(" + std::to_string(g.launch.block.x) +
              ") vdx_mapped(vdx::FftArgs a, vdx::MapArgs m) {\n  vdx::mapped_body<vdx::FixPlan<" +
              std::to_string(g.args.pp.n) + ", " + std::to_string(g.args.pp.T) + ", vdx::RList<" + radices + ">, " +
              std::to_string(maxe) + ">, " + (g.strided ? "true" : "false") + ", " + (g.f64 ? "double" : "float") +
              ", " + std::to_string(mode) + ", VdxHooks>(a, m);\n}\n";
  rc = compile(p->source, g.dev, &p->mod);
  if (rc != VDX_OK) {
    delete p;
    return rc;
  }
  cudaError_t se = cudaMalloc(&p->d_status, sizeof(int));
  if (se == cudaSuccess) se = cudaMemset(p->d_status, 0, sizeof(int));
  if (se != cudaSuccess) {
    delete p;
    return set_error(VDX_ERR_CUDA, (std::string("map plan status word: ") + cudaGetErrorString(se)).c_str());
  }
  if (g.launch.smem > 48 * 1024) {
    cudaError_t e = cudaKernelSetAttributeForDevice(p->mod.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)g.launch.smem, g.dev);
    if (e != cudaSuccess) {
      delete p;
      return set_error(VDX_ERR_CUDA, (std::string("map kernel shared memory: ") + cudaGetErrorString(e)).c_str());
    }
  }
  *plan = p;
  return VDX_OK;
}

int vdx_map_plan_destroy(vdx_map_plan* plan) {
  delete plan;  // the compiled module stays cached for later plans of the same source
  return VDX_OK;
}

int vdx_map_exec(const vdx_map_plan* p, const vdx_map_args* args, void* stream) {
  if (!p || !args) return set_error(VDX_ERR_INVALID, "plan and args must be non-NULL");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->g.dev) return set_error(VDX_ERR_INVALID, "map plan was created on another device");
  for (int i = 0; i < VDX_MAP_MAX_BUFFERS; ++i)
    if (args->counts[i] < 0) return set_error(VDX_ERR_INVALID, "map buffer counts must be >= 0");
  FftArgs a = p->g.args;
  MapArgs m;
  std::memcpy(&m, args, sizeof(vdx_map_args));
  m.status = p->d_status;
  void* kargs[] = {&a, &m};
  const Launch& l = p->g.launch;
  cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(p->mod.kernel), l.grid, l.block, kargs, l.smem,
                                   reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, (std::string("map kernel launch: ") + cudaGetErrorString(e)).c_str());
  return VDX_OK;
}

int vdx_map_plan_status(const vdx_map_plan* p, int* status, int reset) {
  if (!p || !status) return set_error(VDX_ERR_INVALID, "plan and status must be non-NULL");
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, p->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && reset) e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  *status = h;
  return VDX_OK;
}

int vdx_map_plan_source(const vdx_map_plan* p, char* buf, size_t n) {
  if (!p || !buf || n == 0) return set_error(VDX_ERR_INVALID, "plan and a non-empty buffer are required");
  std::snprintf(buf, n, "%s", p->source.c_str());
  return p->source.size() < n ? VDX_OK : set_error(VDX_ERR_INVALID, "buffer too small for the source");
}

}  // extern "C"

static_assert(VDX_RED_ADD == vdx::kRedAdd && VDX_RED_MUL == vdx::kRedMul && VDX_RED_MIN == vdx::kRedMin &&
                  VDX_RED_MAX == vdx::kRedMax && VDX_RED_AND == vdx::kRedAnd && VDX_RED_OR == vdx::kRedOr &&
                  VDX_RED_XOR == vdx::kRedXor,
              "reduction op codes");

struct vdx_reduce_map_plan {
  int dev = 0;
  int out_type = 0;
  Module mod;
  cudaKernel_t final_kernel = nullptr;
  std::string source;
  int* d_status = nullptr;
  ~vdx_reduce_map_plan() {
    if (d_status) cudaFree(d_status);
  }
};

namespace {

// accumulation type and register precision of a map-reduce output type
bool reduce_types(int out_type, const char** acc, const char** re, size_t* bytes) {
  switch (out_type) {
    case VDX_F32: *acc = "float"; *re = "float"; *bytes = 4; return true;
    case VDX_F64: *acc = "double"; *re = "double"; *bytes = 8; return true;
    case VDX_I32: *acc = "int"; *re = "float"; *bytes = 4; return true;
    case VDX_U32: *acc = "unsigned"; *re = "float"; *bytes = 4; return true;
    case VDX_V2F32: *acc = "float2"; *re = "float"; *bytes = 8; return true;
    default: return false;
  }
}

}  // namespace

extern "C" {

int vdx_reduce_map_plan_create(const char* hooks_source, int op, int out_type, vdx_reduce_map_plan** plan) {
  if (!hooks_source || !plan) return set_error(VDX_ERR_INVALID, "hooks_source and plan must be non-NULL");
  *plan = nullptr;
  const char *acc = nullptr, *re = nullptr;
  size_t bytes = 0;
  if (!reduce_types(out_type, &acc, &re, &bytes))
    return set_error(VDX_ERR_INVALID, "out_type must be VDX_F32, VDX_F64, VDX_I32, VDX_U32 or VDX_V2F32");
  if (op < VDX_RED_ADD || op > VDX_RED_XOR) return set_error(VDX_ERR_INVALID, "unknown reduction op");
  if (op >= VDX_RED_AND && out_type != VDX_I32 && out_type != VDX_U32)
    return set_error(VDX_ERR_INVALID, "AND / OR / XOR reductions need an integer output type");
  auto* p = new vdx_reduce_map_plan();
  cudaError_t e = cudaGetDevice(&p->dev);
  if (e != cudaSuccess) {
    delete p;
    return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  }
  p->out_type = out_type;
  const std::string t = acc, r = re, o = std::to_string(op);
  p->source = std::string("#include \"reduce_mapped.cuh\"\n\n") + hooks_source +
              "\n\nextern \"C\" __global__ void __launch_bounds__(512) vdx_mapped(vdx::MapArgs m, long long n, "
              "long long chunk, " + t + "* part, int nparts) {\n  vdx::reduce_mapped_partial<VdxReduceHooks, " + r +
              ", " + t + ", " + o + ">(m, n, chunk, part, nparts);\n}\n\nextern \"C\" __global__ void "
              "__launch_bounds__(512) vdx_mapped_final(const " + t + "* part, int nparts, " + t +
              "* out) {\n  vdx::reduce_mapped_final<" + t + ", " + o + ">(part, nparts, out);\n}\n";
  int rc = compile(p->source, p->dev, &p->mod);
  if (rc != VDX_OK) {
    delete p;
    return rc;
  }
  e = cudaLibraryGetKernel(&p->final_kernel, p->mod.lib, "vdx_mapped_final");
  if (e == cudaSuccess) e = cudaMalloc(&p->d_status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e != cudaSuccess) {
    delete p;
    return set_error(VDX_ERR_CUDA, (std::string("map-reduce plan: ") + cudaGetErrorString(e)).c_str());
  }
  *plan = p;
  return VDX_OK;
}

int vdx_reduce_map_plan_destroy(vdx_reduce_map_plan* plan) {
  delete plan;  // the compiled module stays cached for later plans of the same source
  return VDX_OK;
}

int vdx_reduce_map_exec(const vdx_reduce_map_plan* p, const vdx_map_args* args, int64_t n, int64_t batch, void* out,
                        void* workspace, void* stream) {
  if (!p || !args || !out || !workspace) return set_error(VDX_ERR_INVALID, "plan, args, out and workspace are required");
  if (n < 1 || batch < 1 || batch > 65535) return set_error(VDX_ERR_INVALID, "n >= 1 and 1 <= batch <= 65535 are required");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != p->dev) return set_error(VDX_ERR_INVALID, "map-reduce plan was created on another device");
  for (int i = 0; i < VDX_MAP_MAX_BUFFERS; ++i)
    if (args->counts[i] < 0) return set_error(VDX_ERR_INVALID, "map buffer counts must be >= 0");
  int64_t parts = 0;
  int rc = vdx_reduce_partial_count(n, &parts);
  if (rc != VDX_OK) return rc;
  MapArgs m;
  std::memcpy(&m, args, sizeof(vdx_map_args));
  m.status = p->d_status;
  long long nn = n, chunk = (n + parts - 1) / parts;
  int np = (int)parts;
  void* part = workspace;
  void* a1[] = {&m, &nn, &chunk, &part, &np};
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void*>(p->mod.kernel), dim3((unsigned)parts, (unsigned)batch),
                                   dim3(512), a1, 0, s);
  if (e == cudaSuccess) {
    void* a2[] = {&part, &np, &out};
    e = cudaLaunchKernel(reinterpret_cast<const void*>(p->final_kernel), dim3((unsigned)batch), dim3(512), a2, 0, s);
  }
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, (std::string("map-reduce launch: ") + cudaGetErrorString(e)).c_str());
  return VDX_OK;
}

int vdx_reduce_map_plan_status(const vdx_reduce_map_plan* p, int* status, int reset) {
  if (!p || !status) return set_error(VDX_ERR_INVALID, "plan and status must be non-NULL");
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, p->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && reset) e = cudaMemset(p->d_status, 0, sizeof(int));
  if (e != cudaSuccess) return set_error(VDX_ERR_CUDA, cudaGetErrorString(e));
  *status = h;
  return VDX_OK;
}

int vdx_reduce_map_plan_source(const vdx_reduce_map_plan* p, char* buf, size_t n) {
  if (!p || !buf || n == 0) return set_error(VDX_ERR_INVALID, "plan and a non-empty buffer are required");
  std::snprintf(buf, n, "%s", p->source.c_str());
  return p->source.size() < n ? VDX_OK : set_error(VDX_ERR_INVALID, "buffer too small for the source");
}

}  // extern "C"
