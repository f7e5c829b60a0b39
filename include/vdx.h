/*
 * vdx.h -- C ABI of libvdx, the GB300 (sm_103a) FFT / FFT-convolution /
 * reduction library of vkdispatch_gb300.
 *
 * Conventions
 *   - Every entry point returns an int status: VDX_OK (0) or a VDX_ERR_* code.
 *     On failure nothing is launched and vdx_last_error() returns a message
 *     (thread-local), mirroring the reference's polled last-error string
 *     (vkdispatch/base/errors.py:15-28, vkdispatch/backends/cuda_backend/
 *     helpers.py:42-47).
 *   - All buffers are caller-owned device pointers (torch tensors, CUDA
 *     arrays behind __cuda_array_interface__, cudaMalloc'd memory).  Plans
 *     own only their constant twiddle tables.
 *   - Execution is enqueue-only on the given CUDA stream (a cudaStream_t
 *     passed as void*; NULL = legacy default stream), like the reference's
 *     cuLaunchKernel path (vkdispatch/backends/cuda_backend/
 *     cuda_primitives.py:163-284).  Plans are immutable after creation and
 *     may be shared between host threads.
 *   - Layouts are C order.  complex64 = interleaved (re, im) float32.
 */
#ifndef VDX_H
#define VDX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define VDX_OK 0
#define VDX_ERR_INVALID 1     /* bad argument, shape or plan */
#define VDX_ERR_UNSUPPORTED 2 /* valid request outside what the kernels implement */
#define VDX_ERR_CUDA 3        /* CUDA runtime error (message has the CUDA error string) */
#define VDX_ERR_NOMEM 4       /* device allocation failed (plan tables only) */

/* element types (storage) */
#define VDX_C64 0    /* complex64: 2 x float32 */
#define VDX_C32 1    /* complex32: 2 x float16 (IEEE half) */
#define VDX_C128 2   /* complex128: 2 x float64 */
#define VDX_BF16X2 3 /* complex as 2 x bfloat16 */
#define VDX_F32 4
#define VDX_F64 5
#define VDX_I32 6
#define VDX_U32 7
#define VDX_V2F32 8 /* two float32 lanes (the reference's vec2): map-reduce results only */

/* transform kinds */
#define VDX_KIND_C2C 0  /* complex FFT along one axis, in or out of place */
#define VDX_KIND_R2C 1  /* real FFT of the last axis, packed RFFT layout */
#define VDX_KIND_C2R 2  /* inverse real FFT of the last axis, packed RFFT layout */
#define VDX_KIND_CONV 3 /* fused FFT -> spectrum * op(kernel) -> inverse FFT along one axis */
/* The whole convolve2DR of real images in one launch (vkdispatch/fft/
 * functions.py:614-646): rfft of the last axis -> convolve along axis ndim-2
 * -> irfft, in place on the packed RFFT layout.  shape = the REAL shape
 * (..., H, W), ndim 2 or 3, axis = ndim-2; complex64 only; in == out.
 * normalize scales the column inverse by 1/H and the row inverse by 1/W, as
 * the composed path does.  Plan creation fails with VDX_ERR_UNSUPPORTED for
 * sizes without a fused kernel (today H = W = 512); callers then run the
 * three separate transforms. */
#define VDX_KIND_CONV2D_REAL 4

/* convolution spectrum operations */
#define VDX_KOP_MUL_CONJ 0 /* spectrum * conj(kernel) (the reference default) */
#define VDX_KOP_MUL 1      /* spectrum * kernel */

typedef struct vdx_fft_desc {
  int32_t ndim;       /* 1..4 */
  int64_t shape[4];   /* buffer shape; for R2C/C2R the REAL shape (last dim N) */
  int32_t axis;       /* transformed axis (R2C/C2R: must be ndim-1) */
  int32_t kind;       /* VDX_KIND_* */
  int32_t inverse;    /* C2C: 0 forward (exp(-2 pi i nk/N)), 1 inverse */
  int32_t normalize;  /* C2C / C2R / CONV: 1 = scale the output by 1/N, 2 = by 1/sqrt(N)
                         (orthonormal; keeps fp16-stored spectra of long axes in range),
                         0 = unscaled (R2C: ignored) */
  int32_t io_type;    /* VDX_C64, VDX_C32, VDX_C128 or VDX_BF16X2 */
  int32_t compute_type; /* VDX_C64 (fp32 butterflies) or VDX_C128 (fp64) */
  int64_t signal_lo;  /* input_signal_range: points outside [lo, hi) read as 0; */
  int64_t signal_hi;  /* lo = 0, hi = N (or hi <= 0) means the whole axis       */
  int32_t kernel_op;  /* CONV: VDX_KOP_* */
  int32_t kernel_type;/* CONV: storage type of the kernel spectrum */
  int32_t kernel_broadcast; /* CONV: 1 = one kernel spectrum for every outer batch */
  int32_t flags;      /* VDX_FFT_FLAG_* (0 = defaults) */
} vdx_fft_desc;

/*
 * desc.flags.  VDX_FFT_FLAG_TENSOR_CORE runs the 128-point short transforms
 * of a four-step (long-axis, C2C) plan as BF16 tensor-core GEMMs -- a
 * DFT-16 stage and a DFT-8 stage, each with hi/lo-split three-product
 * compensation and FP32 accumulation -- instead of fp32 butterflies.
 * Available for C2C axes of exactly 16384 points (split 128 x 128) with
 * io_type VDX_C64, VDX_C32 or VDX_BF16X2.  No counterpart in the reference,
 * whose FFT stages are scalar code (vkdispatch/fft/cooley_tukey.py:55-180).
 */
#define VDX_FFT_FLAG_TENSOR_CORE 1
/*
 * VDX_FFT_FLAG_AUTOTUNE: plan creation times the candidate plan choices --
 * threads per CTA (contiguous axes) or columns per tile (strided axes), radix
 * order, compile-time vs runtime pass lists, and four-step vs one-CTA
 * transforms for long C2C axes -- on scratch buffers of the same axis length
 * and stride class (at most VDX_AUTOTUNE_MB, default 256 MB), and keeps the
 * fastest.  Choices are cached per (device, kind, N, stride class, batch
 * class, dtype, direction, kernel op/broadcast, signal range); later plans
 * with the same key reuse them without timing.  The search allocates and
 * synchronises: create autotuned plans outside stream capture.  The
 * reference has no autotuner: its planner picks one configuration by a fixed
 * rule (vkdispatch/fft/config.py:102-190).
 */
#define VDX_FFT_FLAG_AUTOTUNE 2
/*
 * VDX_FFT_FLAG_BLUESTEIN: C2C axes whose length has a prime factor above 13
 * (which the reference rejects, vkdispatch/fft/prime_utils.py:6-10) are
 * planned as Bluestein chirp-z transforms instead of failing: a chirp
 * multiply into a zero-padded workspace of length M (the power of two >=
 * 2N - 1), one fused length-M convolution against the precomputed
 * conj(FFT_M(chirp)), and a chirp multiply out.  The chirps are built in FP64
 * from the exact integer n^2 mod 2N.  Limits: M <= 16384 (fp32 compute) or
 * 8192 (fp64).  Without the flag such lengths fail with VDX_ERR_UNSUPPORTED,
 * as in the reference.
 */
#define VDX_FFT_FLAG_BLUESTEIN 4

typedef struct vdx_plan vdx_plan;

/* Library version (major*10000 + minor*100 + patch).  No counterpart in the
 * reference's path (its version is the Python package's). */
int vdx_version(void);

/* Copies the calling thread's last error message into buf (NUL-terminated):
 * the reference's polled error string (vkdispatch/base/errors.py:15-28). */
int vdx_last_error(char* buf, size_t n);

/* Number of visible CUDA devices; fails when the driver is unusable (the
 * device count behind the reference's get_devices, vkdispatch/backends/
 * cuda_backend/api_context.py:42-50). */
int vdx_device_count(int* count);

/*
 * Plan creation.  Replaces the reference's kernel factory + runtime compile:
 * make_fft_shader / make_convolution_shader (vkdispatch/fft/
 * shader_factories.py:11-60, 107-195) -> FFTConfig plan builder
 * (vkdispatch/fft/config.py:192-277) -> NVRTC compile and module load
 * (vkdispatch/backends/cuda_backend/api_compute.py:30-70).  Builds the radix
 * pass list, launch shape and FP64-built twiddle tables on the current
 * device.
 */
int vdx_fft_plan_create(const vdx_fft_desc* desc, vdx_plan** plan);
int vdx_fft_plan_destroy(vdx_plan* plan);

/* Autotune cache (VDX_FFT_FLAG_AUTOTUNE): number of cached choices and of
 * candidate searches run so far; save to / merge from a text file (one line
 * per key).  No counterpart in the reference. */
int vdx_autotune_entries(int64_t* entries, int64_t* searches);
int vdx_autotune_save(const char* path);
int vdx_autotune_load(const char* path);

/* Human-readable plan (radices, threads per transform, transforms per CTA):
 * what print_shader / ShaderFunction.get_src show in the reference
 * (vkdispatch/shader/shader_function.py:255-275), as JSON. */
int vdx_fft_plan_describe(const vdx_plan* plan, char* buf, size_t n);

/*
 * Executes a plan: one kernel launch on `stream`.  Replaces the reference's
 * ShaderFunction.__call__ -> CommandGraph.record_shader -> cuLaunchKernel
 * path (vkdispatch/shader/shader_function.py:277-380,
 * vkdispatch/execution_pipeline/command_graph.py:193-279,
 * vkdispatch/backends/cuda_backend/cuda_primitives.py:163-284).
 *   in/out : same shape and io_type; in == out is the reference's in-place
 *            mode.  R2C/C2R use the packed RFFT layout: rows of N/2+1
 *            complex elements whose first N reals hold the real signal
 *            (vkdispatch/base/buffer.py:377-448).
 *   kernel : CONV only; spectrum of the buffer's shape (or one batch of it
 *            when kernel_broadcast = 1).
 */
int vdx_fft_exec(const vdx_plan* plan, const void* in, void* out, const void* kernel, void* stream);

/*
 * Fused element-wise operations for the adjoint (autograd) pipelines of FFT
 * convolutions; complex64 plans only, at most one operation per launch.  The
 * weight and auxiliary arrays have the buffer's shape and are indexed like
 * it.  No counterpart in the reference, whose gradients do not exist; these
 * serve the differentiable convolution (vkdispatch_gb300/autograd.py).
 *   in_weight   (C2C)  : each input point is multiplied by
 *                        in_weight[i] * in_weight_scale (* *in_weight_scale_ptr
 *                        when that device pointer is set) as it is loaded
 *   spec_out    (CONV) : receives the forward spectrum S of every transform,
 *                        or, with spec_aux set, spec_aux * conj(S) * spec_scale
 *   loss_weight (C2C)  : each CTA writes sum(loss_weight[i] * |out[i]|^2) over
 *                        its outputs to loss_partials[cta] (vdx_fft_plan_ctas
 *                        entries); fold them with vdx_reduce for the total
 */
typedef struct vdx_exec_ops {
  const float* in_weight;
  const float* in_weight_scale_ptr;
  float in_weight_scale;
  float spec_scale;
  void* spec_out;
  const void* spec_aux;
  const float* loss_weight;
  float* loss_partials;
} vdx_exec_ops;

int vdx_fft_exec_ops(const vdx_plan* plan, const void* in, void* out, const void* kernel, const vdx_exec_ops* ops,
                     void* stream);

/*
 * One signal convolved with kernel_num kernels in one launch (the reference's
 * kernel_num > 1 convolution shader, vkdispatch/fft/shader_factories.py:
 * 166-193, and the kernel_num argument of vd.fft.convolve, vkdispatch/fft/
 * functions.py:476-547): kernel k is read at kernel + k * kernel_stride and
 * output slice k written at out + k * out_stride (strides in elements of the
 * plan's storage type).  The signal is read and transformed once.  `in` must
 * not overlap the output slices of other transforms.  Returns
 * VDX_ERR_UNSUPPORTED for plans without a fused kernel (long four-step axes,
 * Bluestein lengths, the radix-8 plan, 4-byte storage, or when the spectrum
 * does not fit in shared memory); the caller then runs one vdx_fft_exec per
 * kernel.
 */
int vdx_conv_exec_multi(const vdx_plan* plan, const void* in, void* out, const void* kernel, int kernel_num,
                        int64_t kernel_stride, int64_t out_stride, void* stream);

/*
 * convolve2DR of a batch of real images as image groups (the reference's
 * vd.fft.convolve2DR, vkdispatch/fft/functions.py:614-646, which the
 * reference runs as rfft -> convolve(axis 1) -> irfft over the whole batch).
 * desc: VDX_KIND_CONV2D_REAL, ndim 3, REAL shape (B, H, W) with W even,
 * axis 1, io_type = compute_type = VDX_C64, normalize as in
 * VDX_KIND_CONV2D_REAL, kernel_broadcast 1 = one (H, W/2+1) kernel spectrum
 * for every image; flags 0 or VDX_FFT_FLAG_AUTOTUNE.  The images are cut
 * into `groups` (1..8, at most B) runs; each run's three transforms go on a
 * stream the plan owns, forked from and joined back into the caller's stream
 * with events, so that the groups' latency-bound kernels overlap.  Results
 * equal those of one group.  vdx_conv2d_groups_exec runs in place on the
 * packed RFFT layout (data), enqueues only asynchronous work (capturable in a
 * CUDA graph) and must not be called on one plan from two host threads at
 * once.
 */
typedef struct vdx_conv2d_groups_plan vdx_conv2d_groups_plan;

int vdx_conv2d_groups_plan_create(const vdx_fft_desc* desc, int groups, vdx_conv2d_groups_plan** plan);
int vdx_conv2d_groups_plan_destroy(vdx_conv2d_groups_plan* plan);
int vdx_conv2d_groups_plan_describe(const vdx_conv2d_groups_plan* plan, char* buf, size_t n);
int vdx_conv2d_groups_exec(const vdx_conv2d_groups_plan* plan, void* data, const void* kernel, void* stream);

/*
 * The same image groups for any chain of 1-4 in-place per-image transforms
 * of one batch (the reference's fft2 / ifft2 / rfft2 / irfft2 / convolve2D,
 * vkdispatch/fft/functions.py:164-300, 373-448, 549-612, each of which it runs as one
 * launch per transform over the whole batch).  steps[s] describes transform
 * s over the WHOLE batch: ndim 3, shape[0] = the image count (the same in
 * every step), axis 1 or 2, VDX_KIND_C2C, R2C, C2R or CONV, complex64
 * storage and compute, and every step addresses the same bytes per image
 * (R2C / C2R steps take the real shape and the packed RFFT layout).  The plan
 * cuts the batch into `groups` (1..8) runs of images, each with its own plans
 * and stream.  vdx_group_exec runs the chain in place on data; a CONV step
 * reads `kernel` at the image's offset (or at kernel itself when the step
 * has kernel_broadcast = 1).  Same stream, capture and threading rules as
 * vdx_conv2d_groups_exec.
 */
typedef struct vdx_group_plan vdx_group_plan;

int vdx_group_plan_create(const vdx_fft_desc* steps, int nsteps, int groups, vdx_group_plan** plan);
int vdx_group_plan_destroy(vdx_group_plan* plan);
int vdx_group_plan_describe(const vdx_group_plan* plan, char* buf, size_t n);
int vdx_group_exec(const vdx_group_plan* plan, void* data, const void* kernel, void* stream);

/* Number of CTAs one vdx_fft_exec of this plan launches (sizes the loss
 * partials of vdx_fft_exec_ops).  No counterpart in the reference. */
int vdx_fft_plan_ctas(const vdx_plan* plan, int64_t* ctas);

/*
 * Device-side status of a plan's bounded waits (synchronising read): 0 = every
 * wait completed; 1 = a tensor-core MMA completion wait gave up and the
 * affected tile was not written.  Plans without such waits always report 0.
 * No counterpart in the reference (its kernels have no waits).
 */
int vdx_fft_plan_status(const vdx_plan* plan, int* status);

/*
 * Element-wise conversion of `count` elements between VDX_C64, VDX_C128,
 * VDX_C32, VDX_BF16X2, VDX_F32 and VDX_F64 (real -> complex: imaginary part
 * 0; complex -> real: real part).  The load and store ends of the map hooks
 * that change precision or read/write real buffers (vkdispatch/fft/
 * global_memory_iterators.py:71-92, 197-229 with a cast in the map).
 */
int vdx_convert(const void* src, int src_type, void* dst, int dst_type, int64_t count, void* stream);

/*
 * Batched transforms of uneven lengths in one persistent launch.  Each item
 * is `count` contiguous complex64 transforms of `length` points starting at
 * element `offset` of the data buffer.  Lengths up to 16384 run as tiles of
 * whole transforms; longer 13-smooth lengths run as a four-step pair inside
 * the same launch and need a workspace of vdx_batch_workspace_bytes.  Replaces
 * one make_fft_shader kernel and launch per (length, batch) in the reference
 * (vkdispatch/fft/shader_factories.py:11-60, functions.py:104-162).
 * vdx_batch_exec enqueues two memsets and one launch (capturable in a CUDA
 * graph); vdx_batch_status reads (synchronously) whether a dependency wait
 * inside the launch gave up, which leaves the affected items undefined.
 */
typedef struct vdx_batch_item {
  int64_t offset;
  int32_t length;
  int32_t count;
} vdx_batch_item;

typedef struct vdx_batch_plan vdx_batch_plan;

int vdx_batch_plan_create(const vdx_batch_item* items, int nitems, int inverse, int normalize,
                          vdx_batch_plan** plan);
int vdx_batch_plan_destroy(vdx_batch_plan* plan);
int vdx_batch_plan_describe(const vdx_batch_plan* plan, char* buf, size_t n);
int vdx_batch_workspace_bytes(const vdx_batch_plan* plan, size_t* bytes);
int vdx_batch_exec(const vdx_batch_plan* plan, void* data, void* workspace, void* stream);
int vdx_batch_status(const vdx_batch_plan* plan, int* status);
/*
 * Sets the poll limit of the launch's dependency waits (default 2^22 polls of
 * about 100 ns) and clears the plan's status word (synchronous).  A
 * second-pass unit whose column units have not all finished after
 * `wait_limit` polls sets the status to 1, skips its work and the launch goes
 * on.  `extra_dependency` > 0 raises every second-pass unit's dependency
 * count above the number of column units that exist, so those waits can only
 * end at the limit: a host-side way to test that a wait which runs out
 * returns a status instead of hanging (0 restores normal operation).  Not
 * thread-safe against a concurrent vdx_batch_exec of the same plan.  No
 * counterpart in the reference, whose kernels never wait on one another.
 */
int vdx_batch_plan_set_wait(vdx_batch_plan* plan, int64_t wait_limit, int32_t extra_dependency);

/* reduction operations (vkdispatch/reduce/operations.py:17-66) */
#define VDX_RED_ADD 0
#define VDX_RED_MUL 1
#define VDX_RED_MIN 2
#define VDX_RED_MAX 3
#define VDX_RED_AND 4
#define VDX_RED_OR 5
#define VDX_RED_XOR 6

/* element-wise maps applied before reducing (the map-hook menu) */
#define VDX_MAP_IDENTITY 0 /* x                      */
#define VDX_MAP_ABS 1      /* |x|  (complex: modulus) */
#define VDX_MAP_SQUARE 2   /* x^2  (complex: |x|^2)   */
#define VDX_MAP_REAL 3     /* complex: real part      */
#define VDX_MAP_IMAG 4     /* complex: imaginary part */
#define VDX_MAP_SIN 5      /* sin(x)                  */

/*
 * Number of stage-1 partial slots vdx_reduce needs per batch row for a row
 * of `n` elements; the workspace must hold partial_count * batch elements of
 * the output type.  The reference sizes the same stage from its workgroup
 * count (vkdispatch/reduce/reduce_function.py:117-125).
 */
int vdx_reduce_partial_count(int64_t n, int64_t* partial_count);

/*
 * Batched map-reduce over rows: out[b] = op over i < n of map(in[b*n + i]).
 * Replaces ReduceFunction.__call__ and its two generated stages
 * (vkdispatch/reduce/reduce_function.py:73-162, vkdispatch/reduce/
 * stage.py:147-186).  Two launches: per-CTA partials into `workspace`, then
 * one fixed-order pass per row, so results are deterministic for a given n.
 * in_type: VDX_F32, VDX_F64, VDX_I32, VDX_U32 or VDX_C64 (complex input needs
 * a map to a real value).  Output type: F32 for F32/C64 input, otherwise the
 * input type.  Bitwise ops require integer types.
 */
int vdx_reduce(int op, int map, int in_type, const void* in, int64_t n, int64_t batch, void* out,
               void* workspace, void* stream);

/*
 * vdx_reduce without a workspace: the same two launches and results, with
 * the stage-1 partials kept in a fixed device array inside libvdx.  This
 * entry point has no counterpart in the reference.
 *
 * It is for callers that cannot call cudaMalloc on the path that reduces:
 * host applications whose device memory is owned by their own pool
 * allocator, and latency-critical loops that cannot afford cudaMalloc's
 * implicit device-wide synchronisation.  The caller still passes `in` and
 * `out`; nothing is allocated or freed by this call.
 *
 *   - The array holds VDX_REDUCE_NOALLOC_SCRATCH_BYTES (1 MiB) on every GPU
 *     that loads libvdx, for the life of the process.  A request needing
 *     more (vdx_reduce_partial_count(n) * batch * output element size bytes)
 *     fails with VDX_ERR_UNSUPPORTED and launches nothing.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.  The address is cached per device and CUDA
 *     context, so the first call after a device reset looks it up again.
 *   - Every call shares the array, which keeps the last call's partials.
 *     Stage 1 writes every slot stage 2 reads, so nothing needs clearing, but
 *     calls that overlap on the GPU (other streams, other host threads) race
 *     on it: serialise them.
 */
#define VDX_REDUCE_NOALLOC_SCRATCH_BYTES 1048576
int vdx_reduce_noalloc(int op, int map, int in_type, const void* in, int64_t n, int64_t batch, void* out,
                       void* stream);

/*
 * Map hooks compiled at run time.  The reference injects arbitrary user code
 * at the FFT's loads, stores and spectrum multiply: input_map / output_map /
 * kernel_map callbacks traced into its generated shader
 * (vkdispatch/fft/io_manager.py:107-155, vkdispatch/shader/map.py:29-40,
 * compiled by vkdispatch/backends/cuda_backend/api_compute.py:30-70).  Here
 * the caller supplies those callbacks as a C++ source fragment defining
 *
 *   struct VdxHooks {
 *     template <class Re> __device__ static vdx::Cx<Re> load(const vdx::MapArgs& m, long long io, int k, int n);
 *     template <class Re> __device__ static void store(const vdx::MapArgs& m, vdx::Cx<Re> v, long long io,
 *                                                      int k, int n);
 *     template <class Re> __device__ static vdx::Cx<Re> kernel(const vdx::MapArgs& m, vdx::Cx<Re> v,
 *                                                               long long io, int k, int n);
 *   };
 *
 * (io = the element's flat index in the descriptor's shape, the reference's
 * io_index; k = fft_index; n = fft_size; m = the vdx_map_args of the call),
 * and libvdx compiles it with NVRTC into its own Stockham kernel template
 * (csrc/fft_mapped.cuh), specialised to the plan's compile-time radix list.
 * The descriptor is a C2C (load, passes, store) or CONV (load, forward,
 * kernel, inverse, store) descriptor of complex64 or complex128 compute with
 * io_type equal to compute_type; axes that need a four-step or Bluestein
 * plan are refused.  Compilation happens at plan creation (about a second;
 * cached per source, plan shape and device) and needs NVRTC and the CUDA
 * headers at run time (VDX_CUDA_INCLUDE or CUDA_HOME name them when they are
 * not in the default locations); its log is returned through
 * vdx_last_error on failure.  vdx_map_exec is one asynchronous launch.
 */
#define VDX_MAP_MAX_BUFFERS 8
#define VDX_MAP_MAX_SCALARS 8
typedef struct vdx_map_args {
  void* buffers[VDX_MAP_MAX_BUFFERS];  /* device pointers the hooks index */
  int64_t counts[VDX_MAP_MAX_BUFFERS]; /* elements each may be indexed with: an index outside
                                          [0, count) loads 0, skips its store and sets the
                                          plan's status (vdx_map_plan_status) */
  double fscalars[VDX_MAP_MAX_SCALARS]; /* floating-point map arguments */
  int64_t iscalars[VDX_MAP_MAX_SCALARS]; /* integer map arguments */
  int64_t kernel_index;                /* mapped_kernel_index() of a multi-kernel convolution */
} vdx_map_args;

typedef struct vdx_map_plan vdx_map_plan;
/* Plan creation compiles the mapped FFT shader (vkdispatch/fft/
 * shader_factories.py:11-60 with maps; io_manager.py:107-155); exec is its
 * launch (vkdispatch/shader/shader_function.py:277-380). */
int vdx_map_plan_create(const vdx_fft_desc* desc, const char* hooks_source, vdx_map_plan** plan);
int vdx_map_plan_destroy(vdx_map_plan* plan);
int vdx_map_exec(const vdx_map_plan* plan, const vdx_map_args* args, void* stream);
/* The full source NVRTC compiled for the plan (hooks and instantiation): the
 * reference's ShaderFunction.get_src (vkdispatch/shader/shader_function.py:
 * 258-275). */
int vdx_map_plan_source(const vdx_map_plan* plan, char* buf, size_t n);

/*
 * Map-reduce with a compiled map: the reference's vd.reduce.map_reduce (and
 * reduce(mapping_function=...)) with a mapping function outside vdx_reduce's
 * fixed maps, e.g. one that reads several buffers or scalars
 * (vkdispatch/reduce/stage.py:31-186, vkdispatch/reduce/reduce_function.py:
 * 73-162).  hooks_source defines
 *   struct VdxReduceHooks {
 *     template <class Re> __device__ static auto map(const vdx::MapArgs& m, long long io);
 *   };
 * returning the element value for flat index io = row * n + i (a real,
 * integer or vdx::Cx<Re> value; Cx lanes map to VDX_V2F32 components).
 * out_type: VDX_F32, VDX_F64, VDX_I32, VDX_U32 or VDX_V2F32; op: VDX_RED_*
 * (AND/OR/XOR only for VDX_I32 / VDX_U32).  Compiled with NVRTC at plan
 * creation.  vdx_reduce_map_exec runs the same two stages as vdx_reduce:
 * out[row] = op over i < n of map(row * n + i), with
 * vdx_reduce_partial_count(n) partials per row in `workspace` (elements of
 * out_type).  Map buffer indices outside their counts read 0 and set the
 * plan's status (vdx_reduce_map_plan_status).
 */
typedef struct vdx_reduce_map_plan vdx_reduce_map_plan;
int vdx_reduce_map_plan_create(const char* hooks_source, int op, int out_type, vdx_reduce_map_plan** plan);
int vdx_reduce_map_plan_destroy(vdx_reduce_map_plan* plan);
int vdx_reduce_map_exec(const vdx_reduce_map_plan* plan, const vdx_map_args* args, int64_t n, int64_t batch,
                        void* out, void* workspace, void* stream);
int vdx_reduce_map_plan_status(const vdx_reduce_map_plan* plan, int* status, int reset);
int vdx_reduce_map_plan_source(const vdx_reduce_map_plan* plan, char* buf, size_t n);
/* 1 when a launch of the plan indexed a map buffer out of range, else 0
 * (synchronous read; reset != 0 clears it).  No counterpart in the
 * reference. */
int vdx_map_plan_status(const vdx_map_plan* plan, int* status, int reset);

#ifdef __cplusplus
}
#endif

#endif /* VDX_H */
