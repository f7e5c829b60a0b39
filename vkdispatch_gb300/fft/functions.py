"""Public FFT API with the reference's signatures and semantics
(vkdispatch/fft/functions.py:104-713): in-place transforms on Buffers,
per-axis passes for 2-D / 3-D, packed real transforms on RFFTBuffers, and
fused convolutions that multiply by the conjugate kernel spectrum.

Each call resolves precisions (vkdispatch/fft/precision.py:67-99), fetches a
cached plan and records one launch into the graph (immediate by default).
"""

from __future__ import annotations

import math
import os
from typing import Optional, Tuple, Union

from .. import _lib as L
from .. import dtypes as dt
from .. import graph as G
from ..buffer import Buffer, RFFTBuffer
from . import plan as P
from .maps import read_op, write_op  # noqa: F401

_PRECISION_ORDER = (dt.complex32, dt.complex64, dt.complex128)

# validated get_plan arguments of the plain in-place path of fft(), keyed by
# the call's arguments: repeated calls skip the dtype and shape checks
_plain_args = {}


def _validate_complex(t, arg: str) -> None:
    if t not in _PRECISION_ORDER and t != dt.complexbf16:
        raise ValueError(f"{arg} must be one of complex32, complex64, or complex128 (got {t})")


def resolve_compute_precision(io_types, compute_type: Optional[dt.dtype]) -> dt.dtype:
    """Reference rule: explicit compute_type wins; otherwise the widest I/O
    precision, at least complex64."""
    if compute_type is not None:
        _validate_complex(compute_type, "compute_type")
        return compute_type
    if not io_types:
        return dt.complex64
    for t in io_types:
        _validate_complex(t, "io_precision")
    rank = max(_PRECISION_ORDER.index(t) if t in _PRECISION_ORDER else 0 for t in io_types)
    return _PRECISION_ORDER[max(rank, 1)]


def _compute_code(io_type: dt.dtype, compute: dt.dtype) -> int:
    # complex32 compute runs with fp32 butterflies (never less accurate than asked)
    if compute in (dt.complex32, dt.complex64, dt.complexbf16):
        return L.VDX_C64
    return L.VDX_C128


def _norm_axis(axis: Optional[int], ndim: int) -> int:
    if axis is None:
        return ndim - 1
    if axis < 0:
        axis += ndim
    if not 0 <= axis < ndim:
        raise ValueError(f"axis {axis} out of range for {ndim} dimensions")
    return axis


_TORCH_OF = {"complex64": "complex64", "complex128": "complex128"}


def _native_pair(io_t: dt.dtype, compute: dt.dtype) -> bool:
    """(storage, compute) pairs the kernels run directly."""
    c = _compute_code(io_t, compute)
    if io_t == dt.complex128:
        return c == L.VDX_C128
    return c == L.VDX_C64 and io_t in (dt.complex64, dt.complex32, dt.complexbf16)


def _compute_torch(compute: dt.dtype):
    import torch

    return torch.complex128 if _compute_code(None, compute) == L.VDX_C128 else torch.complex64


def _split_buffers(buffers, input_map, output_map, kernel_map=None, conv=False):
    """The reference's argument order: output-map buffers (or the output
    buffer), input-map buffers (or, with only an output map, one input buffer),
    kernel-map buffers (or the kernel buffer) -- vkdispatch/fft/
    io_manager.py:58-105."""
    n_out = len(output_map.buffer_types) if output_map is not None else 1
    outs = list(buffers[:n_out])
    rest = list(buffers[n_out:])
    if input_map is not None:
        n_in = len(input_map.buffer_types)
        ins, rest = rest[:n_in], rest[n_in:]
    elif output_map is not None:
        if not rest:
            raise ValueError("When output_map is used without input_map, an input buffer argument must be provided "
                             "after output_map arguments")
        ins, rest = rest[:1], rest[1:]
    else:
        ins = None
    if conv:
        n_k = len(kernel_map.buffer_types) if kernel_map is not None else 1
        kers, rest = rest[:n_k], rest[n_k:]
    else:
        kers = []
    return outs, ins, kers


def _io_ends(outs, ins, input_map, output_map):
    """(out buffer, out kind, in buffer, in kind) after map recognition."""
    from . import maps as M

    if output_map is not None:
        om = M.classify_output(output_map)
        out_buf, out_kind = outs[om.buffer], om.kind
        if out_buf.var_type != om.var_type:
            raise ValueError(f"output map buffer type {out_buf.var_type.name} does not match its annotation")
    else:
        out_buf, out_kind = outs[0], "complex"
    if input_map is not None:
        im = M.classify_input(input_map)
        in_buf, in_kind = ins[im.buffer], im.kind
        if in_buf.var_type != im.var_type:
            raise ValueError(f"input map buffer type {in_buf.var_type.name} does not match its annotation")
    elif ins is not None:
        in_buf, in_kind = ins[0], "complex"
    else:
        in_buf, in_kind = out_buf, out_kind
    return out_buf, out_kind, in_buf, in_kind


def _staged(plan_fn, out_buf, out_kind, in_buf, in_kind, shape, compute, graph, ker=None, keep=(), pre=None):
    """Runs a compute-precision plan between buffers of other types: the
    input is converted into a compute-type buffer unless it already is one,
    the plan runs out of place into the output (or a staging buffer), and the
    staging buffer is converted into the output's type."""
    import torch

    ct = _compute_torch(compute)
    code = L.VDX_C128 if ct == torch.complex128 else L.VDX_C64
    count = math.prod(shape)
    in_direct = in_kind == "complex" and in_buf.var_type.vdx_code == code
    out_direct = out_kind == "complex" and out_buf.var_type.vdx_code == code
    stage_in = None if in_direct else torch.empty(count, dtype=ct, device=in_buf.tensor.device)
    stage_out = None if out_direct else torch.empty(count, dtype=ct, device=out_buf.tensor.device)
    plan = plan_fn(code)
    in_ptr, in_type = in_buf.ptr, in_buf.var_type.vdx_code
    out_ptr, out_type = out_buf.ptr, out_buf.var_type.vdx_code
    if in_kind == "real":
        in_type = L.VDX_F32 if in_buf.var_type == dt.float32 else L.VDX_F64
    if out_kind == "real":
        out_type = L.VDX_F32 if out_buf.var_type == dt.float32 else L.VDX_F64

    def launch(s):
        if pre is not None:
            pre(s)
        src = in_ptr
        if stage_in is not None:
            L.convert(in_ptr, in_type, stage_in.data_ptr(), code, count, s)
            src = stage_in.data_ptr()
        dst = out_ptr if stage_out is None else stage_out.data_ptr()
        plan.exec(src, dst, ker, s)
        if stage_out is not None:
            L.convert(stage_out.data_ptr(), code, out_ptr, out_type, count, s)

    _record(graph, launch, (in_buf, out_buf, stage_in, stage_out) + tuple(keep))


def _strided(*groups) -> bool:
    """Whether any Buffer among the arguments addresses a non-contiguous array."""
    return any(isinstance(b, Buffer) and not b.contiguous for g in groups for b in (g or ()))


def _check_strided_defaults(shape, slab, bufs, kernel) -> None:
    """A non-contiguous buffer read or written without a map is addressed by
    the transform's own io_index, so it must have the transform's shape (a
    broadcast kernel: the shape of one slab)."""
    for b in bufs:
        if isinstance(b, Buffer) and not b.contiguous and tuple(b.shape) != tuple(shape):
            raise ValueError(f"a non-contiguous buffer of shape {b.shape} needs buffer_shape == its shape")
    if isinstance(kernel, Buffer) and not kernel.contiguous and kernel.size not in (math.prod(shape), slab):
        raise ValueError(f"a non-contiguous kernel of shape {kernel.shape} must hold one slab or the whole signal")


def _signal(sr, N: int) -> Optional[Tuple[int, int]]:
    if sr is None:
        return None
    lo, hi = sr
    lo = 0 if lo is None else int(lo)
    hi = N if hi is None else int(hi)
    if lo == 0 and hi == N:
        return None
    return (lo, hi)


def _record(graph, launch, keep=()) -> None:
    G.resolve(graph).record(launch, keep)


def fft(
    *buffers: Buffer,
    buffer_shape: Tuple = None,
    graph: G.CommandGraph = None,
    print_shader: bool = False,
    axis: int = None,
    name: str = None,
    inverse: bool = False,
    normalize_inverse: bool = True,
    r2c: bool = False,
    input_map=None,
    output_map=None,
    output_type: dt.dtype = None,
    input_type: dt.dtype = None,
    compute_type: dt.dtype = None,
    input_signal_range: Union[Tuple[Optional[int], Optional[int]], None] = None,
):
    if len(buffers) < 1:
        raise ValueError("At least one buffer must be provided")
    if input_map is None and output_map is None and len(buffers) != 1:
        raise ValueError("fft() expects exactly one buffer unless input_map/output_map are used")
    if input_map is not None or output_map is not None:
        if r2c:
            raise NotImplementedError("map hooks on real (r2c) transforms are not in the supported menu")
        if input_map is not None and input_type is not None:
            raise ValueError("input_type cannot be provided when input_map is used")
        if output_map is not None and output_type is not None:
            raise ValueError("output_type cannot be provided when output_map is used")
        outs, ins, _ = _split_buffers(buffers, input_map, output_map)
        try:
            if _strided(outs, ins):
                raise NotImplementedError("non-contiguous buffers")
            out_buf, out_kind, in_buf, in_kind = _io_ends(outs, ins, input_map, output_map)
        except NotImplementedError as menu:
            _jit_transform(outs, ins, [], input_map, output_map, None, False, buffer_shape, axis, inverse,
                           bool(inverse and normalize_inverse), compute_type, input_signal_range, graph, print_shader,
                           menu)
            return
        io = []
        if output_map is None:
            io.append(out_buf.var_type)
        if input_map is None:
            io.append(in_buf.var_type if input_type is None else input_type)
        compute = resolve_compute_precision(io, compute_type)
        shape = tuple(int(x) for x in (buffer_shape if buffer_shape is not None else buffers[0].shape))
        ax = _norm_axis(axis, len(shape))
        sr = _signal(input_signal_range, shape[ax])
        _staged(lambda code: P.get_plan(shape, ax, L.VDX_KIND_C2C, inverse, bool(inverse and normalize_inverse), code,
                                        code, sr),
                out_buf, out_kind, in_buf, in_kind, shape, compute, graph)
        return
    buf = buffers[0]
    if not buf.contiguous:
        if r2c:
            raise ValueError("R2C/C2R transforms need a contiguous buffer")
        _jit_transform([buf], [], [], None, None, None, False, buffer_shape, axis, inverse,
                       bool(inverse and normalize_inverse), compute_type, input_signal_range, graph, print_shader,
                       "non-contiguous buffer")
        return
    memo_key = (buf.var_type, buf.shape, buf.size, None if buffer_shape is None else tuple(buffer_shape), axis,
                bool(inverse), bool(normalize_inverse), bool(r2c), output_type, input_type, compute_type,
                None if input_signal_range is None else tuple(input_signal_range))
    args = _plain_args.get(memo_key)
    if args is not None:
        plan = P.get_plan(*args)
        if print_shader:
            print(plan.describe())
        ptr = buf.ptr
        _record(graph, lambda s: plan.exec(ptr, ptr, None, s), (buf,))
        return
    if buffer_shape is None:
        buffer_shape = buf.shape
    buffer_shape = tuple(int(s) for s in buffer_shape)
    out_t = buf.var_type if output_type is None else output_type
    _validate_complex(out_t, "output_type")
    in_t = out_t if input_type is None else input_type
    _validate_complex(in_t, "input_type")
    if in_t != out_t:
        raise ValueError("input_type must match output_type when input_map is None (default FFT path is in-place)")
    if out_t != buf.var_type:
        raise ValueError(f"output_type {out_t.name} does not match the buffer type {buf.var_type.name}")
    compute = resolve_compute_precision([out_t, in_t], compute_type)
    ax = _norm_axis(axis, len(buffer_shape))
    N = buffer_shape[ax]
    if not r2c and not _native_pair(out_t, compute):
        # e.g. complex64 storage with complex128 compute: stage through the compute type
        _staged(lambda code: P.get_plan(buffer_shape, ax, L.VDX_KIND_C2C, inverse, bool(inverse and normalize_inverse),
                                        code, code, _signal(input_signal_range, N)),
                buf, "complex", buf, "complex", buffer_shape, compute, graph)
        return
    if r2c:
        if ax != len(buffer_shape) - 1:
            raise ValueError("R2C io only supported for contiguous data")
        expect = buffer_shape[:-1] + (buffer_shape[-1] // 2 + 1,)
        if tuple(buf.shape) != expect:
            raise ValueError(f"R2C buffer of shape {buf.shape} does not match real shape {buffer_shape}")
        kind = L.VDX_KIND_C2R if inverse else L.VDX_KIND_R2C
    else:
        if math.prod(buffer_shape) > buf.size:
            raise ValueError(f"buffer_shape {buffer_shape} exceeds the buffer size {buf.size}")
        kind = L.VDX_KIND_C2C
    args = (buffer_shape, ax, kind, inverse, bool(inverse and normalize_inverse), out_t.vdx_code,
            _compute_code(out_t, compute), _signal(input_signal_range, N))
    plan = P.get_plan(*args)
    _plain_args[memo_key] = args
    if print_shader:
        print(plan.describe())
    ptr = buf.ptr
    _record(graph, lambda s: plan.exec(ptr, ptr, None, s), (buf,))


def fft2(buffer: Buffer, graph=None, print_shader=False, input_map=None, output_map=None, output_type=None,
         input_type=None, compute_type=None):
    if len(buffer.shape) not in (2, 3):
        raise ValueError("Buffer must have 2 or 3 dimensions")
    if (input_map is None and output_map is None and output_type in (None, dt.complex64)
            and input_type in (None, dt.complex64) and compute_type in (None, dt.complex64) and _groupable(buffer)
            and _axes_split(buffer, [(L.VDX_KIND_C2C, 1, False, False, None), (L.VDX_KIND_C2C, 2, False, False, None)],
                            graph, print_shader)):
        return
    kw = dict(graph=graph, print_shader=print_shader, output_type=output_type, input_type=input_type,
              compute_type=compute_type)
    fft(buffer, axis=len(buffer.shape) - 2, input_map=input_map, **kw)
    fft(buffer, axis=len(buffer.shape) - 1, output_map=output_map, **kw)


def fft3(buffer: Buffer, graph=None, print_shader=False, input_map=None, output_map=None, output_type=None,
         input_type=None, compute_type=None):
    if len(buffer.shape) != 3:
        raise ValueError("Buffer must have 3 dimensions")
    kw = dict(graph=graph, print_shader=print_shader, output_type=output_type, input_type=input_type,
              compute_type=compute_type)
    fft(buffer, axis=0, input_map=input_map, **kw)
    fft(buffer, axis=1, **kw)
    fft(buffer, axis=2, output_map=output_map, **kw)


def ifft(buffer: Buffer, graph=None, print_shader=False, axis=None, name=None, normalize=True, input_map=None,
         output_map=None, output_type=None, input_type=None, compute_type=None):
    fft(buffer, graph=graph, print_shader=print_shader, axis=axis, name=name, inverse=True,
        normalize_inverse=normalize, input_map=input_map, output_map=output_map, output_type=output_type,
        input_type=input_type, compute_type=compute_type)


def ifft2(buffer: Buffer, graph=None, print_shader=False, normalize=True, input_map=None, output_map=None,
          output_type=None, input_type=None, compute_type=None):
    if len(buffer.shape) not in (2, 3):
        raise ValueError("Buffer must have 2 or 3 dimensions")
    if (input_map is None and output_map is None and output_type in (None, dt.complex64)
            and input_type in (None, dt.complex64) and compute_type in (None, dt.complex64) and _groupable(buffer)
            and _axes_split(buffer, [(L.VDX_KIND_C2C, 1, True, bool(normalize), None),
                                     (L.VDX_KIND_C2C, 2, True, bool(normalize), None)], graph, print_shader)):
        return
    kw = dict(graph=graph, print_shader=print_shader, normalize=normalize, output_type=output_type,
              input_type=input_type, compute_type=compute_type)
    ifft(buffer, axis=len(buffer.shape) - 2, input_map=input_map, **kw)
    ifft(buffer, axis=len(buffer.shape) - 1, output_map=output_map, **kw)


def ifft3(buffer: Buffer, graph=None, print_shader=False, normalize=True, input_map=None, output_map=None,
          output_type=None, input_type=None, compute_type=None):
    if len(buffer.shape) != 3:
        raise ValueError("Buffer must have 3 dimensions")
    kw = dict(graph=graph, print_shader=print_shader, normalize=normalize, output_type=output_type,
              input_type=input_type, compute_type=compute_type)
    ifft(buffer, axis=0, input_map=input_map, **kw)
    ifft(buffer, axis=1, **kw)
    ifft(buffer, axis=2, output_map=output_map, **kw)


def rfft(buffer: RFFTBuffer, graph=None, print_shader=False, name=None, compute_type=None):
    fft(buffer, buffer_shape=buffer.real_shape, graph=graph, print_shader=print_shader, name=name, r2c=True,
        output_type=buffer.var_type, input_type=buffer.var_type, compute_type=compute_type)


def rfft2(buffer: RFFTBuffer, graph=None, print_shader=False, compute_type=None):
    if len(buffer.real_shape) not in (2, 3):
        raise ValueError("Buffer must have 2 or 3 dimensions")
    if (compute_type in (None, dt.complex64) and len(buffer.real_shape) == 3 and _groupable(buffer)
            and _axes_split(buffer, [(L.VDX_KIND_R2C, 2, False, False, buffer.real_shape),
                                     (L.VDX_KIND_C2C, 1, False, False, None)], graph, print_shader)):
        return
    rfft(buffer, graph=graph, print_shader=print_shader, compute_type=compute_type)
    fft(buffer, graph=graph, print_shader=print_shader, axis=len(buffer.real_shape) - 2,
        output_type=buffer.var_type, input_type=buffer.var_type, compute_type=compute_type)


def rfft3(buffer: RFFTBuffer, graph=None, print_shader=False, compute_type=None):
    if len(buffer.real_shape) != 3:
        raise ValueError("Buffer must have 3 dimensions")
    rfft(buffer, graph=graph, print_shader=print_shader, compute_type=compute_type)
    for ax in (1, 0):
        fft(buffer, graph=graph, print_shader=print_shader, axis=ax, output_type=buffer.var_type,
            input_type=buffer.var_type, compute_type=compute_type)


def irfft(buffer: RFFTBuffer, graph=None, print_shader=False, name=None, normalize=True, compute_type=None):
    fft(buffer, buffer_shape=buffer.real_shape, graph=graph, print_shader=print_shader, name=name, inverse=True,
        normalize_inverse=normalize, r2c=True, output_type=buffer.var_type, input_type=buffer.var_type,
        compute_type=compute_type)


def irfft2(buffer: RFFTBuffer, graph=None, print_shader=False, normalize=True, compute_type=None):
    if len(buffer.real_shape) not in (2, 3):
        raise ValueError("Buffer must have 2 or 3 dimensions")
    if (compute_type in (None, dt.complex64) and len(buffer.real_shape) == 3 and _groupable(buffer)
            and _axes_split(buffer, [(L.VDX_KIND_C2C, 1, True, bool(normalize), None),
                                     (L.VDX_KIND_C2R, 2, True, bool(normalize), buffer.real_shape)], graph,
                            print_shader)):
        return
    ifft(buffer, graph=graph, print_shader=print_shader, axis=len(buffer.real_shape) - 2, normalize=normalize,
         output_type=buffer.var_type, input_type=buffer.var_type, compute_type=compute_type)
    irfft(buffer, graph=graph, print_shader=print_shader, normalize=normalize, compute_type=compute_type)


def irfft3(buffer: RFFTBuffer, graph=None, print_shader=False, normalize=True, compute_type=None):
    if len(buffer.real_shape) != 3:
        raise ValueError("Buffer must have 3 dimensions")
    for ax in (0, 1):
        ifft(buffer, graph=graph, print_shader=print_shader, axis=ax, normalize=normalize,
             output_type=buffer.var_type, input_type=buffer.var_type, compute_type=compute_type)
    irfft(buffer, graph=graph, print_shader=print_shader, normalize=normalize, compute_type=compute_type)


def convolve(
    *buffers: Buffer,
    kernel_map=None,
    kernel_num: int = 1,
    buffer_shape: Tuple = None,
    graph: G.CommandGraph = None,
    print_shader: bool = False,
    axis: int = None,
    normalize: bool = True,
    name: str = None,
    transposed_kernel: bool = False,
    kernel_inner_only: bool = False,
    input_map=None,
    output_map=None,
    output_type: dt.dtype = None,
    input_type: dt.dtype = None,
    kernel_type: dt.dtype = None,
    compute_type: dt.dtype = None,
    input_signal_range=None,
):
    """In-place FFT -> spectrum * conj(kernel) -> inverse FFT along `axis`, in
    one kernel.  The kernel spectrum is read at the signal's own index
    (vkdispatch/fft/io_manager.py:181-187), or from one slab shared by all
    outer batches when kernel_inner_only is set (or when the kernel buffer
    holds exactly one slab)."""
    if len(buffers) < 1:
        raise ValueError("At least one buffer must be provided")
    if kernel_map is None and len(buffers) < 2:
        raise ValueError("convolve() requires at least an output buffer and kernel buffer")
    if kernel_num < 1:
        raise ValueError("kernel_num must be >= 1")
    if kernel_num > 1:
        _convolve_multi(buffers, kernel_map, kernel_num, buffer_shape, graph, axis, normalize, kernel_inner_only,
                        input_map, output_map, compute_type, input_signal_range)
        return
    if input_map is not None or output_map is not None or kernel_map is not None:
        _convolve_mapped(buffers, kernel_map, buffer_shape, graph, axis, normalize, kernel_inner_only, input_map,
                         output_map, compute_type, input_signal_range)
        return
    buf, ker = buffers[0], buffers[1]
    if _strided([buf, ker]):
        _jit_transform([buf], [], [ker], None, None, None, True, buffer_shape, axis, False, bool(normalize),
                       compute_type, input_signal_range, graph, print_shader, "non-contiguous buffer",
                       kernel_inner_only=kernel_inner_only)
        return
    if buffer_shape is None:
        buffer_shape = buf.shape
    buffer_shape = tuple(int(s) for s in buffer_shape)
    out_t = buf.var_type if output_type is None else output_type
    in_t = out_t if input_type is None else input_type
    k_t = ker.var_type if kernel_type is None else kernel_type
    for t, nm in ((out_t, "output_type"), (in_t, "input_type"), (k_t, "kernel_type")):
        _validate_complex(t, nm)
    if in_t != out_t:
        raise ValueError("input_type must match output_type when input_map is None (default FFT path is in-place)")
    if k_t != ker.var_type or out_t != buf.var_type:
        raise ValueError("kernel_type/output_type must match the buffers' types")
    compute = resolve_compute_precision([out_t, in_t, k_t], compute_type)
    ax = _norm_axis(axis, len(buffer_shape))
    total = math.prod(buffer_shape)
    slab = math.prod(buffer_shape[ax:])
    broadcast = bool(kernel_inner_only)
    if not broadcast and ker.size < total:
        if ker.size >= slab:
            broadcast = True
        else:
            raise ValueError(f"kernel buffer of {ker.size} elements is smaller than the signal ({total})")
    plan = P.get_plan(
        buffer_shape,
        ax,
        L.VDX_KIND_CONV,
        False,
        normalize,
        out_t.vdx_code,
        _compute_code(out_t, compute),
        _signal(input_signal_range, buffer_shape[ax]),
        L.VDX_KOP_MUL_CONJ,
        k_t.vdx_code,
        broadcast,
    )
    if print_shader:
        print(plan.describe())
    ptr, kptr = buf.ptr, ker.ptr
    _record(graph, lambda s: plan.exec(ptr, ptr, kptr, s), (buf, ker))


def _convolve_mapped(buffers, kernel_map, buffer_shape, graph, axis, normalize, kernel_inner_only, input_map,
                     output_map, compute_type, input_signal_range):
    import torch

    from . import maps as M

    outs, ins, kers = _split_buffers(buffers, input_map, output_map, kernel_map, conv=True)
    try:
        if _strided(outs, ins, kers):
            raise NotImplementedError("non-contiguous buffers")
        out_buf, out_kind, in_buf, in_kind = _io_ends(outs, ins, input_map, output_map)
        km = M.classify_kernel(kernel_map) if kernel_map is not None else M.KernelMap("conj_mul", 0,
                                                                                     kers[0].var_type)
    except NotImplementedError as menu:
        _jit_transform(outs, ins, kers, input_map, output_map, kernel_map, True, buffer_shape, axis, False,
                       bool(normalize), compute_type, input_signal_range, graph, False, menu,
                       kernel_inner_only=kernel_inner_only)
        return
    io = []
    if output_map is None:
        io.append(out_buf.var_type)
    if input_map is None:
        io.append(in_buf.var_type)
    if kernel_map is None:
        io.append(kers[0].var_type)
    compute = resolve_compute_precision(io, compute_type)
    shape = tuple(int(x) for x in (buffer_shape if buffer_shape is not None else buffers[0].shape))
    ax = _norm_axis(axis, len(shape))
    sr = _signal(input_signal_range, shape[ax])
    total, slab = math.prod(shape), math.prod(shape[ax:])
    if km.kind == "identity":
        # no spectrum operation: the forward and inverse transforms cancel up to 1/N
        def plan_fn(code):
            class _Pair:
                def __init__(self):
                    self.f = P.get_plan(shape, ax, L.VDX_KIND_C2C, False, False, code, code, sr)
                    self.i = P.get_plan(shape, ax, L.VDX_KIND_C2C, True, bool(normalize), code, code)

                def exec(self, src, dst, ker, s):
                    self.f.exec(src, dst, None, s)
                    self.i.exec(dst, dst, None, s)

            return _Pair()

        _staged(plan_fn, out_buf, out_kind, in_buf, in_kind, shape, compute, graph)
        return
    kbuf = kers[km.buffer]
    ct = _compute_torch(compute)
    code = L.VDX_C128 if ct == torch.complex128 else L.VDX_C64
    pre = None
    if kbuf.var_type.vdx_code == code and km.kind != "real_scale":
        kptr, keep = kbuf.ptr, (kbuf,)
    else:
        # real scale buffers (or other precisions) become a compute-type
        # spectrum, converted inside the launch so recorded graphs see the
        # kernel buffer's contents at submit time
        kt = torch.empty(kbuf.size, dtype=ct, device=kbuf.tensor.device)
        src_type = {dt.float32: L.VDX_F32, dt.float64: L.VDX_F64}.get(kbuf.var_type, kbuf.var_type.vdx_code)
        kptr, keep = kt.data_ptr(), (kbuf, kt)
        kb_ptr, kb_n = kbuf.ptr, kbuf.size

        def pre(s):
            L.convert(kb_ptr, src_type, kptr, code, kb_n, s)
    kop = L.VDX_KOP_MUL_CONJ if km.kind == "conj_mul" else L.VDX_KOP_MUL
    if kop == L.VDX_KOP_MUL and code != L.VDX_C64:
        raise NotImplementedError("plain-product kernel maps need complex64 compute")
    broadcast = bool(kernel_inner_only) or (kbuf.size < total and kbuf.size >= slab)
    if not broadcast and kbuf.size < total:
        raise ValueError(f"kernel buffer of {kbuf.size} elements is smaller than the signal ({total})")
    _staged(lambda c: P.get_plan(shape, ax, L.VDX_KIND_CONV, False, normalize, c, c, sr, kop, c, broadcast),
            out_buf, out_kind, in_buf, in_kind, shape, compute, graph, ker=kptr, keep=keep, pre=pre)


def _convolve_multi(buffers, kernel_map, kernel_num, buffer_shape, graph, axis, normalize, kernel_inner_only,
                    input_map, output_map, compute_type, input_signal_range):
    """kernel_num convolutions of one signal (vkdispatch/fft/shader_factories.py:
    166-193): for kernel k the kernel map reads, and the output map writes,
    ``io_index + mapped_kernel_index() * C`` -- C * k elements along their
    buffers (C = 0 when the map does not use the index).  One fused
    convolution launch for all kernels (the signal read and transformed
    once) where the plan has such a kernel, else one fused convolution launch
    per kernel; the signal is read from a copy when an output slice overlaps
    it, so every kernel sees the original signal, as in the reference's
    single pass over the input."""
    import torch

    from . import maps as M

    outs, ins, kers = _split_buffers(buffers, input_map, output_map, kernel_map, conv=True)
    try:
        if _strided(outs, ins, kers):
            raise NotImplementedError("non-contiguous buffers")
        _classify_multi(input_map, output_map, kernel_map)
    except NotImplementedError as menu:
        _jit_transform(outs, ins, kers, input_map, output_map, kernel_map, True, buffer_shape, axis, False,
                       bool(normalize), compute_type, input_signal_range, graph, False, menu,
                       kernel_inner_only=kernel_inner_only, kernel_num=kernel_num)
        return
    if output_map is not None:
        om = M.classify_output(output_map)
        if om.kind != "complex":
            raise NotImplementedError("multi-kernel convolutions write complex outputs")
        out_buf, ostride = outs[om.buffer], om.stride
    else:
        out_buf, ostride = outs[0], 0
    if input_map is not None:
        im = M.classify_input(input_map)
        if im.kind != "complex":
            raise NotImplementedError("multi-kernel convolutions read complex inputs")
        in_buf = ins[im.buffer]
    else:
        in_buf = ins[0] if ins else out_buf
    if kernel_map is not None:
        km = M.classify_kernel(kernel_map)
        if km.kind not in ("conj_mul", "mul"):
            raise NotImplementedError(f"kernel map {kernel_map.func.__name__}: multi-kernel convolutions take a "
                                      "(conjugate) product with a kernel buffer")
        kbuf, kstride, kind = kers[km.buffer], km.stride, km.kind
    else:
        kbuf, kstride, kind = kers[0], 0, "conj_mul"
    vt = out_buf.var_type
    if in_buf.var_type != vt or kbuf.var_type != vt or vt not in (dt.complex64, dt.complex128):
        raise NotImplementedError("multi-kernel convolutions need complex64 (or complex128) signal, kernel and output")
    compute = resolve_compute_precision([vt], compute_type)
    code = vt.vdx_code
    if _compute_code(vt, compute) != code:
        raise NotImplementedError("multi-kernel convolutions compute in their storage precision")
    shape = tuple(int(x) for x in (buffer_shape if buffer_shape is not None else in_buf.shape))
    ax = _norm_axis(axis, len(shape))
    total, slab = math.prod(shape), math.prod(shape[ax:])
    broadcast = bool(kernel_inner_only) or (kbuf.size - (kernel_num - 1) * kstride < total)
    need_k = (kernel_num - 1) * kstride + (slab if broadcast else total)
    if kbuf.size < need_k:
        raise ValueError(f"kernel buffer of {kbuf.size} elements is smaller than the {need_k} the kernels need")
    if out_buf.size < (kernel_num - 1) * ostride + total or in_buf.size < total:
        raise ValueError("output buffer too small for kernel_num slices of the signal shape")
    kop = L.VDX_KOP_MUL_CONJ if kind == "conj_mul" else L.VDX_KOP_MUL
    plan = P.get_plan(shape, ax, L.VDX_KIND_CONV, False, normalize, code, code, _signal(input_signal_range, shape[ax]),
                      kop, code, broadcast)
    es = vt.item_size
    in_ptr, out_ptr, k_ptr = in_buf.ptr, out_buf.ptr, kbuf.ptr
    in_end, out_end = in_ptr + total * es, out_ptr + ((kernel_num - 1) * ostride + total) * es
    # the first kernel_num - 1 outputs must not overwrite the signal the later kernels read
    overlap = in_ptr < out_end and out_ptr < in_end
    stage = torch.empty(total, dtype=vt.torch_dtype, device=in_buf.tensor.device) if overlap else None

    def launch(s):
        src = in_ptr
        if stage is not None:
            L.convert(in_ptr, code, stage.data_ptr(), code, total, s)
            src = stage.data_ptr()
        if plan.exec_multi(src, out_ptr, k_ptr, kernel_num, kstride, ostride, s):
            return
        for k in range(kernel_num):
            plan.exec(src, out_ptr + k * ostride * es, k_ptr + k * kstride * es, s)

    _record(graph, launch, (in_buf, out_buf, kbuf, stage))


def _classify_multi(input_map, output_map, kernel_map) -> None:
    """Raises NotImplementedError when a multi-kernel convolution's maps are
    outside what the fused multi-kernel launch implements."""
    from . import maps as M

    if output_map is not None and M.classify_output(output_map).kind != "complex":
        raise NotImplementedError("multi-kernel convolutions write complex outputs")
    if input_map is not None and M.classify_input(input_map).kind != "complex":
        raise NotImplementedError("multi-kernel convolutions read complex inputs")
    if kernel_map is not None and M.classify_kernel(kernel_map).kind not in ("conj_mul", "mul"):
        raise NotImplementedError("multi-kernel convolutions take a (conjugate) product with a kernel buffer")


def _first_buffer(*groups):
    for g in groups:
        for b in g or ():
            if isinstance(b, Buffer):
                return b
    raise ValueError("at least one Buffer argument is required")


def _jit_transform(outs, ins, kers, input_map, output_map, kernel_map, conv, buffer_shape, axis, inverse, normalize,
                   compute_type, input_signal_range, graph, print_shader, menu_error, kernel_inner_only=False,
                   kernel_num=1):
    """An FFT or convolution whose maps are outside the functor menu: the
    maps are lowered to a C++ hooks struct and compiled with NVRTC into the
    FFT kernel template (vkdispatch_gb300/fft/jit.py).  A multi-kernel
    convolution runs one launch per kernel index; when the output may
    overwrite the signal it reads, the signal is read from a copy, so every
    kernel sees the original signal."""
    import torch

    from . import jit as J

    io = []
    if output_map is None:
        io.append(outs[0].var_type)
    if input_map is None:
        io.append((ins[0] if ins else outs[0]).var_type)
    if conv and kernel_map is None:
        io.append(kers[0].var_type)
    for t in io:
        if t not in _PRECISION_ORDER:
            raise ValueError(f"buffers without a map must be complex (got {t.name})")
    compute = resolve_compute_precision(io, compute_type)
    code = _compute_code(None, compute)
    first = _first_buffer(outs, ins, kers)
    shape = tuple(int(x) for x in (buffer_shape if buffer_shape is not None else first.shape))
    ax = _norm_axis(axis, len(shape))
    total, slab = math.prod(shape), math.prod(shape[ax:])
    _check_strided_defaults(shape, slab,
                            ([outs[0]] if output_map is None else []) + ([(ins or outs)[0]] if input_map is None else []),
                            kers[0] if conv and kernel_map is None else None)
    bslab = 0
    if conv and kernel_map is None:
        kb = kers[0]
        if kernel_inner_only or kb.size < total:
            if kb.size < slab:
                raise ValueError(f"kernel buffer of {kb.size} elements is smaller than the signal ({total})")
            bslab = slab
    stage = stage_src = None
    if kernel_num > 1 and input_map is None:
        # the signal the default load reads, copied when an output buffer aliases it
        src = ins[0] if ins else outs[0]
        if any(isinstance(b, Buffer) and b.ptr == src.ptr for b in outs):
            stage, stage_src = Buffer(src.shape, src.var_type), src
            ins = [stage]
    try:
        spec = J.build_hooks(outs, ins, kers, input_map, output_map, kernel_map, conv, bslab)
    except NotImplementedError as e:
        raise NotImplementedError(f"{menu_error}; and the map-hook compiler: {e}") from e
    plan = J.get_plan(shape, ax, conv, inverse, 1 if normalize else 0, code, _signal(input_signal_range, shape[ax]),
                      spec.source)
    if print_shader:
        print(plan.source())
    slots = spec.slots

    def launch(s):
        if stage is not None:
            n = stage_src.tensor.numel()
            with torch.cuda.stream(torch.cuda.ExternalStream(s) if s else torch.cuda.current_stream()):
                stage.tensor.reshape(-1)[:n].copy_(stage_src.tensor.reshape(-1), non_blocking=True)
        for k in range(kernel_num):
            plan.exec(J.make_args(slots, k), s)

    _record(graph, launch, tuple(slots.buffers) + ((stage,) if stage is not None else ()))


def convolve2D(buffer: Buffer, kernel: Buffer, kernel_map=None, buffer_shape=None, graph=None, print_shader=False,
               normalize=True, transposed_kernel=False, kernel_inner_only=False, input_map=None, output_map=None,
               output_type=None, input_type=None, kernel_type=None, compute_type=None):
    if len(buffer.shape) not in (2, 3):
        raise ValueError("Buffer must have 2 or 3 dimensions")
    if (kernel_map is None and buffer_shape is None and not transposed_kernel and input_map is None
            and output_map is None and output_type in (None, dt.complex64) and input_type in (None, dt.complex64)
            and kernel_type in (None, dt.complex64) and compute_type in (None, dt.complex64)
            and _groupable(buffer, kernel) and len(buffer.shape) == 3):
        broadcast = _kernel_broadcast(buffer, kernel, kernel_inner_only)
        shape = tuple(int(x) for x in buffer.shape)
        steps = [(shape, 2, L.VDX_KIND_C2C, False, False, False),
                 (shape, 1, L.VDX_KIND_CONV, False, bool(normalize), broadcast),
                 (shape, 2, L.VDX_KIND_C2C, True, bool(normalize), False)]
        if _image_groups(buffer, graph, (buffer, kernel), steps, print_shader, kernel):
            return
    fft(buffer, graph=graph, print_shader=print_shader, input_map=input_map, output_type=output_type,
        input_type=input_type, compute_type=compute_type)
    convolve(buffer, kernel, kernel_map=kernel_map, buffer_shape=buffer_shape, graph=graph,
             transposed_kernel=transposed_kernel, kernel_inner_only=kernel_inner_only, print_shader=print_shader,
             axis=len(buffer.shape) - 2, normalize=normalize, output_type=output_type, input_type=input_type,
             kernel_type=kernel_type, compute_type=compute_type)
    ifft(buffer, graph=graph, print_shader=print_shader, normalize=normalize, output_map=output_map,
         output_type=output_type if output_map is None else None,
         input_type=input_type if output_map is None else None, compute_type=compute_type)


_conv2d_refused = set()  # plan keys that have no fused 2-D kernel


def _conv2d_fused(buffer, kernel, kernel_inner_only, normalize, graph, print_shader) -> bool:
    """The whole convolve2DR in one launch (VDX_KIND_CONV2D_REAL: rows, then
    columns through a thread-block cluster's shared memory, then rows), for
    the sizes that have a fused kernel, when VDX_FUSED_CONV2D=1.  It is off by
    default: it moves 43 % of the composed path's HBM bytes, but each image's
    half spectrum fills the shared memory of an 8-CTA cluster, so only 15
    images are in flight on a GB300 and every phase's latency is exposed
    (64 x 512^2: 0.224 ms against 0.129 ms for the three launches).
    Returns False when the caller must run the three separate transforms."""
    if os.environ.get("VDX_FUSED_CONV2D", "0") != "1":
        return False
    real_shape = tuple(int(x) for x in buffer.real_shape)
    total = math.prod(buffer.shape)
    slab = math.prod(buffer.shape[-2:])
    broadcast = bool(kernel_inner_only)
    if not broadcast and kernel.size < total:
        if kernel.size < slab:
            raise ValueError(f"kernel buffer of {kernel.size} elements is smaller than the signal ({total})")
        broadcast = True
    key = (torch_device_index(), real_shape, bool(normalize), broadcast)
    if key in _conv2d_refused:
        return False
    try:
        plan = P.get_plan(real_shape, len(real_shape) - 2, L.VDX_KIND_CONV2D_REAL, False, bool(normalize),
                          L.VDX_C64, L.VDX_C64, None, L.VDX_KOP_MUL_CONJ, L.VDX_C64, broadcast)
    except ValueError:
        _conv2d_refused.add(key)
        return False
    if print_shader:
        print(plan.describe())
    ptr, kptr = buffer.ptr, kernel.ptr
    _record(graph, lambda s: plan.exec(ptr, ptr, kptr, s), (buffer, kernel))
    return True


def _conv2d_split_parts() -> int:
    """How many image groups a batched convolve2DR runs as, each on its own
    stream (VDX_CONV2D_STREAMS, default 2; 1 = one group on the caller's
    stream)."""
    try:
        return max(1, min(8, int(os.environ.get("VDX_CONV2D_STREAMS", "2"))))
    except ValueError:
        return 2


def _image_groups(buffer, graph, keep, steps, print_shader=False, kernel=None) -> bool:
    """Runs a batch of 2-D images as `parts` groups of images, each group's
    chain of launches on its own plan-owned stream, forked from and joined
    back into the caller's stream (vdx_group_plan, one C call per execution).
    Every kernel of such a chain is latency-bound at partial occupancy, so one
    group's kernels fill the SMs that another group's kernel leaves idle while
    it drains (convolve2DR of 64 x 512^2 on GB300: 0.0944 ms for two groups of
    32 against 0.1019 ms for one group of 64).  Each image goes through the
    same arithmetic, so the results are those of one group.

    steps: (shape, axis, kind, inverse, normalize, kernel_broadcast) of each
    transform over the whole batch, in place on `buffer`; a CONV step reads
    `kernel`.  Returns False (nothing recorded) for a buffer that is not a
    batch of at least 8 images of 16 MiB or more in all, or with
    VDX_CONV2D_STREAMS=1."""
    parts = _conv2d_split_parts()
    if parts < 2 or len(buffer.shape) != 3 or int(buffer.shape[0]) < 8 or buffer.mem_size < (16 << 20):
        return False
    plan = P.get_group_plan(tuple(steps), min(parts, int(buffer.shape[0]) // 4))
    if print_shader:
        print(plan.describe())
    data = buffer.ptr
    ker = kernel.ptr if kernel is not None else None

    def launch(s):
        plan.exec(data, ker, s)

    _record(graph, launch, tuple(keep) + (plan,))
    return True


def _groupable(*buffers) -> bool:
    """complex64 storage, contiguous: the buffers the image-group split takes."""
    return all(b.var_type == dt.complex64 and b.contiguous for b in buffers)


def _kernel_broadcast(buffer, kernel, kernel_inner_only) -> bool:
    """Whether one kernel spectrum serves every image: kernel_inner_only, or a
    kernel buffer of one image (smaller buffers are refused)."""
    if kernel_inner_only or kernel.size >= buffer.size:
        return bool(kernel_inner_only)
    img = math.prod(buffer.shape[1:])
    if kernel.size < img:
        raise ValueError(f"kernel buffer of {kernel.size} elements is smaller than the signal ({buffer.size})")
    return True


def _conv2d_split(buffer, kernel, kernel_inner_only, normalize, graph, print_shader) -> bool:
    """convolve2DR as image groups: rfft rows -> column convolution -> irfft
    rows per group (see _image_groups)."""
    real_shape = tuple(int(x) for x in buffer.real_shape)
    if len(real_shape) != 3 or real_shape[2] % 2:
        return False
    broadcast = _kernel_broadcast(buffer, kernel, kernel_inner_only)
    shape = tuple(int(x) for x in buffer.shape)
    steps = [(real_shape, 2, L.VDX_KIND_R2C, False, False, False),
             (shape, 1, L.VDX_KIND_CONV, False, bool(normalize), broadcast),
             (real_shape, 2, L.VDX_KIND_C2R, True, bool(normalize), False)]
    return _image_groups(buffer, graph, (buffer, kernel), steps, print_shader, kernel)


def _axes_split(buffer, steps, graph, print_shader) -> bool:
    """A chain of per-image transforms of a (batch, H, W) buffer as image
    groups; steps = [(kind, axis, inverse, normalize, real_shape_or_None)]."""
    if any(real is not None and int(real[-1]) % 2 for *_, real in steps):
        return False
    full = [(tuple(int(x) for x in (real if real is not None else buffer.shape)), ax, kind, inv, norm, False)
            for kind, ax, inv, norm, real in steps]
    return _image_groups(buffer, graph, (buffer,), full, print_shader)


def torch_device_index() -> int:
    import torch

    return torch.cuda.current_device()


def convolve2DR(buffer: RFFTBuffer, kernel: RFFTBuffer, kernel_map=None, buffer_shape=None, transposed_kernel=False,
                kernel_inner_only=False, graph=None, print_shader=False, normalize=True, compute_type=None):
    if len(buffer.real_shape) not in (2, 3):
        raise ValueError("Buffer must have 2 or 3 dimensions")
    if (kernel_map is None and buffer_shape is None and not transposed_kernel
            and compute_type in (None, dt.complex64) and buffer.var_type == dt.complex64
            and kernel.var_type == dt.complex64
            and _conv2d_fused(buffer, kernel, kernel_inner_only, normalize, graph, print_shader)):
        return
    if (kernel_map is None and buffer_shape is None and not transposed_kernel
            and compute_type in (None, dt.complex64) and buffer.var_type == dt.complex64
            and _groupable(buffer, kernel)
            and _conv2d_split(buffer, kernel, kernel_inner_only, normalize, graph, print_shader)):
        return
    rfft(buffer, graph=graph, print_shader=print_shader, compute_type=compute_type)
    convolve(buffer, kernel, kernel_map=kernel_map, buffer_shape=buffer_shape, graph=graph,
             transposed_kernel=transposed_kernel, kernel_inner_only=kernel_inner_only, print_shader=print_shader,
             axis=len(buffer.shape) - 2, normalize=normalize, output_type=buffer.var_type,
             input_type=buffer.var_type, kernel_type=kernel.var_type, compute_type=compute_type)
    irfft(buffer, graph=graph, print_shader=print_shader, normalize=normalize, compute_type=compute_type)


def get_transposed_size(buffer_shape: Tuple, axis: int = None, compute_type=dt.complex64) -> int:
    """Elements of the kernel layout that ``transpose`` produces.  This build
    reads kernel spectra in natural order, so the layout is the spectrum
    itself."""
    return math.prod(buffer_shape)


def transpose(in_buffer: Buffer, conv_shape: Tuple = None, axis: int = None, out_buffer: Buffer = None,
              graph=None, kernel_inner_only: bool = False, print_shader: bool = False, input_type=None,
              output_type=None, compute_type=None) -> Buffer:
    """Re-lays a kernel spectrum for ``convolve(..., transposed_kernel=True)``
    (vkdispatch/fft/functions.py:648-713).  The fused kernels here read the
    spectrum in natural order, so this is an ordered copy into out_buffer."""
    import torch

    size = get_transposed_size(tuple(in_buffer.shape), axis)
    out_t = (out_buffer.var_type if out_buffer is not None else in_buffer.var_type) if output_type is None else output_type
    if out_buffer is None:
        out_buffer = Buffer((size,), out_t)
    if out_buffer.var_type != out_t:
        raise ValueError(f"out_buffer type ({out_buffer.var_type.name}) does not match output_type ({out_t.name})")
    if out_buffer.size < size:
        raise ValueError(f"Output buffer size {out_buffer.size} is smaller than expected transposed size {size}")
    src, dst = in_buffer, out_buffer

    def launch(stream):
        s = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            n = src.tensor.numel()
            dst.tensor.reshape(-1)[:n].copy_(src.tensor.reshape(-1), non_blocking=True)

    _record(graph, launch, (src, dst))
    return out_buffer


def cache_clear() -> None:
    from . import shader_factories

    P.cache_clear()
    shader_factories.cache_clear()
