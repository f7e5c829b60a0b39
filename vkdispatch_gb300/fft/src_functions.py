"""Source inspection for the FFT path: the reference's ``*_src`` and
``*_print_src`` functions (vkdispatch/fft/src_functions.py) and ``pad_dim``
(vkdispatch/fft/prime_utils.py:50-64), with the same names and arguments.

The reference generates one shader per transform and returns its source.
Here the kernels are compiled ahead of time into libvdx, so a transform
without maps returns a description of the plan that would run: the kernel
template, its launch shape and the plan's radix passes.  A transform with
maps returns the C++ hooks struct that the map-hook compiler lowers the maps
to and compiles into the FFT kernel template (vkdispatch_gb300/fft/jit.py).
Either way the call only plans; nothing is launched."""

from __future__ import annotations

import json
import math
from dataclasses import dataclass
from typing import Optional, Tuple, Union

from .. import _lib as L
from .. import dtypes as dt
from . import plan as P
from .functions import _norm_axis, _signal

_OP_KERNEL = {
    "c2c_fwd": "vdx::k_c2c",
    "c2c_inv": "vdx::k_c2c",
    "conv": "vdx::k_conv",
    "r2c_even": "vdx::k_r2c_even",
    "c2r_even": "vdx::k_c2r_even",
    "r2c_odd": "vdx::k_real_odd",
    "c2r_odd": "vdx::k_real_odd",
}


@dataclass
class ShaderSource:
    """What one transform runs: name, code and CTA shape (the fields of the
    reference's vd.ShaderSource, vkdispatch/shader/shader_function.py:139-145)."""

    name: str
    code: str
    local_size: Tuple[int, int, int]

    def __repr__(self):
        return f"// ---- {self.name}, CTA shape {self.local_size} ----\n{self.code}"


def _numbered(code: str, line_numbers: bool) -> str:
    if not line_numbers:
        return code
    lines = code.splitlines()
    width = len(str(len(lines)))
    return "\n".join(f"{i + 1:>{width}} {ln}" for i, ln in enumerate(lines))


def _plan_source(plan, what: str, shape, axis, line_numbers) -> ShaderSource:
    d = plan.describe()
    op = d.get("op", "")
    block = d.get("block", 0)
    if isinstance(block, list):
        block = block[0]
    if "fourstep" in d:
        n1, n0 = d["fourstep"]
        name = "vdx::k_fs"
        body = [f"// two launches of {name}: {n1}-point transforms of every column b0 of the {n1} x {n0} split,",
                f"// times W_N^(b0 k1), into the plan's workspace; then {n0}-point transforms written to",
                f"// X[k1 + {n1} k2]" + (" (tensor-core DFT stages)" if d.get("tensor_core") else "")]
    elif "bluestein" in d:
        name = "vdx::k_bs_in + convolution + vdx::k_bs_out"
        body = [f"// Bluestein: chirp-in into a {d['bluestein']}-point zero-padded workspace, a",
                "// length-M convolution against the chirp spectrum, chirp-out"]
    elif op == "conv2d_real":
        name = "vdx::k_conv2d_real"
        body = ["// rows, columns through the shared memory of an 8-CTA cluster, rows: one launch"]
    else:
        name = _OP_KERNEL.get(op, "vdx::k_c2c")
        plan_kind = ("compile-time plan" if d.get("fixed") else "runtime-radix plan")
        body = [f"// {plan_kind}: radix passes {d.get('radices')}, {d.get('threads_per_transform')} threads per "
                f"transform, {d.get('transforms_per_cta')} transform(s) per CTA" +
                (", strided column tiles" if d.get("strided") else ""),
                f"// grid {d.get('grid')} x {block} threads, {d.get('smem')} bytes of dynamic shared memory"]
    code = "\n".join([f"// {what} of the {shape[axis]}-point axis {axis} of a {tuple(shape)} buffer",
                      "// ahead-of-time CUDA kernel of libvdx.so (sm_103a)", *body,
                      "// plan: " + json.dumps(d)])
    return ShaderSource(name, _numbered(code, line_numbers), (int(block or 1), 1, 1))


class _Placeholder:
    """A buffer argument of a map whose buffers are bound only at call time."""

    def __init__(self, var_type=None):
        self.var_type = var_type
        self.strides = None


def _map_args(mf):
    return [0.0 if sc else _Placeholder() for sc in mf.arg_is_scalar()]


def _maps_source(shape, axis, conv, input_map, output_map, kernel_map, kernel_broadcast_slab, line_numbers,
                 what) -> ShaderSource:
    from . import jit as J

    io = _Placeholder(dt.complex64)
    outs = _map_args(output_map) if output_map is not None else [io]
    ins = _map_args(input_map) if input_map is not None else []
    kers = (_map_args(kernel_map) if kernel_map is not None else [_Placeholder(dt.complex64)]) if conv else []
    spec = J.build_hooks(outs, ins, kers, input_map, output_map, kernel_map, conv, kernel_broadcast_slab)
    head = [f"// {what} of the {shape[axis]}-point axis {axis} of a {tuple(shape)} buffer: hooks compiled with",
            "// NVRTC into the FFT kernel template (vkdispatch_gb300/csrc/fft_mapped.cuh)"]
    return ShaderSource("vdx::k_mapped<VdxHooks>", _numbered("\n".join(head) + "\n" + spec.source, line_numbers),
                        (0, 1, 1))


def fft_src(buffer_shape: Tuple, axis: int = None, inverse: bool = False, normalize_inverse: bool = True,
            r2c: bool = False, input_map=None, output_map=None,
            input_signal_range: Union[Tuple[Optional[int], Optional[int]], None] = None,
            line_numbers: bool = False) -> ShaderSource:
    shape = tuple(int(s) for s in buffer_shape)
    ax = _norm_axis(axis, len(shape))
    what = ("inverse " if inverse else "forward ") + ("real FFT" if r2c else "FFT")
    if input_map is not None or output_map is not None:
        if r2c:
            raise NotImplementedError("map hooks on real (r2c) transforms are not in the supported menu")
        return _maps_source(shape, ax, False, input_map, output_map, None, 0, line_numbers, what)
    if r2c:
        if ax != len(shape) - 1:
            raise ValueError("R2C io only supported for contiguous data")
        kind = L.VDX_KIND_C2R if inverse else L.VDX_KIND_R2C
    else:
        kind = L.VDX_KIND_C2C
    plan = P.get_plan(shape, ax, kind, inverse, bool(inverse and normalize_inverse), L.VDX_C64, L.VDX_C64,
                      _signal(input_signal_range, shape[ax]))
    return _plan_source(plan, what, shape, ax, line_numbers)


def _check_dims(buffer_shape, dims):
    if len(buffer_shape) not in dims:
        raise ValueError("Buffer Shape must have " + " or ".join(str(d) for d in dims) + " dimensions")


def fft2_src(buffer_shape: Tuple, input_map=None, output_map=None):
    _check_dims(buffer_shape, (2, 3))
    n = len(buffer_shape)
    return (fft_src(buffer_shape, axis=n - 2, input_map=input_map),
            fft_src(buffer_shape, axis=n - 1, output_map=output_map))


def fft3_src(buffer_shape: Tuple, input_map=None, output_map=None):
    _check_dims(buffer_shape, (3,))
    return (fft_src(buffer_shape, axis=0, input_map=input_map), fft_src(buffer_shape, axis=1),
            fft_src(buffer_shape, axis=2, output_map=output_map))


def ifft_src(buffer_shape: Tuple, axis: int = None, normalize: bool = True, input_map=None, output_map=None):
    return fft_src(buffer_shape, axis=axis, inverse=True, normalize_inverse=normalize, input_map=input_map,
                   output_map=output_map)


def ifft2_src(buffer_shape: Tuple, normalize: bool = True, input_map=None, output_map=None):
    _check_dims(buffer_shape, (2, 3))
    n = len(buffer_shape)
    return (ifft_src(buffer_shape, axis=n - 2, normalize=normalize, input_map=input_map),
            ifft_src(buffer_shape, axis=n - 1, normalize=normalize, output_map=output_map))


def ifft3_src(buffer_shape: Tuple, normalize: bool = True, input_map=None, output_map=None):
    _check_dims(buffer_shape, (3,))
    return (ifft_src(buffer_shape, axis=0, normalize=normalize, input_map=input_map),
            ifft_src(buffer_shape, axis=1, normalize=normalize),
            ifft_src(buffer_shape, axis=2, normalize=normalize, output_map=output_map))


def _fourier_shape(real_shape):
    return tuple(real_shape[:-1]) + (int(real_shape[-1]) // 2 + 1,)


def rfft_src(buffer_shape: Tuple):
    return fft_src(buffer_shape, r2c=True)


def rfft2_src(buffer_shape: Tuple):
    _check_dims(buffer_shape, (2, 3))
    return rfft_src(buffer_shape), fft_src(_fourier_shape(buffer_shape), axis=len(buffer_shape) - 2)


def rfft3_src(buffer_shape: Tuple):
    _check_dims(buffer_shape, (3,))
    fs = _fourier_shape(buffer_shape)
    return rfft_src(buffer_shape), fft_src(fs, axis=1), fft_src(fs, axis=0)


def irfft_src(buffer_shape: Tuple, normalize: bool = True):
    return fft_src(buffer_shape, inverse=True, normalize_inverse=normalize, r2c=True)


def irfft2_src(buffer_shape: Tuple, normalize: bool = True):
    _check_dims(buffer_shape, (2, 3))
    return (ifft_src(_fourier_shape(buffer_shape), axis=len(buffer_shape) - 2, normalize=normalize),
            irfft_src(buffer_shape, normalize=normalize))


def irfft3_src(buffer_shape: Tuple, normalize: bool = True):
    _check_dims(buffer_shape, (3,))
    fs = _fourier_shape(buffer_shape)
    return (ifft_src(fs, axis=0, normalize=normalize), ifft_src(fs, axis=1, normalize=normalize),
            irfft_src(buffer_shape, normalize=normalize))


def convolve_src(buffer_shape: Tuple, kernel_map=None, kernel_num: int = 1, axis: int = None,
                 normalize: bool = True, transposed_kernel: bool = False, kernel_inner_only: bool = False,
                 input_map=None, output_map=None,
                 input_signal_range: Union[Tuple[Optional[int], Optional[int]], None] = None,
                 line_numbers: bool = False) -> ShaderSource:
    shape = tuple(int(s) for s in buffer_shape)
    ax = _norm_axis(axis, len(shape))
    if kernel_num < 1:
        raise ValueError("kernel_num must be >= 1")
    slab = math.prod(shape[ax:])
    if input_map is not None or output_map is not None or kernel_map is not None:
        return _maps_source(shape, ax, True, input_map, output_map, kernel_map,
                            slab if kernel_inner_only else 0, line_numbers, "FFT convolution")
    plan = P.get_plan(shape, ax, L.VDX_KIND_CONV, False, bool(normalize), L.VDX_C64, L.VDX_C64,
                      _signal(input_signal_range, shape[ax]), L.VDX_KOP_MUL_CONJ, L.VDX_C64, bool(kernel_inner_only))
    src = _plan_source(plan, "FFT convolution" + (f" with {kernel_num} kernels" if kernel_num > 1 else ""), shape, ax,
                       line_numbers)
    return src


def convolve2D_src(buffer_shape: Tuple, kernel_map=None, normalize: bool = True, transposed_kernel: bool = False,
                   kernel_inner_only: bool = False, input_map=None, output_map=None):
    _check_dims(buffer_shape, (2, 3))
    n = len(buffer_shape)
    return (fft_src(buffer_shape, axis=n - 1, input_map=input_map),
            convolve_src(buffer_shape, kernel_map=kernel_map, transposed_kernel=transposed_kernel,
                         kernel_inner_only=kernel_inner_only, axis=n - 2, normalize=normalize),
            ifft_src(buffer_shape, axis=n - 1, normalize=normalize, output_map=output_map))


def convolve2DR_src(buffer_shape: Tuple, kernel_map=None, transposed_kernel: bool = False,
                    kernel_inner_only: bool = False, normalize: bool = True):
    _check_dims(buffer_shape, (2, 3))
    return (rfft_src(buffer_shape),
            convolve_src(_fourier_shape(buffer_shape), kernel_map=kernel_map, transposed_kernel=transposed_kernel,
                         kernel_inner_only=kernel_inner_only, axis=len(buffer_shape) - 2, normalize=normalize),
            irfft_src(buffer_shape, normalize=normalize))


def transpose_src(buffer_shape: Tuple, axis: int = None, kernel_inner_only: bool = False,
                  line_numbers: bool = False) -> ShaderSource:
    """transpose() is an ordered copy here (the kernels read spectra in natural
    order): no kernel of this package runs for it."""
    shape = tuple(int(s) for s in buffer_shape)
    code = (f"// transpose of a {shape} kernel spectrum: an ordered device copy (torch copy_),\n"
            "// since the convolution kernels read the spectrum in natural order")
    return ShaderSource("ordered copy", _numbered(code, line_numbers), (0, 1, 1))


def _printer(fn):
    def print_src(*args, **kwargs):
        out = fn(*args, **kwargs)
        for s in (out if isinstance(out, tuple) else (out,)):
            print(s)

    print_src.__name__ = fn.__name__.replace("_src", "_print_src")
    print_src.__doc__ = f"Prints what {fn.__name__} returns."
    return print_src


fft_print_src = _printer(fft_src)
fft2_print_src = _printer(fft2_src)
fft3_print_src = _printer(fft3_src)
ifft_print_src = _printer(ifft_src)
ifft2_print_src = _printer(ifft2_src)
ifft3_print_src = _printer(ifft3_src)
rfft_print_src = _printer(rfft_src)
rfft2_print_src = _printer(rfft2_src)
rfft3_print_src = _printer(rfft3_src)
irfft_print_src = _printer(irfft_src)
irfft2_print_src = _printer(irfft2_src)
irfft3_print_src = _printer(irfft3_src)
convolve_print_src = _printer(convolve_src)
convolve2D_print_src = _printer(convolve2D_src)
convolve2DR_print_src = _printer(convolve2DR_src)


def pad_dim(dim: int, max_register_count: int = None) -> int:
    """The smallest length >= dim whose prime factors are all at most
    max_register_count (default 16, i.e. 13-smooth): the padding the
    reference's planner needs (vkdispatch/fft/prime_utils.py:50-64).  This
    build also plans the other lengths, as Bluestein transforms."""
    if max_register_count is None:
        max_register_count = 16
    if dim <= 0:
        raise ValueError("Dimension must be greater than 0")
    n = int(dim)
    while True:
        m = n
        p = 2
        while p * p <= m and p <= max_register_count:
            while m % p == 0:
                m //= p
            p += 1
        if m == 1 or m <= max_register_count:
            return n
        n += 1


def get_cache_info():
    """Plan-cache counters (hits, misses, maxsize, currsize)."""
    return P.cache_info()


def print_cache_info() -> None:
    print(get_cache_info())
