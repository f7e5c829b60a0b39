"""FFT plan cache over the C ABI (the role of the reference's lru_cache'd
kernel factories, vkdispatch/fft/shader_factories.py:11, 107)."""

from __future__ import annotations

import collections
import contextlib
import ctypes
import json
import threading
from typing import Dict, Optional, Tuple

import torch

from .. import _lib as L

_cache: Dict[tuple, "Plan"] = {}
_mu = threading.Lock()
_stats = [0, 0]  # plan-cache hits, misses
_tls = threading.local()

# storage types whose 16384-point C2C axes can run their short transforms on
# the tensor cores (include/vdx.h: VDX_FFT_FLAG_TENSOR_CORE)
_TC_IO = (L.VDX_C64, L.VDX_C32, L.VDX_BF16X2)


@contextlib.contextmanager
def autotune(enabled: bool = True):
    """Within the block, new plans time their candidate choices (threads per
    CTA or columns per tile, radix order, compile-time kernels, four-step
    split) on scratch buffers and keep the fastest, cached per (kind, N,
    stride class, batch class, dtype, direction).  Create such plans outside
    CUDA-graph capture: the search allocates and synchronises.  Per thread."""
    old = getattr(_tls, "tune", False)
    _tls.tune = bool(enabled)
    try:
        yield
    finally:
        _tls.tune = old


def bluestein_enabled() -> bool:
    """Whether C2C axes with a prime factor above 13 plan as Bluestein
    transforms on this thread (the default)."""
    return getattr(_tls, "bluestein", True)


@contextlib.contextmanager
def bluestein(enabled: bool = True):
    """C2C axes whose length has a prime factor above 13 (which the
    reference's planner rejects, vkdispatch/fft/prime_utils.py:6-10) are
    planned as Bluestein chirp-z transforms by default; ``with
    vd.fft.bluestein(False):`` restores the reference's ValueError for such
    lengths inside the block.  Per thread."""
    old = bluestein_enabled()
    _tls.bluestein = bool(enabled)
    try:
        yield
    finally:
        _tls.bluestein = old


def autotune_stats() -> Tuple[int, int]:
    """(cached choices, candidate searches run) of this process."""
    a, b = ctypes.c_int64(), ctypes.c_int64()
    L.check(L.lib().vdx_autotune_entries(ctypes.byref(a), ctypes.byref(b)), "autotune stats")
    return int(a.value), int(b.value)


def autotune_save(path: str) -> None:
    L.check(L.lib().vdx_autotune_save(str(path).encode()), "autotune save")


def autotune_load(path: str) -> None:
    L.check(L.lib().vdx_autotune_load(str(path).encode()), "autotune load")


@contextlib.contextmanager
def tensor_core_stages(enabled: bool = True):
    """Within the block, C2C transforms along axes of 16384 points run their
    128-point short transforms as BF16 tensor-core GEMMs with hi/lo-split
    compensation and FP32 accumulation.  Other plans are unaffected.  The
    setting is per thread, like the reference's per-thread graph state."""
    old = getattr(_tls, "tc", False)
    _tls.tc = bool(enabled)
    try:
        yield
    finally:
        _tls.tc = old


class Plan:
    def __init__(self, desc: L.FftDesc):
        self.desc = desc
        h = ctypes.c_void_p()
        L.check(L.lib().vdx_fft_plan_create(ctypes.byref(desc), ctypes.byref(h)), "FFT plan")
        self.handle = h

    def describe(self) -> dict:
        buf = ctypes.create_string_buffer(1024)
        L.check(L.lib().vdx_fft_plan_describe(self.handle, buf, len(buf)), "FFT plan describe")
        return json.loads(buf.value.decode())

    def exec(self, in_ptr: int, out_ptr: int, ker_ptr: Optional[int], stream: int) -> None:
        L.check(L.lib().vdx_fft_exec(self.handle, in_ptr, out_ptr, ker_ptr, stream), "FFT exec")

    def exec_multi(self, in_ptr: int, out_ptr: int, ker_ptr: int, kernel_num: int, kernel_stride: int,
                   out_stride: int, stream: int) -> bool:
        """One launch for kernel_num kernels (strides in elements); False when
        the plan has no fused multi-kernel kernel (nothing was launched)."""
        rc = L.lib().vdx_conv_exec_multi(self.handle, in_ptr, out_ptr, ker_ptr, kernel_num, kernel_stride,
                                         out_stride, stream)
        if rc == L.VDX_ERR_UNSUPPORTED:
            return False
        L.check(rc, "multi-kernel convolution")
        return True

    def exec_ops(self, in_ptr: int, out_ptr: int, ker_ptr: Optional[int], ops: L.ExecOps, stream: int) -> None:
        L.check(L.lib().vdx_fft_exec_ops(self.handle, in_ptr, out_ptr, ker_ptr, ctypes.byref(ops), stream),
                "FFT exec")

    def status(self) -> int:
        """0, or 1 if a bounded device-side wait of this plan gave up."""
        c = ctypes.c_int()
        L.check(L.lib().vdx_fft_plan_status(self.handle, ctypes.byref(c)), "FFT plan status")
        return int(c.value)

    def ctas(self) -> int:
        c = ctypes.c_int64()
        L.check(L.lib().vdx_fft_plan_ctas(self.handle, ctypes.byref(c)), "FFT plan ctas")
        return int(c.value)

    def __del__(self):
        try:
            if self.handle:
                L.lib().vdx_fft_plan_destroy(self.handle)
        except Exception:
            pass


def _default_flags(shape, axis: int, kind: int, io_type: int, compute_type: int, signal_range) -> int:
    """Plan flags from the calling thread's settings (tensor-core stages,
    autotuning, Bluestein)."""
    flags = 0
    if (getattr(_tls, "tc", False) and kind == L.VDX_KIND_C2C and int(shape[axis]) == 16384
            and io_type in _TC_IO and compute_type == L.VDX_C64 and signal_range is None):
        flags = L.VDX_FFT_FLAG_TENSOR_CORE
    if getattr(_tls, "tune", False):
        flags |= L.VDX_FFT_FLAG_AUTOTUNE
    if bluestein_enabled() and kind == L.VDX_KIND_C2C:
        flags |= L.VDX_FFT_FLAG_BLUESTEIN
    return flags


def get_plan(
    shape: Tuple[int, ...],
    axis: int,
    kind: int,
    inverse: bool,
    normalize: bool,
    io_type: int,
    compute_type: int,
    signal_range: Optional[Tuple[int, int]] = None,
    kernel_op: int = L.VDX_KOP_MUL_CONJ,
    kernel_type: Optional[int] = None,
    kernel_broadcast: bool = False,
    flags: Optional[int] = None,
) -> Plan:
    dev = torch.cuda.current_device()
    if flags is None:
        flags = _default_flags(shape, axis, kind, io_type, compute_type, signal_range)
    key = (dev, tuple(shape), axis, kind, bool(inverse), int(normalize), io_type, compute_type, signal_range,
           kernel_op, kernel_type, bool(kernel_broadcast), int(flags))
    p = _cache.get(key)
    if p is not None:
        _stats[0] += 1
        return p
    with _mu:
        p = _cache.get(key)
        if p is not None:
            _stats[0] += 1
            return p
        _stats[1] += 1
        d = L.FftDesc()
        d.ndim = len(shape)
        for i, s in enumerate(shape):
            d.shape[i] = int(s)
        d.axis = axis
        d.kind = kind
        d.inverse = int(bool(inverse))
        d.normalize = int(normalize)  # 0, 1 (1/N) or 2 (1/sqrt(N))
        d.io_type = io_type
        d.compute_type = compute_type
        if signal_range is None:
            d.signal_lo, d.signal_hi = -1, -1
        else:
            d.signal_lo, d.signal_hi = int(signal_range[0]), int(signal_range[1])
        d.kernel_op = kernel_op
        d.kernel_type = io_type if kernel_type is None else kernel_type
        d.kernel_broadcast = int(bool(kernel_broadcast))
        d.flags = int(flags)
        p = Plan(d)
        _cache[key] = p
        return p


class GroupPlan:
    """vdx_group_plan: a chain of in-place per-image transforms of a
    (B, H, W) batch, cut into image groups on streams the plan owns (one C
    call per execution forks, runs and joins the groups)."""

    def __init__(self, steps: Tuple[tuple, ...], groups: int):
        arr = (L.FftDesc * len(steps))()
        for d, (shape, axis, kind, inverse, normalize, broadcast) in zip(arr, steps):
            d.ndim = len(shape)
            for i, x in enumerate(shape):
                d.shape[i] = int(x)
            d.axis = axis
            d.kind = kind
            d.inverse = int(bool(inverse))
            d.normalize = int(normalize)
            d.io_type = d.compute_type = L.VDX_C64
            d.signal_lo = d.signal_hi = -1
            d.kernel_op = L.VDX_KOP_MUL_CONJ
            d.kernel_type = L.VDX_C64
            d.kernel_broadcast = int(bool(broadcast))
            d.flags = _default_flags(shape, axis, kind, L.VDX_C64, L.VDX_C64, None)
        self.steps = arr
        h = ctypes.c_void_p()
        L.check(L.lib().vdx_group_plan_create(arr, len(steps), int(groups), ctypes.byref(h)), "image-group plan")
        self.handle = h

    def describe(self) -> dict:
        buf = ctypes.create_string_buffer(1024)
        L.check(L.lib().vdx_group_plan_describe(self.handle, buf, len(buf)), "image-group plan describe")
        return json.loads(buf.value.decode())

    def exec(self, data_ptr: int, ker_ptr: Optional[int], stream: int) -> None:
        L.check(L.lib().vdx_group_exec(self.handle, data_ptr, ker_ptr, stream), "image-group exec")

    def __del__(self):
        try:
            if self.handle:
                L.lib().vdx_group_plan_destroy(self.handle)
        except Exception:
            pass


def get_group_plan(steps: Tuple[tuple, ...], groups: int) -> GroupPlan:
    """The calling thread's image-group plan for this chain of steps
    ((shape, axis, kind, inverse, normalize, kernel_broadcast) each): a
    plan's streams and events serve one host thread at a time, so each
    thread keeps its own plans."""
    key = (torch.cuda.current_device(), tuple(steps), int(groups),
           tuple(_default_flags(st[0], st[1], st[2], L.VDX_C64, L.VDX_C64, None) for st in steps))
    cache = getattr(_tls, "groups", None)
    if cache is None:
        cache = _tls.groups = {}
    p = cache.get(key)
    if p is None:
        _stats[1] += 1
        p = cache[key] = GroupPlan(tuple(steps), groups)
    else:
        _stats[0] += 1
    return p


def cache_clear() -> None:
    with _mu:
        _cache.clear()
        _stats[0] = _stats[1] = 0
    if getattr(_tls, "groups", None):
        _tls.groups.clear()


CacheInfo = collections.namedtuple("CacheInfo", ["hits", "misses", "maxsize", "currsize"])


def cache_info() -> CacheInfo:
    """Plan-cache counters in the form of functools' cache_info (the
    reference reports its shader caches this way,
    vkdispatch/fft/shader_factories.py:197-205); the cache is unbounded."""
    return CacheInfo(_stats[0], _stats[1], None, len(_cache))
