"""ctypes wrapper of the C restatement of the reference algorithms
(oracle/vdx_ref.c).  Test infrastructure only."""

from __future__ import annotations

import ctypes

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(str(path))
        vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        L.vdxref_plan_describe.argtypes = [i32, ctypes.POINTER(ctypes.c_int), i32]
        L.vdxref_plan_describe.restype = i32
        L.vdxref_fft_c2c.argtypes = [vp, i64, i32, i64, i32, i32, i32, i32]
        L.vdxref_fft_c2c.restype = i32
        L.vdxref_fft_real.argtypes = [vp, i64, i32, i32, i32, i32, i32]
        L.vdxref_fft_real.restype = i32
        L.vdxref_convolve.argtypes = [vp, vp, i64, i32, i64, i64, i32]
        L.vdxref_convolve.restype = i32
        L.vdxref_reduce_f32.argtypes = [vp, i32, i64, i64, i32, i32, vp]
        L.vdxref_reduce_f32.restype = i32
        L.vdxref_reduce_f64.argtypes = [vp, i64, i64, i32, vp]
        L.vdxref_reduce_f64.restype = i32
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    """Sets the OpenMP threads of the restatement's batched loops (a launcher
    such as torchrun may have set OMP_NUM_THREADS=1 for the process) and
    returns the count now in effect."""
    L = lib()
    L.omp_set_num_threads(ctypes.c_int(int(n)))
    L.omp_get_max_threads.restype = ctypes.c_int
    return int(L.omp_get_max_threads())


def plan(n: int):
    """The reference planner's stage prime groups for length n, or None when
    the reference rejects n."""
    buf = (ctypes.c_int * 512)()
    k = lib().vdxref_plan_describe(n, buf, 512)
    if k < 0:
        return None
    vals = list(buf[:k])
    nst, regs, threads = vals[0], vals[1], vals[2]
    groups, i = [], 3
    for _ in range(nst):
        npr = vals[i]
        groups.append(vals[i + 1 : i + 1 + npr])
        i += 1 + npr
    return {"groups": groups, "register_count": regs, "batch_threads": threads}


def _split(shape, axis):
    outer = int(np.prod(shape[:axis])) if axis > 0 else 1
    inner = int(np.prod(shape[axis + 1 :])) if axis + 1 < len(shape) else 1
    return outer, shape[axis], inner


def fft(x, axis=-1, inverse=False, normalize=True, signal_range=None):
    """The reference's in-place C2C transform (complex64) along `axis`."""
    a = np.ascontiguousarray(np.array(x, dtype=np.complex64, copy=True))
    axis = axis % a.ndim
    outer, n, inner = _split(a.shape, axis)
    lo, hi = (0, n) if signal_range is None else signal_range
    rc = lib().vdxref_fft_c2c(a.ctypes.data, outer, n, inner, int(inverse), int(normalize), lo, hi)
    if rc != 0:
        raise ValueError(f"the reference planner rejects length {n}")
    return a


def packed_from_real(x):
    """Real array (..., N) -> packed RFFT layout (..., N/2+1) complex64."""
    x = np.asarray(x, dtype=np.float32)
    n = x.shape[-1]
    h = n // 2 + 1
    p = np.zeros(x.shape[:-1] + (2 * h,), dtype=np.float32)
    p[..., :n] = x
    return p.view(np.complex64)


def real_from_packed(p, n):
    return np.ascontiguousarray(p).view(np.float32)[..., :n]


def rfft_packed(p, n, signal_range=None):
    """The reference's R2C on the packed layout (in place on a copy)."""
    a = np.ascontiguousarray(np.array(p, dtype=np.complex64, copy=True))
    rows = int(np.prod(a.shape[:-1])) if a.ndim > 1 else 1
    lo, hi = (0, n) if signal_range is None else signal_range
    if lib().vdxref_fft_real(a.ctypes.data, rows, n, 0, 1, lo, hi) != 0:
        raise ValueError(f"the reference planner rejects length {n}")
    return a


def irfft_packed(p, n, normalize=True):
    a = np.ascontiguousarray(np.array(p, dtype=np.complex64, copy=True))
    rows = int(np.prod(a.shape[:-1])) if a.ndim > 1 else 1
    if lib().vdxref_fft_real(a.ctypes.data, rows, n, 1, int(normalize), 0, n) != 0:
        raise ValueError(f"the reference planner rejects length {n}")
    return a


def convolve(x, kernel, axis=-1, normalize=True, broadcast=False):
    """The reference's fused convolution along `axis` (multiply by conj(K))."""
    a = np.ascontiguousarray(np.array(x, dtype=np.complex64, copy=True))
    k = np.ascontiguousarray(np.asarray(kernel, dtype=np.complex64))
    axis = axis % a.ndim
    outer, n, inner = _split(a.shape, axis)
    kstride = 0 if broadcast else n * inner
    if lib().vdxref_convolve(a.ctypes.data, k.ctypes.data, outer, n, inner, kstride, int(normalize)) != 0:
        raise ValueError(f"the reference planner rejects length {n}")
    return a


def convolve2DR(images, kernel_spec_packed, normalize=True):
    """rfft (last axis) -> convolve (axis ndim-2) -> irfft, on packed data."""
    n = images.shape[-1]
    p = rfft_packed(packed_from_real(images), n)
    p = convolve(p, kernel_spec_packed, axis=p.ndim - 2, normalize=normalize,
                 broadcast=kernel_spec_packed.size < p.size)
    p = irfft_packed(p, n, normalize=normalize)
    return real_from_packed(p, n)


_OPS = {"add": 0, "mul": 1, "min": 2, "max": 3}
_MAPS = {"identity": 0, "abs": 1, "square": 2, "real": 3, "imag": 4, "sin": 5}


def reduce_f32(x, op="add", map="identity", batch=1):  # noqa: A002
    """The reference's two-stage float reduction, in its order."""
    x = np.ascontiguousarray(x)
    typ = 0 if np.iscomplexobj(x) else 4
    x = x.astype(np.complex64 if typ == 0 else np.float32)
    n = x.size // batch
    out = np.zeros(batch, dtype=np.float32)
    lib().vdxref_reduce_f32(x.ctypes.data, typ, n, batch, _OPS[op], _MAPS[map], out.ctypes.data)
    return out
