"""Device buffers with the reference's Buffer / RFFTBuffer surface
(vkdispatch/base/buffer.py:40-466), backed by PyTorch device memory.

A Buffer owns (or aliases) one torch tensor on the current CUDA device;
``ptr`` is what the C ABI receives.  ``from_cuda_array`` aliases any object
exposing ``__cuda_array_interface__`` without copying, with the reference's
checks: C-contiguous (unless ``require_contiguous=False``), dtype match,
read-only flag.  A buffer over a non-contiguous array records its element
strides (``strides``); the FFT functions then address it through its
strides instead of assuming C order.
"""

from __future__ import annotations

import math
import typing
from typing import Optional, Tuple

import numpy as np
import torch

from . import dtypes as dt

MAX_ELEMENTS = 2**30  # the reference caps buffers at 2^30 elements (buffer.py:86-87)


_cuda_checked = False


def _device() -> torch.device:
    global _cuda_checked
    if not _cuda_checked:
        if not torch.cuda.is_available():
            raise RuntimeError("vkdispatch_gb300 needs a CUDA device (no CPU fallback)")
        _cuda_checked = True
    return torch.device("cuda", torch.cuda.current_device())


class Buffer:
    def __init__(self, shape, var_type: dt.dtype = dt.complex64, external=None, writable: bool = True):
        if isinstance(shape, int):
            shape = (shape,)
        shape = tuple(int(s) for s in shape)
        if len(shape) < 1 or len(shape) > 4:
            raise ValueError("Buffer shape must have 1 to 4 dimensions")
        if any(s < 1 for s in shape):
            raise ValueError("Buffer dimensions must be positive")
        size = math.prod(shape)
        if size > MAX_ELEMENTS:
            raise ValueError(f"Buffer of {size} elements exceeds the 2^30 element limit")
        self.shape = shape
        self.var_type = var_type
        self.size = size
        self.writable = writable
        self._keepalive = None
        self.strides = None  # element strides of a non-contiguous external array, else None (C order)
        lane_shape = shape + ((var_type.lanes,) if var_type.lanes > 1 else ())
        if external is None:
            self._t = torch.empty(lane_shape, dtype=var_type.torch_dtype, device=_device())
        else:
            t, keep = external
            self._t = t
            self._keepalive = keep

    @classmethod
    def _empty(cls, shape: Tuple[int, ...], var_type: dt.dtype) -> "Buffer":
        """A new device buffer of a shape already checked by the caller (the
        result buffers of repeated reductions)."""
        b = cls.__new__(cls)
        b.shape = shape
        b.var_type = var_type
        b.size = math.prod(shape)
        b.writable = True
        b._keepalive = None
        b.strides = None
        lane_shape = shape + ((var_type.lanes,) if var_type.lanes > 1 else ())
        b._t = torch.empty(lane_shape, dtype=var_type.torch_dtype, device=_device())
        return b

    # -- properties -----------------------------------------------------
    @property
    def ptr(self) -> int:
        return int(self._t.data_ptr())

    @property
    def contiguous(self) -> bool:
        return self.strides is None

    @property
    def tensor(self) -> torch.Tensor:
        """The backing torch tensor (lanes of multi-lane types in the last dim)."""
        return self._t

    @property
    def mem_size(self) -> int:
        return self.size * self.var_type.item_size

    @property
    def __cuda_array_interface__(self):
        if self.var_type in (dt.complex32, dt.complexbf16, dt.vec2):
            return self._t.__cuda_array_interface__
        return self._t.__cuda_array_interface__

    # -- host transfers -------------------------------------------------
    def _to_lanes(self, data) -> torch.Tensor:
        vt = self.var_type
        a = np.asarray(data)
        if vt in (dt.complex32, dt.complexbf16):
            if np.iscomplexobj(a):
                a = a.astype(np.complex64)
                pairs = np.stack([a.real, a.imag], axis=-1).astype(np.float32)
            else:
                pairs = a.astype(np.float32)
            t = torch.from_numpy(np.ascontiguousarray(pairs)).to(vt.torch_dtype)
        elif vt == dt.vec2:
            t = torch.from_numpy(np.ascontiguousarray(a.astype(np.float32)))
        else:
            t = torch.from_numpy(np.ascontiguousarray(a.astype(vt.np_dtype)))
        return t

    def write(self, data, index: Optional[int] = None) -> None:
        if not self.writable:
            raise ValueError("Buffer is read-only")
        t = self._to_lanes(data)
        if t.numel() * t.element_size() != self._t.numel() * self._t.element_size():
            raise ValueError(f"data of {t.numel()} lanes does not match buffer of shape {self.shape}")
        self._t.copy_(t.reshape(self._t.shape), non_blocking=False)

    def read(self, index: Optional[int] = None):
        vt = self.var_type
        h = self._t.detach().to("cpu")
        if vt in (dt.complex32, dt.complexbf16):
            f = h.float().numpy()
            out = (f[..., 0] + 1j * f[..., 1]).astype(np.complex64)
        elif vt == dt.uint32 and h.dtype == torch.int32:
            out = h.numpy().view(np.uint32)
        else:
            out = h.numpy()
        if index is None:
            return [out]
        return out

    def destroy(self) -> None:
        self._t = None
        self._keepalive = None

    def __repr__(self):
        return f"Buffer(shape={self.shape}, var_type={self.var_type.name})"


def asbuffer(array) -> Buffer:
    a = np.asarray(array)
    buf = Buffer(a.shape, dt.from_numpy_dtype(a.dtype))
    buf.write(a)
    return buf


_TYPESTR = {
    "<f4": dt.float32,
    "<f8": dt.float64,
    "<i4": dt.int32,
    "<u4": dt.uint32,
    "<c8": dt.complex64,
    "<c16": dt.complex128,
    "<f2": dt.float16,
}


def from_cuda_array(
    obj: typing.Any,
    var_type: Optional[dt.dtype] = None,
    require_contiguous: bool = True,
    writable: Optional[bool] = None,
    keepalive: bool = True,
) -> Buffer:
    """Zero-copy Buffer over a ``__cuda_array_interface__`` object
    (vkdispatch/base/buffer.py:309-375)."""
    if not hasattr(obj, "__cuda_array_interface__"):
        raise TypeError("Expected an object with __cuda_array_interface__")
    iface = obj.__cuda_array_interface__
    if not isinstance(iface, dict):
        raise TypeError("__cuda_array_interface__ must be a dictionary")
    for k in ("shape", "typestr", "data"):
        if k not in iface:
            raise ValueError("__cuda_array_interface__ is missing required fields (shape/typestr/data)")
    shape = tuple(int(d) for d in iface["shape"]) or (1,)
    data = iface["data"]
    if not (isinstance(data, tuple) and len(data) >= 2):
        raise ValueError("__cuda_array_interface__['data'] must be a tuple (ptr, read_only)")
    read_only = bool(data[1])
    typestr = iface["typestr"].replace("|", "<").replace("=", "<")
    inferred = _TYPESTR.get(typestr)
    if inferred is None:
        raise ValueError(f"unsupported CAI typestr {iface['typestr']}")
    if var_type is None:
        var_type = inferred
    if var_type != inferred:
        raise ValueError(f"CAI dtype ({iface['typestr']}) does not match requested dtype ({var_type.name}).")
    strides = iface.get("strides")
    elem_strides = None
    if strides is not None:
        itemsize = np.dtype(inferred.np_dtype).itemsize
        expected, s = [], itemsize
        for d in reversed(shape):
            expected.insert(0, s)
            s *= d
        strides = tuple(int(x) for x in strides)
        if strides != tuple(expected) and not all(d == 1 or st == ex for d, st, ex in zip(shape, strides, expected)):
            if require_contiguous:
                raise ValueError("Only contiguous C-order CUDA arrays are supported in from_cuda_array().")
            if any(st < 0 or st % itemsize for st in strides):
                raise ValueError("strided CUDA arrays need non-negative strides that are multiples of the item size")
            elem_strides = tuple(st // itemsize for st in strides)
    buf_writable = (not read_only) if writable is None else bool(writable)
    if buf_writable and read_only:
        raise ValueError("Requested writable=True for a read-only CUDA array.")
    t = torch.as_tensor(obj, device=_device())
    if int(t.data_ptr()) != int(data[0]):
        raise ValueError("could not alias the CUDA array without a copy")
    buf = Buffer(shape, var_type, external=(t, obj if keepalive else None), writable=buf_writable)
    buf.strides = elem_strides
    return buf


class RFFTBuffer(Buffer):
    """Packed real/half-spectrum buffer: shape (..., N//2+1) complex; the
    first N reals of each row hold the real signal."""

    def __init__(self, shape: Tuple[int, ...], fourier_type: dt.dtype = dt.complex64):
        if not fourier_type.is_complex or fourier_type == dt.complexbf16:
            raise ValueError("RFFTBuffer fourier_type must be complex32, complex64, or complex128")
        shape = tuple(int(s) for s in shape)
        super().__init__(shape[:-1] + (shape[-1] // 2 + 1,), fourier_type)
        self.real_shape = shape
        self.fourier_shape = self.shape
        self.real_type = fourier_type.child_type

    def _real_view(self) -> torch.Tensor:
        if self.var_type == dt.complex32:
            return self._t.reshape(self.shape[:-1] + (self.shape[-1] * 2,))
        return torch.view_as_real(self._t).reshape(self.shape[:-1] + (self.shape[-1] * 2,))

    def read_real(self, index: Optional[int] = None):
        r = self._real_view()[..., : self.real_shape[-1]].detach().to("cpu")
        out = r.float().numpy() if self.var_type == dt.complex32 else r.numpy()
        return [out] if index is None else out

    def read_fourier(self, index: Optional[int] = None):
        return self.read(index)

    def write_real(self, data, index: Optional[int] = None) -> None:
        a = np.asarray(data)
        if a.shape != self.real_shape:
            raise ValueError(f"Data shape {a.shape} must match real shape {self.real_shape}!")
        if np.iscomplexobj(a):
            raise ValueError("Data dtype must be real, not complex!")
        view = self._real_view()
        packed = torch.zeros(view.shape, dtype=view.dtype)
        packed[..., : self.real_shape[-1]] = torch.from_numpy(np.ascontiguousarray(a)).to(view.dtype)
        view.copy_(packed)

    def write_fourier(self, data, index: Optional[int] = None) -> None:
        a = np.asarray(data)
        if a.shape != self.fourier_shape:
            raise ValueError(f"Data shape {a.shape} must match fourier shape {self.fourier_shape}!")
        if not np.iscomplexobj(a):
            raise ValueError("Data dtype must be complex!")
        self.write(a)


def asrfftbuffer(data, fourier_type: Optional[dt.dtype] = None) -> RFFTBuffer:
    a = np.asarray(data)
    if np.iscomplexobj(a):
        raise ValueError("Input data to asrfftbuffer must be real-valued!")
    if fourier_type is None:
        scalar = dt.from_numpy_dtype(a.dtype) if a.dtype in (np.float32, np.float64, np.float16) else dt.float32
        fourier_type = dt.complex_from_float(scalar)
    buf = RFFTBuffer(a.shape, fourier_type=fourier_type)
    buf.write_real(a)
    return buf
