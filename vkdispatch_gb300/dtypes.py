"""Element types of Buffers (the subset of vkdispatch/base/dtype.py:94-130 and
:709-731 the FFT / reduction path uses, plus a bf16 complex pair)."""

from __future__ import annotations

import numpy as np
import torch

from . import _lib as L


class dtype:
    def __init__(self, name, item_size, np_dtype, torch_dtype, lanes, vdx_code, child=None, is_complex=False):
        self.name = name
        self.item_size = item_size
        self.np_dtype = np.dtype(np_dtype)
        self.torch_dtype = torch_dtype  # storage dtype of one lane
        self.lanes = lanes  # torch elements per logical element
        self.vdx_code = vdx_code
        self.child_type = child
        self.is_complex = is_complex

    def __repr__(self):
        return f"vkdispatch_gb300.{self.name}"

    def __hash__(self):
        return hash(self.name)

    def __eq__(self, other):
        return self is other or (isinstance(other, dtype) and other.name == self.name)


float16 = dtype("float16", 2, np.float16, torch.float16, 1, None)
bfloat16 = dtype("bfloat16", 2, np.float32, torch.bfloat16, 1, None)
float32 = dtype("float32", 4, np.float32, torch.float32, 1, L.VDX_F32)
float64 = dtype("float64", 8, np.float64, torch.float64, 1, L.VDX_F64)
int32 = dtype("int32", 4, np.int32, torch.int32, 1, L.VDX_I32)
uint32 = dtype("uint32", 4, np.uint32, torch.uint32 if hasattr(torch, "uint32") else torch.int32, 1, L.VDX_U32)
complex32 = dtype("complex32", 4, np.complex64, torch.float16, 2, L.VDX_C32, float16, True)
complex64 = dtype("complex64", 8, np.complex64, torch.complex64, 1, L.VDX_C64, float32, True)
complex128 = dtype("complex128", 16, np.complex128, torch.complex128, 1, L.VDX_C128, float64, True)
# complex value stored as two bfloat16 (not in the reference; storage for the
# reduced-precision FFT path)
complexbf16 = dtype("complexbf16", 4, np.complex64, torch.bfloat16, 2, L.VDX_BF16X2, bfloat16, True)
# two-lane float vector (the reference's vec2 / v2)
vec2 = dtype("vec2", 8, np.float32, torch.float32, 2, None, float32, False)

_NUMPY_MAP = {
    np.dtype(np.float16): float16,
    np.dtype(np.float32): float32,
    np.dtype(np.float64): float64,
    np.dtype(np.int32): int32,
    np.dtype(np.uint32): uint32,
    np.dtype(np.complex64): complex64,
    np.dtype(np.complex128): complex128,
}


def from_numpy_dtype(d) -> dtype:
    d = np.dtype(d)
    if d not in _NUMPY_MAP:
        raise ValueError(f"unsupported numpy dtype {d}")
    return _NUMPY_MAP[d]


def complex_from_float(t: dtype) -> dtype:
    return {float16: complex32, float32: complex64, float64: complex128}[t]


def is_complex(t: dtype) -> bool:
    return t.is_complex
