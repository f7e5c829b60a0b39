"""The reference's short names for map annotations and element types
(vkdispatch/codegen/abbreviations.py), importable as
``vkdispatch_gb300.codegen.abbreviations`` for the types this path has."""

from . import dtypes as _dt
from .codegen import Buffer as Buff  # noqa: F401
from .codegen import Var  # noqa: F401

Const = Var  # compile-time constants are passed like scalar map arguments here

f16 = _dt.float16
f32 = _dt.float32
f64 = _dt.float64
i32 = _dt.int32
u32 = _dt.uint32
c32 = _dt.complex32
c64 = _dt.complex64
c128 = _dt.complex128
v2 = _dt.vec2

__all__ = ["Buff", "Var", "Const", "f16", "f32", "f64", "i32", "u32", "c32", "c64", "c128", "v2"]
