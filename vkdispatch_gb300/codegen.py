"""Tracing stand-ins for the parts of ``vkdispatch.codegen`` that reduction
and map functions use (type annotations ``Buff[f32]`` and a few math
functions).

There is no code generation here: a user function is called once with
symbolic arguments, the expression it builds is matched against the menu of
device functors libvdx implements (identity, abs / complex modulus, square /
|z|^2, real, imag, sin; add, mul, min, max, and, or, xor), and anything
outside the menu raises NotImplementedError naming the function.
"""

from __future__ import annotations

from . import dtypes as dt

f16, f32, f64 = dt.float16, dt.float32, dt.float64
i32, u32 = dt.int32, dt.uint32
c32, c64, c128 = dt.complex32, dt.complex64, dt.complex128
v2 = dt.vec2


class _BufferType:
    def __init__(self, t):
        self.var_type = t
        self.__args__ = (t,)

    def __repr__(self):
        return f"Buffer[{self.var_type.name}]"


class _BufferFactory:
    def __getitem__(self, t):
        return _BufferType(t)


Buffer = _BufferFactory()
Buff = Buffer


class Sym:
    """Symbolic value: ``op`` with operand tuple ``args``."""

    def __init__(self, op, *args):
        self.op = op
        self.args = args

    def _bin(self, op, other):
        return Sym(op, self, other)

    def __add__(self, o):
        return self._bin("add", o)

    __radd__ = __add__

    def __mul__(self, o):
        return self._bin("mul", o)

    __rmul__ = __mul__

    def __and__(self, o):
        return self._bin("and", o)

    def __or__(self, o):
        return self._bin("or", o)

    def __xor__(self, o):
        return self._bin("xor", o)

    def __sub__(self, o):
        return self._bin("sub", o)

    def __neg__(self):
        return Sym("neg", self)

    def __abs__(self):
        return Sym("abs", self)

    def __pow__(self, o):
        return self._bin("pow", o)

    @property
    def real(self):
        return Sym("real", self)

    @property
    def imag(self):
        return Sym("imag", self)

    @property
    def x(self):
        return Sym("real", self)

    @property
    def y(self):
        return Sym("imag", self)

    def __repr__(self):
        return f"{self.op}({', '.join(map(repr, self.args))})"


class SymBuffer:
    def __init__(self, index, var_type):
        self.index = index
        self.var_type = var_type

    def __getitem__(self, idx):
        return Sym("load", self.index)


class _IoIndex:
    def __repr__(self):
        return "io_index"


def mapped_io_index():
    return _IoIndex()


def sin(x):
    return Sym("sin", x)


def cos(x):
    return Sym("cos", x)


def sqrt(x):
    return Sym("sqrt", x)


def length(x):
    return Sym("length", x)


def abs(x):  # noqa: A001 - mirrors vc.abs
    return Sym("abs", x)


def min(a, b):  # noqa: A001
    return Sym("min", a, b)


def max(a, b):  # noqa: A001
    return Sym("max", a, b)


# --- used by FFT map hooks (vkdispatch_gb300/fft/maps.py traces them) -------
def to_dtype(var_type, *args):
    """Cast (one argument) or build a value of var_type from components."""
    if len(args) == 1:
        return Sym("cast", args[0])
    return Sym("make", *args)


def to_complex(x):
    return Sym("to_complex", x)


def mult_complex(a, b):
    return Sym("cmul", a, b)


def new_register(var_type, *args, var_name=None):
    from .fft import maps

    return maps.new_trace_register(var_type)
