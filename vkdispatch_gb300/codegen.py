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

import contextlib

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

    # comparisons build traced conditions (for if_block and friends);
    # == and != keep Python's identity meaning when Python itself asks
    # (containers, `in`), so the equality overloads do not break lookups
    __hash__ = object.__hash__

    def __lt__(self, o):
        return _Cmp("lt", self, o)

    def __le__(self, o):
        return _Cmp("le", self, o)

    def __gt__(self, o):
        return _Cmp("gt", self, o)

    def __ge__(self, o):
        return _Cmp("ge", self, o)

    def __eq__(self, o):
        return _Cmp("eq", self, o)

    def __ne__(self, o):
        return _Cmp("ne", self, o)

    def __invert__(self):
        return Sym("invert", self)

    def _bin(self, op, other):
        return Sym(op, self, other)

    def __add__(self, o):
        return self._bin("add", o)

    __radd__ = __add__

    def __mul__(self, o):
        return self._bin("mul", o)

    __rmul__ = __mul__

    def __rsub__(self, o):
        return Sym("sub", o, self)

    def __truediv__(self, o):
        return self._bin("div", o)

    def __rtruediv__(self, o):
        return Sym("div", o, self)

    def __floordiv__(self, o):
        return self._bin("floordiv", o)

    def __rfloordiv__(self, o):
        return Sym("floordiv", o, self)

    def __mod__(self, o):
        return self._bin("mod", o)

    def __rmod__(self, o):
        return Sym("mod", o, self)

    def to_register(self, var_name=None):
        return self

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


class _Cmp(Sym):
    """A traced comparison.  As a Python bool, == and != mean identity;
    ordering comparisons refuse, as the reference's variables do
    (vkdispatch/codegen/variables/variables.py:338-339)."""

    def __bool__(self):
        if self.op == "eq":
            return self.args[0] is self.args[1]
        if self.op == "ne":
            return self.args[0] is not self.args[1]
        raise ValueError("traced values cannot be cast to a Python bool: use vc.if_block and friends")


class SymBuffer:
    def __init__(self, index, var_type):
        self.index = index
        self.var_type = var_type

    def __getitem__(self, idx):
        return Sym("load", self.index, idx)


class SymVec(tuple):
    """Integer vector of index components (ravel_index's result)."""

    def to_register(self, var_name=None):
        return self


class _VarType:
    """Annotation of a scalar map argument (``vc.Var[vc.f32]``)."""

    def __init__(self, t):
        self.var_type = t
        self.__args__ = (t,)
        self.is_scalar = True

    def __repr__(self):
        return f"Var[{self.var_type.name}]"


class _VarFactory:
    def __getitem__(self, t):
        return _VarType(t)


Var = _VarFactory()


class _IoIndex(Sym):
    """mapped_io_index() of a reduction map: the element's flat index."""

    def __init__(self):
        Sym.__init__(self, "io_index")

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


def _unary(name):
    def f(x):
        return Sym(name, x)

    f.__name__ = name
    return f


tan, asin, acos, atan, sinh, cosh, tanh = (_unary(n) for n in ("tan", "asin", "acos", "atan", "sinh", "cosh", "tanh"))
exp, exp2, log, log2, inversesqrt = (_unary(n) for n in ("exp", "exp2", "log", "log2", "inversesqrt"))
floor, ceil, trunc, fract, sign = (_unary(n) for n in ("floor", "ceil", "trunc", "fract", "sign"))
round = _unary("round")  # noqa: A001 - mirrors vc.round


def atan2(y, x):
    return Sym("atan2", y, x)


def pow(x, y):  # noqa: A001 - mirrors vc.pow
    return Sym("pow", x, y)


def mod(x, y):
    return Sym("mod", x, y)


def fma(a, b, c):
    return Sym("fma", a, b, c)


def clamp(x, lo, hi):
    return Sym("clamp", x, lo, hi)


clip = clamp


def mix(x, y, a):
    return Sym("mix", x, y, a)


def complex_from_euler_angle(angle):
    return Sym("make", cos(angle), sin(angle))


def ravel_index(index, shape):
    """Flat index -> (x, y[, z]) components in a 2-D or 3-D shape
    (vkdispatch/codegen/functions/index_raveling.py:55-77)."""
    shape = tuple(int(v) for v in shape)
    if len(shape) == 2:
        return SymVec((index // shape[1], index % shape[1]))
    if len(shape) == 3:
        return SymVec((index // (shape[1] * shape[2]), (index // shape[2]) % shape[1], index % shape[2]))
    raise ValueError(f"Shape must have 2 or 3 elements, not '{shape}'!")


def unravel_index(index, shape):
    """(x, y[, z]) components -> flat index in a 2-D or 3-D shape
    (vkdispatch/codegen/functions/index_raveling.py:79-96)."""
    shape = tuple(int(v) for v in shape)
    if not isinstance(index, (tuple, list)):
        return index
    if len(index) > len(shape):
        raise ValueError(f"Index ({index}) must have the same number of elements as shape ({shape})!")
    if len(index) == 2:
        return index[0] * shape[1] + index[1]
    if len(index) == 3:
        return index[0] * (shape[1] * shape[2]) + index[1] * shape[2] + index[2]
    return index[0]


def length(x):
    return Sym("length", x)


def abs(x):  # noqa: A001 - mirrors vc.abs
    return Sym("abs", x)


def min(a, b):  # noqa: A001
    return Sym("min", a, b)


def max(a, b):  # noqa: A001
    return Sym("max", a, b)


# --- control flow inside FFT maps (vkdispatch/codegen/functions/control_flow.py)
# Each block is recorded as events around the statements traced inside it
# and lowered to the same C++ block in the map's hook.
@contextlib.contextmanager
def if_block(cond):
    from .fft import maps

    maps.trace_control("if", cond)
    yield
    maps.trace_control("end")


@contextlib.contextmanager
def else_if_block(cond):
    from .fft import maps

    maps.trace_control("elif", cond)
    yield
    maps.trace_control("end")


@contextlib.contextmanager
def else_block():
    from .fft import maps

    maps.trace_control("else")
    yield
    maps.trace_control("end")


@contextlib.contextmanager
def while_block(cond):
    from .fft import maps

    maps.trace_control("while", cond)
    yield
    maps.trace_control("end")


def any(*args):  # noqa: A001 - mirrors vc.any
    """Logical or of traced conditions."""
    return Sym("lor", *args)


def all(*args):  # noqa: A001 - mirrors vc.all
    """Logical and of traced conditions."""
    return Sym("land", *args)


# --- used by FFT map hooks (vkdispatch_gb300/fft/maps.py traces them) -------
def to_dtype(var_type, *args):
    """Cast (one argument) or build a value of var_type from components."""
    if len(args) == 1:
        return Sym("cast", args[0], var_type)
    return Sym("make", *args)


def to_complex(x):
    return Sym("to_complex", x)


def mult_complex(a, b):
    return Sym("cmul", a, b)


def new_register(var_type, *args, var_name=None):
    from .fft import maps

    return maps.new_trace_register(var_type, *args)


def new_complex_register(*args, var_name=None):
    return new_register(c64, *args)


new_complex64_register = new_complex_register


def new_float_register(*args, var_name=None):
    return new_register(f32, *args)


def new_int_register(*args, var_name=None):
    return new_register(i32, *args)
