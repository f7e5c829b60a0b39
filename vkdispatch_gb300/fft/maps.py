"""Map hooks for FFTs and convolutions: `vd.fft.read_op()` / `write_op()` and
the recognition of user map functions (vkdispatch/fft/io_manager.py:23-37,
vkdispatch/shader/map.py:10-68).

A map function is called once with symbolic buffers and read/write-op
objects that record what it does.  The record is first matched against the
menu of maps that libvdx's ahead-of-time kernels implement; a map outside
the menu is lowered to C++ and compiled at run time instead
(vkdispatch_gb300/fft/jit.py), and only constructs that compiler lacks raise
NotImplementedError naming the map.

  input maps   read_op().read_from_buffer(buf)           complex load of buf's type
               register.real = buf[io_index]; .imag = 0  real load (imaginary 0)
  output maps  write_op().write_to_buffer(buf)           complex store in buf's type
               buf[io_index] = write_op().register.real  real-part store
  kernel maps  read into a register k, register *= conj(k)   conjugate product (the default)
               read into a register k, register *= k         plain product
               register *= to_complex(scale[io_index])       real scale buffer
               (empty body)                                  no spectrum operation

With kernel_num > 1 (vkdispatch/fft/shader_factories.py:166-193) a kernel
map's read_from_buffer and an output map's write_to_buffer may index
``io_index + mapped_kernel_index() * C``: kernel k then reads (or writes)
C * k elements further along its buffer.
"""

from __future__ import annotations

import threading
from dataclasses import dataclass
from typing import Optional

from .. import codegen as vc
from .. import dtypes as dt

_tls = threading.local()


class TraceRegister(vc.Sym):
    """An FFT register (or a new_register temporary) while a map is traced:
    arithmetic on it builds expressions over ``reg(name)``; assignments to
    ``.real``, ``.imag`` or ``[:]`` are recorded as events."""

    def __init__(self, name: str, events: list):
        vc.Sym.__init__(self, "reg", name)
        object.__setattr__(self, "_name", name)
        object.__setattr__(self, "_events", events)

    @property
    def real(self):
        return vc.Sym("reg_real", self._name)

    @real.setter
    def real(self, value):
        self._events.append(("set_real", self._name, value))

    @property
    def imag(self):
        return vc.Sym("reg_imag", self._name)

    @imag.setter
    def imag(self, value):
        self._events.append(("set_imag", self._name, value))

    @property
    def x(self):
        return self.real

    @property
    def y(self):
        return self.imag

    def __setitem__(self, key, value):
        self._events.append(("set", self._name, value))

    # in-place arithmetic assigns the register, as the reference's variables
    # do (vkdispatch/codegen/variables/variables.py:399-402); Python then
    # rebinds the name to the register itself
    def _assign(self, value):
        self._events.append(("set", self._name, value))
        return self

    def __iadd__(self, other):
        return self._assign(vc.Sym.__add__(self, other))

    def __isub__(self, other):
        return self._assign(vc.Sym.__sub__(self, other))

    def __imul__(self, other):
        return self._assign(vc.Sym.__mul__(self, other))

    def __itruediv__(self, other):
        return self._assign(vc.Sym.__truediv__(self, other))

    def conjugate(self):
        return vc.Sym("conj", vc.Sym("reg", self._name))

    @property
    def var_type(self):
        return dt.complex64

    def __repr__(self):
        return f"reg({self._name})"


class _TraceBuffer:
    def __init__(self, index: int, var_type, events: list):
        self.index = index
        self.var_type = var_type
        self._events = events

    def __getitem__(self, idx):
        return vc.Sym("load", self.index, idx)

    def __setitem__(self, idx, value):
        self._events.append(("store", self.index, value, idx))


class _TraceScalar(vc.Sym):
    """A scalar map argument (``vc.Var[...]``)."""

    def __init__(self, index: int, var_type):
        vc.Sym.__init__(self, "scalar", index)
        self.var_type = var_type


class _TraceOp:
    def __init__(self, events: list):
        self._events = events
        self.register = TraceRegister("reg", events)
        self.io_index = vc.Sym("io_index")
        self.fft_index = vc.Sym("fft_index")
        self.fft_size = vc.Sym("fft_size")

    def read_from_buffer(self, buffer, register=None, io_index=None):
        name = register._name if isinstance(register, TraceRegister) else "reg"
        stride = kernel_stride(io_index)
        self._events.append(("read", buffer.index, name, stride is not None, stride or 0, io_index))

    def write_to_buffer(self, buffer, register=None, io_index=None):
        stride = kernel_stride(io_index)
        self._events.append(("write", buffer.index, stride is not None, stride or 0, register, io_index))


def mapped_kernel_index():
    """The kernel index of a multi-kernel convolution while its maps are
    traced (a symbol to index buffers with), else None
    (vkdispatch/fft/shader_factories.py:99-105)."""
    return getattr(_tls, "kidx", None)


def _is_io_index(e) -> bool:
    return isinstance(e, vc.Sym) and e.op == "io_index"


def kernel_stride(expr):
    """Elements per kernel index of an io_index expression: 0 for None or
    io_index itself, C for io_index + mapped_kernel_index() * C (either operand
    order), None for any other expression."""
    if expr is None or _is_io_index(expr):
        return 0
    if isinstance(expr, vc.Sym) and expr.op == "add" and len(expr.args) == 2:
        a, b = expr.args
        if _is_io_index(b):
            a, b = b, a
        if _is_io_index(a) and isinstance(b, vc.Sym) and b.op == "mul" and len(b.args) == 2:
            x, y = b.args
            if isinstance(y, vc.Sym) and y.op == "kidx":
                x, y = y, x
            if isinstance(x, vc.Sym) and x.op == "kidx" and isinstance(y, int) and y >= 0:
                return y
    return None


def read_op():
    op = getattr(_tls, "read", None)
    if op is None:
        raise ValueError("No global read operation is set for the current thread!")
    return op


def write_op():
    op = getattr(_tls, "write", None)
    if op is None:
        raise ValueError("No global write operation is set for the current thread!")
    return op


def trace_control(kind: str, cond=None) -> None:
    """Records the start ("if", "elif", "else", "while") or the end ("end")
    of a control-flow block of the map being traced."""
    events = getattr(_tls, "events", None)
    if events is None:
        raise NotImplementedError("control-flow blocks are traced only inside FFT map functions")
    events.append((kind,) if cond is None else (kind, cond))


def new_trace_register(var_type, *args):
    events = getattr(_tls, "events", None)
    if events is None:
        raise ValueError("new_register is only available while a map function is traced")
    n = getattr(_tls, "nreg", 0)
    _tls.nreg = n + 1
    name = f"tmp{n}"
    events.append(("new", name, var_type, args))
    return TraceRegister(name, events)


def _trace(mf, role: str):
    events: list = []
    types = mf.input_dtypes()
    scalar = mf.arg_is_scalar()
    bufs = [_TraceScalar(i, t) if sc else _TraceBuffer(i, t, events) for i, (t, sc) in enumerate(zip(types, scalar))]
    _tls.events, _tls.nreg = events, 0
    _tls.kidx = vc.Sym("kidx")
    _tls.read = _TraceOp(events) if role in ("input", "kernel") else None
    _tls.write = _TraceOp(events) if role == "output" else None
    try:
        mf.func(*bufs)
    except NotImplementedError:
        raise
    except Exception as e:  # noqa: BLE001
        raise NotImplementedError(f"{role} map {mf.func.__name__} could not be traced: {e}") from e
    finally:
        _tls.events = _tls.read = _tls.write = _tls.kidx = None
    return events, types


def _has(expr, op, arg=None) -> bool:
    if not isinstance(expr, vc.Sym):
        return False
    if expr.op == op and (arg is None or arg in expr.args):
        return True
    return any(_has(a, op, arg) for a in expr.args)


_CONTROL = ("if", "elif", "else", "while", "end")


def _menu_events(ev):
    """The events the menu matchers look at: new_register temporaries
    declared without an initial value carry no operation of their own.  A map
    with control flow is outside the menu (the map-hook compiler takes it)."""
    if any(e[0] in _CONTROL for e in ev):
        raise NotImplementedError("maps with control flow are outside the functor menu")
    return [e for e in ev if not (e[0] == "new" and not e[3])]


def _loads_at_io(expr) -> bool:
    """Every buffer load inside expr reads at io_index itself."""
    if not isinstance(expr, vc.Sym):
        return True
    if expr.op == "load":
        return len(expr.args) > 1 and isinstance(expr.args[1], vc.Sym) and expr.args[1].op == "io_index"
    return all(_loads_at_io(a) for a in expr.args)


def _is_reg_real(expr) -> bool:
    """expr is the FFT register's real part, possibly cast."""
    while isinstance(expr, vc.Sym) and expr.op == "cast":
        expr = expr.args[0]
    return isinstance(expr, vc.Sym) and expr.op == "reg_real" and expr.args == ("reg",)


def _plain_cast_of_load(expr, buf) -> bool:
    """expr is buf[io_index], possibly cast: the menu's real-input load."""
    while isinstance(expr, vc.Sym) and expr.op == "cast":
        expr = expr.args[0]
    return (isinstance(expr, vc.Sym) and expr.op == "load" and expr.args[0] == buf
            and isinstance(expr.args[1], vc.Sym) and expr.args[1].op == "io_index")


def _is_zero(expr) -> bool:
    if isinstance(expr, (int, float)):
        return expr == 0
    return isinstance(expr, vc.Sym) and expr.op == "cast" and _is_zero(expr.args[0])


@dataclass
class IoMap:
    kind: str  # "complex" or "real"
    buffer: int  # index among the map's buffers
    var_type: object
    stride: int = 0  # elements per kernel index (multi-kernel convolutions)


@dataclass
class KernelMap:
    kind: str  # "conj_mul", "mul", "real_scale" or "identity"
    buffer: Optional[int]
    var_type: object
    stride: int = 0  # elements per kernel index (multi-kernel convolutions)


def classify_input(mf) -> IoMap:
    ev, types = _trace(mf, "input")
    ev = _menu_events(ev)
    name = mf.func.__name__
    if len(ev) == 1 and ev[0][0] == "read" and ev[0][2] == "reg" and ev[0][3] and ev[0][4] == 0:
        i = ev[0][1]
        if not types[i].is_complex:
            raise NotImplementedError(f"input map {name}: read_from_buffer needs a complex buffer")
        return IoMap("complex", i, types[i])
    sets = {e[0]: e for e in ev if e[1] == "reg"}
    if len(ev) == 2 and set(sets) == {"set_real", "set_imag"} and _is_zero(sets["set_imag"][2]):
        loads = [a for a in range(len(types)) if _has(sets["set_real"][2], "load", a)]
        if (len(loads) == 1 and types[loads[0]] in (dt.float32, dt.float64)
                and _plain_cast_of_load(sets["set_real"][2], loads[0])):
            return IoMap("real", loads[0], types[loads[0]])
    raise NotImplementedError(f"input map {name} is not in the supported map menu: {ev}")


def classify_output(mf) -> IoMap:
    ev, types = _trace(mf, "output")
    ev = _menu_events(ev)
    name = mf.func.__name__
    if len(ev) == 1 and ev[0][0] == "write" and ev[0][2] and ev[0][4] is None:
        i = ev[0][1]
        if not types[i].is_complex:
            raise NotImplementedError(f"output map {name}: write_to_buffer needs a complex buffer")
        return IoMap("complex", i, types[i], ev[0][3])
    if (len(ev) == 1 and ev[0][0] == "store" and _is_reg_real(ev[0][2])
            and isinstance(ev[0][3], vc.Sym) and ev[0][3].op == "io_index"):
        i = ev[0][1]
        if types[i] in (dt.float32, dt.float64):
            return IoMap("real", i, types[i])
    raise NotImplementedError(f"output map {name} is not in the supported map menu: {ev}")


def classify_kernel(mf) -> KernelMap:
    ev, types = _trace(mf, "kernel")
    ev = _menu_events(ev)
    name = mf.func.__name__
    if not ev:
        return KernelMap("identity", None, None)
    if len(ev) == 2 and ev[0][0] == "read" and ev[1][0] == "set" and ev[1][1] == "reg" and ev[0][3]:
        i, reg, stride = ev[0][1], ev[0][2], ev[0][4]
        prod = ev[1][2]
        if isinstance(prod, vc.Sym) and prod.op == "cmul" and types[i].is_complex:
            a, b = prod.args
            if isinstance(a, TraceRegister) and a._name == "reg":
                if isinstance(b, vc.Sym) and b.op == "conj" and b.args[0].args == (reg,):
                    return KernelMap("conj_mul", i, types[i], stride)
                if isinstance(b, TraceRegister) and b._name == reg:
                    return KernelMap("mul", i, types[i], stride)
    if len(ev) == 1 and ev[0][0] == "set" and ev[0][1] == "reg":
        prod = ev[0][2]
        if isinstance(prod, vc.Sym) and prod.op == "cmul" and _has(prod.args[1], "to_complex"):
            loads = [a for a in range(len(types)) if _has(prod.args[1], "load", a)]
            if (len(loads) == 1 and types[loads[0]] in (dt.float32, dt.float64) and _loads_at_io(prod.args[1])
                    and isinstance(prod.args[0], TraceRegister) and prod.args[0]._name == "reg"):
                return KernelMap("real_scale", loads[0], types[loads[0]])
    raise NotImplementedError(f"kernel map {name} is not in the supported map menu: {ev}")
