"""Map hooks that the functor menu does not cover, compiled at run time.

The reference traces input_map / output_map / kernel_map callbacks into the
FFT shader it generates (vkdispatch/fft/io_manager.py:107-155,
vkdispatch/shader/map.py:29-40).  Here the same callbacks are traced once
with symbolic values (vkdispatch_gb300/fft/maps.py) and the recorded events
are lowered to a C++ hooks struct -- load (input map), store (output map)
and kernel (kernel map) functions of one element -- that libvdx compiles
with NVRTC into its own FFT kernel template (vdx_map_plan_create, csrc/
fft_mapped.cuh).  The FFT passes stay hand-written; only the element I/O and
the spectrum operation are user code.

Buffers over non-contiguous arrays (from_cuda_array with
require_contiguous=False) run through the same hooks: every index into
them, default or user-written, becomes the sum of coordinate * stride.

Supported inside maps: buffer loads and stores at any integer index
expression (io_index, fft_index, fft_size, mapped_kernel_index(), integer
arithmetic, vc.ravel_index / vc.unravel_index), scalar map arguments
(vc.Var[...]), read_from_buffer / write_to_buffer with an io_index, register
and component assignments, new_register temporaries, + - * / // % and
unary minus, vc.mult_complex, conjugate(), to_dtype / to_complex and the
math functions of vkdispatch_gb300.codegen, and control flow: vc.if_block,
else_if_block, else_block and while_block around traced statements, with
conditions built from comparisons, vc.any / vc.all and integer ~ (lowered to
the same C++ blocks; a value used as a condition is true when nonzero).
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

from .. import _lib as L
from .. import codegen as vc
from .. import dtypes as dt
from . import maps as M

MAX_BUFFERS = 8
MAX_SCALARS = 8

# element types the hooks can load and store: dtype -> (C++ storage type, kind)
_STORAGE = {
    dt.complex64: ("vdx::Cx<float>", "c"),
    dt.complex128: ("vdx::Cx<double>", "c"),
    dt.complex32: ("vdx::c32s", "c"),
    dt.float32: ("float", "f"),
    dt.float64: ("double", "f"),
    dt.int32: ("int", "i"),
    dt.uint32: ("unsigned", "i"),
    dt.vec2: ("vdx::Cx<float>", "c"),  # two float lanes, laid out as complex64
}

_UNARY = {"sin", "cos", "tan", "asin", "acos", "atan", "sinh", "cosh", "tanh", "exp", "exp2", "log", "log2", "sqrt",
          "inversesqrt", "abs", "floor", "ceil", "trunc", "round", "fract", "sign"}


def phys_index(buf, ix: str) -> str:
    """The element offset of flat index ix (in the buffer's shape) of a
    buffer: ix itself in C order, else the sum of coordinate * stride."""
    strides = getattr(buf, "strides", None)
    if strides is None:
        return ix
    shape = tuple(int(d) for d in buf.shape)
    terms = []
    for i, (d, st) in enumerate(zip(shape, strides)):
        inner = 1
        for x in shape[i + 1:]:
            inner *= x
        c = f"(({ix}) / {inner}LL)" if inner > 1 else f"({ix})"
        if i > 0 and d > 1:
            c = f"({c} % {d}LL)"
        if d > 1 and st:
            terms.append(f"{c} * {st}LL")
    return "(" + (" + ".join(terms) or "0LL") + ")"


_COMPARE = {"lt": "<", "le": "<=", "gt": ">", "ge": ">=", "eq": "==", "ne": "!="}


def _wider(*kinds: str) -> str:
    return "c" if "c" in kinds else "f" if "f" in kinds else "i"


@dataclass
class Slots:
    """Where each map argument lives in vdx_map_args."""

    buffers: List[object] = field(default_factory=list)  # Buffer objects, slot order
    fscalars: List[float] = field(default_factory=list)
    iscalars: List[int] = field(default_factory=list)

    def add_buffer(self, buf) -> int:
        if len(self.buffers) >= MAX_BUFFERS:
            raise NotImplementedError(f"map hooks take at most {MAX_BUFFERS} buffers")
        self.buffers.append(buf)
        return len(self.buffers) - 1

    def add_scalar(self, value, var_type) -> Tuple[str, int]:
        if var_type in (dt.int32, dt.uint32):
            if len(self.iscalars) >= MAX_SCALARS:
                raise NotImplementedError(f"map hooks take at most {MAX_SCALARS} integer scalars")
            self.iscalars.append(int(value))
            return "i", len(self.iscalars) - 1
        if len(self.fscalars) >= MAX_SCALARS:
            raise NotImplementedError(f"map hooks take at most {MAX_SCALARS} floating-point scalars")
        self.fscalars.append(float(value))
        return "f", len(self.fscalars) - 1


class _Lower:
    """Lowers one traced map (its events and argument bindings) to C++
    statements inside a hook whose register variable is ``reg``."""

    def __init__(self, name: str, types, scalar_flags, args, slots: Slots):
        self.name = name
        self.types = types
        self.bind: Dict[int, Tuple[str, int]] = {}
        self.objs: Dict[int, object] = {}
        self.regs: Dict[str, str] = {"reg": "c"}
        for i, (t, sc, a) in enumerate(zip(types, scalar_flags, args)):
            if sc:
                self.bind[i] = ("s",) + slots.add_scalar(a, t)
            else:
                if t not in _STORAGE:
                    raise NotImplementedError(f"map {name}: buffers of {t.name} are not supported by map hooks")
                if getattr(a, "var_type", None) is not None and a.var_type != t:
                    raise ValueError(f"map {name}: buffer of type {a.var_type.name} passed for a {t.name} argument")
                self.bind[i] = ("b", slots.add_buffer(a))
                self.objs[i] = a

    def fail(self, what):
        raise NotImplementedError(f"map {self.name}: {what} is not supported by the map-hook compiler")

    # ---- expressions: (C++ code, kind) with kind in i (integer), f (real), c (complex)
    def expr(self, e) -> Tuple[str, str]:
        if isinstance(e, bool):
            return ("1" if e else "0"), "i"
        if isinstance(e, int):
            return f"(long long)({e})", "i"
        if isinstance(e, float):
            return f"Re({e!r})", "f"
        if isinstance(e, complex):
            return f"vdx::mk<Re>(Re({e.real!r}), Re({e.imag!r}))", "c"
        if isinstance(e, vc.SymVec):
            self.fail("an index vector used as a value (pass it to vc.unravel_index)")
        if isinstance(e, vc._IoIndex):
            return "io", "i"
        if not isinstance(e, vc.Sym):
            self.fail(f"the value {e!r}")
        op, a = e.op, e.args
        if op == "io_index":
            return "io", "i"
        if op == "fft_index":
            return "(long long)k", "i"
        if op == "fft_size":
            return "(long long)n", "i"
        if op == "kidx":
            return "m.kidx", "i"
        if op == "scalar":
            kind, slot = self.bind[a[0]][1:]
            return (f"m.is[{slot}]", "i") if kind == "i" else (f"Re(m.fs[{slot}])", "f")
        if op == "reg":
            kind = self.regs.get(a[0])
            if kind is None:
                self.fail(f"register {a[0]}")
            return a[0], kind
        if op in ("reg_real", "reg_imag"):
            return f"{a[0]}.{'x' if op == 'reg_real' else 'y'}", "f"
        if op == "load":
            return self.load(a[0], a[1] if len(a) > 1 else vc.Sym("io_index"))
        if op in ("real", "imag"):
            c, k = self.expr(a[0])
            if k == "c":
                return f"({c}).{'x' if op == 'real' else 'y'}", "f"
            return (c, k) if op == "real" else ("Re(0)", "f")
        if op in ("add", "sub", "mul", "div"):
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            k = _wider(ka, kb)
            if k == "i":  # integer (index) arithmetic stays integer
                return f"({ca} {dict(add='+', sub='-', mul='*', div='/')[op]} {cb})", "i"
            return f"vdx::mapops::{op}({self.real(ca, ka)}, {self.real(cb, kb)})", k
        if op == "floordiv":
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            if ka == kb == "i":
                return f"({ca} / {cb})", "i"
            return f"vdx::mapops::m_floor(vdx::mapops::div({self.real(ca, ka)}, {self.real(cb, kb)}))", _wider(ka, kb)
        if op == "mod":
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            if ka == kb == "i":
                return f"({ca} % {cb})", "i"
            if "c" in (ka, kb):
                self.fail("% on complex values")
            return f"vdx::mapops::m_mod({self.real(ca, ka)}, {self.real(cb, kb)})", "f"
        if op in _COMPARE:
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            if "c" in (ka, kb):
                self.fail(f"a comparison ({op}) of complex values")
            k = _wider(ka, kb)
            return f"({self.as_kind(ca, ka, k)} {_COMPARE[op]} {self.as_kind(cb, kb, k)})", "i"
        if op in ("lor", "land"):
            return "(" + (" || " if op == "lor" else " && ").join(self.cond(x) for x in a) + ")", "i"
        if op == "invert":
            c, k = self.expr(a[0])
            if k != "i":
                self.fail("~ on a non-integer value")
            return f"(~{c})", "i"
        if op in ("and", "or", "xor"):
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            if ka != "i" or kb != "i":
                self.fail(f"bitwise {op} on non-integer values")
            return f"({ca} {'&' if op == 'and' else '|' if op == 'or' else '^'} {cb})", "i"
        if op == "neg":
            c, k = self.expr(a[0])
            return f"vdx::mapops::neg({c})", k
        if op in _UNARY:
            c, k = self.expr(a[0])
            if k == "i" and op in ("abs",):
                return f"vdx::mapops::m_abs({c})", "i"
            return f"vdx::mapops::m_{op}({self.real(c, k) if k == 'i' else c})", "f" if k == "i" else k
        if op == "length":
            c, k = self.expr(a[0])
            return f"vdx::mapops::m_length({self.real(c, k)})", "f"
        if op in ("min", "max"):
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            k = _wider(ka, kb)
            return f"vdx::mapops::m_{op}({self.as_kind(ca, ka, k)}, {self.as_kind(cb, kb, k)})", k
        if op == "clamp":
            parts = [self.expr(x) for x in a]
            k = _wider(*(p[1] for p in parts))
            return "vdx::mapops::m_clamp(" + ", ".join(self.as_kind(c, kk, k) for c, kk in parts) + ")", k
        if op == "mix":
            (cx, kx), (cy, ky), (ca, ka) = (self.expr(x) for x in a)
            k = _wider(kx, ky)
            return (f"vdx::mapops::m_mix({self.as_kind(cx, kx, k)}, {self.as_kind(cy, ky, k)}, "
                    f"{self.as_kind(ca, ka, 'f')})"), k
        if op in ("pow", "atan2"):
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            if "c" in (ka, kb):
                self.fail(f"{op} on complex values")
            return f"vdx::mapops::m_{op}({self.real(ca, ka)}, {self.real(cb, kb)})", "f"
        if op == "fma":
            parts = [self.expr(x) for x in a]
            if any(k == "c" for _, k in parts):
                self.fail("fma on complex values")
            return "vdx::mapops::m_fma(" + ", ".join(self.real(c, k) for c, k in parts) + ")", "f"
        if op == "cmul":
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            return f"vdx::mapops::cplx_mul({self.as_kind(ca, ka, 'c')}, {self.as_kind(cb, kb, 'c')})", "c"
        if op == "conj":
            c, k = self.expr(a[0])
            return f"vdx::mapops::cplx_conj({self.as_kind(c, k, 'c')})", "c"
        if op == "to_complex":
            c, k = self.expr(a[0])
            return (c, k) if k == "c" else (f"vdx::mk<Re>({self.real(c, k)}, Re(0))", "c")
        if op == "make":
            if len(a) != 2:
                self.fail("to_dtype with more than two components")
            (ca, ka), (cb, kb) = self.expr(a[0]), self.expr(a[1])
            if "c" in (ka, kb):
                self.fail("a complex value built from complex components")
            return f"vdx::mk<Re>({self.real(ca, ka)}, {self.real(cb, kb)})", "c"
        if op == "cast":
            c, k = self.expr(a[0])
            target = a[1] if len(a) > 1 else None
            if target is None or getattr(target, "is_complex", False):
                return self.as_kind(c, k, "c"), "c"
            if target in (dt.int32, dt.uint32):
                if k == "c":
                    self.fail("a complex value cast to an integer")
                return f"(long long)({c})", "i"
            if k == "c":
                self.fail("a complex value cast to a real type")
            return self.real(c, k), "f"
        self.fail(f"the operation {op}")

    def real(self, code, kind):
        return f"Re({code})" if kind == "i" else code

    def as_kind(self, code, kind, want):
        if kind == want:
            return code
        if want == "c":
            return f"vdx::mapops::to_cx<Re>({code})"
        if want == "f":
            if kind == "c":
                self.fail("a complex value where a real one is needed")
            return f"Re({code})"
        if kind != "i":
            self.fail("a floating-point value where an integer is needed")
        return code

    def index(self, idx) -> str:
        if idx is None:
            return "io"
        c, k = self.expr(idx)
        if k != "i":
            self.fail("a non-integer buffer index")
        return c

    def buffer(self, i):
        b = self.bind.get(i)
        if b is None or b[0] != "b":
            self.fail(f"argument {i} used as a buffer")
        return b[1], _STORAGE[self.types[i]]

    def load(self, i, idx) -> Tuple[str, str]:
        slot, (ctype, kind) = self.buffer(i)
        ix = phys_index(self.objs[i], self.index(idx))
        if kind == "c":
            return self.ldc(ctype, slot, ix), "c"
        if kind == "f":
            return f"vdx::map_ld<{ctype}>(m, {slot}, {ix})", "f"
        return f"(long long)vdx::map_ld<{ctype}>(m, {slot}, {ix})", "i"

    @staticmethod
    def ldc(ctype, slot, ix) -> str:
        if ctype == "vdx::c32s":  # complex32 converts through float
            return f"vdx::mapops::to_cx<Re>(vdx::map_ldc<vdx::c32s, float>(m, {slot}, {ix}))"
        return f"vdx::map_ldc<{ctype}, Re>(m, {slot}, {ix})"

    @staticmethod
    def stc(ctype, slot, ix, val) -> str:
        if ctype == "vdx::c32s":
            return f"vdx::map_stc<vdx::c32s, float>(m, {slot}, {ix}, vdx::mapops::to_cx<float>({val}));"
        return f"vdx::map_stc<{ctype}, Re>(m, {slot}, {ix}, {val});"

    def store(self, i, idx, value) -> str:
        slot, (ctype, kind) = self.buffer(i)
        ix = phys_index(self.objs[i], self.index(idx))
        c, k = self.expr(value)
        if kind == "c":
            return self.stc(ctype, slot, ix, self.as_kind(c, k, "c"))
        if k == "c":
            self.fail("a complex value stored to a real buffer")
        return f"vdx::map_st<{ctype}>(m, {slot}, {ix}, ({ctype})({c}));"

    # ---- statements
    def cond(self, e) -> str:
        """A traced value used as a condition: nonzero is true."""
        c, k = self.expr(e)
        if k == "c":
            self.fail("a complex value as a condition")
        return f"({c} != {'0' if k == 'i' else 'Re(0)'})"

    def statements(self, events) -> List[str]:
        out = []
        depth = 0
        for ev in events:
            kind = ev[0]
            start = len(out)
            if kind in ("if", "elif", "while"):
                if kind == "elif" and not (out and out[-1].strip() == "}"):
                    self.fail("else_if_block without an if_block right before it")
                word = {"if": "if", "elif": "else if", "while": "while"}[kind]
                out.append(f"{word} ({self.cond(ev[1])}) {{")
                depth += 1
            elif kind == "else":
                if not (out and out[-1].strip() == "}"):
                    self.fail("else_block without an if_block right before it")
                out.append("else {")
                depth += 1
            elif kind == "end":
                out.append("}")
                depth -= 1
            elif kind == "new":
                _, name, var_type, init = ev
                if getattr(var_type, "is_complex", False):
                    self.regs[name] = "c"
                    if not init:
                        out.append(f"vdx::Cx<Re> {name} = vdx::mk<Re>(Re(0), Re(0));")
                    elif len(init) == 1:
                        c, k = self.expr(init[0])
                        out.append(f"vdx::Cx<Re> {name} = {self.as_kind(c, k, 'c')};")
                    else:
                        c, _ = self.expr(vc.Sym("make", *init))
                        out.append(f"vdx::Cx<Re> {name} = {c};")
                else:
                    k = "i" if var_type in (dt.int32, dt.uint32) else "f"
                    self.regs[name] = k
                    init_code = self.as_kind(*self.expr(init[0]), k) if init else "0"
                    out.append(f"{'long long' if k == 'i' else 'Re'} {name} = {init_code};")
            elif kind == "read":
                _, i, reg, _, _, idx = ev
                c, k = self.load(i, idx)
                out.append(f"{reg} = {self.as_kind(c, k, 'c')};")
            elif kind == "write":
                _, i, _, _, reg, idx = ev
                out.append(self.store(i, idx, vc.Sym("reg", "reg") if reg is None else reg))
            elif kind in ("set_real", "set_imag"):
                _, reg, value = ev
                if self.regs.get(reg) != "c":
                    self.fail(f"a component assignment to {reg}")
                c, k = self.expr(value)
                out.append(f"{reg}.{'x' if kind == 'set_real' else 'y'} = {self.as_kind(c, k, 'f')};")
            elif kind == "set":
                _, reg, value = ev
                c, k = self.expr(value)
                out.append(f"{reg} = {self.as_kind(c, k, self.regs.get(reg, 'c'))};")
            elif kind == "store":
                _, i, value, idx = ev
                out.append(self.store(i, idx, value))
            else:
                self.fail(f"the event {kind}")
            # statements inside blocks are indented by their depth
            lead = "  " * (depth - (1 if kind in ("if", "elif", "while", "else") else 0))
            if lead:
                out[start:] = [lead + ln for ln in out[start:]]
        if depth != 0:
            self.fail("an unterminated control-flow block")
        return out


def _trace_events(mf, role):
    events, _ = M._trace(mf, role)
    return events


def _hook(signature: str, body: List[str]) -> str:
    lines = "\n".join("    " + b for b in body)
    return f"  template <class Re>\n  __device__ static {signature} {{\n{lines}\n  }}\n"


@dataclass
class MapSpec:
    """One call's hooks: the C++ source and the argument slots it reads."""

    source: str
    slots: Slots
    stage_input: Optional[object] = None  # a buffer the default load reads from a staged copy


def build_hooks(outs, ins, kers, input_map, output_map, kernel_map, conv: bool, kernel_broadcast_slab: int = 0,
                ) -> MapSpec:
    """Lowers the call's maps (None for absent ones) to one hooks struct.

    outs / ins / kers are the call's buffers (and scalars) in the
    reference's argument order (vkdispatch/fft/io_manager.py:58-105): the
    output map's arguments or the output buffer, the input map's arguments
    or the input buffer, the kernel map's arguments or the kernel buffer."""
    slots = Slots()

    def lowered(mf, role, args):
        if len(args) != len(mf.buffer_types):
            raise ValueError(f"{role} map {mf.func.__name__} takes {len(mf.buffer_types)} arguments, "
                             f"{len(args)} given")
        low = _Lower(mf.func.__name__, mf.input_dtypes(), mf.arg_is_scalar(), args, slots)
        return low.statements(_trace_events(mf, role))

    def complex_buffer(b, what):
        if b is None or getattr(b, "var_type", None) not in _STORAGE or _STORAGE[b.var_type][1] != "c":
            raise ValueError(f"the {what} buffer must be a complex Buffer")
        return slots.add_buffer(b), _STORAGE[b.var_type][0]

    # store (output map)
    if output_map is not None:
        body = ["using namespace vdx::mapops;", "vdx::Cx<Re> reg = v;"] + lowered(output_map, "output", outs)
        body.append("(void)reg;")
    else:
        slot, ctype = complex_buffer(outs[0], "output")
        body = [_Lower.stc(ctype, slot, phys_index(outs[0], "io"), "v")]
    store = _hook("void store(const vdx::MapArgs& m, vdx::Cx<Re> v, long long io, int k, int n)",
                  body + ["(void)k; (void)n; (void)m;"])
    # load (input map)
    if input_map is not None:
        body = ["using namespace vdx::mapops;", "vdx::Cx<Re> reg = vdx::mk<Re>(Re(0), Re(0));"]
        body += lowered(input_map, "input", ins) + ["return reg;"]
    else:
        src = ins[0] if ins else outs[0]
        slot, ctype = complex_buffer(src, "input")
        body = [f"return {_Lower.ldc(ctype, slot, phys_index(src, 'io'))};"]
    load = _hook("vdx::Cx<Re> load(const vdx::MapArgs& m, long long io, int k, int n)",
                 ["(void)k; (void)n; (void)m;"] + body)
    # kernel (kernel map), convolutions only
    if not conv:
        body = ["return v;"]
    elif kernel_map is not None:
        body = ["using namespace vdx::mapops;", "vdx::Cx<Re> reg = v;"] + lowered(kernel_map, "kernel", kers)
        body.append("return reg;")
    else:
        slot, ctype = complex_buffer(kers[0] if kers else None, "kernel")
        kio = f"(io % {kernel_broadcast_slab}LL)" if kernel_broadcast_slab else "io"
        body = [f"return vdx::cmulc(v, {_Lower.ldc(ctype, slot, phys_index(kers[0], kio))});"]
    kernel = _hook("vdx::Cx<Re> kernel(const vdx::MapArgs& m, vdx::Cx<Re> v, long long io, int k, int n)",
                   ["(void)k; (void)n; (void)m; (void)io;"] + body)
    src = "struct VdxHooks {\n" + load + store + kernel + "};\n"
    return MapSpec(src, slots)


# ---------------------------------------------------------------------------
# plans and launches
# ---------------------------------------------------------------------------
_plans: Dict[tuple, object] = {}


class MapPlan:
    def __init__(self, desc, source: str):
        h = ctypes.c_void_p()
        L.check(L.lib().vdx_map_plan_create(ctypes.byref(desc), source.encode(), ctypes.byref(h)), "map plan")
        self.handle = h

    def source(self) -> str:
        buf = ctypes.create_string_buffer(1 << 18)
        L.check(L.lib().vdx_map_plan_source(self.handle, buf, len(buf)), "map source")
        return buf.value.decode()

    def exec(self, args, stream) -> None:
        L.check(L.lib().vdx_map_exec(self.handle, ctypes.byref(args), stream), "map exec")

    def status(self, reset: bool = False) -> int:
        """1 when a launch of this plan indexed a map buffer out of range
        (synchronous); reset clears it."""
        st = ctypes.c_int()
        L.check(L.lib().vdx_map_plan_status(self.handle, ctypes.byref(st), int(reset)), "map status")
        return int(st.value)

    def __del__(self):
        try:
            if self.handle:
                L.lib().vdx_map_plan_destroy(self.handle)
        except Exception:
            pass


def out_of_range(reset: bool = True) -> bool:
    """Whether any compiled map plan of the current device indexed a map
    buffer outside its extent since the last reset (synchronous)."""
    import torch

    dev = torch.cuda.current_device()
    return any(p.status(reset) for k, p in list(_plans.items()) if k[0] == dev)


def get_plan(shape, axis, conv, inverse, normalize, code, sig, source) -> MapPlan:
    import torch

    key = (torch.cuda.current_device(), tuple(shape), axis, conv, inverse, normalize, code, sig, source)
    p = _plans.get(key)
    if p is None:
        d = L.FftDesc()
        d.ndim = len(shape)
        for i, s in enumerate(shape):
            d.shape[i] = int(s)
        d.axis = axis
        d.kind = L.VDX_KIND_CONV if conv else L.VDX_KIND_C2C
        d.inverse = int(bool(inverse))
        d.normalize = int(normalize)
        d.io_type = d.compute_type = code
        d.kernel_type = code
        d.signal_lo, d.signal_hi = (-1, -1) if sig is None else sig
        p = MapPlan(d, source)
        _plans[key] = p
    return p


def extent(buf) -> int:
    """Elements a buffer may be indexed with: its size in C order, else one
    past its largest strided offset."""
    strides = getattr(buf, "strides", None)
    if strides is None:
        return int(buf.size)
    return 1 + sum((int(d) - 1) * int(s) for d, s in zip(buf.shape, strides))


def make_args(slots: Slots, kernel_index: int = 0):
    a = L.MapArgs()
    for i, b in enumerate(slots.buffers):
        a.buffers[i] = b.ptr
        a.counts[i] = extent(b)
    for i, v in enumerate(slots.fscalars):
        a.fscalars[i] = v
    for i, v in enumerate(slots.iscalars):
        a.iscalars[i] = v
    a.kernel_index = kernel_index
    return a
