"""vd.reduce-compatible map-reduce API (vkdispatch/reduce/decorator.py:22-64,
operations.py:17-66, reduce_function.py:73-162).

``@reduce(identity)`` and ``@map_reduce(op)`` return a ReduceFunction whose
call enqueues the two libvdx reduction launches and returns a new Buffer in
the reference's layout: shape ``(parts + 1[, batch])`` with the results in
the first ``batch`` elements (``res.read(0)[0]`` for one row) and the
stage-1 partials after them.
"""

from __future__ import annotations

import ctypes
import dataclasses
import inspect
import re
from typing import List, Optional, Union

import numpy as np

from .. import _lib as L
from .. import codegen as vc
from .. import dtypes as dt
from .. import graph as G
from ..buffer import Buffer


@dataclasses.dataclass
class ReduceOp:
    name: str
    code: int
    identity: Union[int, float, str]


SubgroupAdd = ReduceOp("add", L.VDX_RED_ADD, 0)
SubgroupMul = ReduceOp("mul", L.VDX_RED_MUL, 1)
SubgroupMin = ReduceOp("min", L.VDX_RED_MIN, "inf")
SubgroupMax = ReduceOp("max", L.VDX_RED_MAX, "-inf")
SubgroupAnd = ReduceOp("and", L.VDX_RED_AND, -1)
SubgroupOr = ReduceOp("or", L.VDX_RED_OR, 0)
SubgroupXor = ReduceOp("xor", L.VDX_RED_XOR, 0)

_OPS = {"add": SubgroupAdd, "mul": SubgroupMul, "min": SubgroupMin, "max": SubgroupMax, "and": SubgroupAnd,
        "or": SubgroupOr, "xor": SubgroupXor}

mapped_io_index = vc.mapped_io_index


def _trace_reduction(func) -> ReduceOp:
    a, b = vc.Sym("a"), vc.Sym("b")
    try:
        r = func(a, b)
    except Exception as e:  # noqa: BLE001
        raise NotImplementedError(f"reduction {func.__name__} could not be traced: {e}") from e
    if isinstance(r, vc.Sym) and r.op in _OPS and len(r.args) == 2:
        ids = {x.op if isinstance(x, vc.Sym) else None for x in r.args}
        if ids == {"a", "b"}:
            return _OPS[r.op]
    raise NotImplementedError(f"reduction {func.__name__} is not one of add, mul, min, max, and, or, xor")


def _trace_map(func, in_types) -> int:
    bufs = [vc.SymBuffer(i, t) for i, t in enumerate(in_types)]
    try:
        r = func(*bufs)
    except Exception as e:  # noqa: BLE001
        raise NotImplementedError(f"map {func.__name__} could not be traced: {e}") from e

    def is_load(x):
        return (isinstance(x, vc.Sym) and x.op == "load" and x.args[:1] == (0,)
                and (len(x.args) == 1 or isinstance(x.args[1], vc._IoIndex)))

    if len(in_types) != 1:
        raise NotImplementedError(f"map {func.__name__}: maps over more than one buffer are not in the menu")
    if is_load(r):
        return L.VDX_MAP_IDENTITY
    if isinstance(r, vc.Sym):
        if r.op == "sin" and is_load(r.args[0]):
            return L.VDX_MAP_SIN
        if r.op in ("abs", "length") and is_load(r.args[0]):
            return L.VDX_MAP_ABS
        if r.op == "mul" and is_load(r.args[0]) and is_load(r.args[1]):
            return L.VDX_MAP_SQUARE
        if r.op == "real" and is_load(r.args[0]):
            return L.VDX_MAP_REAL
        if r.op == "imag" and is_load(r.args[0]):
            return L.VDX_MAP_IMAG
        if r.op == "sqrt":  # sqrt(re*re + im*im)
            s = r.args[0]
            if isinstance(s, vc.Sym) and s.op == "add":
                parts = {p.args[0].op if isinstance(p, vc.Sym) and p.op == "mul" and isinstance(p.args[0], vc.Sym)
                         else None for p in s.args}
                if parts == {"real", "imag"}:
                    return L.VDX_MAP_ABS
        if r.op == "add" and all(isinstance(p, vc.Sym) and p.op == "mul" for p in r.args):
            ops = {p.args[0].op for p in r.args if isinstance(p.args[0], vc.Sym)}
            if ops == {"real", "imag"}:
                return L.VDX_MAP_SQUARE
    raise NotImplementedError(f"map {func.__name__} ({r!r}) is not in the supported map menu")


def _signature(func):
    """Signature with string annotations (``from __future__ import
    annotations``) evaluated in the function's module."""
    try:
        return inspect.signature(func, eval_str=True)
    except (NameError, TypeError, SyntaxError, AttributeError):
        return inspect.signature(func)


def _named_dtype(name: str):
    t = getattr(vc, name, None)
    if isinstance(t, dt.dtype):
        return t
    t = getattr(dt, name, None)
    return t if isinstance(t, dt.dtype) else None


def _resolve_annotation(a):
    """String annotations that could not be evaluated (they name objects
    local to an enclosing function) resolve by dtype name:
    'x.Buff[x.complex64]' -> Buffer[complex64], 'x.float32' -> float32."""
    if not isinstance(a, str):
        return a
    m = re.fullmatch(r"\s*(?:[\w.]*\.)?(?:Buff|Buffer)\[\s*(?:[\w.]*\.)?(\w+)\s*\]\s*", a)
    if m and _named_dtype(m.group(1)) is not None:
        return vc.Buffer[_named_dtype(m.group(1))]
    m = re.fullmatch(r"\s*(?:[\w.]*\.)?Var\[\s*(?:[\w.]*\.)?(\w+)\s*\]\s*", a)
    if m and _named_dtype(m.group(1)) is not None:
        return vc.Var[_named_dtype(m.group(1))]
    m = re.fullmatch(r"\s*(?:[\w.]*\.)?(\w+)\s*", a)
    if m and _named_dtype(m.group(1)) is not None:
        return _named_dtype(m.group(1))
    raise ValueError(f"cannot resolve the annotation {a!r} to a buffer or element type")


class MappingFunction:
    """The reference's vd.map object: a function plus its buffer types."""

    def __init__(self, func, return_type=None, input_types=None):
        self.func = func
        sig = _signature(func)
        if return_type is None and sig.return_annotation is not inspect.Parameter.empty:
            return_type = _resolve_annotation(sig.return_annotation)
        self.return_type = return_type
        if input_types is None:
            input_types = [_resolve_annotation(p.annotation) for p in sig.parameters.values()]
        self.buffer_types = list(input_types)

    def arg_is_scalar(self) -> List[bool]:
        """Per argument: a scalar (``vc.Var[...]``) rather than a buffer."""
        return [bool(getattr(t, "is_scalar", False)) for t in self.buffer_types]

    def input_dtypes(self) -> List[dt.dtype]:
        out = []
        for t in self.buffer_types:
            if hasattr(t, "var_type"):
                out.append(t.var_type)
            elif hasattr(t, "__args__"):
                out.append(t.__args__[0])
            else:
                raise ValueError(f"map argument annotation {t} is not a Buffer[...] type")
        return out


def map(func=None, return_type=None, input_types=None):  # noqa: A001 - mirrors vd.map
    if func is None:
        return lambda f: MappingFunction(f, return_type, input_types)
    return MappingFunction(func, return_type, input_types)


_partial_counts: dict = {}  # n -> partial sums of the first stage (vdx_reduce_partial_count)


_OUT_CODES = {dt.float32: L.VDX_F32, dt.float64: L.VDX_F64, dt.int32: L.VDX_I32, dt.uint32: L.VDX_U32,
              dt.vec2: L.VDX_V2F32}


class _CompiledReducePlan:
    """A libvdx map-reduce plan whose map was compiled with NVRTC."""

    def __init__(self, source: str, op: int, out_code: int):
        h = ctypes.c_void_p()
        L.check(L.lib().vdx_reduce_map_plan_create(source.encode(), op, out_code, ctypes.byref(h)), "map-reduce plan")
        self.handle = h

    def status(self, reset: bool = True) -> int:
        c = ctypes.c_int()
        L.check(L.lib().vdx_reduce_map_plan_status(self.handle, ctypes.byref(c), int(reset)), "map-reduce status")
        return int(c.value)

    def source(self) -> str:
        buf = ctypes.create_string_buffer(1 << 16)
        L.check(L.lib().vdx_reduce_map_plan_source(self.handle, buf, len(buf)), "map-reduce source")
        return buf.value.decode()

    def __del__(self):
        try:
            if self.handle:
                L.lib().vdx_reduce_map_plan_destroy(self.handle)
        except Exception:
            pass


_compiled_plans = {}  # (hooks source, op, output code, device) -> _CompiledReducePlan


def _reduce_hooks(mf: "MappingFunction", args):
    """Lowers a mapping function to the VdxReduceHooks struct that
    vdx_reduce_map_plan_create compiles (csrc/reduce_mapped.cuh); returns the
    source and the argument slots of this call."""
    from ..fft import jit as J
    from ..fft import maps as M

    types = mf.input_dtypes()
    flags = mf.arg_is_scalar()
    if len(args) != len(types):
        raise ValueError(f"map {mf.func.__name__} takes {len(types)} arguments, {len(args)} given")
    syms = [M._TraceScalar(i, t) if sc else vc.SymBuffer(i, t) for i, (t, sc) in enumerate(zip(types, flags))]
    # registers, their assignments and control-flow blocks the map runs
    # before its return value are recorded as events and lowered to the
    # statements that precede the hook's return
    events: list = []
    M._tls.events, M._tls.nreg = events, 0
    try:
        r = mf.func(*syms)
    except NotImplementedError:
        raise
    except Exception as e:  # noqa: BLE001
        raise NotImplementedError(f"map {mf.func.__name__} could not be traced: {e}") from e
    finally:
        M._tls.events = None
    if r is None:
        raise NotImplementedError(f"map {mf.func.__name__} returns no value to reduce")
    slots = J.Slots()
    low = J._Lower(mf.func.__name__, types, flags, list(args), slots)
    stmts = low.statements(events)
    code, _ = low.expr(r)
    body = ["using namespace vdx::mapops;", "const long long k = 0, n = 0;", "(void)k; (void)n; (void)m;",
            *stmts, f"return {code};"]
    src = "struct VdxReduceHooks {\n" + J._hook("auto map(const vdx::MapArgs& m, long long io)", body) + "};\n"
    return src, slots


class ReduceFunction:
    def __init__(self, reduction: ReduceOp, group_size: Optional[int] = None, axes: Optional[List[int]] = None,
                 mapping_function: Optional[MappingFunction] = None):
        self.reduction = reduction
        self.group_size = group_size
        self.axes = axes
        self.map_func = mapping_function
        self.out_type = mapping_function.return_type if mapping_function is not None else None
        self._map_code = None
        self._compiled_only = False  # the map is outside the fixed maps: always compiled
        # (input type, shape) -> validated launch layout of a call
        self._layouts = {}

    def _needs_compiled_map(self, args) -> bool:
        """Maps outside vdx_reduce's fixed maps (several arguments, other
        expressions, other element types) run as a compiled map."""
        if self.map_func is None:
            return False
        if self._compiled_only or len(args) != 1 or not isinstance(args[0], Buffer):
            return True
        t = args[0].var_type
        if t.vdx_code is None or t.vdx_code in (L.VDX_C32, L.VDX_C128, L.VDX_BF16X2):
            return True
        try:
            self._resolve_map(t)
        except NotImplementedError:
            self._compiled_only = True
            return True
        out_type = dt.float32 if t == dt.complex64 else t
        return self.out_type is not None and self.out_type != out_type

    def get_src(self, line_numbers: bool = None):
        """The two stages as [stage 1, stage 2] sources (the reference's
        ReduceFunction.get_src, vkdispatch/reduce/reduce_function.py:53-59):
        the ahead-of-time kernels a fixed map runs on, or the compiled
        map's hooks and instantiations."""
        from ..fft.src_functions import ShaderSource, _numbered, _Placeholder

        name = self.reduction.name
        out_t = self.out_type
        if self.map_func is None:
            maps, compiled = "identity", False
        else:
            types = self.map_func.input_dtypes()
            try:
                if len(types) != 1:
                    raise NotImplementedError("several arguments")
                code = _trace_map(self.map_func.func, types)
                maps = {L.VDX_MAP_IDENTITY: "identity", L.VDX_MAP_ABS: "abs", L.VDX_MAP_SQUARE: "square",
                        L.VDX_MAP_REAL: "real", L.VDX_MAP_IMAG: "imag", L.VDX_MAP_SIN: "sin"}[code]
                compiled = False
            except NotImplementedError:
                compiled = True
        if not compiled:
            s1 = (f"// stage 1: vdx::k_reduce_partial<In, T, {name}, {maps}> of libvdx.so (sm_103a):\n"
                  "// grid (parts, rows) x 512 threads; each CTA folds one contiguous chunk of a row")
            s2 = (f"// stage 2: vdx::k_reduce_final<T, {name}>: one CTA per row folds its partials in a fixed "
                  "order")
        else:
            args = [0.0 if sc else _Placeholder(t) for t, sc in zip(self.map_func.input_dtypes(),
                                                                    self.map_func.arg_is_scalar())]
            hooks, _ = _reduce_hooks(self.map_func, args)
            acc = {dt.float32: "float", dt.float64: "double", dt.int32: "int", dt.uint32: "unsigned",
                   dt.vec2: "float2"}.get(out_t, "float")
            s1 = ("// stage 1, compiled with NVRTC (csrc/reduce_mapped.cuh)\n" + hooks +
                  f"// vdx::reduce_mapped_partial<VdxReduceHooks, Re, {acc}, {name}>")
            s2 = f"// stage 2: vdx::reduce_mapped_final<{acc}, {name}>"
        return [ShaderSource("reduction stage 1", _numbered(s1, bool(line_numbers)), (512, 1, 1)),
                ShaderSource("reduction stage 2", _numbered(s2, bool(line_numbers)), (512, 1, 1))]

    def print_src(self, line_numbers: bool = None):
        srcs = self.get_src(line_numbers)
        print(f"// Reduction Stage 1:\n{srcs[0]}\n// Reduction Stage 2:\n{srcs[1]}")

    def _rows(self, src):
        """(n, batch): elements per reduced row and rows, from the axes."""
        if self.axes is None:
            return src.size, 1
        shape = src.shape
        batched = []
        for i in range(len(shape)):
            if i in self.axes:
                break
            batched.append(i)
        skipped = []
        for i in range(len(shape) - 1, -1, -1):
            if i in self.axes:
                break
            skipped.append(i)
        if skipped:
            raise ValueError("Reduction axes must be contiguous!")
        batch = int(np.prod([shape[i] for i in batched])) if batched else 1
        return src.size // batch, batch

    def _call_compiled(self, args, graph) -> Buffer:
        import torch

        from ..fft import jit as J

        src = next((a for a in args if isinstance(a, Buffer)), None)
        if src is None:
            raise ValueError("a map-reduce needs at least one buffer argument")
        out_type = self.out_type
        if out_type not in _OUT_CODES:
            raise NotImplementedError(f"map-reduce results of type {getattr(out_type, 'name', out_type)} "
                                      "(float32, float64, int32, uint32 and vec2 are supported)")
        op = self.reduction.code
        if op >= L.VDX_RED_AND and out_type not in (dt.int32, dt.uint32):
            raise ValueError(f"{self.reduction.name} reductions need an integer result type")
        n, batch = self._rows(src)
        source, slots = _reduce_hooks(self.map_func, args)
        key = (source, op, _OUT_CODES[out_type], torch.cuda.current_device())
        plan = _compiled_plans.get(key)
        if plan is None:
            plan = _compiled_plans[key] = _CompiledReducePlan(source, op, _OUT_CODES[out_type])
        nparts = _partial_counts.get(n)
        if nparts is None:
            parts = ctypes.c_int64()
            L.check(L.lib().vdx_reduce_partial_count(n, ctypes.byref(parts)), "reduce")
            nparts = _partial_counts[n] = int(parts.value)
        res = Buffer._empty((nparts + 1,) + ((batch,) if batch > 1 else ()), out_type)
        margs = J.make_args(slots)
        out = res.ptr
        ws = out + batch * out_type.item_size
        handle = plan.handle

        def launch(stream):
            L.check(L.lib().vdx_reduce_map_exec(handle, ctypes.byref(margs), n, batch, out, ws, stream),
                    "map-reduce")

        G.resolve(graph).record(launch, (plan, res, margs) + tuple(a for a in args if isinstance(a, Buffer)))
        self.last_plan = plan
        return res

    def _resolve_map(self, in_type: dt.dtype) -> int:
        if self.map_func is None:
            return L.VDX_MAP_IDENTITY
        if self._map_code is None:
            self._map_code = _trace_map(self.map_func.func, self.map_func.input_dtypes())
        return self._map_code

    def __call__(self, *args, graph: Optional[G.CommandGraph] = None, **kwargs) -> Buffer:
        if self._needs_compiled_map(args):
            return self._call_compiled(args, graph)
        src = args[0]
        lay = self._layouts.get((src.var_type, src.shape))
        if lay is None:
            lay = self._layouts[(src.var_type, src.shape)] = self._layout(src)
        map_code, n, batch, out_type, shape = lay
        res = Buffer._empty(shape, out_type)
        op = self.reduction.code
        in_code = src.var_type.vdx_code
        ptr, out = src.ptr, res.ptr
        ws = out + batch * out_type.item_size
        if not src.contiguous:
            # a non-contiguous array is reduced from a C-order copy made in the launch
            import torch

            tmp = torch.empty(src.tensor.shape, dtype=src.tensor.dtype, device=src.tensor.device)
            ptr = tmp.data_ptr()

            def launch(stream):
                with torch.cuda.stream(torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()):
                    tmp.copy_(src.tensor, non_blocking=True)
                L.check(L.lib().vdx_reduce(op, map_code, in_code, ptr, n, batch, out, ws, stream), "reduce")

            G.resolve(graph).record(launch, (src, res, tmp))
            return res

        def launch(stream):
            L.check(L.lib().vdx_reduce(op, map_code, in_code, ptr, n, batch, out, ws, stream), "reduce")

        G.resolve(graph).record(launch, (src, res))
        return res

    def _layout(self, src):
        """Checks a call's input and derives (map code, n, batch, output type,
        output shape)."""
        in_type = src.var_type
        if in_type.vdx_code is None or in_type.vdx_code in (L.VDX_C32, L.VDX_C128, L.VDX_BF16X2):
            raise NotImplementedError(f"reductions over {in_type.name} buffers are not in the supported menu")
        map_code = self._resolve_map(in_type)
        if self.axes is None:
            n, batch = src.size, 1
        else:
            shape = src.shape
            batched = []
            for i in range(len(shape)):
                if i in self.axes:
                    break
                batched.append(i)
            skipped = []
            for i in range(len(shape) - 1, -1, -1):
                if i in self.axes:
                    break
                skipped.append(i)
            if skipped:
                raise ValueError("Reduction axes must be contiguous!")
            batch = int(np.prod([shape[i] for i in batched])) if batched else 1
            n = src.size // batch
        out_type = dt.float32 if in_type == dt.complex64 else in_type
        if self.out_type is not None and self.out_type != out_type:
            raise NotImplementedError(f"map return type {self.out_type} does not match the reduction type {out_type}")
        nparts = _partial_counts.get(n)
        if nparts is None:
            parts = ctypes.c_int64()
            L.check(L.lib().vdx_reduce_partial_count(n, ctypes.byref(parts)), "reduce")
            nparts = _partial_counts[n] = int(parts.value)
        shape = (nparts + 1,) + ((batch,) if batch > 1 else ())
        return map_code, n, batch, out_type, shape


def reduce(identity, axes=None, group_size=None, mapping_function: MappingFunction = None):
    def decorator(func):
        sig = _signature(func)
        if sig.return_annotation is inspect.Parameter.empty:
            raise ValueError("Return type must be annotated")
        ret = _resolve_annotation(sig.return_annotation)
        op = _trace_reduction(func)
        mf = mapping_function
        if mf is not None and mf.return_type != ret:
            raise ValueError("Mapping function return type must match the return type of the reduction function")
        return ReduceFunction(op, group_size=group_size, axes=axes, mapping_function=mf)

    return decorator


def map_reduce(reduction: ReduceOp, axes=None, group_size=None):
    def decorator(func):
        return ReduceFunction(reduction, group_size=group_size, axes=axes, mapping_function=MappingFunction(func))

    return decorator
