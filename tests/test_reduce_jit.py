"""CPU tests of compiled map-reduce (vkdispatch_gb300/reduce: _reduce_hooks ->
csrc/reduce_mapped.cuh): maps outside vdx_reduce's fixed maps are traced and
lowered to a VdxReduceHooks struct, and the generated source compiles with
NVRTC against the two-stage reduction template.  No GPU is used."""

import os
from pathlib import Path

import numpy as np
import pytest

import vkdispatch_gb300 as vd
import vkdispatch_gb300.codegen as vc
from vkdispatch_gb300.reduce import _reduce_hooks

CSRC = Path(__file__).resolve().parent.parent / "vkdispatch_gb300" / "csrc"


class FakeBuffer(vd.Buffer):
    def __init__(self, shape, var_type):  # noqa: D107 - no device memory
        self.shape, self.var_type, self.strides = tuple(shape), var_type, None
        self.size = int(np.prod(shape))

    @property
    def ptr(self):
        return 0


def _compile(hooks, acc="float", re="float", op=0):
    nvrtc = pytest.importorskip("cuda.bindings.nvrtc")
    inc = os.environ.get("VDX_CUDA_INCLUDE") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                                                             "include")
    if not os.path.exists(os.path.join(inc, "cuda_fp16.h")):
        pytest.skip("CUDA headers not found")
    src = ('#include "reduce_mapped.cuh"\n' + hooks +
           f'\nextern "C" __global__ void vdx_mapped(vdx::MapArgs m, long long n, long long chunk, {acc}* part, '
           f'int nparts) {{ vdx::reduce_mapped_partial<VdxReduceHooks, {re}, {acc}, {op}>(m, n, chunk, part, '
           f'nparts); }}\n'
           f'extern "C" __global__ void vdx_mapped_final(const {acc}* part, int nparts, {acc}* out) '
           f'{{ vdx::reduce_mapped_final<{acc}, {op}>(part, nparts, out); }}\n')
    err, prog = nvrtc.nvrtcCreateProgram(src.encode(), b"r.cu", 0, [], [])
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", f"-I{CSRC}".encode(), f"-I{inc}".encode(),
            b"-default-device"]
    (err,) = nvrtc.nvrtcCompileProgram(prog, len(opts), opts)
    if err != nvrtc.nvrtcResult.NVRTC_SUCCESS:
        _, size = nvrtc.nvrtcGetProgramLogSize(prog)
        log = b" " * size
        nvrtc.nvrtcGetProgramLog(prog, log)
        pytest.fail(log.decode(errors="replace"))


def test_listed_reduction_map_over_two_vec2_buffers():
    """The reference's test_listed_reductions map: sin of the sum of two
    vec2 buffers, reduced component-wise."""

    def sum_map(buffer: vc.Buffer[vd.vec2], buffer2: vc.Buffer[vd.vec2]) -> vd.vec2:
        ind = vd.reduce.mapped_io_index()
        return vc.sin(buffer[ind] + buffer2[ind])

    mf = vd.reduce.MappingFunction(sum_map)
    a, b = FakeBuffer((1024,), vd.vec2), FakeBuffer((1024,), vd.vec2)
    src, slots = _reduce_hooks(mf, (a, b))
    assert "struct VdxReduceHooks" in src and "m_sin" in src and len(slots.buffers) == 2
    _compile(src, acc="float2")


def test_scalar_argument_and_integer_reduction():
    def scaled(buf: vc.Buffer[vc.f32], s: vc.Var[vc.f32]) -> vc.f32:
        return buf[vd.reduce.mapped_io_index()] * s + 1.0

    src, slots = _reduce_hooks(vd.reduce.MappingFunction(scaled), (FakeBuffer((64,), vd.float32), 2.5))
    assert "m.fs[0]" in src and slots.fscalars == [2.5]
    _compile(src, acc="float", op=3)

    def mixed(u: vc.Buffer[vc.u32]) -> vc.u32:
        i = vd.reduce.mapped_io_index()
        return u[i] ^ (i * 3)

    src, _ = _reduce_hooks(vd.reduce.MappingFunction(mixed), (FakeBuffer((64,), vd.uint32),))
    _compile(src, acc="unsigned", op=6)


def test_argument_count_checked():
    def one(buf: vc.Buffer[vc.f32]) -> vc.f32:
        return buf[vd.reduce.mapped_io_index()]

    with pytest.raises(ValueError):
        _reduce_hooks(vd.reduce.MappingFunction(one), ())


def test_get_src_of_fixed_and_compiled_maps(capsys):
    """ReduceFunction.get_src returns both stages (the reference's
    test_min_max_codegen_stage_creation), for a fixed map and a compiled one."""

    @vd.reduce.map_reduce(vd.reduce.SubgroupMin)
    def min_map(buffer: vc.Buffer[vc.f32]) -> vc.f32:
        return buffer[vd.reduce.mapped_io_index()]

    @vd.reduce.map_reduce(vd.reduce.SubgroupMax)
    def max_map(buffer: vc.Buffer[vc.f32], s: vc.Var[vc.f32]) -> vc.f32:
        return buffer[vd.reduce.mapped_io_index()] * s

    s1, s2 = min_map.get_src()
    assert s1 and s2 and "k_reduce_partial" in s1.code
    c1, c2 = max_map.get_src(line_numbers=True)
    assert "VdxReduceHooks" in c1.code and "reduce_mapped_final" in c2.code
    max_map.print_src()
    assert "Reduction Stage 2" in capsys.readouterr().out


def test_map_with_registers_and_control_flow():
    """A mapping function that declares registers, assigns them in place and
    branches before returning (the statements the reference's codegen emits
    for such a map, vkdispatch/codegen/functions/control_flow.py) lowers to
    the same statements ahead of the hook's return."""

    def clipped(buf: vc.Buffer[vc.f32], lim: vc.Var[vc.f32]) -> vc.f32:
        i = vd.reduce.mapped_io_index()
        r = vc.new_float_register(buf[i])
        with vc.if_block(r > lim):
            r[:] = lim
        with vc.else_if_block(r < -lim):
            r[:] = -lim
        with vc.else_block():
            r += 1.0
        c = vc.new_int_register(0)
        with vc.while_block(c < 3):
            c += 1
            r *= 0.5
        return r

    src, slots = _reduce_hooks(vd.reduce.MappingFunction(clipped), (FakeBuffer((64,), vd.float32), 2.0))
    assert "if (" in src and "else if (" in src and "while (" in src and slots.fscalars == [2.0]
    assert src.index("while (") < src.index("return")
    _compile(src, acc="float", op=0)


def test_map_without_a_return_value_is_refused():
    def nothing(buf: vc.Buffer[vc.f32]) -> vc.f32:
        vc.new_float_register(buf[vd.reduce.mapped_io_index()])

    with pytest.raises(NotImplementedError):
        _reduce_hooks(vd.reduce.MappingFunction(nothing), (FakeBuffer((64,), vd.float32),))
