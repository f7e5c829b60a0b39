"""CPU tests of the map-hook compiler (vkdispatch_gb300/fft/jit.py): user
maps outside the functor menu are traced and lowered to a C++ hooks struct;
the generated source must compile with NVRTC against the kernel template
(csrc/fft_mapped.cuh).  No GPU is used: buffers are stand-ins that carry a
shape and a dtype."""

from pathlib import Path

import numpy as np
import pytest

import vkdispatch_gb300 as vd
import vkdispatch_gb300.codegen as vc
from vkdispatch_gb300.fft import jit as J

CSRC = Path(__file__).resolve().parent.parent / "vkdispatch_gb300" / "csrc"


class FakeBuffer:
    def __init__(self, shape, var_type):
        self.shape, self.var_type, self.ptr = tuple(shape), var_type, 0
        self.size = int(np.prod(shape))


def _nvrtc_compile(hooks_src, n=10, T=2, radices="5, 2", strided="true", mode=2, re="float"):
    nvrtc = pytest.importorskip("cuda.bindings.nvrtc")
    import os

    inc = os.environ.get("VDX_CUDA_INCLUDE") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                                                             "include")
    if not os.path.exists(os.path.join(inc, "cuda_fp16.h")):
        pytest.skip("CUDA headers not found")
    src = ('#include "fft_mapped.cuh"\n' + hooks_src +
           f'\nextern "C" __global__ void vdx_mapped(vdx::FftArgs a, vdx::MapArgs m) {{\n'
           f'  vdx::mapped_body<vdx::FixPlan<{n}, {T}, vdx::RList<{radices}>, 16>, {strided}, {re}, {mode}, '
           f'VdxHooks>(a, m);\n}}\n')
    err, prog = nvrtc.nvrtcCreateProgram(src.encode(), b"m.cu", 0, [], [])
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", f"-I{CSRC}".encode(), f"-I{inc}".encode(),
            b"-default-device"]
    (err,) = nvrtc.nvrtcCompileProgram(prog, len(opts), opts)
    _, size = nvrtc.nvrtcGetProgramLogSize(prog)
    log = b" " * size
    nvrtc.nvrtcGetProgramLog(prog, log)
    assert err == nvrtc.nvrtcResult.NVRTC_SUCCESS, log.decode()


def _padded_maps(full, trimmed):
    def remap(io_index):
        return vc.unravel_index(vc.ravel_index(io_index, trimmed).to_register(), full)

    @vd.map
    def input_map(input_buffer: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        op.read_from_buffer(input_buffer, io_index=remap(op.io_index))

    @vd.map
    def output_map(output_buffer: vc.Buffer[vc.c64]):
        op = vd.fft.write_op()
        op.write_to_buffer(output_buffer, io_index=remap(op.io_index))

    return input_map, output_map


def test_padded_region_index_remap_lowers_to_integer_arithmetic():
    buf = FakeBuffer((4, 24, 16), vd.complex64)
    im, om = _padded_maps(buf.shape, (4, 10, 16))
    spec = J.build_hooks([buf], [buf], [], im, om, None, False)
    # b * 384 + s * 16 + c with (b, s, c) the trimmed coordinates of io
    assert "(io / (long long)(160)) * (long long)(384)" in spec.source
    assert "Re(" not in spec.source.split("map_ldc")[1].split(";")[0].split(",", 1)[1]
    assert len(spec.slots.buffers) == 2
    _nvrtc_compile(spec.source, mode=0)


def test_scalar_kernel_map_and_menu_refusal():
    @vd.map
    def scale_spectrum(scale_factor: vc.Var[vc.f32]):
        op = vd.fft.read_op()
        op.register[:] = op.register * scale_factor

    from vkdispatch_gb300.fft import maps as M

    with pytest.raises(NotImplementedError):
        M.classify_kernel(scale_spectrum)
    buf = FakeBuffer((8, 10), vd.complex64)
    spec = J.build_hooks([buf], [], [np.float32(0.5)], None, None, scale_spectrum, True)
    assert spec.slots.fscalars == [0.5]
    assert "m.fs[0]" in spec.source
    _nvrtc_compile(spec.source)


def test_general_maps_compile():
    @vd.map
    def in_map(a: vc.Buffer[vc.c64], w: vc.Buffer[vc.f32], s: vc.Var[vc.f32]):
        op = vd.fft.read_op()
        t = vc.new_register(vc.c64)
        t[:] = a[op.io_index] * 2.0 + vc.to_complex(w[op.io_index]) * s
        op.register[:] = vc.mult_complex(t, t.conjugate()) - t
        op.register.imag = vc.sin(op.register.real) + vc.sqrt(vc.abs(w[op.fft_size - 1 - op.fft_index]))

    @vd.map
    def out_map(p: vc.Buffer[vc.f32]):
        op = vd.fft.write_op()
        p[op.io_index] = op.register.real * op.register.real + op.register.imag * op.register.imag

    @vd.map
    def ker_map(h: vc.Buffer[vc.c64], n: vc.Var[vc.i32]):
        op = vd.fft.read_op()
        f = vc.to_dtype(vc.f32, op.fft_index)
        g = vc.exp(-(f * f) / 8.0)
        op.register[:] = vc.mult_complex(op.register, h[op.io_index % n]) * g

    a, w, p, h = (FakeBuffer((6, 10), t) for t in (vd.complex64, vd.float32, vd.float32, vd.complex64))
    spec = J.build_hooks([p], [a, w, np.float32(1.5)], [h, 10], in_map, out_map, ker_map, True)
    assert spec.slots.fscalars == [1.5] and spec.slots.iscalars == [10]
    _nvrtc_compile(spec.source, strided="false")


def test_multi_kernel_index_and_complex32_buffers():
    @vd.map
    def ker_map(h: vc.Buffer[vc.c32]):
        op = vd.fft.read_op()
        k = vc.new_register(vc.c64)
        op.read_from_buffer(h, register=k, io_index=op.io_index + vd.fft.mapped_kernel_index() * 60)
        op.register[:] = vc.mult_complex(op.register, k)

    @vd.map
    def out_map(o: vc.Buffer[vc.c32]):
        op = vd.fft.write_op()
        op.write_to_buffer(o, io_index=op.io_index + vd.fft.mapped_kernel_index() * 60)

    h, o, x = FakeBuffer((3, 6, 10), vd.complex32), FakeBuffer((3, 6, 10), vd.complex32), FakeBuffer((6, 10),
                                                                                                     vd.complex64)
    spec = J.build_hooks([o], [x], [h], None, out_map, ker_map, True)
    assert "m.kidx" in spec.source
    _nvrtc_compile(spec.source, strided="false", re="double")


def test_untraceable_maps_raise():
    @vd.map
    def bad(a: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        op.register[:] = a[op.io_index] * "x"

    buf = FakeBuffer((4, 8), vd.complex64)
    with pytest.raises(NotImplementedError):
        J.build_hooks([buf], [buf], [], bad, None, None, False)

    @vd.map
    def cplx_mod(a: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        op.register[:] = a[op.io_index] % 2.0

    with pytest.raises(NotImplementedError):
        J.build_hooks([buf], [buf], [], cplx_mod, None, None, False)


def test_menu_refuses_real_store_of_an_expression():
    """Only a store of the register's real part at io_index is the menu's
    real output map; |reg|^2 must go to the compiler."""
    from vkdispatch_gb300.fft import maps as M

    @vd.map
    def power(p: vc.Buffer[vc.f32]):
        op = vd.fft.write_op()
        p[op.io_index] = op.register.real * op.register.real + op.register.imag * op.register.imag

    @vd.map
    def real_part(p: vc.Buffer[vc.f32]):
        op = vd.fft.write_op()
        p[op.io_index] = vc.to_dtype(p.var_type, op.register.real)

    with pytest.raises(NotImplementedError):
        M.classify_output(power)
    assert M.classify_output(real_part).kind == "real"


def test_control_flow_blocks_lower_and_compile():
    """vc.if_block / else_if_block / else_block / while_block around traced
    statements become the same C++ blocks in the hooks."""
    import vkdispatch_gb300.codegen as vc2

    buf = FakeBuffer((4, 10), vd.complex64)

    @vd.map
    def masked(b: vc2.Buffer[vc2.c64], lim: vc2.Var[vc2.i32]):
        op = vd.fft.read_op()
        op.read_from_buffer(b)
        with vc2.if_block(vc2.any(op.fft_index >= lim, op.io_index < 3)):
            op.register[:] = 0.0
        with vc2.else_if_block(op.fft_index == 0):
            op.register *= 2.0
        with vc2.else_block():
            n = vc2.new_register(vc2.i32, 0)
            with vc2.while_block(n < 2):
                op.register *= 1.5
                n += 1

    spec = J.build_hooks([buf], [buf, 4], [], masked, None, None, False)
    src = spec.source
    assert "if (" in src and "else if (" in src and "else {" in src and "while (" in src
    assert src.count("{") == src.count("}")
    _nvrtc_compile(spec.source, mode=0)


def test_control_flow_misuse_is_refused():
    import vkdispatch_gb300.codegen as vc2

    buf = FakeBuffer((4, 10), vd.complex64)

    @vd.map
    def dangling_else(b: vc2.Buffer[vc2.c64]):
        op = vd.fft.read_op()
        op.read_from_buffer(b)
        with vc2.else_block():
            op.register *= 2.0

    with pytest.raises(NotImplementedError):
        J.build_hooks([buf], [buf], [], dangling_else, None, None, False)

    @vd.map
    def python_if(b: vc2.Buffer[vc2.c64]):
        op = vd.fft.read_op()
        op.read_from_buffer(b)
        if op.fft_index < 3:  # a traced value has no Python truth value
            op.register *= 2.0

    with pytest.raises(NotImplementedError):
        J.build_hooks([buf], [buf], [], python_if, None, None, False)
    with pytest.raises(NotImplementedError):
        with vc2.if_block(1):  # outside a traced map
            pass


def test_every_traced_math_function_lowers_and_compiles():
    """Each function of the codegen surface (the reference's vc math,
    vkdispatch/codegen/functions/*) lowers to C++ that NVRTC compiles inside
    the kernel template: unary and binary math, clamps and mixes, integer
    arithmetic and bit operations, casts, complex helpers."""
    @vd.map
    def in_map(a: vc.Buffer[vc.c64], s: vc.Var[vc.f32], n: vc.Var[vc.i32]):
        op = vd.fft.read_op()
        x = vc.new_float_register(a[op.io_index].real)
        y = vc.new_float_register(vc.abs(a[op.io_index].imag) + 1.0)
        u = (vc.tan(x) + vc.asin(vc.clamp(x, -1.0, 1.0)) + vc.acos(vc.clamp(x, -1.0, 1.0)) + vc.atan(x)
             + vc.sinh(x) + vc.cosh(x) + vc.tanh(x) + vc.exp(x) + vc.exp2(x) + vc.log(y) + vc.log2(y)
             + vc.inversesqrt(y) + vc.floor(x) + vc.ceil(x) + vc.trunc(x) + vc.fract(x) + vc.sign(x)
             + vc.round(x))
        b = (vc.atan2(x, y) + vc.pow(y, s) + vc.mod(y, 3.0) + vc.fma(x, y, s) + vc.mix(x, y, 0.25)
             + vc.min(x, y) + vc.max(x, y) + vc.length(a[op.io_index]) + y ** 2.0 - (-x))
        i = vc.new_int_register(op.io_index)
        j = ((i // 3) % n + (i & 7) + (i | 1) + (i ^ 5)) * 2 - i
        z = vc.complex_from_euler_angle(x * s)
        op.register[:] = vc.mult_complex(a[op.io_index], z) + vc.to_complex(u + b + vc.to_dtype(vc.f32, j))

    a = FakeBuffer((6, 10), vd.complex64)
    spec = J.build_hooks([a], [a, np.float32(0.5), 3], [], in_map, None, None, False)
    for fn in ("tan", "asin", "acos", "atan", "sinh", "cosh", "tanh", "exp", "exp2", "log", "log2", "inversesqrt",
               "floor", "ceil", "trunc", "fract", "sign", "round", "atan2", "pow", "mod", "fma", "mix", "min", "max",
               "length", "clamp", "abs"):
        assert f"m_{fn}(" in spec.source, fn
    _nvrtc_compile(spec.source, strided="false")
    _nvrtc_compile(spec.source, strided="true", re="double")  # the fp64-compute instantiation


def test_control_flow_in_output_and_kernel_maps_compiles():
    """Blocks in the store and spectrum hooks too: an output map that writes
    one of two buffers by a condition, and a kernel map whose loop and
    complex register updates run between the forward and inverse passes."""
    out_a, out_b = FakeBuffer((6, 10), vd.complex64), FakeBuffer((6, 10), vd.complex64)
    sig, ker = FakeBuffer((6, 10), vd.complex64), FakeBuffer((6, 10), vd.complex64)
    mask = FakeBuffer((6, 10), vd.int32)

    @vd.map
    def split_store(a: vc.Buffer[vc.c64], b: vc.Buffer[vc.c64], keep: vc.Buffer[vc.i32]):
        op = vd.fft.write_op()
        with vc.if_block(vc.all(keep[op.io_index] != 0, op.fft_index < op.fft_size - 1)):
            op.write_to_buffer(a)
        with vc.else_block():
            b[op.io_index] = op.register.conjugate()

    @vd.map
    def shaped_kernel(h: vc.Buffer[vc.c64], taps: vc.Var[vc.i32]):
        op = vd.fft.read_op()
        acc = vc.new_complex_register(0.0, 0.0)
        t = vc.new_int_register(0)
        with vc.while_block(t < taps):
            acc += h[(op.io_index + t) % 60] * 0.5
            t += 1
        with vc.if_block(vc.abs(acc.real) > 1.0):
            acc.real = vc.sign(acc.real)
        op.register[:] = vc.mult_complex(op.register, acc.conjugate())

    spec = J.build_hooks([out_a, out_b, mask], [sig], [ker, 3], None, split_store, shaped_kernel, True)
    src = spec.source
    assert src.count("{") == src.count("}") and "while (" in src and "else {" in src
    _nvrtc_compile(src, strided="false", mode=2)  # the fused convolution runs the kernel hook
    _nvrtc_compile(src, strided="true", mode=2, re="double")
