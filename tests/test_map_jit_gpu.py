"""GPU tests of map hooks outside the functor menu, compiled at run time
(vkdispatch_gb300/fft/jit.py -> vdx_map_plan_create): the reference's
padded-region workflow (docs/tutorials/reductions_and_fft.rst:177-205), a
scalar kernel map (the tutorial's scale_spectrum, :133-148), and general
input / output / kernel maps, each against FP64 numpy within the fp32 bound."""

import numpy as np
import pytest

from helpers import crandn, rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

vd = pytest.importorskip("vkdispatch_gb300")
import vkdispatch_gb300.codegen as vc  # noqa: E402


def padded_axis_fft(buffer, signal_cols):
    """The reference tutorial's padded-region FFT: an FFT of the first
    signal_cols rows of axis 1, read and written through io_index remaps."""
    trimmed_shape = (buffer.shape[0], signal_cols, buffer.shape[2])

    def remap(io_index):
        return vc.unravel_index(vc.ravel_index(io_index, trimmed_shape).to_register(), buffer.shape)

    @vd.map
    def input_map(input_buffer: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        op.read_from_buffer(input_buffer, io_index=remap(op.io_index))

    @vd.map
    def output_map(output_buffer: vc.Buffer[vc.c64]):
        op = vd.fft.write_op()
        op.write_to_buffer(output_buffer, io_index=remap(op.io_index))

    vd.fft.fft(buffer, buffer, buffer_shape=trimmed_shape, axis=1, input_map=input_map, output_map=output_map,
               input_signal_range=(0, signal_cols))


@pytest.mark.parametrize("shape,cols", [((4, 24, 16), 10), ((3, 64, 33), 48), ((2, 512, 8), 300)])
def test_padded_region_fft(shape, cols):
    rng = np.random.default_rng(cols)
    x = crandn(rng, shape)
    b = vd.asbuffer(x)
    padded_axis_fft(b, cols)
    got = b.read(0)
    want = x.astype(np.complex128).copy()
    want[:, :cols, :] = np.fft.fft(want[:, :cols, :], axis=1)
    assert rel_l2(got[:, :cols], want[:, :cols]) <= tol_fp32(cols)
    assert np.array_equal(got[:, cols:], x[:, cols:])  # rows outside the region are untouched


def test_padded_cross_correlation_workflow():
    """Forward padded FFT, a conjugate product with a template spectrum
    through a kernel map, inverse padded FFT: cross-correlation of each
    region column with a template, as the tutorial's workflow does."""
    rng = np.random.default_rng(7)
    shape, cols = (2, 40, 12), 24
    x = crandn(rng, shape)
    t = crandn(rng, (shape[0], cols, shape[2]))
    b = vd.asbuffer(x)
    tb = vd.asbuffer(np.fft.fft(t.astype(np.complex128), axis=1).astype(np.complex64))
    trimmed = (shape[0], cols, shape[2])

    def remap(io_index):
        return vc.unravel_index(vc.ravel_index(io_index, trimmed).to_register(), shape)

    @vd.map
    def input_map(inb: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        op.read_from_buffer(inb, io_index=remap(op.io_index))

    @vd.map
    def output_map(outb: vc.Buffer[vc.c64]):
        op = vd.fft.write_op()
        op.write_to_buffer(outb, io_index=remap(op.io_index))

    @vd.map
    def kernel_map(tspec: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        k = vc.new_register(vc.c64)
        op.read_from_buffer(tspec, register=k)
        op.register[:] = vc.mult_complex(op.register, k.conjugate())

    vd.fft.convolve(b, b, tb, buffer_shape=trimmed, axis=1, input_map=input_map, output_map=output_map,
                    kernel_map=kernel_map)
    got = b.read(0)
    xs = x[:, :cols].astype(np.complex128)
    want = np.fft.ifft(np.fft.fft(xs, axis=1) * np.conj(np.fft.fft(t.astype(np.complex128), axis=1)), axis=1)
    assert rel_l2(got[:, :cols], want) <= tol_fp32(cols, cols) * 2
    assert np.array_equal(got[:, cols:], x[:, cols:])


def test_scalar_kernel_map():
    """vd.fft.convolve(buf, np.float32(0.5), kernel_map=scale_spectrum):
    forward FFT, spectrum * 0.5, inverse FFT = 0.5 x."""

    @vd.map
    def scale_spectrum(scale_factor: vc.Var[vc.f32]):
        op = vd.fft.read_op()
        op.register[:] = op.register * scale_factor

    rng = np.random.default_rng(3)
    x = crandn(rng, (16, 360))
    b = vd.asbuffer(x)
    vd.fft.convolve(b, np.float32(0.5), kernel_map=scale_spectrum)
    assert rel_l2(b.read(0), 0.5 * x.astype(np.complex128)) <= tol_fp32(360, 360)


def test_general_input_output_kernel_maps():
    rng = np.random.default_rng(5)
    R, N = 12, 100
    a = crandn(rng, (R, N))
    w = rng.standard_normal((R, N)).astype(np.float32)
    h = crandn(rng, (R, N))
    s = 1.5

    @vd.map
    def in_map(ab: vc.Buffer[vc.c64], wb: vc.Buffer[vc.f32], sc: vc.Var[vc.f32]):
        op = vd.fft.read_op()
        op.register[:] = ab[op.io_index] * 2.0 + vc.to_complex(wb[op.io_index]) * sc

    @vd.map
    def out_map(pb: vc.Buffer[vc.f32]):
        op = vd.fft.write_op()
        pb[op.io_index] = op.register.real * op.register.real + op.register.imag * op.register.imag

    @vd.map
    def ker_map(hb: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        f = vc.to_dtype(vc.f32, op.fft_index)
        g = vc.exp(-(f * f) / 50.0)
        op.register[:] = vc.mult_complex(op.register, hb[op.io_index]) * g

    pb = vd.Buffer((R, N), vd.float32)
    ab, wb, hb = vd.asbuffer(a), vd.asbuffer(w), vd.asbuffer(h)
    vd.fft.convolve(pb, ab, wb, np.float32(s), hb, input_map=in_map, output_map=out_map, kernel_map=ker_map)
    x = 2.0 * a.astype(np.complex128) + s * w
    g = np.exp(-(np.arange(N) ** 2) / 50.0)
    y = np.fft.ifft(np.fft.fft(x, axis=1) * h * g, axis=1)
    want = np.abs(y) ** 2
    assert rel_l2(pb.read(0), want) <= 4 * tol_fp32(N, N)


def test_fft_output_map_with_fft_index_and_inverse():
    """An inverse FFT whose output map writes a reversed, scaled copy."""
    rng = np.random.default_rng(9)
    x = crandn(rng, (5, 7, 48))
    src, dst = vd.asbuffer(x), vd.Buffer((5, 7, 48), vd.complex64)

    @vd.map
    def out_map(ob: vc.Buffer[vc.c64]):
        op = vd.fft.write_op()
        # axis 1 of (5, 7, 48): points are 48 elements apart
        ob[op.io_index - op.fft_index * 48 + (op.fft_size - 1 - op.fft_index) * 48] = op.register * 3.0

    vd.fft.fft(dst, src, axis=1, inverse=True, output_map=out_map)
    want = 3.0 * np.fft.ifft(x.astype(np.complex128), axis=1)[:, ::-1, :]
    assert rel_l2(dst.read(0), want) <= tol_fp32(7) * 2


def test_multi_kernel_with_compiled_maps():
    """kernel_num = 3 with a kernel map outside the menu (a plain product
    scaled by the kernel index): kernel k writes output slice k."""
    rng = np.random.default_rng(11)
    R, N, K = 4, 64, 3
    x = crandn(rng, (R, N))
    h = crandn(rng, (K, R, N))
    xb, hb = vd.asbuffer(x), vd.asbuffer(h)
    ob = vd.Buffer((K, R, N), vd.complex64)

    @vd.map
    def ker_map(kb: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        kk = vd.fft.mapped_kernel_index()
        op.register[:] = vc.mult_complex(op.register, kb[op.io_index + kk * (R * N)]) * (vc.to_dtype(vc.f32, kk) + 1.0)

    @vd.map
    def out_map(o: vc.Buffer[vc.c64]):
        op = vd.fft.write_op()
        op.write_to_buffer(o, io_index=op.io_index + vd.fft.mapped_kernel_index() * (R * N))

    vd.fft.convolve(ob, xb, hb, kernel_map=ker_map, output_map=out_map, kernel_num=K)
    X = np.fft.fft(x.astype(np.complex128), axis=1)
    want = np.stack([np.fft.ifft(X * h[k] * (k + 1), axis=1) for k in range(K)])
    assert rel_l2(ob.read(0), want) <= tol_fp32(N, N)


def test_complex128_compute_with_compiled_map():
    rng = np.random.default_rng(13)
    x = (rng.standard_normal((6, 90)) + 1j * rng.standard_normal((6, 90))).astype(np.complex128)
    b = vd.asbuffer(x)

    @vd.map
    def in_map(ib: vc.Buffer[vc.c128]):
        op = vd.fft.read_op()
        op.register[:] = vc.mult_complex(ib[op.io_index], ib[op.io_index])

    out = vd.Buffer((6, 90), vd.complex128)

    @vd.map
    def out_map(ob: vc.Buffer[vc.c128]):
        op = vd.fft.write_op()
        op.write_to_buffer(ob)

    vd.fft.fft(out, b, input_map=in_map, output_map=out_map, compute_type=vd.complex128)
    want = np.fft.fft(x * x, axis=1)
    assert rel_l2(out.read(0), want) <= 1e-12


def test_hooks_that_do_not_compile_report_the_compiler_log():
    """vdx_map_plan_create with C++ that NVRTC rejects returns
    VDX_ERR_INVALID (ValueError) whose message carries the compiler's log;
    nothing is launched."""
    from vkdispatch_gb300 import _lib as L
    from vkdispatch_gb300.fft import jit as J

    bad = "struct VdxHooks { this is not C++; };"
    with pytest.raises(ValueError, match="do not compile"):
        J.get_plan((4, 64), 1, False, False, 0, L.VDX_C64, None, bad)


def test_compiled_plan_source_and_status_reset():
    """The compiled source is readable back, and the out-of-range status
    resets: a map reading one element past its buffer sets it once."""
    from vkdispatch_gb300.fft import jit as J

    rng = np.random.default_rng(17)
    x = crandn(rng, (2, 16))
    src = vd.asbuffer(x)
    dst = vd.Buffer((2, 16), vd.complex64)

    @vd.map
    def shifted(ib: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        op.register[:] = ib[op.io_index + 1]  # the last element reads index 32 of a 32-element buffer

    J.out_of_range(reset=True)
    vd.fft.fft(dst, src, input_map=shifted)
    assert J.out_of_range(reset=True)
    assert not J.out_of_range()
    shifted_x = np.concatenate([x.reshape(-1)[1:], [0]]).reshape(2, 16).astype(np.complex128)
    assert rel_l2(dst.read(0), np.fft.fft(shifted_x, axis=1)) <= tol_fp32(16)
    plan = next(p for k, p in J._plans.items() if "(io + (long long)(1))" in k[-1])
    assert "vdx_mapped" in plan.source() and "FixPlan<16" in plan.source()


def test_in_place_register_arithmetic():
    """`op.register *= s` and `+=` assign the register (the reference's
    in-place variable operators); a scalar added to the complex register adds
    to both components, as on a vec2."""
    rng = np.random.default_rng(71)
    x = crandn(rng, (6, 360))
    src = vd.asbuffer(x)
    out = vd.Buffer((6, 360), vd.complex64)

    @vd.map
    def scaled_shift(buf: vc.Buffer[vc.c64], s: vc.Var[vc.f32]):
        op = vd.fft.read_op()
        op.read_from_buffer(buf)
        op.register *= s
        op.register += 0.5
        op.register -= 0.25

    vd.fft.fft(out, src, 1.5, input_map=scaled_shift)
    ref = np.fft.fft(x.astype(np.complex128) * 1.5 + (0.25 + 0.25j), axis=1)
    assert rel_l2(out.read(0), ref) <= tol_fp32(360)


def test_control_flow_maps():
    """An input map that truncates the transform input past a length given
    at call time (if_block), scales the first point (else_if_block) and runs
    a counted loop (while_block); and an output map that writes two
    different scalings by the output index (if / else)."""
    rng = np.random.default_rng(72)
    n, lim = 240, 150
    x = crandn(rng, (5, n))
    src = vd.asbuffer(x)
    out = vd.Buffer((5, n), vd.complex64)

    @vd.map
    def truncate(buf: vc.Buffer[vc.c64], limit: vc.Var[vc.i32]):
        op = vd.fft.read_op()
        op.read_from_buffer(buf)
        with vc.if_block(op.fft_index >= limit):
            op.register[:] = 0.0
        with vc.else_if_block(op.fft_index == 0):
            op.register *= 3.0
        with vc.else_block():
            c = vc.new_register(vc.i32, 0)
            with vc.while_block(c < 2):
                op.register *= 2.0
                c += 1

    vd.fft.fft(out, src, lim, input_map=truncate)
    y = x.astype(np.complex128) * 4.0
    y[:, lim:] = 0.0
    y[:, 0] = x[:, 0] * 3.0
    ref = np.fft.fft(y, axis=1)
    assert rel_l2(out.read(0), ref) <= tol_fp32(n)

    dst = vd.Buffer((5, n), vd.complex64)

    @vd.map
    def split_scale(buf: vc.Buffer[vc.c64]):
        op = vd.fft.write_op()
        with vc.if_block(vc.all(op.fft_index > 0, op.fft_index < 10)):
            buf[op.io_index] = op.register * 0.5
        with vc.else_block():
            buf[op.io_index] = op.register

    b = vd.asbuffer(x)
    vd.fft.fft(dst, b, output_map=split_scale)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    ref[:, 1:10] *= 0.5
    assert rel_l2(dst.read(0), ref) <= tol_fp32(n)
