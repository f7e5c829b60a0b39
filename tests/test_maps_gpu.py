"""GPU tests of the FFT map hooks and precision pairs, mirroring the
reference's tests/test_fft_mixed_precision.py (same seeds and tolerances)."""

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

vd = pytest.importorskip("vkdispatch_gb300")
import vkdispatch_gb300.codegen as vc  # noqa: E402


def _q32(values):
    return (values.real.astype(np.float16).astype(np.float32)
            + 1j * values.imag.astype(np.float16).astype(np.float32)).astype(np.complex64)


def test_map_complex32_input_to_complex128_output_auto_compute():
    rng = np.random.default_rng(11)
    data = (rng.standard_normal(32) + 1j * rng.standard_normal(32)).astype(np.complex64)
    inb = vd.Buffer(data.shape, vd.complex32)
    inb.write(data)
    outb = vd.Buffer(data.shape, vd.complex128)

    def input_map(buffer: vc.Buffer[vd.complex32]):
        vd.fft.read_op().read_from_buffer(buffer)

    def output_map(buffer: vc.Buffer[vd.complex128]):
        vd.fft.write_op().write_to_buffer(buffer)

    vd.fft.fft(outb, inb, input_map=vd.map(input_map), output_map=vd.map(output_map))
    ref = np.fft.fft(_q32(data)).astype(np.complex128)
    got = outb.read(0)
    assert got.dtype == np.complex128
    assert np.allclose(got, ref, atol=3e-1, rtol=2e-2)
    assert rel_l2(got, ref) < 1e-6


def test_float32_input_output_maps():
    rng = np.random.default_rng(23)
    data = rng.standard_normal(64).astype(np.float32)
    inb = vd.asbuffer(data)
    outb = vd.Buffer(data.shape, vd.float32)

    def input_map(buffer: vc.Buffer[vd.float32]):
        op = vd.fft.read_op()
        value = vc.to_dtype(op.register.var_type.child_type, buffer[op.io_index])
        op.register.real = value
        op.register.imag = vc.to_dtype(op.register.var_type.child_type, 0)

    def output_map(buffer: vc.Buffer[vd.float32]):
        op = vd.fft.write_op()
        buffer[op.io_index] = vc.to_dtype(buffer.var_type, op.register.real)

    vd.fft.fft(outb, inb, input_map=vd.map(input_map), output_map=vd.map(output_map))
    ref = np.fft.fft(data.astype(np.complex64)).real.astype(np.float32)
    assert np.allclose(outb.read(0), ref, atol=2e-3, rtol=1e-3)


def test_kernel_map_float32_scale():
    rng = np.random.default_rng(31)
    data = (rng.standard_normal(64) + 1j * rng.standard_normal(64)).astype(np.complex64)
    sig = vd.asbuffer(data.copy())
    scale = vd.asbuffer(np.full(data.shape, np.float32(0.5)))

    def kernel_map(scale_values: vc.Buffer[vd.float32]):
        op = vd.fft.read_op()
        sv = vc.to_dtype(op.register.var_type, vc.to_complex(scale_values[op.io_index]))
        op.register[:] = vc.mult_complex(op.register, sv)

    vd.fft.convolve(sig, scale, kernel_map=vd.map(kernel_map))
    assert np.allclose(sig.read(0), data * np.float32(0.5), atol=2e-3, rtol=1e-3)


def test_kernel_maps_conj_mul_identity():
    rng = np.random.default_rng(5)
    x = (rng.standard_normal((3, 48)) + 1j * rng.standard_normal((3, 48))).astype(np.complex64)
    k = (rng.standard_normal((3, 48)) + 1j * rng.standard_normal((3, 48))).astype(np.complex64)
    kspec = np.fft.fft(k.astype(np.complex128), axis=-1).astype(np.complex64)

    def conj_map(kb: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        kv = vc.new_register(vd.complex64)
        op.read_from_buffer(kb, register=kv)
        op.register[:] = vc.mult_complex(op.register, kv.conjugate())

    def mul_map(kb: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        kv = vc.new_register(vd.complex64)
        op.read_from_buffer(kb, register=kv)
        op.register[:] = vc.mult_complex(op.register, kv)

    def nothing():
        return

    s = np.fft.fft(x.astype(np.complex128), axis=-1)
    for m, want in ((conj_map, np.fft.ifft(s * np.conj(kspec), axis=-1)), (mul_map, np.fft.ifft(s * kspec, axis=-1))):
        b, kb = vd.asbuffer(x), vd.asbuffer(kspec)
        vd.fft.convolve(b, kb, kernel_map=vd.map(m))
        assert rel_l2(b.read(0), want) < 1e-5, m.__name__
    b = vd.asbuffer(x)
    vd.fft.convolve(b, kernel_map=vd.map(nothing))
    assert rel_l2(b.read(0), x) < 1e-5


def test_output_map_without_input_map_uses_explicit_input_buffer():
    rng = np.random.default_rng(37)
    data = (rng.standard_normal(64) + 1j * rng.standard_normal(64)).astype(np.complex64)
    inb = vd.asbuffer(data.copy())
    outb = vd.Buffer(data.shape, vd.complex64)

    def output_map(buffer: vc.Buffer[vd.complex64]):
        vd.fft.write_op().write_to_buffer(buffer)

    vd.fft.fft(outb, inb, output_map=vd.map(output_map))
    assert np.allclose(outb.read(0), np.fft.fft(data).astype(np.complex64), atol=2e-3, rtol=1e-3)
    assert np.array_equal(inb.read(0), data)  # the input is left untouched


def test_complex64_io_with_complex128_compute():
    rng = np.random.default_rng(29)
    data = (rng.standard_normal(64) + 1j * rng.standard_normal(64)).astype(np.complex64)
    b = vd.asbuffer(data)
    vd.fft.fft(b, compute_type=vd.complex128)
    got = b.read(0)
    assert np.allclose(got, np.fft.fft(data).astype(np.complex64), atol=2e-3, rtol=1e-3)
    # fp64 butterflies: only the final complex64 rounding remains
    assert rel_l2(got, np.fft.fft(data.astype(np.complex128))) < 1e-7


def test_map_outside_the_menu_is_compiled_and_unsupported_ones_name_themselves():
    """A map outside the functor menu runs through the run-time compiler (an
    input map that squares the still-zero register gives a zero transform);
    a construct the compiler lacks raises NotImplementedError naming the map."""

    def weird(buffer: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        op.register[:] = vc.mult_complex(op.register, op.register)

    b = vd.asbuffer(np.ones(8, np.complex64))
    vd.fft.fft(b, b, input_map=vd.map(weird))
    assert np.array_equal(b.read(0), np.zeros(8, np.complex64))

    def odd(buffer: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        op.register[:] = buffer[op.io_index] % 2.0

    with pytest.raises(NotImplementedError, match="odd"):
        vd.fft.fft(b, b, input_map=vd.map(odd))
