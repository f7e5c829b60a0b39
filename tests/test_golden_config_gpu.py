"""GPU parity at the benchmark configurations' lengths and stride classes
against the reference's own generated kernels (tests/golden/config_vectors.npz,
produced by tests/golden/make_golden.py config): 1024-point rows forward and
inverse with the magnitude-sum reduction (the plain C2C workload), 512-point
R2C / C2R rows and the 512 x 257 strided convolution (the 2-D convolution
workload), a 32^3 FFT3, and the reference's integer and float reductions.

Inputs are regenerated from oracle/inputs.py; large outputs are compared at
the fixture's sampled indices.  Bounds: relative L2 <= 5e-7 log2 N per pass
(summed over the passes of a chain), integer reductions bit-exact, float sums
within 2 eps log2(n) sum|x| plus the input difference of a chained case."""

import json
from pathlib import Path

import numpy as np
import pytest

from helpers import rel_l2, tol_fp32
from oracle import inputs

pytestmark = pytest.mark.gpu

vd = pytest.importorskip("vkdispatch_gb300")
from vkdispatch_gb300.codegen import Buff, c64, f32, i32, u32  # noqa: E402
import vkdispatch_gb300.codegen as vc  # noqa: E402

G = np.load(Path(__file__).resolve().parent / "golden" / "config_vectors.npz")
META = json.loads(bytes(G["__meta__"]).decode())


def _at(name, arr):
    flat = np.ascontiguousarray(arr).reshape(-1)
    return flat if META[name]["full"] else flat[G[name + "__idx"]]


def test_cfg1_rows_forward_inverse_and_magnitude_sum():
    b = vd.asbuffer(inputs.complex_uniform(101, (256, 1024)))
    vd.fft.fft(b)
    assert rel_l2(_at("cfg1_fwd", b.read(0)), G["cfg1_fwd"]) <= tol_fp32(1024)
    vd.fft.ifft(b)
    z = b.read(0)
    assert rel_l2(_at("cfg1_inv", z), G["cfg1_inv"]) <= tol_fp32(1024, 1024)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def mag(buffer: Buff[c64]) -> f32:
        v = buffer[vd.reduce.mapped_io_index()]
        return vc.sqrt(v.real * v.real + v.imag * v.imag)

    got = float(mag(b).read(0)[0])
    want = float(G["cfg1_magsum"][0])
    n = z.size
    bound = 2 * np.finfo(np.float32).eps * np.log2(n) * want + tol_fp32(1024, 1024) * np.sqrt(n) * np.linalg.norm(z)
    assert abs(got - want) <= bound


def test_512_point_real_rows():
    xr = inputs.uniform(102, (8, 512))
    rb = vd.asrfftbuffer(xr)
    vd.fft.rfft(rb)
    assert rel_l2(_at("r2c_8x512", rb.read_fourier(0)), G["r2c_8x512"]) <= tol_fp32(512)
    spec = inputs.complex_uniform(103, (8, 257))
    cb = vd.RFFTBuffer((8, 512))
    cb.write_fourier(spec)
    vd.fft.irfft(cb)
    assert rel_l2(_at("c2r_8x512", cb.read_real(0)), G["c2r_8x512"]) <= tol_fp32(512)


def test_strided_conv_512x257_axis1():
    b = vd.asbuffer(inputs.complex_uniform(104, (2, 512, 257)))
    k = vd.asbuffer(inputs.complex_uniform(105, (2, 512, 257)))
    vd.fft.convolve(b, k, axis=1)
    assert rel_l2(_at("conv_2x512x257_ax1", b.read(0)), G["conv_2x512x257_ax1"]) <= tol_fp32(512, 512)


def test_fft3_32():
    b = vd.asbuffer(inputs.complex_uniform(106, (32, 32, 32)))
    vd.fft.fft3(b)
    assert rel_l2(_at("fft3_32", b.read(0)), G["fft3_32"]) <= tol_fp32(32, 32, 32)


def test_integer_reductions_bit_exact():
    u = vd.asbuffer(inputs.uint32(107, (3, 100003)))

    @vd.reduce.reduce(0, axes=[1])
    def xor_u(a: u32, b: u32) -> u32:
        return a ^ b

    assert np.array_equal(xor_u(u).read(0).reshape(-1)[:3].astype(np.uint32), G["xor_u32_3x100003"][:3])
    i = inputs.uint32(109, (3 * 100003,)).view(np.int32) | np.int32(0x10204081)
    ib = vd.asbuffer(i.reshape(3, 100003))

    @vd.reduce.reduce(-1, axes=[1])
    def and_i(a: i32, b: i32) -> i32:
        return a & b

    assert np.array_equal(and_i(ib).read(0).reshape(-1)[:3].astype(np.int32), G["and_i32_3x100003"][:3])


def test_float_sum_rows():
    f = inputs.uniform(108, (3, 300001))
    fb = vd.asbuffer(f)

    @vd.reduce.reduce(0, axes=[1])
    def sum_f(a: f32, b: f32) -> f32:
        return a + b

    got = sum_f(fb).read(0).reshape(-1)[:3].astype(np.float64)
    want = G["sum_f32_3x300001"][:3].astype(np.float64)
    bound = 2 * np.finfo(np.float32).eps * np.log2(300001) * np.abs(f.astype(np.float64)).sum(axis=1)
    assert np.all(np.abs(got - want) <= bound)
