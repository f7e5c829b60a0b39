"""Bluestein (chirp-z) transforms for lengths with prime factors above 13
(VDX_FFT_FLAG_BLUESTEIN; on by default in vd.fft), which the reference
rejects (vkdispatch/fft/prime_utils.py:6-10), against FP64 numpy.fft.

Tolerance: the transform is a length-M convolution (M = the power of two
>= 2N - 1) between two chirp multiplications, so fp32 compute is held to
three times the per-pass bound of a length-M transform."""

import numpy as np
import pytest

from helpers import crandn, rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

vd = pytest.importorskip("vkdispatch_gb300")


def _m(n):
    m = 1
    while m < 2 * n - 1:
        m *= 2
    return m


@pytest.mark.parametrize("n", [17, 97, 127, 646, 1009, 4099])
def test_contiguous_forward_and_inverse(n):
    rng = np.random.default_rng(n)
    x = crandn(rng, (5, n))
    buf = vd.asbuffer(x)
    with vd.fft.bluestein():
        vd.fft.fft(buf)
        got = buf.read(0)
        vd.fft.ifft(buf)
    assert rel_l2(got, np.fft.fft(x.astype(np.complex128), axis=1)) <= 3 * tol_fp32(_m(n))
    assert rel_l2(buf.read(0), x) <= 6 * tol_fp32(_m(n))


@pytest.mark.parametrize("shape,axis", [((131, 24), 0), ((3, 211, 5), 1)])
def test_strided_axes(shape, axis):
    rng = np.random.default_rng(sum(shape))
    x = crandn(rng, shape)
    buf = vd.asbuffer(x)
    with vd.fft.bluestein():
        vd.fft.fft(buf, axis=axis)
    n = shape[axis]
    assert rel_l2(buf.read(0), np.fft.fft(x.astype(np.complex128), axis=axis)) <= 3 * tol_fp32(_m(n))


def test_fp64_compute():
    rng = np.random.default_rng(31)
    x = (rng.standard_normal((4, 1009)) + 1j * rng.standard_normal((4, 1009))).astype(np.complex128)
    buf = vd.asbuffer(x)
    with vd.fft.bluestein():
        vd.fft.fft(buf)
    assert rel_l2(buf.read(0), np.fft.fft(x, axis=1)) < 1e-12


def test_bf16_storage():
    rng = np.random.default_rng(37)
    x = crandn(rng, (4, 257)) * 0.25
    buf = vd.Buffer(x.shape, vd.complexbf16)
    buf.write(x)
    q = buf.read(0).astype(np.complex128)
    with vd.fft.bluestein():
        vd.fft.fft(buf)
    assert rel_l2(buf.read(0), np.fft.fft(q, axis=1)) < 5e-3


def test_default_on_and_refusal_on_request():
    rng = np.random.default_rng(41)
    x = crandn(rng, (2, 17))
    b = vd.asbuffer(x)
    vd.fft.fft(b)  # Bluestein by default
    assert rel_l2(b.read(0), np.fft.fft(x.astype(np.complex128), axis=1)) <= 3 * tol_fp32(_m(17))
    with vd.fft.bluestein(False), pytest.raises(ValueError):
        vd.fft.fft(vd.Buffer((2, 17), vd.complex64))  # the reference's behaviour
    with pytest.raises(ValueError):
        vd.fft.fft(vd.Buffer((1, 8209), vd.complex128))  # fp64: single-CTA convolutions only (M <= 8192)


@pytest.mark.parametrize("n,rows", [(8209, 3), (16411, 2), (65537, 1)])
def test_long_lengths_through_four_step(n, rows):
    """M > 16384: the convolution runs as a four-step forward transform, a
    spectrum product and a four-step inverse."""
    rng = np.random.default_rng(n)
    x = crandn(rng, (rows, n))
    b = vd.asbuffer(x)
    vd.fft.fft(b)
    got = b.read(0)
    assert rel_l2(got, np.fft.fft(x.astype(np.complex128), axis=1)) <= 3 * tol_fp32(_m(n))
    vd.fft.ifft(b)
    assert rel_l2(b.read(0), x) <= 6 * tol_fp32(_m(n))


def test_long_strided_axis():
    rng = np.random.default_rng(43)
    x = crandn(rng, (10007, 4))
    b = vd.asbuffer(x)
    vd.fft.fft(b, axis=0)
    assert rel_l2(b.read(0), np.fft.fft(x.astype(np.complex128), axis=0)) <= 3 * tol_fp32(_m(10007))
