"""A seeded sweep of transform shapes against FP64 numpy: lengths from the
compile-time plans, the runtime-radix plans, the four-step pair (partial
column tiles included) and Bluestein; every axis of 1-3-D buffers; forward
and inverse; complex64, complex32 and bf16-pair storage; and convolutions of
the same shapes.  Each case is small (at most 2^21 points)."""

import numpy as np
import pytest

import vkdispatch_gb300 as vd

from helpers import crandn, rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

LENGTHS = [2, 3, 5, 7, 8, 11, 13, 16, 17, 24, 31, 64, 100, 127, 243, 256, 343, 512, 625, 1000, 1024, 2187,
           2401, 4096, 6561, 8192, 12005, 16384, 20000, 50421]
STORAGE = {"c64": (vd.complex64, 1.0), "c32": (vd.complex32, 2.5e-3), "bf16": (vd.complexbf16, 1.6e-2)}


def _case(seed):
    rng = np.random.default_rng(1000 + seed)
    ndim = int(rng.integers(1, 4))
    axis = int(rng.integers(0, ndim))
    n = int(rng.choice(LENGTHS))
    shape = [int(rng.choice([1, 2, 3, 5, 8, 17])) for _ in range(ndim)]
    shape[axis] = n
    while np.prod(shape) > (1 << 21) and max(shape) > 1:
        i = int(np.argmax([s if j != axis else 0 for j, s in enumerate(shape)]))
        if shape[i] == 1:
            break
        shape[i] = max(1, shape[i] // 2)
    storage = str(rng.choice(["c64", "c64", "c32", "bf16"]))
    inverse = bool(rng.integers(0, 2))
    return tuple(shape), axis, storage, inverse, rng


@pytest.mark.parametrize("seed", range(48))
def test_fft_sweep(seed):
    shape, axis, storage, inverse, rng = _case(seed)
    vt, tol_half = STORAGE[storage]
    x = crandn(rng, shape) * 0.5
    buf = vd.Buffer(shape, vt)
    buf.write(x)
    q = buf.read(0).astype(np.complex128)  # the stored (rounded) input
    (vd.fft.ifft if inverse else vd.fft.fft)(buf, axis=axis)
    ref = (np.fft.ifft if inverse else np.fft.fft)(q, axis=axis)
    tol = 2 * tol_fp32(shape[axis]) if storage == "c64" else tol_half
    assert rel_l2(buf.read(0), ref) <= tol, (shape, axis, storage, inverse)


@pytest.mark.parametrize("seed", range(16))
def test_convolve_sweep(seed):
    shape, axis, _, _, rng = _case(500 + seed)
    if shape[axis] > 16384:  # convolutions run one CTA per transform
        pytest.skip("axis above the one-CTA convolution limit")
    x = crandn(rng, shape)
    k = crandn(rng, shape) * 0.1
    b, kb = vd.asbuffer(x), vd.asbuffer(k)
    if vd.fft.pad_dim(shape[axis]) != shape[axis]:
        # prime factors above 13: the fused convolution has no Bluestein form
        # and refuses them, as the reference's planner does
        with pytest.raises(ValueError):
            vd.fft.convolve(b, kb, axis=axis)
        return
    vd.fft.convolve(b, kb, axis=axis)
    x64 = x.astype(np.complex128)
    ref = np.fft.ifft(np.fft.fft(x64, axis=axis) * np.conj(k), axis=axis)
    assert rel_l2(b.read(0), ref) <= 3 * tol_fp32(shape[axis]), (shape, axis)


@pytest.mark.parametrize("seed", range(16))
def test_real_sweep(seed):
    """rfft then irfft along the last axis: even lengths (half-length complex
    FFT with the split) and odd ones (the full-length rule)."""
    rng = np.random.default_rng(3000 + seed)
    n = int(rng.choice([2, 6, 9, 16, 25, 100, 243, 512, 1000, 1001, 2187, 4096, 12005, 16384]))
    rows = int(rng.choice([1, 3, 17]))
    x = rng.standard_normal((rows, n)).astype(np.float32)
    buf = vd.RFFTBuffer((rows, n))
    buf.write_real(x)
    vd.fft.rfft(buf)
    spec = buf.read_fourier(0)
    ref = np.fft.rfft(x.astype(np.float64), axis=-1)
    assert rel_l2(spec, ref) <= 2 * tol_fp32(n), (rows, n)
    vd.fft.irfft(buf)
    assert rel_l2(buf.read_real(0), x) <= 4 * tol_fp32(n), (rows, n)
