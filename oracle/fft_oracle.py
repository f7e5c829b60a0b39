"""FFT oracles (test infrastructure only; see oracle/__init__.py).

* FP64 oracle: numpy.fft on complex128 / float64 inputs, the oracle the
  reference's own tests use (tests/test_fft.py, tests/test_conv.py).
* Reference-semantics helpers: the packed RFFT layout, input_signal_range
  masking and the conjugate-kernel convolution convention of the reference
  (vkdispatch/fft/global_memory_iterators.py:17-49, 167-229;
  vkdispatch/fft/shader_factories.py:136-145).
"""

from __future__ import annotations

import numpy as np


def rel_l2(got, ref) -> float:
    got = np.asarray(got, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    den = np.linalg.norm(ref.ravel())
    if den == 0:
        return float(np.linalg.norm(got.ravel()))
    return float(np.linalg.norm((got - ref).ravel()) / den)


def fft_fp64(x, axis=-1, inverse=False, normalize=True):
    x = np.asarray(x).astype(np.complex128)
    if not inverse:
        return np.fft.fft(x, axis=axis)
    y = np.fft.ifft(x, axis=axis)
    return y if normalize else y * x.shape[axis]


def convolve_fp64(signal, kernel, axes=(-1,)):
    """ifft(fft(signal) * conj(fft(kernel))) over `axes` (the reference's
    default kernel map multiplies by the conjugate kernel spectrum)."""
    s = np.fft.fftn(np.asarray(signal).astype(np.complex128), axes=axes)
    k = np.fft.fftn(np.asarray(kernel).astype(np.complex128), axes=axes)
    return np.fft.ifftn(s * np.conj(k), axes=axes)


def mask_signal(x, axis, lo, hi):
    """input_signal_range: samples outside [lo, hi) along `axis` read as 0."""
    z = np.array(x, copy=True)
    sl = [slice(None)] * z.ndim
    sl[axis] = slice(0, lo)
    z[tuple(sl)] = 0
    sl[axis] = slice(hi, z.shape[axis])
    z[tuple(sl)] = 0
    return z
