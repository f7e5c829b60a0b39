"""Shared helpers for the parity tests: seeded inputs, error metrics and the
tolerance rule.

Tolerance (complex64 with fp32 butterflies): relative L2 error against the
FP64 numpy.fft result <= 5e-7 * max(1, log2 N) for a transform of length N,
accumulated per pass for multi-axis transforms.
"""

import math

import numpy as np


def rel_l2(got, ref) -> float:
    got = np.asarray(got, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    den = np.linalg.norm(ref.ravel())
    if den == 0:
        return float(np.linalg.norm(got.ravel()))
    return float(np.linalg.norm((got - ref).ravel()) / den)


def tol_fp32(*lengths) -> float:
    return sum(5e-7 * max(1.0, math.log2(n)) for n in lengths)


def crandn(rng, shape, dtype=np.complex64):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


def smooth_sizes(primes=(2, 3, 5, 7, 11, 13), limit=4096):
    out = set()

    def rec(v, i):
        if v > limit:
            return
        out.add(v)
        for j in range(i, len(primes)):
            rec(v * primes[j], j)

    rec(1, 0)
    return sorted(out)
