"""Portable seeded inputs for fixtures whose inputs are regenerated instead of
stored (test infrastructure only).

numpy's Generator distributions may change between numpy releases, so the
config-shape golden fixtures draw their inputs from splitmix64 (Steele, Lea
and Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014)
over the element index, in plain uint64 arithmetic: every host and numpy
version produces the same bits.
"""

from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """`count` 64-bit outputs of splitmix64 started at state `seed`."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + _GAMMA * (np.arange(count, dtype=np.uint64) + np.uint64(1))
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, shape) -> np.ndarray:
    """float32 in [-1, 1) with 24 random bits each."""
    n = int(np.prod(shape))
    top = (splitmix64(seed, n) >> np.uint64(40)).astype(np.float64)
    return (top * (2.0 / 16777216.0) - 1.0).astype(np.float32).reshape(shape)


def complex_uniform(seed: int, shape) -> np.ndarray:
    """complex64 with real and imaginary parts from uniform(), interleaved."""
    flat = uniform(seed, (int(np.prod(shape)) * 2,))
    return flat.view(np.complex64).reshape(shape)


def uint32(seed: int, shape) -> np.ndarray:
    n = int(np.prod(shape))
    return (splitmix64(seed, n) >> np.uint64(32)).astype(np.uint32).reshape(shape)


def sample_indices(seed: int, size: int, count: int = 4096) -> np.ndarray:
    """Sorted distinct flat indices < size at which sampled outputs are kept."""
    idx = np.unique(splitmix64(seed ^ 0x5A5A, count) % np.uint64(size)).astype(np.int64)
    return idx
