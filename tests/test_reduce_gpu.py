"""GPU parity tests of vd.reduce (mirrors the reference's
tests/test_reductions.py): integer reductions bit-exact, float reductions
within an order-dependent tolerance against an FP64 sum."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

vd = pytest.importorskip("vkdispatch_gb300")
from vkdispatch_gb300.codegen import Buff, c64, f32, i32, u32  # noqa: E402
import vkdispatch_gb300.codegen as vc  # noqa: E402


def float_sum_tol(x):
    # |fp32 sum - exact| <= n * eps * sum|x| (worst case); the tree order gives ~sqrt(log n) in practice
    return 2 * np.finfo(np.float32).eps * np.log2(max(2, x.size)) * np.abs(x.astype(np.float64)).sum() + 1e-30


@pytest.mark.parametrize("n", [1, 7, 1024, 1536, 300000, 4096 * 1024 + 3])
def test_sum_map_reduce(n):
    rng = np.random.default_rng(n)
    data = rng.random(n).astype(np.float32)
    buf = vd.asbuffer(data)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def sum_map(buffer: Buff[f32]) -> f32:
        return buffer[vd.reduce.mapped_io_index()]

    res = sum_map(buf).read(0)[0]
    assert abs(float(res) - data.astype(np.float64).sum()) <= float_sum_tol(data)


def test_pure_reduce_and_sin_map():
    rng = np.random.default_rng(1)
    data = rng.random(300000).astype(np.float32)
    buf = vd.asbuffer(data)

    @vd.reduce.reduce(0)
    def sum_reduce(a: f32, b: f32) -> f32:
        return a + b

    r = sum_reduce(buf).read(0)[0]
    assert abs(r - data.sum(dtype=np.float64)) / data.sum(dtype=np.float64) < 1e-5

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def sin_map(buffer: Buff[f32]) -> f32:
        return vc.sin(buffer[vd.reduce.mapped_io_index()])

    r = sin_map(buf).read(0)[0]
    ref = np.sin(data.astype(np.float64)).sum()
    assert abs(r - ref) / abs(ref) < 1e-5


def test_min_max_batched():
    rng = np.random.default_rng(2)
    data = rng.standard_normal((10, 300000)).astype(np.float32)
    buf = vd.asbuffer(data)

    @vd.reduce.reduce("inf", axes=[1])
    def rmin(a: f32, b: f32) -> f32:
        return vc.min(a, b)

    @vd.reduce.reduce("-inf", axes=[1])
    def rmax(a: f32, b: f32) -> f32:
        return vc.max(a, b)

    assert np.array_equal(rmin(buf).read(0).ravel()[:10], data.min(axis=1))
    assert np.array_equal(rmax(buf).read(0).ravel()[:10], data.max(axis=1))


def test_batched_sum_axes():
    rng = np.random.default_rng(3)
    data = rng.random((10, 30000)).astype(np.float32)
    buf = vd.asbuffer(data)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd, axes=[1])
    def s(buffer: Buff[f32]) -> f32:
        return buffer[vd.reduce.mapped_io_index()]

    got = s(buf).read(0).ravel()[:10]
    ref = data.astype(np.float64).sum(axis=1)
    assert np.all(np.abs(got - ref) <= 1e-5 * ref)


@pytest.mark.parametrize("op", ["and", "or", "xor", "add", "min", "max"])
def test_integer_reductions_bit_exact(op):
    rng = np.random.default_rng(4)
    data = rng.integers(0, 2**31 - 1, size=123457, dtype=np.int32)
    buf = vd.asbuffer(data)
    fns = {
        "and": (lambda a, b: a & b, -1, np.bitwise_and.reduce),
        "or": (lambda a, b: a | b, 0, np.bitwise_or.reduce),
        "xor": (lambda a, b: a ^ b, 0, np.bitwise_xor.reduce),
        "add": (lambda a, b: a + b, 0, lambda d: np.add.reduce(d, dtype=np.int32)),
        "min": (lambda a, b: vc.min(a, b), 2**31 - 1, np.min),
        "max": (lambda a, b: vc.max(a, b), -(2**31), np.max),
    }
    f, ident, ref = fns[op]

    def red(a: i32, b: i32) -> i32:
        return f(a, b)

    red.__name__ = f"red_{op}"
    rf = vd.reduce.reduce(ident)(red)
    with np.errstate(over="ignore"):
        assert rf(buf).read(0)[0] == ref(data)


def test_uint_xor():
    rng = np.random.default_rng(5)
    data = rng.integers(0, 2**32 - 1, size=70001, dtype=np.uint32)
    buf = vd.asbuffer(data)

    @vd.reduce.reduce(0)
    def rx(a: u32, b: u32) -> u32:
        return a ^ b

    assert int(rx(buf).read(0)[0]) == int(np.bitwise_xor.reduce(data))


def test_complex_magnitude_sum():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal((256, 1024)) + 1j * rng.standard_normal((256, 1024))).astype(np.complex64)
    buf = vd.asbuffer(x)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def mag(buffer: Buff[c64]) -> f32:
        v = buffer[vd.reduce.mapped_io_index()]
        return vc.sqrt(v.real * v.real + v.imag * v.imag)

    got = mag(buf).read(0)[0]
    ref = np.abs(x.astype(np.complex128)).sum()
    assert abs(got - ref) / ref < 1e-6
