"""CPU tests: the oracle (C restatement of the reference algorithms) pinned
against fixtures generated from the reference itself
(tests/golden/make_golden.py): the reference planner's own plans, and
outputs of the reference's own generated kernels."""

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import fft_oracle as fo
from oracle import ref

GOLDEN = Path(__file__).resolve().parent / "golden"


def _vectors():
    g = np.load(GOLDEN / "vectors.npz")
    meta = json.loads(bytes(g["__meta__"]).decode())
    return g, meta


def test_planner_matches_reference_plans():
    plans = json.loads((GOLDEN / "plans.json").read_text())
    assert len(plans) > 1000
    for key, want in plans.items():
        n = int(key.split("/")[0])
        got = ref.plan(n)
        if "error" in want:
            assert got is None, key
        else:
            assert got is not None, key
            assert got["groups"] == want["groups"], key
            assert got["register_count"] == want["register_count"], key
            assert got["batch_threads"] == want["batch_threads"], key


G, META = _vectors()


@pytest.mark.parametrize("name", sorted(META))
def test_restatement_bit_exact_vs_reference_kernels(name):
    m = META[name]
    x, y = G[name + "__in"], G[name + "__out"]
    shape, axis, sr = tuple(m["shape"]), m["axis"], m["signal_range"]
    ax = len(shape) - 1 if axis is None else axis
    kind = m["kind"]
    if kind in ("fft", "ifft"):
        got = ref.fft(x, axis=ax, inverse=kind == "ifft", signal_range=None if sr is None else tuple(sr))
    elif kind == "rfft":
        got = ref.rfft_packed(x, shape[-1], signal_range=None if sr is None else tuple(sr))
    elif kind == "irfft":
        got = ref.real_from_packed(ref.irfft_packed(x, shape[-1]), shape[-1])
        y = ref.real_from_packed(y, shape[-1])
    else:
        got = ref.convolve(x, G[name + "__kernel"], axis=ax)
    assert np.array_equal(np.asarray(got), np.asarray(y))


@pytest.mark.parametrize("name", sorted(META))
def test_reference_vectors_vs_fp64(name):
    """The golden outputs themselves sit within the fp32 tolerance of FP64."""
    m = META[name]
    x, y = G[name + "__in"], G[name + "__out"]
    shape, axis, sr = tuple(m["shape"]), m["axis"], m["signal_range"]
    ax = len(shape) - 1 if axis is None else axis
    n = shape[ax]
    kind = m["kind"]
    if kind in ("fft", "ifft"):
        xx = x if sr is None else fo.mask_signal(x, ax, *sr)
        want = fo.fft_fp64(xx, axis=ax, inverse=kind == "ifft")
    elif kind == "rfft":
        xr = ref.real_from_packed(x, n)
        xx = xr if sr is None else fo.mask_signal(xr, -1, *sr)
        want = np.fft.rfft(xx.astype(np.float64), axis=-1)
    elif kind == "irfft":
        h = x.astype(np.complex128).copy()
        h[..., 0] = h[..., 0].real
        if n % 2 == 0:
            h[..., -1] = h[..., -1].real
        want = np.fft.irfft(h, n=n, axis=-1)
        y = ref.real_from_packed(y, n)
    else:
        k = G[name + "__kernel"]
        want = np.fft.ifft(np.fft.fft(x.astype(np.complex128), axis=ax) * np.conj(k.astype(np.complex128)), axis=ax)
    assert fo.rel_l2(y, want) <= 2 * 5e-7 * max(1, np.log2(n))


@pytest.mark.parametrize("n", [2, 3, 5, 7, 11, 13, 16, 45, 81, 100, 162, 343, 512, 1024, 1331, 4096, 16384])
def test_restatement_accuracy(n):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))).astype(np.complex64)
    y = ref.fft(x)
    assert fo.rel_l2(y, np.fft.fft(x.astype(np.complex128), axis=-1)) <= 5e-7 * max(1, np.log2(n))
    assert fo.rel_l2(ref.fft(y, inverse=True), x) <= 1e-6 * max(1, np.log2(n))


def test_restatement_rejects_like_reference():
    with pytest.raises(ValueError):
        ref.fft(np.zeros((2, 17), np.complex64))  # prime above 13
    with pytest.raises(ValueError):
        ref.fft(np.zeros((1, 15625), np.complex64))  # needs more than 1024 threads


def test_convolve2dr_restatement():
    rng = np.random.default_rng(1)
    img = rng.uniform(-1, 1, (3, 32, 32)).astype(np.float32)
    ker = rng.uniform(-1, 1, (32, 32)).astype(np.float32)
    kp = ref.packed_from_real(ker)
    kspec = ref.rfft_packed(kp, 32)
    kspec = ref.fft(kspec, axis=0)
    got = ref.convolve2DR(img, kspec)
    want = fo.convolve_fp64(img, np.broadcast_to(ker, img.shape), axes=(-2, -1)).real
    assert fo.rel_l2(got, want) < 1e-5


def test_reduce_restatement():
    rng = np.random.default_rng(2)
    d = rng.random(300001).astype(np.float32)
    s = ref.reduce_f32(d)[0]
    assert abs(s - d.astype(np.float64).sum()) / d.sum() < 1e-6
    assert ref.reduce_f32(d, op="max")[0] == d.max()
    assert ref.reduce_f32(d, op="min")[0] == d.min()
    c = (rng.standard_normal(5000) + 1j * rng.standard_normal(5000)).astype(np.complex64)
    assert abs(ref.reduce_f32(c, map="abs")[0] - np.abs(c.astype(np.complex128)).sum()) < 1e-3
