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


# ---------------------------------------------------------------------------
# config-shape fixtures (tests/golden/config_vectors.npz): inputs regenerated
# from oracle/inputs.py, outputs of the reference's own generated kernels
# (sampled where large)
# ---------------------------------------------------------------------------
from oracle import inputs  # noqa: E402

CG = np.load(GOLDEN / "config_vectors.npz")
CMETA = json.loads(bytes(CG["__meta__"]).decode())


def _at(name, arr):
    flat = np.ascontiguousarray(arr).reshape(-1)
    return flat if CMETA[name]["full"] else flat[CG[name + "__idx"]]


def _cfg1_chain():
    x = inputs.complex_uniform(101, (256, 1024))
    y = ref.fft(x, axis=1)
    return y, ref.fft(y, axis=1, inverse=True)


def test_config_cfg1_forward_inverse_bit_exact():
    y, z = _cfg1_chain()
    assert np.array_equal(_at("cfg1_fwd", y), CG["cfg1_fwd"])
    assert np.array_equal(_at("cfg1_inv", z), CG["cfg1_inv"])


def test_config_cfg1_magnitude_sum_bit_exact():
    """The reference's two-stage map_reduce (sqrt(re^2 + im^2), add) over the
    inverse output: the restatement's fold order gives its exact bits."""
    _, z = _cfg1_chain()
    got = ref.reduce_f32(z.reshape(-1), "add", "abs")
    assert got[0] == CG["cfg1_magsum"][0]


def test_config_512_point_real_rows_bit_exact():
    xr = inputs.uniform(102, (8, 512))
    assert np.array_equal(_at("r2c_8x512", ref.rfft_packed(ref.packed_from_real(xr), 512)), CG["r2c_8x512"])
    spec = inputs.complex_uniform(103, (8, 257))
    got = ref.real_from_packed(ref.irfft_packed(spec, 512), 512)
    assert np.array_equal(_at("c2r_8x512", got), CG["c2r_8x512"])


def test_config_strided_conv_512x257_bit_exact():
    xs = inputs.complex_uniform(104, (2, 512, 257))
    ks = inputs.complex_uniform(105, (2, 512, 257))
    assert np.array_equal(_at("conv_2x512x257_ax1", ref.convolve(xs, ks, axis=1)), CG["conv_2x512x257_ax1"])


def test_config_fft3_32_bit_exact():
    b = inputs.complex_uniform(106, (32, 32, 32))
    for ax in (0, 1, 2):
        b = ref.fft(b, axis=ax)
    assert np.array_equal(_at("fft3_32", b), CG["fft3_32"])


def test_config_reductions():
    u = inputs.uint32(107, (3, 100003))
    assert np.array_equal(CG["xor_u32_3x100003"][:3], np.bitwise_xor.reduce(u, axis=1))
    i = inputs.uint32(109, (3 * 100003,)).view(np.int32) | np.int32(0x10204081)
    assert np.array_equal(CG["and_i32_3x100003"][:3], np.bitwise_and.reduce(i.reshape(3, -1), axis=1))
    f = inputs.uniform(108, (3 * 300001,))
    assert np.array_equal(ref.reduce_f32(f, "add", "identity", batch=3), CG["sum_f32_3x300001"][:3])
