"""Long axes: the four-step pair of launches (csrc/fft_large.cu) against FP64
numpy.fft, for contiguous and strided axes, every storage type, chunked and
unchunked workspaces, and lengths above the single-CTA limit of 16384 (which
the reference's planner rejects, vkdispatch/fft/config.py:185-190)."""

import contextlib
import os

import numpy as np
import pytest
import torch

import vkdispatch_gb300 as vd
from vkdispatch_gb300 import _lib as L
from vkdispatch_gb300.fft import plan as P

from helpers import crandn, rel_l2, tol_fp32

pytestmark = pytest.mark.gpu


@contextlib.contextmanager
def _env(**kv):
    old = {k: os.environ.get(k) for k in kv}
    try:
        for k, v in kv.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = str(v)
        yield
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _plan(shape, axis, inverse=False, normalize=False, io=L.VDX_C64, **env):
    """An uncached plan created under the given environment."""
    d = L.FftDesc()
    d.ndim = len(shape)
    for i, s in enumerate(shape):
        d.shape[i] = int(s)
    d.axis = axis
    d.kind = L.VDX_KIND_C2C
    d.inverse = int(inverse)
    d.normalize = int(normalize)
    d.io_type = io
    d.compute_type = L.VDX_C64
    d.signal_lo, d.signal_hi = -1, -1
    d.kernel_op = L.VDX_KOP_MUL_CONJ
    d.kernel_type = io
    with _env(**env):
        return P.Plan(d)


def _run(plan, t):
    plan.exec(t.data_ptr(), t.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()


# 12005 = 245 x 49 and 50421 = 343 x 147: the first pass's last column tile
# is partial (49 and 147 columns in tiles of 16)
@pytest.mark.parametrize("n", [8192, 12005, 12500, 16384, 20000, 24576, 32768, 50421, 65536])
def test_contiguous_lengths(n):
    rng = np.random.default_rng(n)
    x = crandn(rng, (3, n))
    t = torch.from_numpy(x).cuda()
    p = _plan((3, n), 1)
    d = p.describe()
    assert d["fourstep"][0] * d["fourstep"][1] == n
    _run(p, t)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    assert rel_l2(t.cpu().numpy(), ref) <= tol_fp32(n)
    pi = _plan((3, n), 1, inverse=True, normalize=True)
    _run(pi, t)
    assert rel_l2(t.cpu().numpy(), x) <= 2 * tol_fp32(n)


def test_length_2_pow_20():
    n = 1 << 20
    rng = np.random.default_rng(20)
    x = crandn(rng, (1, n))
    t = torch.from_numpy(x).cuda()
    _run(_plan((1, n), 1), t)
    assert rel_l2(t.cpu().numpy(), np.fft.fft(x.astype(np.complex128))) <= tol_fp32(n)


@pytest.mark.parametrize("shape,axis", [((16384, 40), 0), ((3, 8192, 24), 1), ((2, 16384, 5), 1)])
@pytest.mark.parametrize("ws_mb", [None, 1, 0])
def test_strided_axes_and_chunks(shape, axis, ws_mb):
    rng = np.random.default_rng(sum(shape) + (ws_mb or 7))
    x = crandn(rng, shape)
    t = torch.from_numpy(x).cuda()
    p = _plan(shape, axis, VDX_FOURSTEP_WS_MB=ws_mb, VDX_FOURSTEP_FUSED=None if ws_mb is None else 0)
    assert p.describe()["strided"] is True
    _run(p, t)
    ref = np.fft.fft(x.astype(np.complex128), axis=axis)
    assert rel_l2(t.cpu().numpy(), ref) <= tol_fp32(shape[axis])


@pytest.mark.parametrize("ws_mb", [1, 0])
def test_contiguous_chunks(ws_mb):
    rng = np.random.default_rng(5)
    x = crandn(rng, (20, 16384))
    t = torch.from_numpy(x).cuda()
    # workspace chunks belong to the two-launch form
    p = _plan((20, 16384), 1, VDX_FOURSTEP_WS_MB=ws_mb, VDX_FOURSTEP_FUSED=0)
    d = p.describe()
    assert d["chunk_outer"] == (8 if ws_mb == 1 else 20)
    _run(p, t)
    assert rel_l2(t.cpu().numpy(), np.fft.fft(x.astype(np.complex128), axis=1)) <= tol_fp32(16384)


def test_threshold_env_keeps_single_cta_path():
    p = _plan((2, 16384), 1, VDX_FOURSTEP_MIN=0)
    assert "fourstep" not in p.describe()
    q = _plan((2, 32768), 1, VDX_FOURSTEP_MIN=0)  # above the single-CTA limit: four-step regardless
    assert q.describe()["fourstep"] == [256, 128]


@pytest.mark.parametrize("vt,tol", [(vd.complexbf16, 5e-3), (vd.complex32, 1.2e-3)])
@pytest.mark.parametrize("axis", [0, 1])
def test_half_storage(vt, tol, axis):
    rng = np.random.default_rng(11 + axis)
    shape = (16384, 32) if axis == 0 else (4, 16384)
    x = crandn(rng, shape)
    buf = vd.Buffer(shape, vt)
    buf.write(x)
    q = buf.read(0).astype(np.complex128)
    vd.fft.fft(buf, axis=axis)
    got = buf.read(0)
    # storage rounding of the workspace and of the outputs dominates
    assert rel_l2(got, np.fft.fft(q, axis=axis)) < tol


def test_fft2_through_the_api():
    rng = np.random.default_rng(3)
    x = crandn(rng, (16384, 64))
    buf = vd.asbuffer(x)
    vd.fft.fft2(buf)
    ref = np.fft.fft2(x.astype(np.complex128))
    assert rel_l2(buf.read(0), ref) <= tol_fp32(16384, 64)
    vd.fft.ifft2(buf)
    assert rel_l2(buf.read(0), x) <= 2 * tol_fp32(16384, 64)


def test_fused_ops_rejected_on_fourstep_plans():
    p = _plan((1, 16384), 1)
    t = torch.zeros((1, 16384), dtype=torch.complex64, device="cuda")
    w = torch.ones((1, 16384), dtype=torch.float32, device="cuda")
    ops = L.ExecOps()
    ops.in_weight = w.data_ptr()
    ops.in_weight_scale = 1.0
    with pytest.raises(ValueError):
        p.exec_ops(t.data_ptr(), t.data_ptr(), None, ops, torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("vt", [vd.complexbf16, vd.complex32])
@pytest.mark.parametrize("shape,axis,ws_mb", [((16384, 40), 0, None), ((3, 16384, 36), 1, None),
                                              ((16384, 100), 0, 1)])
def test_half_storage_strided_tiles(vt, shape, axis, ws_mb):
    """Strided axes with 4-byte storage stage their tiles with TMA copies:
    partial last tiles (zero-filled columns), outer batches (rank-4 maps) and
    chunked workspaces (moved base pointers)."""
    rng = np.random.default_rng(sum(shape) + axis)
    x = crandn(rng, shape) * 0.25
    buf = vd.Buffer(shape, vt)
    buf.write(x)
    q = buf.read(0).astype(np.complex128)
    with _env(VDX_FOURSTEP_WS_MB=ws_mb):
        P.cache_clear()
        vd.fft.fft(buf, axis=axis)
    got = buf.read(0)
    tol = 5e-3 if vt == vd.complexbf16 else 1.2e-3
    assert rel_l2(got, np.fft.fft(q, axis=axis)) < tol
    P.cache_clear()


@pytest.mark.parametrize("shape,axis", [((16384, 40), 0), ((2, 16384, 37), 1), ((5, 16384), 1), ((4096, 70), 0),
                                        ((9, 4096), 1), ((3, 65536), 1), ((65536, 3), 0)])
@pytest.mark.parametrize("inverse", [False, True])
def test_fused_four_step_matches_numpy_and_two_launch_form(shape, axis, inverse):
    """The opt-in fused form (VDX_FOURSTEP_FUSED=1: both passes of a square
    split in one persistent launch with an L2-resident ring, csrc/
    fft_fused4.cu) against FP64 numpy and against the default two-launch
    form, out of place."""
    rng = np.random.default_rng(sum(shape) + axis + inverse)
    x = crandn(rng, shape)
    src = torch.from_numpy(x).cuda()
    # VDX_FOURSTEP_MIN=1: four-step for the 4096-point axes too (64 x 64 splits)
    fused = _plan(shape, axis, inverse=inverse, normalize=inverse, VDX_FOURSTEP_MIN=1, VDX_FOURSTEP_FUSED=1)
    plain = _plan(shape, axis, inverse=inverse, normalize=inverse, VDX_FOURSTEP_MIN=1, VDX_FOURSTEP_FUSED=0)
    assert fused.describe()["fused"] and not plain.describe()["fused"]
    outs = []
    for p in (fused, plain):
        out = torch.empty_like(src)
        p.exec(src.data_ptr(), out.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    assert fused.status() == 0
    x64 = x.astype(np.complex128)
    ref = np.fft.ifft(x64, axis=axis) if inverse else np.fft.fft(x64, axis=axis)
    n = shape[axis]
    assert rel_l2(outs[0], ref) <= tol_fp32(n)
    assert rel_l2(outs[0], outs[1]) <= tol_fp32(n)


@pytest.mark.parametrize("vt,tol", [(vd.complexbf16, 5e-3), (vd.complex32, 1.2e-3)])
@pytest.mark.parametrize("shape,axis", [((16384, 48), 0), ((3, 16384), 1)])
def test_fused_four_step_half_storage(vt, tol, shape, axis):
    rng = np.random.default_rng(77 + axis)
    x = crandn(rng, shape) * 0.25
    buf = vd.Buffer(shape, vt)
    buf.write(x)
    q = buf.read(0).astype(np.complex128)
    io = L.VDX_BF16X2 if vt == vd.complexbf16 else L.VDX_C32
    p = _plan(shape, axis, io=io, VDX_FOURSTEP_FUSED=1)
    assert p.describe()["fused"]
    _run(p, buf.tensor)
    assert p.status() == 0
    assert rel_l2(buf.read(0), np.fft.fft(q, axis=axis)) < tol
