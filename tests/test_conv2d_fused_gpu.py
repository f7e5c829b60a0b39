"""The one-launch convolve2DR (csrc/fft_conv2d.cu, VDX_KIND_CONV2D_REAL)
against FP64 numpy and against the composed rfft -> convolve -> irfft path
(vkdispatch/fft/functions.py:614-646), whose result it must reproduce,
including the post-convolution Nyquist bin left in each packed row."""

import os

import numpy as np
import pytest
import torch

import vkdispatch_gb300 as vd
from vkdispatch_gb300 import _lib as L
from vkdispatch_gb300.fft import plan as P

from helpers import crandn, rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

TOL = 4 * tol_fp32(512)  # row rfft, column FFT and inverse, row irfft


def _ref(x, K, normalize=True):
    """FP64 restatement of the composed path: rfft rows, columns * conj(K), irfft rows."""
    S = np.fft.rfft(x.astype(np.float64), axis=-1)
    T = np.fft.ifft(np.fft.fft(S, axis=-2) * np.conj(K), axis=-2)
    y = np.fft.irfft(T, n=x.shape[-1], axis=-1)
    if not normalize:
        y = y * x.shape[-2] * x.shape[-1]
    return y


def _gaussian_spectrum(H, W, sigma=5.0, size=31):
    ax = np.arange(size) - size // 2
    g = np.exp(-(ax[:, None] ** 2 + ax[None, :] ** 2) / (2 * sigma ** 2))
    k = np.zeros((H, W))
    k[:size, :size] = g / g.sum()
    return np.fft.rfft2(k)


def _run(x, K, fused=True, **kw):
    buf = vd.RFFTBuffer(x.shape)
    buf.write_real(x.astype(np.float32))
    kb = vd.RFFTBuffer(K.shape[:-1] + (2 * (K.shape[-1] - 1),))  # the real shape whose spectrum K is
    kb.write_fourier(K.astype(np.complex64))
    old = os.environ.get("VDX_FUSED_CONV2D")
    os.environ["VDX_FUSED_CONV2D"] = "1" if fused else "0"
    try:
        vd.fft.convolve2DR(buf, kb, **kw)
    finally:
        if old is None:
            os.environ.pop("VDX_FUSED_CONV2D")
        else:
            os.environ["VDX_FUSED_CONV2D"] = old
    torch.cuda.synchronize()
    return buf


def test_plan_is_the_fused_kind():
    p = P.get_plan((4, 512, 512), 1, L.VDX_KIND_CONV2D_REAL, False, True, L.VDX_C64, L.VDX_C64, None,
                   L.VDX_KOP_MUL_CONJ, L.VDX_C64, False)
    d = p.describe()
    assert d["op"] == "conv2d_real" and d["cluster"] == 8 and d["images"] == 4


@pytest.mark.parametrize("random_kernel", [False, True])
def test_matches_fp64_and_the_composed_path(random_kernel):
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (3, 512, 512))
    if random_kernel:
        K = crandn(rng, (3, 512, 257)).astype(np.complex128) * 0.1
    else:
        K = np.broadcast_to(_gaussian_spectrum(512, 512), (3, 512, 257)).copy()
    fused = _run(x, K)
    composed = _run(x, K, fused=False)
    ref = _ref(x, K)
    assert rel_l2(fused.read_real(0), ref) <= TOL
    # the whole packed buffer, the rows' last complex slot included
    assert rel_l2(fused.tensor.cpu().numpy(), composed.tensor.cpu().numpy()) <= TOL


def test_broadcast_kernel_and_2d_buffer():
    rng = np.random.default_rng(2)
    K = _gaussian_spectrum(512, 512)
    x3 = rng.uniform(-1, 1, (2, 512, 512))
    b3 = _run(x3, K, kernel_inner_only=True)
    assert rel_l2(b3.read_real(0), _ref(x3, K)) <= TOL
    x2 = rng.uniform(-1, 1, (512, 512))
    b2 = _run(x2, K)
    assert rel_l2(b2.read_real(0), _ref(x2, K)) <= TOL


def test_unnormalised():
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (1, 512, 512))
    K = crandn(rng, (1, 512, 257)).astype(np.complex128) * 1e-3
    b = _run(x, K, normalize=False)
    assert rel_l2(b.read_real(0), _ref(x, K, normalize=False)) <= TOL


def test_other_sizes_use_the_composed_path():
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (2, 256, 128))
    K = crandn(rng, (2, 256, 65)).astype(np.complex128) * 0.1
    with pytest.raises(ValueError):
        P.get_plan((2, 256, 128), 1, L.VDX_KIND_CONV2D_REAL, False, True, L.VDX_C64, L.VDX_C64, None,
                   L.VDX_KOP_MUL_CONJ, L.VDX_C64, False)
    b = _run(x, K)
    assert rel_l2(b.read_real(0), _ref(x, K)) <= 4 * tol_fp32(256)


def test_cuda_graph_capture(monkeypatch):
    monkeypatch.setenv("VDX_FUSED_CONV2D", "1")
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (2, 512, 512)).astype(np.float32)
    K = np.broadcast_to(_gaussian_spectrum(512, 512), (2, 512, 257)).astype(np.complex64).copy()
    buf = vd.RFFTBuffer(x.shape)
    kb = vd.RFFTBuffer(x.shape)
    kb.write_fourier(K)
    buf.write_real(x)
    vd.fft.convolve2DR(buf, kb)  # plan created before capture
    torch.cuda.synchronize()
    buf.write_real(x)
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            with vd.cuda_graph_capture(torch.cuda.current_stream()):
                vd.fft.convolve2DR(buf, kb)
    torch.cuda.current_stream().wait_stream(s)
    buf.write_real(x)
    g.replay()
    torch.cuda.synchronize()
    assert rel_l2(buf.read_real(0), _ref(x.astype(np.float64), K)) <= TOL
