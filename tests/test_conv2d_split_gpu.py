"""convolve2DR over a batch of images split into groups, each group's
rfft -> convolution -> irfft chain on its own stream (fft/functions.py
_conv2d_split, through vdx_group_plan): the same results as one group on the caller's stream, for
replicated and broadcast kernels, uneven groups, CUDA-graph capture and
deferred CommandGraph recording."""

import numpy as np
import pytest
import torch

import vkdispatch_gb300 as vd

from helpers import rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

TOL = 4 * tol_fp32(512)


def _gaussian_spectrum(H, W, sigma=5.0, size=31):
    ax = np.arange(size) - size // 2
    g = np.exp(-(ax[:, None] ** 2 + ax[None, :] ** 2) / (2 * sigma ** 2))
    k = np.zeros((H, W))
    k[:size, :size] = g / g.sum()
    return np.fft.rfft2(k)


def _ref(x, K):
    S = np.fft.rfft(x.astype(np.float64), axis=-1)
    T = np.fft.ifft(np.fft.fft(S, axis=-2) * np.conj(K), axis=-2)
    return np.fft.irfft(T, n=x.shape[-1], axis=-1)


def _inputs(n, seed, broadcast=False):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 512, 512)).astype(np.float32)
    if broadcast:
        K = _gaussian_spectrum(512, 512)
        kb = vd.RFFTBuffer((1, 512, 512))
        kb.write_fourier(K.astype(np.complex64)[None])
    else:
        K = (rng.standard_normal((n, 512, 257)) + 1j * rng.standard_normal((n, 512, 257))) * 0.01
        kb = vd.RFFTBuffer((n, 512, 512))
        kb.write_fourier(K.astype(np.complex64))
    buf = vd.RFFTBuffer((n, 512, 512))
    buf.write_real(x)
    return x, K, buf, kb


def _conv(buf, kb, parts, monkeypatch, **kw):
    monkeypatch.setenv("VDX_CONV2D_STREAMS", str(parts))
    vd.fft.convolve2DR(buf, kb, **kw)
    torch.cuda.synchronize()
    return buf.tensor.cpu().numpy()


@pytest.mark.parametrize("n,parts", [(16, 2), (18, 4), (24, 3)])
def test_groups_match_one_group(n, parts, monkeypatch):
    x, K, buf, kb = _inputs(n, n + parts)
    got = _conv(buf, kb, parts, monkeypatch)
    buf.write_real(x)
    one = _conv(buf, kb, 1, monkeypatch)
    assert rel_l2(got, one) <= TOL
    buf.tensor.copy_(torch.from_numpy(got))
    assert rel_l2(buf.read_real(0), _ref(x, K)) <= TOL


def test_broadcast_kernel(monkeypatch):
    x, K, buf, kb = _inputs(16, 7, broadcast=True)
    got = _conv(buf, kb, 2, monkeypatch, kernel_inner_only=True)
    buf.write_real(x)
    one = _conv(buf, kb, 1, monkeypatch, kernel_inner_only=True)
    assert rel_l2(got, one) <= TOL
    assert rel_l2(buf.read_real(0), _ref(x, K)) <= TOL


def test_cuda_graph_capture(monkeypatch):
    monkeypatch.setenv("VDX_CONV2D_STREAMS", "2")
    x, K, buf, kb = _inputs(16, 8)
    vd.fft.convolve2DR(buf, kb)  # plans created before capture
    torch.cuda.synchronize()
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
    assert rel_l2(buf.read_real(0), _ref(x, K)) <= TOL


def test_deferred_command_graph(monkeypatch):
    monkeypatch.setenv("VDX_CONV2D_STREAMS", "2")
    x, K, buf, kb = _inputs(16, 9)
    cg = vd.CommandGraph()
    vd.fft.convolve2DR(buf, kb, graph=cg)
    torch.cuda.synchronize()
    assert rel_l2(buf.read_real(0), x) == 0.0  # nothing ran yet
    cg.submit()
    torch.cuda.synchronize()
    assert rel_l2(buf.read_real(0), _ref(x, K)) <= TOL


def _crand(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("parts", [2, 3])
def test_rfft2_irfft2_groups(parts, monkeypatch):
    rng = np.random.default_rng(20 + parts)
    x = rng.uniform(-1, 1, (16, 512, 512)).astype(np.float32)
    buf = vd.RFFTBuffer(x.shape)
    buf.write_real(x)
    monkeypatch.setenv("VDX_CONV2D_STREAMS", str(parts))
    vd.fft.rfft2(buf)
    torch.cuda.synchronize()
    spec = buf.read_fourier(0)
    assert rel_l2(spec, np.fft.rfft2(x.astype(np.float64))) <= 2 * tol_fp32(512)
    vd.fft.irfft2(buf)
    torch.cuda.synchronize()
    assert rel_l2(buf.read_real(0), x) <= 4 * tol_fp32(512)


@pytest.mark.parametrize("parts", [2, 4])
def test_fft2_ifft2_and_convolve2d_groups(parts, monkeypatch):
    rng = np.random.default_rng(30 + parts)
    x = _crand(rng, (16, 256, 512))
    K = _crand(rng, (16, 256, 512)) * 0.05
    buf = vd.asbuffer(x)
    monkeypatch.setenv("VDX_CONV2D_STREAMS", str(parts))
    vd.fft.fft2(buf)
    torch.cuda.synchronize()
    assert rel_l2(buf.read(0), np.fft.fft2(x.astype(np.complex128))) <= 2 * tol_fp32(256, 512)
    vd.fft.ifft2(buf)
    torch.cuda.synchronize()
    assert rel_l2(buf.read(0), x) <= 4 * tol_fp32(256, 512)
    kb = vd.asbuffer(K)
    vd.fft.convolve2D(buf, kb)
    torch.cuda.synchronize()
    x64 = x.astype(np.complex128)
    S = np.fft.fft(x64, axis=2)
    ref = np.fft.ifft(np.fft.ifft(np.fft.fft(S, axis=1) * np.conj(K), axis=1), axis=2)
    assert rel_l2(buf.read(0), ref) <= 4 * tol_fp32(256, 512)


def test_long_axes_keep_one_group(monkeypatch):
    """Axes of 8192 points and up plan as four-step pairs that own a
    workspace; each image group has its own plans, so those chains split
    too."""
    rng = np.random.default_rng(40)
    x = _crand(rng, (8, 64, 16384))
    buf = vd.asbuffer(x)
    monkeypatch.setenv("VDX_CONV2D_STREAMS", "2")
    vd.fft.fft2(buf)
    torch.cuda.synchronize()
    assert rel_l2(buf.read(0), np.fft.fft2(x.astype(np.complex128))) <= 2 * tol_fp32(64, 16384)


def test_two_host_threads(monkeypatch):
    """Each host thread forks its own side streams and events: concurrent
    calls from two threads on their own torch streams keep their results."""
    import threading

    monkeypatch.setenv("VDX_CONV2D_STREAMS", "2")
    cases = [_inputs(16, 50 + i) for i in range(2)]
    for _, _, buf, kb in cases:  # plans created before the threads start
        vd.fft.convolve2DR(buf, kb)
    torch.cuda.synchronize()
    for x, _, buf, _ in cases:
        buf.write_real(x)
    errors = []

    def work(i):
        try:
            x, K, buf, kb = cases[i]
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(3):
                    buf.write_real(x)
                    vd.fft.convolve2DR(buf, kb)
            s.synchronize()
        except Exception as e:  # reported by the main thread
            errors.append(e)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors
    torch.cuda.synchronize()
    for x, K, buf, _ in cases:
        assert rel_l2(buf.read_real(0), _ref(x, K)) <= TOL
