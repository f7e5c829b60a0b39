"""The reference's kernel factories as callables (vkdispatch/fft/
shader_factories.py:11-195, called the way vkdispatch/fft/functions.py:
144-162, 526-547 and 699-709 call them): the same results as vd.fft.fft,
convolve and transpose, bit for bit (the same plans run), and printable."""

import numpy as np
import pytest
import torch

import vkdispatch_gb300 as vd

from helpers import crandn

pytestmark = pytest.mark.gpu


def test_fft_shader_matches_fft():
    rng = np.random.default_rng(1)
    x = crandn(rng, (8, 1000))
    a, b = vd.asbuffer(x), vd.asbuffer(x)
    shader = vd.fft.make_fft_shader((8, 1000), 1)
    shader(a)
    vd.fft.fft(b, axis=1)
    torch.cuda.synchronize()
    assert np.array_equal(a.read(0), b.read(0))
    inv = vd.fft.make_fft_shader((8, 1000), 1, inverse=True)
    inv(a)
    torch.cuda.synchronize()
    assert np.allclose(a.read(0), x, atol=1e-5)
    assert "CTA shape" in repr(shader) and "1000" in repr(shader)


def test_fft_shader_deferred_graph():
    rng = np.random.default_rng(2)
    x = crandn(rng, (4, 256))
    a = vd.asbuffer(x)
    g = vd.CommandGraph()
    vd.fft.make_fft_shader((4, 256), 1)(a, graph=g)
    torch.cuda.synchronize()
    assert np.array_equal(a.read(0), x)  # recorded, not run
    g.submit()
    torch.cuda.synchronize()
    assert np.allclose(a.read(0), np.fft.fft(x.astype(np.complex128), axis=1), rtol=1e-4, atol=1e-3)


def test_convolution_and_transpose_shaders():
    rng = np.random.default_rng(3)
    x = crandn(rng, (16, 512))
    k = crandn(rng, (16, 512)) * 0.1
    s1, s2 = vd.asbuffer(x), vd.asbuffer(x)
    kb = vd.asbuffer(k)
    vd.fft.fft(kb)
    for s in (s1, s2):
        vd.fft.fft(s)
    vd.fft.make_convolution_shader((16, 512), axis=1)(s1, kb)
    vd.fft.convolve(s2, kb, axis=1)
    torch.cuda.synchronize()
    assert np.array_equal(s1.read(0), s2.read(0))
    size = vd.fft.get_transposed_size((16, 512), axis=1)
    out = vd.Buffer((size,), vd.complex64)
    vd.fft.make_transpose_shader((16, 512), axis=1)(out, kb)
    torch.cuda.synchronize()
    assert np.array_equal(out.read(0)[: 16 * 512].reshape(16, 512), kb.read(0))


def test_runtime_helpers_on_gpu():
    """get_devices, the typed buffer allocators and the capture state that
    cuda_graph_capture yields (vkdispatch/execution_pipeline/
    cuda_graph_capture.py:9-41)."""
    devs = vd.get_devices()
    assert devs and devs[0].dev_index == 0 and devs[0].sub_group_size == 32
    assert devs[0].device_name in repr(devs[0])
    b = vd.buffer_c64((4, 8))
    assert b.shape == (4, 8) and b.var_type == vd.complex64
    assert vd.buffer_f32((3,)).var_type == vd.float32
    s = torch.cuda.Stream()
    with vd.cuda_graph_capture(s) as cap:
        assert vd.get_cuda_capture() is cap and cap.cuda_stream is s
        with vd.suspend_cuda_capture():
            assert vd.get_cuda_capture() is None
        assert vd.get_cuda_capture() is cap
    assert vd.get_cuda_capture() is None
