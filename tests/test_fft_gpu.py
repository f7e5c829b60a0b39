"""GPU parity tests of the FFT path through the C ABI (vd-compatible API) vs
the FP64 numpy.fft oracle, mirroring the reference's tests/test_fft.py,
test_fft_padded.py and test_fft_mixed_precision.py checks, with seeded
inputs and the relative-L2 bound of tests/helpers.py.
"""

import numpy as np
import pytest

from helpers import crandn, rel_l2, smooth_sizes, tol_fp32

pytestmark = pytest.mark.gpu

vd = pytest.importorskip("vkdispatch_gb300")

SIZES_SMALL = smooth_sizes(limit=128)
SIZES_SAMPLED = [160, 192, 243, 256, 343, 512, 625, 768, 1000, 1024, 1331, 2048, 2197, 3072, 4096, 6561, 8192,
                 10000, 12288, 12500, 16384]


@pytest.mark.parametrize("n", SIZES_SMALL + SIZES_SAMPLED)
def test_c2c_1d_forward_inverse(n):
    rng = np.random.default_rng(n)
    batch = 3 if n > 1024 else 7
    x = crandn(rng, (batch, n))
    buf = vd.asbuffer(x)
    vd.fft.fft(buf)
    y = buf.read(0)
    assert rel_l2(y, np.fft.fft(x.astype(np.complex128), axis=-1)) <= tol_fp32(n)
    vd.fft.ifft(buf)
    z = buf.read(0)
    assert rel_l2(z, x) <= 2 * tol_fp32(n)
    # the reference's own acceptance check (tests/test_fft.py:49)
    assert np.allclose(y, np.fft.fft(x, axis=-1), atol=1e-3 * max(1, np.sqrt(n) / 8))


@pytest.mark.parametrize(
    "shape,axis",
    [((4, 16, 3), 1), ((2, 512, 257), 1), ((5, 81, 17), 1), ((64, 32), 0), ((13, 7, 11), 0), ((3, 1024, 16), 1),
     ((2, 2048, 5), 1), ((6, 10, 26), 1), ((3, 4096, 2), 1)],
)
def test_c2c_strided_axis(shape, axis):
    rng = np.random.default_rng(sum(shape) + axis)
    x = crandn(rng, shape)
    buf = vd.asbuffer(x)
    vd.fft.fft(buf, axis=axis)
    ref = np.fft.fft(x.astype(np.complex128), axis=axis)
    assert rel_l2(buf.read(0), ref) <= tol_fp32(shape[axis])
    vd.fft.ifft(buf, axis=axis)
    assert rel_l2(buf.read(0), x) <= 2 * tol_fp32(shape[axis])


@pytest.mark.parametrize("shape", [(32, 64), (48, 80), (9, 13, 25), (16, 16, 16), (100, 5, 12)])
def test_fft2_fft3(shape):
    rng = np.random.default_rng(len(shape) * 100 + shape[0])
    x = crandn(rng, shape)
    buf = vd.asbuffer(x)
    if len(shape) == 3:
        vd.fft.fft3(buf)
        ref = np.fft.fftn(x.astype(np.complex128))
        tol = tol_fp32(*shape)
    else:
        vd.fft.fft2(buf)
        ref = np.fft.fft2(x.astype(np.complex128))
        tol = tol_fp32(*shape[-2:])
    assert rel_l2(buf.read(0), ref) <= tol
    if len(shape) == 3:
        vd.fft.ifft3(buf)
    else:
        vd.fft.ifft2(buf)
    assert rel_l2(buf.read(0), x) <= 2 * tol


@pytest.mark.parametrize("shape", [(4, 2), (3, 16), (5, 30), (2, 81), (8, 512), (3, 1000), (2, 13), (4, 45),
                                   (2, 4096), (2, 8190), (1, 16384), (64, 512)])
def test_rfft_irfft_1d(shape):
    rng = np.random.default_rng(shape[-1])
    x = rng.uniform(-1, 1, shape).astype(np.float32)
    buf = vd.asrfftbuffer(x)
    vd.fft.rfft(buf)
    ref = np.fft.rfft(x.astype(np.float64), axis=-1)
    assert rel_l2(buf.read_fourier(0), ref) <= tol_fp32(shape[-1])
    vd.fft.irfft(buf)
    assert rel_l2(buf.read_real(0), x) <= 2 * tol_fp32(shape[-1])


def test_irfft_keeps_padding_and_ignores_dc_nyquist_imag():
    rng = np.random.default_rng(5)
    n = 64
    spec = crandn(rng, (3, n // 2 + 1))
    buf = vd.RFFTBuffer((3, n))
    buf.write_fourier(spec)
    vd.fft.irfft(buf)
    herm = spec.astype(np.complex128).copy()
    herm[:, 0] = herm[:, 0].real
    herm[:, -1] = herm[:, -1].real
    ref = np.fft.irfft(herm, n=n, axis=-1)
    assert rel_l2(buf.read_real(0), ref) <= 2 * tol_fp32(n)
    # reals N..N+1 of each row are untouched (the spectrum's last bin)
    raw = buf.read(0)
    assert np.array_equal(raw[:, -1], spec[:, -1])


@pytest.mark.parametrize("shape", [(16, 32), (30, 64), (6, 45, 26), (8, 24, 10), (162, 13)])
def test_rfft2_rfft3_roundtrip(shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.uniform(-1, 1, shape).astype(np.float32)
    buf = vd.asrfftbuffer(x)
    if len(shape) == 3:
        vd.fft.rfft3(buf)
        ref = np.fft.rfftn(x.astype(np.float64))
        tol = tol_fp32(*shape)
    else:
        vd.fft.rfft2(buf)
        ref = np.fft.rfft2(x.astype(np.float64))
        tol = tol_fp32(*shape)
    assert rel_l2(buf.read_fourier(0), ref) <= tol
    if len(shape) == 3:
        vd.fft.irfft3(buf)
    else:
        vd.fft.irfft2(buf)
    assert rel_l2(buf.read_real(0), x) <= 2 * tol


@pytest.mark.parametrize("n,lo,hi", [(64, 3, 40), (100, 0, 17), (243, 200, 243), (1024, 1, 1023)])
def test_signal_range(n, lo, hi):
    rng = np.random.default_rng(n + lo)
    x = crandn(rng, (5, n))
    buf = vd.asbuffer(x)
    vd.fft.fft(buf, input_signal_range=(lo, hi))
    z = x.copy()
    z[:, :lo] = 0
    z[:, hi:] = 0
    assert rel_l2(buf.read(0), np.fft.fft(z.astype(np.complex128), axis=-1)) <= tol_fp32(n)
    # r2c form (tests/test_fft_padded.py:71-96)
    xr = rng.uniform(0, 1, (4, n)).astype(np.float32)
    rb = vd.asrfftbuffer(xr)
    vd.fft.fft(rb, buffer_shape=rb.real_shape, r2c=True, input_signal_range=(lo, hi))
    zr = xr.copy()
    zr[:, :lo] = 0
    zr[:, hi:] = 0
    assert rel_l2(rb.read_fourier(0), np.fft.rfft(zr.astype(np.float64), axis=-1)) <= tol_fp32(n)


def _np_conv(sig, ker, axes):
    s = np.fft.fftn(sig.astype(np.complex128), axes=axes)
    k = np.fft.fftn(ker.astype(np.complex128), axes=axes)
    return np.fft.ifftn(s * np.conj(k), axes=axes)


@pytest.mark.parametrize("shape", [(8, 64), (3, 100), (4, 1024), (2, 13, 11), (5, 243)])
def test_convolve_1d(shape):
    rng = np.random.default_rng(shape[-1] * 3)
    x = crandn(rng, shape)
    k = crandn(rng, shape)
    sig, ker = vd.asbuffer(x), vd.asbuffer(k)
    vd.fft.fft(ker)
    vd.fft.convolve(sig, ker)
    assert rel_l2(sig.read(0), _np_conv(x, k, (-1,))) <= 3 * tol_fp32(shape[-1])


@pytest.mark.parametrize("shape", [(32, 32), (3, 64, 48), (26, 20), (2, 81, 16)])
def test_convolve2d(shape):
    rng = np.random.default_rng(sum(shape) * 7)
    x = crandn(rng, shape)
    k = crandn(rng, shape)
    sig, ker = vd.asbuffer(x), vd.asbuffer(k)
    vd.fft.fft2(ker)
    vd.fft.convolve2D(sig, ker)
    assert rel_l2(sig.read(0), _np_conv(x, k, (-2, -1))) <= 3 * tol_fp32(*shape[-2:])


def test_convolve2d_transposed_kernel():
    rng = np.random.default_rng(11)
    shape = (40, 24)
    x, k = crandn(rng, shape), crandn(rng, shape)
    sig, ker = vd.asbuffer(x), vd.asbuffer(k)
    vd.fft.fft2(ker)
    tsize = vd.fft.get_transposed_size(shape, axis=0)
    tbuf = vd.Buffer((tsize,), vd.complex64)
    vd.fft.transpose(ker, out_buffer=tbuf, axis=0)
    vd.fft.convolve2D(sig, tbuf, transposed_kernel=True)
    assert rel_l2(sig.read(0), _np_conv(x, k, (-2, -1))) <= 3 * tol_fp32(*shape)


@pytest.mark.parametrize("shape", [(2, 64, 64), (32, 32), (162, 13), (3, 30, 26), (4, 512, 512)])
def test_convolve2dr(shape):
    rng = np.random.default_rng(sum(shape) * 5)
    x = rng.uniform(-1, 1, shape).astype(np.float32)
    k = rng.uniform(-1, 1, shape).astype(np.float32)
    sig, ker = vd.asrfftbuffer(x), vd.asrfftbuffer(k)
    vd.fft.rfft2(ker)
    vd.fft.convolve2DR(sig, ker)
    ref = _np_conv(x, k, (-2, -1)).real
    assert rel_l2(sig.read_real(0), ref) <= 3 * tol_fp32(*shape[-2:])
    assert np.allclose(sig.read_real(0), ref, atol=1e-3 * max(1, shape[-1] / 64))


def test_convolve_kernel_inner_only_broadcast():
    rng = np.random.default_rng(21)
    x = crandn(rng, (6, 48, 20))
    k = crandn(rng, (48, 20))
    sig, ker = vd.asbuffer(x), vd.asbuffer(k)
    vd.fft.fft2(ker)
    vd.fft.convolve2D(sig, ker, kernel_inner_only=True)
    ref = _np_conv(x, np.broadcast_to(k, x.shape), (-2, -1))
    assert rel_l2(sig.read(0), ref) <= 3 * tol_fp32(48, 20)


def test_complex32_io_fp32_compute():
    rng = np.random.default_rng(7)
    data = crandn(rng, 64)
    q = (data.real.astype(np.float16).astype(np.float32) + 1j * data.imag.astype(np.float16).astype(np.float32))
    buf = vd.Buffer(data.shape, vd.complex32)
    buf.write(data)
    vd.fft.fft(buf, compute_type=vd.complex64)
    ref = np.fft.fft(q.astype(np.complex128))
    # tests/test_fft_mixed_precision.py:89 bound plus a relative check
    got = buf.read(0)
    assert np.allclose(got, ref, atol=3e-1, rtol=2e-2)
    assert rel_l2(got, ref) < 2e-3


def test_complex128_compute():
    rng = np.random.default_rng(29)
    x = (rng.standard_normal((4, 1536)) + 1j * rng.standard_normal((4, 1536))).astype(np.complex128)
    buf = vd.asbuffer(x)
    vd.fft.fft(buf)
    assert rel_l2(buf.read(0), np.fft.fft(x, axis=-1)) < 1e-14
    vd.fft.ifft(buf)
    assert rel_l2(buf.read(0), x) < 1e-14


def test_bf16_storage_fft():
    rng = np.random.default_rng(4)
    x = crandn(rng, (8, 1024))
    buf = vd.Buffer(x.shape, vd.complexbf16)
    buf.write(x)
    q = buf.read(0).astype(np.complex128)
    vd.fft.fft(buf)
    got = buf.read(0)
    # bf16 storage rounding of the outputs dominates (2^-9 relative)
    assert rel_l2(got, np.fft.fft(q, axis=-1)) < 4e-3


def test_prime_above_13_rejected_on_request():
    """The reference's planner rejects a prime factor above 13; here such
    lengths plan as Bluestein transforms unless vd.fft.bluestein(False)."""
    buf = vd.Buffer((4, 17), vd.complex64)
    with vd.fft.bluestein(False), pytest.raises(ValueError):
        vd.fft.fft(buf)


def test_command_graph_and_cuda_graph_capture():
    import torch

    rng = np.random.default_rng(3)
    x = crandn(rng, (16, 256))
    t = torch.from_numpy(x).cuda()
    buf = vd.from_cuda_array(t)
    g = vd.CommandGraph()
    vd.fft.fft(buf, graph=g)
    vd.fft.ifft(buf, graph=g)
    vd.fft.fft(buf, graph=g)
    assert len(g) == 3
    g.submit()
    torch.cuda.synchronize()
    assert rel_l2(t.cpu().numpy(), np.fft.fft(x.astype(np.complex128), axis=-1)) <= 3 * tol_fp32(256)
    # capture the recorded graph into a torch CUDA graph and replay it
    t.copy_(torch.from_numpy(x))
    cg = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(cg, stream=s):
            with vd.cuda_graph_capture(torch.cuda.current_stream()):
                g.submit()
    torch.cuda.current_stream().wait_stream(s)
    t.copy_(torch.from_numpy(x))
    cg.replay()
    torch.cuda.synchronize()
    assert rel_l2(t.cpu().numpy(), np.fft.fft(x.astype(np.complex128), axis=-1)) <= 3 * tol_fp32(256)


def test_from_cuda_array_checks():
    import torch

    t = torch.zeros((4, 8), dtype=torch.complex64, device="cuda")
    b = vd.from_cuda_array(t)
    assert b.ptr == t.data_ptr() and b.shape == (4, 8)
    with pytest.raises(ValueError):
        vd.from_cuda_array(t.t())  # non-contiguous
    with pytest.raises(ValueError):
        vd.from_cuda_array(t, var_type=vd.complex128)


@pytest.mark.parametrize("pts", [8, 32])
@pytest.mark.parametrize("kop_conj", [True, False])
def test_strided_convolution_points_per_thread(monkeypatch, kop_conj, pts):
    """The alternative compile-time plans of the strided fused convolution
    (radix 8 x 8 x 8 with 64 threads per 512-point column, radix 32 x 16 with
    16) match FP64 numpy, conjugate and plain product."""
    import torch

    from vkdispatch_gb300 import _lib as L
    from vkdispatch_gb300.fft import plan as P

    monkeypatch.setenv("VDX_POINTS_PER_THREAD", str(pts))
    P.cache_clear()
    rng = np.random.default_rng(31 + kop_conj + pts)
    shape = (3, 512, 257)
    x = crandn(rng, shape)
    k = crandn(rng, shape)
    xt, kt = torch.from_numpy(x).cuda(), torch.from_numpy(k).cuda()
    kop = L.VDX_KOP_MUL_CONJ if kop_conj else L.VDX_KOP_MUL
    p = P.get_plan(shape, 1, L.VDX_KIND_CONV, False, True, L.VDX_C64, L.VDX_C64, None, kop, L.VDX_C64)
    d = p.describe()
    assert d["threads_per_transform"] == 512 // pts and d["fixed"] is True
    assert d["radices"] == {8: "8x8x8", 32: "32x16"}[pts]
    p.exec(xt.data_ptr(), xt.data_ptr(), kt.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    s = np.fft.fft(x.astype(np.complex128), axis=1)
    ref = np.fft.ifft(s * (np.conj(k) if kop_conj else k), axis=1)
    assert rel_l2(xt.cpu().numpy(), ref) <= 2 * tol_fp32(512)
    P.cache_clear()


@pytest.mark.parametrize("shape,axis", [((96, 1024), 1), ((1024, 40), 0), ((3, 1024, 5), 1), ((70, 512), 1),
                                        ((512, 33), 0)])
def test_c2c_two_pass_plans(monkeypatch, shape, axis):
    """The two-pass compile-time plans (radix 32 x 32, one warp per
    1024-point transform; radix 32 x 16 for 512 points) match FP64 numpy
    forward and inverse, contiguous and strided."""
    import torch

    from vkdispatch_gb300 import _lib as L
    from vkdispatch_gb300.fft import plan as P

    monkeypatch.setenv("VDX_POINTS_PER_THREAD", "32")
    P.cache_clear()
    rng = np.random.default_rng(sum(shape) + axis)
    x = crandn(rng, shape)
    t = torch.from_numpy(x).cuda()
    s = torch.cuda.current_stream().cuda_stream
    fwd = P.get_plan(shape, axis, L.VDX_KIND_C2C, False, False, L.VDX_C64, L.VDX_C64)
    d = fwd.describe()
    n = shape[axis]
    assert d["threads_per_transform"] == n // 32 and d["fixed"] is True
    assert d["radices"] == {512: "32x16", 1024: "32x32"}[n]
    fwd.exec(t.data_ptr(), t.data_ptr(), None, s)
    torch.cuda.synchronize()
    ref = np.fft.fft(x.astype(np.complex128), axis=axis)
    assert rel_l2(t.cpu().numpy(), ref) <= tol_fp32(n)
    inv = P.get_plan(shape, axis, L.VDX_KIND_C2C, True, True, L.VDX_C64, L.VDX_C64)
    inv.exec(t.data_ptr(), t.data_ptr(), None, s)
    torch.cuda.synchronize()
    assert rel_l2(t.cpu().numpy(), x) <= 2 * tol_fp32(n)
    P.cache_clear()


@pytest.mark.parametrize("N", [1024, 2048])
def test_real_transforms_two_pass_plan(monkeypatch, N):
    """R2C / C2R of 1024 and 2048 real samples (512 / 1024 complex points) on
    the two-pass radix-32 compile-time plans match FP64 numpy."""
    monkeypatch.setenv("VDX_POINTS_PER_THREAD", "32")
    from vkdispatch_gb300.fft import plan as P

    P.cache_clear()
    rng = np.random.default_rng(N)
    r = rng.standard_normal((24, N)).astype(np.float32)
    rb = vd.asrfftbuffer(r)
    vd.fft.rfft(rb)
    spec = np.fft.rfft(r.astype(np.float64), axis=-1)
    assert rel_l2(rb.read_fourier(0), spec) <= tol_fp32(N)
    vd.fft.irfft(rb)
    assert rel_l2(rb.read_real(0), r) <= 2 * tol_fp32(N)
    P.cache_clear()


@pytest.mark.parametrize("n", [512, 1024])
def test_contiguous_convolution_two_pass_plan(monkeypatch, n):
    """The fused convolution along the contiguous axis on the two-pass plans."""
    monkeypatch.setenv("VDX_POINTS_PER_THREAD", "32")
    from vkdispatch_gb300.fft import plan as P

    P.cache_clear()
    rng = np.random.default_rng(n + 5)
    x = crandn(rng, (20, n))
    k = crandn(rng, (20, n))
    b = vd.asbuffer(x)
    vd.fft.convolve(b, vd.asbuffer(k))
    ref = np.fft.ifft(np.fft.fft(x.astype(np.complex128), axis=1) * np.conj(k), axis=1)
    assert rel_l2(b.read(0), ref) <= 2 * tol_fp32(n)
    P.cache_clear()
