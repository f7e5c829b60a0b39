"""The torch.fft-compatible front end (vkdispatch_gb300.torch_fft) against
torch.fft itself (cuFFT) on the same GPU inputs: values for every function,
n / s padding and trimming, the three norm modes and non-contiguous inputs,
and gradients against torch.fft autograd on complex128."""

import numpy as np
import pytest

from helpers import rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
tf = pytest.importorskip("vkdispatch_gb300.torch_fft")


def _c(shape, seed, dtype=torch.complex64):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(shape, dtype=dtype, device="cuda", generator=g)


def _r(shape, seed, dtype=torch.float32):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(shape, dtype=dtype, device="cuda", generator=g)


def _err(a, b):
    return rel_l2(a.detach().cpu().numpy(), b.detach().cpu().numpy())


@pytest.mark.parametrize("norm", [None, "forward", "ortho"])
@pytest.mark.parametrize("n,dim", [(None, -1), (300, -1), (60, 0), (None, 1)])
def test_c2c_one_dim(norm, n, dim):
    x = _c((96, 200), 1)
    for ours, ref in ((tf.fft, torch.fft.fft), (tf.ifft, torch.fft.ifft)):
        got = ours(x, n=n, dim=dim, norm=norm)
        assert got.shape == ref(x, n=n, dim=dim, norm=norm).shape
        assert _err(got, ref(x, n=n, dim=dim, norm=norm)) <= 2 * tol_fp32(got.shape[dim])


@pytest.mark.parametrize("norm", [None, "forward", "ortho"])
@pytest.mark.parametrize("n,dim", [(None, -1), (513, -1), (256, 0), (None, 0)])
def test_real_one_dim(norm, n, dim):
    x = _r((64, 512), 2)
    y = tf.rfft(x, n=n, dim=dim, norm=norm)
    yr = torch.fft.rfft(x, n=n, dim=dim, norm=norm)
    assert y.shape == yr.shape and _err(y, yr) <= 2 * tol_fp32(512)
    z = tf.irfft(yr, n=n, dim=dim, norm=norm)
    zr = torch.fft.irfft(yr, n=n, dim=dim, norm=norm)
    assert z.shape == zr.shape and _err(z, zr) <= 2 * tol_fp32(512)


@pytest.mark.parametrize("n", [97, 38, 1000, 2 * 19 * 23])
def test_lengths_beyond_the_radix_set(n):
    """Lengths with prime factors above 13 (Bluestein), C2C and real."""
    x = _c((5, n), 12)
    assert _err(tf.fft(x), torch.fft.fft(x)) <= 4 * tol_fp32(n)
    assert _err(tf.ifft(x, norm="ortho"), torch.fft.ifft(x, norm="ortho")) <= 4 * tol_fp32(n)
    r = _r((5, n), 13)
    h = torch.fft.rfft(r)
    assert _err(tf.rfft(r), h) <= 4 * tol_fp32(n)
    assert _err(tf.irfft(h, n=n), torch.fft.irfft(h, n=n)) <= 4 * tol_fp32(n)


@pytest.mark.parametrize("norm", [None, "ortho"])
def test_multi_dim(norm):
    x = _c((12, 40, 64), 3)
    assert _err(tf.fft2(x, norm=norm), torch.fft.fft2(x, norm=norm)) <= 3 * tol_fp32(64)
    assert _err(tf.ifftn(x, norm=norm), torch.fft.ifftn(x, norm=norm)) <= 3 * tol_fp32(64)
    assert _err(tf.fftn(x, s=(50, 60), norm=norm), torch.fft.fftn(x, s=(50, 60), norm=norm)) <= 3 * tol_fp32(64)
    r = _r((10, 48, 96), 4)
    assert _err(tf.rfft2(r, norm=norm), torch.fft.rfft2(r, norm=norm)) <= 3 * tol_fp32(96)
    h = torch.fft.rfftn(r, norm=norm)
    assert _err(tf.rfftn(r, norm=norm), h) <= 3 * tol_fp32(96)
    assert _err(tf.irfftn(h, s=r.shape, norm=norm), torch.fft.irfftn(h, s=r.shape, norm=norm)) <= 3 * tol_fp32(96)
    assert _err(tf.irfft2(h[0], norm=norm), torch.fft.irfft2(h[0], norm=norm)) <= 3 * tol_fp32(96)


def test_non_contiguous_and_real_promotion():
    x = _c((64, 128), 5).t()  # a transposed view
    assert not x.is_contiguous()
    assert _err(tf.fft(x, dim=0), torch.fft.fft(x, dim=0)) <= 2 * tol_fp32(128)
    r = _r((32, 100), 6)
    assert tf.fft(r).dtype == torch.complex64
    assert _err(tf.fft(r), torch.fft.fft(r)) <= 2 * tol_fp32(100)
    r64 = _r((8, 64), 7, torch.float64)
    assert tf.rfft(r64).dtype == torch.complex128


@pytest.mark.parametrize("norm", [None, "forward", "ortho"])
def test_gradients_vs_torch_fp64(norm):
    x0 = _c((6, 48), 8, torch.complex128)
    r0 = _r((6, 50), 9, torch.float64)
    w = _r((6, 48), 10, torch.float64).abs()

    def loss(mod, x, r):
        y = mod.fft(x, norm=norm) + mod.ifft(x, n=48, norm=norm).conj()
        h = mod.rfft(r, norm=norm)
        z = mod.irfft(h * 1.5, n=50, norm=norm)
        return (w * (y.real ** 2 + y.imag ** 2)).sum() + (z * r).sum()

    grads = []
    for mod in (tf, torch.fft):
        x = x0.clone().requires_grad_(True)
        r = r0.clone().requires_grad_(True)
        loss(mod, x, r).backward()
        grads.append((x.grad, r.grad))
    assert _err(grads[0][0], grads[1][0]) < 1e-10
    assert _err(grads[0][1], grads[1][1]) < 1e-10


def test_invalid_arguments():
    x = _c((4, 16), 11)
    with pytest.raises(ValueError):
        tf.fft(x, norm="none")
    with pytest.raises(ValueError):
        tf.fftn(x, s=(4,), dim=(0, 1))
    with pytest.raises(ValueError):
        tf.fft(x.cpu())


@pytest.mark.parametrize("norm", [None, "forward", "ortho"])
@pytest.mark.parametrize("n", [None, 30, 64])
def test_hermitian_pair_and_shifts(norm, n):
    """hfft / ihfft against torch.fft (values, and the hfft gradient in
    FP64), fftshift / ifftshift and the frequency generators."""
    g = torch.Generator(device="cuda").manual_seed(9)
    h = torch.randn(4, 33, dtype=torch.complex64, device="cuda", generator=g)
    got = tf.hfft(h, n=n, norm=norm)
    ref = torch.fft.hfft(h, n=n, norm=norm)
    assert got.shape == ref.shape
    assert torch.linalg.norm(got - ref) <= 1e-5 * torch.linalg.norm(ref)
    x = torch.randn(3, 48, dtype=torch.float32, device="cuda", generator=g)
    got = tf.ihfft(x, n=n, norm=norm)
    ref = torch.fft.ihfft(x, n=n, norm=norm)
    assert got.shape == ref.shape
    assert torch.linalg.norm(got - ref) <= 1e-5 * torch.linalg.norm(ref)
    h64 = torch.randn(2, 17, dtype=torch.complex128, device="cuda", generator=g, requires_grad=True)
    (tf.hfft(h64, n=n, norm=norm) ** 2).sum().backward()
    ga = h64.grad.clone()
    h64.grad = None
    (torch.fft.hfft(h64, n=n, norm=norm) ** 2).sum().backward()
    assert torch.allclose(ga, h64.grad, rtol=1e-9, atol=1e-9)
    y = torch.randn(5, 6, 7, device="cuda", generator=g)
    assert torch.equal(tf.fftshift(y), torch.fft.fftshift(y))
    assert torch.equal(tf.ifftshift(y, dim=(0, 2)), torch.fft.ifftshift(y, dim=(0, 2)))
    assert torch.equal(tf.fftshift(y, dim=1), torch.fft.fftshift(y, dim=1))
    assert torch.equal(tf.fftfreq(10, 0.5), torch.fft.fftfreq(10, 0.5))
