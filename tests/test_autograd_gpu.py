"""GPU tests of the hand-written adjoints (vkdispatch_gb300.autograd): against
torch.fft autograd on complex128 (FP64 reference), and against FP64 central
finite differences (eps = 1e-4) of the loss at random coordinates."""

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
ag = pytest.importorskip("vkdispatch_gb300.autograd")


def crand(shape, seed, scale=1.0):
    g = torch.Generator().manual_seed(seed)
    re = torch.randn(shape, generator=g, dtype=torch.float64)
    im = torch.randn(shape, generator=g, dtype=torch.float64)
    return (scale * (re + 1j * im)).to(torch.complex128)


@pytest.mark.parametrize("n,dim", [(64, -1), (100, -1), (48, 0), (1024, -1), (243, 1)])
def test_fft_ifft_grad_vs_torch(n, dim):
    shape = (3, n) if dim in (-1, 1) else (n, 5)
    x64 = crand(shape, n)
    x = x64.to(torch.complex64).cuda().requires_grad_(True)
    up = crand(shape, n + 1).to(torch.complex64).cuda()
    for fwd, ref in ((ag.fft, torch.fft.fft), (ag.ifft, torch.fft.ifft)):
        x.grad = None
        y = fwd(x, dim=dim)
        (y * up.conj()).real.sum().backward()
        xr = x64.cuda().requires_grad_(True)
        yr = ref(xr, dim=dim)
        (yr * up.to(torch.complex128).conj()).real.sum().backward()
        assert rel_l2(y.detach().cpu().numpy(), yr.detach().cpu().numpy()) < 1e-5
        assert rel_l2(x.grad.cpu().numpy(), xr.grad.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("n", [64, 100, 45, 512])
def test_rfft_irfft_grad_vs_torch(n):
    g = torch.Generator().manual_seed(n)
    x64 = torch.randn((4, n), generator=g, dtype=torch.float64)
    x = x64.float().cuda().requires_grad_(True)
    h = n // 2 + 1
    up = crand((4, h), n + 3).to(torch.complex64).cuda()
    y = ag.rfft(x)
    (y * up.conj()).real.sum().backward()
    xr = x64.cuda().requires_grad_(True)
    yr = torch.fft.rfft(xr)
    (yr * up.to(torch.complex128).conj()).real.sum().backward()
    assert rel_l2(y.detach().cpu().numpy(), yr.detach().cpu().numpy()) < 1e-5
    assert rel_l2(x.grad.cpu().numpy(), xr.grad.cpu().numpy()) < 1e-5
    # irfft of a Hermitian-consistent spectrum
    spec64 = torch.fft.rfft(torch.randn((3, n), generator=g, dtype=torch.float64))
    hs = spec64.to(torch.complex64).cuda().requires_grad_(True)
    upr = torch.randn((3, n), generator=g, dtype=torch.float64)
    z = ag.irfft(hs, n)
    (z * upr.float().cuda()).sum().backward()
    hr = spec64.cuda().requires_grad_(True)
    zr = torch.fft.irfft(hr, n)
    (zr * upr.cuda()).sum().backward()
    assert rel_l2(z.detach().cpu().numpy(), zr.detach().cpu().numpy()) < 1e-5
    assert rel_l2(hs.grad.cpu().numpy(), hr.grad.cpu().numpy()) < 1e-5


def _torch_loss(x, khat, w):
    dims = tuple(range(x.dim()))
    y = torch.fft.ifftn(torch.fft.fftn(x, dim=dims) * khat.conj(), dim=dims)
    return (w * (y.real ** 2 + y.imag ** 2)).sum(), y


@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 24, 40), (64, 64, 64), (8, 128)])
def test_fft_convolve_and_fused_loss_vs_torch_fp64(shape):
    x64 = crand(shape, 2)
    k64 = crand(shape, 3, 0.1)
    g = torch.Generator().manual_seed(4)
    w64 = torch.rand(shape, generator=g, dtype=torch.float64)
    # FP64 reference with torch autograd
    xr, kr = x64.cuda().requires_grad_(True), k64.cuda().requires_grad_(True)
    lr, yr = _torch_loss(xr, kr, w64.cuda())
    lr.backward()
    x = x64.to(torch.complex64).cuda()
    k = k64.to(torch.complex64).cuda()
    w = w64.float().cuda()
    for fn in (ag.conv_weighted_sqnorm, ag.conv_weighted_sqnorm_plain):
        xa, ka = x.clone().requires_grad_(True), k.clone().requires_grad_(True)
        loss = fn(xa, ka, w)
        loss.backward()
        assert abs(loss.item() - lr.item()) / abs(lr.item()) < 1e-5, fn.__name__
        assert rel_l2(xa.grad.cpu().numpy(), xr.grad.cpu().numpy()) < 1e-5, fn.__name__
        assert rel_l2(ka.grad.cpu().numpy(), kr.grad.cpu().numpy()) < 1e-5, fn.__name__
    # the convolution alone, with an upstream gradient
    xa, ka = x.clone().requires_grad_(True), k.clone().requires_grad_(True)
    y = ag.fft_convolve(xa, ka)
    assert rel_l2(y.detach().cpu().numpy(), yr.detach().cpu().numpy()) < 1e-5
    (w * (y.real ** 2 + y.imag ** 2)).sum().backward()
    assert rel_l2(xa.grad.cpu().numpy(), xr.grad.cpu().numpy()) < 1e-5
    assert rel_l2(ka.grad.cpu().numpy(), kr.grad.cpu().numpy()) < 1e-5


def test_fused_loss_finite_differences_fp64():
    """Central differences of the FP64 loss (numpy) at 64 random coordinates
    against the fp32 hand-written gradient."""
    shape = (12, 10, 16)
    x64 = crand(shape, 7).numpy()
    k64 = crand(shape, 8, 0.1).numpy()
    rng = np.random.default_rng(9)
    w64 = rng.uniform(0, 1, shape)

    def loss(xx, kk):
        y = np.fft.ifftn(np.fft.fftn(xx) * np.conj(kk))
        return float((w64 * np.abs(y) ** 2).sum())

    x = torch.from_numpy(x64).to(torch.complex64).cuda().requires_grad_(True)
    k = torch.from_numpy(k64).to(torch.complex64).cuda().requires_grad_(True)
    ag.conv_weighted_sqnorm(x, k, torch.from_numpy(w64).float().cuda()).backward()
    gx, gk = x.grad.cpu().numpy(), k.grad.cpu().numpy()
    eps = 1e-4
    flat = rng.choice(x64.size, 64, replace=False)
    for which, base, grad in (("x", x64, gx), ("k", k64, gk)):
        for f in flat:
            idx = np.unravel_index(f, shape)
            fd = []
            for d in (1.0, 1j):
                p, m = base.copy(), base.copy()
                p[idx] += eps * d
                m[idx] -= eps * d
                lp = loss(p, k64) if which == "x" else loss(x64, p)
                lm = loss(m, k64) if which == "x" else loss(x64, m)
                fd.append((lp - lm) / (2 * eps))
            fd = fd[0] + 1j * fd[1]  # PyTorch convention: dL/dRe + i dL/dIm
            assert abs(grad[idx] - fd) <= 1e-4 * max(1.0, abs(fd)), (which, idx, grad[idx], fd)


@pytest.mark.parametrize("shape", [(6, 512), (4, 1024), (512, 6)])
def test_fused_loss_on_two_pass_plans(monkeypatch, shape):
    """The fused loss and its adjoints (spectrum-saving and kernel-gradient
    convolution variants, weighted-|y|^2 partials) on the two-pass radix-32
    compile-time plans of 512 and 1024 points."""
    from vkdispatch_gb300.fft import plan as P

    monkeypatch.setenv("VDX_POINTS_PER_THREAD", "32")
    P.cache_clear()
    x64 = crand(shape, 5)
    k64 = crand(shape, 6, 0.1)
    g = torch.Generator().manual_seed(7)
    w64 = torch.rand(shape, generator=g, dtype=torch.float64)
    xr, kr = x64.cuda().requires_grad_(True), k64.cuda().requires_grad_(True)
    lr, _ = _torch_loss(xr, kr, w64.cuda())
    lr.backward()
    xa = x64.to(torch.complex64).cuda().requires_grad_(True)
    ka = k64.to(torch.complex64).cuda().requires_grad_(True)
    loss = ag.conv_weighted_sqnorm(xa, ka, w64.float().cuda())
    loss.backward()
    assert abs(loss.item() - lr.item()) / abs(lr.item()) < 1e-5
    assert rel_l2(xa.grad.cpu().numpy(), xr.grad.cpu().numpy()) < 1e-5
    assert rel_l2(ka.grad.cpu().numpy(), kr.grad.cpu().numpy()) < 1e-5
    P.cache_clear()


def test_lazy_conjugate_and_negative_views():
    """conj() and neg() views (PyTorch's lazy bits, raw memory unchanged) are
    resolved before the kernels read memory, in the forward and the backward."""
    x = crand((8, 64), 21).to(torch.complex64).cuda()
    got = ag.fft(x.conj())
    assert rel_l2(got.cpu().numpy(), torch.fft.fft(x.conj()).cpu().numpy()) < 1e-6
    got = ag.fft(torch.neg(x.conj()))
    assert rel_l2(got.cpu().numpy(), torch.fft.fft(-x.conj()).cpu().numpy()) < 1e-6
    xa = x.clone().requires_grad_(True)
    xr = x.clone().requires_grad_(True)
    (ag.ifft(xa).conj().real.sum() + ag.fft(xa).conj().imag.sum()).backward()
    (torch.fft.ifft(xr).conj().real.sum() + torch.fft.fft(xr).conj().imag.sum()).backward()
    assert rel_l2(xa.grad.cpu().numpy(), xr.grad.cpu().numpy()) < 1e-6
