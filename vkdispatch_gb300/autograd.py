"""Differentiable FFTs and FFT convolutions: torch.autograd.Function wrappers
whose backward passes are the hand-derived adjoints, run on libvdx kernels.

Conventions (PyTorch's, for real losses of complex tensors): the gradient of
a linear map y = A x is A^H g.
  * C2C transform with output scale c (1 or 1/N): adjoint = the transform in
    the opposite direction with the same scale.
  * rfft (bins 0..N/2 of the unscaled forward transform of a real row):
    grad_x[n] = Re sum_{k<=N/2} g_k W^{-nk}, i.e. the unscaled C2R of g with
    the interior bins halved (C2R doubles them, DC and Nyquist appear once).
  * irfft (1/N-scaled C2R of a half spectrum): grad_h = rfft(g) / N with the
    interior bins doubled and DC / Nyquist kept once.
  * FFT convolution y = IFFTn(FFTn(x) * conj(K)) (the reference's convention,
    vkdispatch/fft/shader_factories.py:136-145):
        grad_x = IFFTn(FFTn(g) * K),  grad_K = FFTn(x) * conj(FFTn(g)) / N.
The convolution's forward keeps the spectrum FFTn(x) (written by the fused
convolution kernel as it passes through) for the kernel gradient, and the
backward's fused convolution kernel writes grad_K while it multiplies by K.
`conv_weighted_sqnorm` additionally fuses the loss sum(w |y|^2) into the last
inverse pass and the loss gradient 2 w y into the first backward pass.
"""

from __future__ import annotations

from typing import Optional, Sequence

import torch

from . import _lib as L
from . import graph as G
from .fft import plan as P

_IO = {torch.complex64: (L.VDX_C64, L.VDX_C64), torch.complex128: (L.VDX_C128, L.VDX_C128)}


def _stream() -> int:
    return G.current_stream_handle()


def _raw(t: torch.Tensor) -> torch.Tensor:
    """t with PyTorch's lazy conjugate / negative views applied and C-contiguous:
    the kernels read raw memory, which a conj() or neg() view does not change."""
    return t.resolve_conj().resolve_neg().contiguous()


def _check_tensor(t: torch.Tensor, name: str) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (there is no CPU path)")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be C-contiguous")


def smooth13(n: int) -> bool:
    """True when n has no prime factor above 13 (the radix kernels' lengths)."""
    for p in (2, 3, 5, 7, 11, 13):
        while n % p == 0:
            n //= p
    return n == 1


def _c2c_plan(shape, axis, inverse, scale_1n, dtype):
    # lengths with larger prime factors run as Bluestein transforms; the flag
    # is explicit so that the backward pass (on autograd's own thread) plans
    # the same way as the forward
    io, comp = _IO[dtype]
    flags = None if smooth13(int(shape[axis])) else L.VDX_FFT_FLAG_BLUESTEIN
    return P.get_plan(tuple(shape), axis, L.VDX_KIND_C2C, inverse, scale_1n, io, comp, flags=flags)


def _conv_plan(shape, axis, kop, dtype):
    io, comp = _IO[dtype]
    return P.get_plan(tuple(shape), axis, L.VDX_KIND_CONV, False, True, io, comp, None, kop, io, False)


def _ops(**kw) -> L.ExecOps:
    o = L.ExecOps()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


# ---------------------------------------------------------------------------
# C2C transforms
# ---------------------------------------------------------------------------
def _c2c(x: torch.Tensor, dim: int, inverse: bool, scale_1n: bool) -> torch.Tensor:
    x = _raw(x)
    _check_tensor(x, "input")
    if x.dtype not in _IO:
        raise ValueError("complex64 or complex128 input required")
    dim = dim % x.dim()
    y = torch.empty_like(x)
    _c2c_plan(x.shape, dim, inverse, scale_1n, x.dtype).exec(x.data_ptr(), y.data_ptr(), None, _stream())
    return y


class FFTFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, dim: int, inverse: bool, scale_1n: bool):
        ctx.cfg = (dim, inverse, scale_1n)
        return _c2c(_raw(x), dim, inverse, scale_1n)

    @staticmethod
    def backward(ctx, g):
        dim, inverse, scale_1n = ctx.cfg
        return _c2c(_raw(g), dim, not inverse, scale_1n), None, None, None


def fft(x: torch.Tensor, dim: int = -1) -> torch.Tensor:
    """Unscaled forward transform along `dim` (torch.fft.fft semantics)."""
    return FFTFunction.apply(x, dim, False, False)


def ifft(x: torch.Tensor, dim: int = -1) -> torch.Tensor:
    """1/N-scaled inverse transform along `dim` (torch.fft.ifft semantics)."""
    return FFTFunction.apply(x, dim, True, True)


# ---------------------------------------------------------------------------
# real transforms of the last dimension
# ---------------------------------------------------------------------------
def _packed(shape_real, dtype):
    n = shape_real[-1]
    return torch.empty(tuple(shape_real[:-1]) + (n // 2 + 1,), dtype=dtype, device="cuda")


def _rfft_raw(x: torch.Tensor) -> torch.Tensor:
    n = x.shape[-1]
    cdt = torch.complex64 if x.dtype == torch.float32 else torch.complex128
    buf = _packed(x.shape, cdt)
    torch.view_as_real(buf).reshape(buf.shape[:-1] + (2 * buf.shape[-1],))[..., :n].copy_(x)
    io, comp = _IO[cdt]
    P.get_plan(tuple(x.shape), x.dim() - 1, L.VDX_KIND_R2C, False, False, io, comp).exec(
        buf.data_ptr(), buf.data_ptr(), None, _stream())
    return buf


def _irfft_raw(h: torch.Tensor, n: int, scale_1n: bool) -> torch.Tensor:
    buf = _raw(h).clone()
    io, comp = _IO[h.dtype]
    shape = tuple(h.shape[:-1]) + (n,)
    P.get_plan(shape, len(shape) - 1, L.VDX_KIND_C2R, True, scale_1n, io, comp).exec(
        buf.data_ptr(), buf.data_ptr(), None, _stream())
    return torch.view_as_real(buf).reshape(buf.shape[:-1] + (2 * buf.shape[-1],))[..., :n].contiguous()


def _interior(n: int) -> slice:
    # bins that appear twice in the Hermitian extension: 1 .. ceil(N/2)-1
    return slice(1, (n + 1) // 2)


class RFFTFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        x = _raw(x)
        _check_tensor(x, "input")
        ctx.n = x.shape[-1]
        return _rfft_raw(x)

    @staticmethod
    def backward(ctx, g):
        n = ctx.n
        h = _raw(g).clone()
        h[..., _interior(n)] *= 0.5
        return _irfft_raw(h, n, scale_1n=False)


class IRFFTFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, h, n: int):
        h = _raw(h)
        _check_tensor(h, "input")
        ctx.n = n
        return _irfft_raw(h, n, scale_1n=True)

    @staticmethod
    def backward(ctx, g):
        n = ctx.n
        gh = _rfft_raw(_raw(g))
        gh[..., _interior(n)] *= 2.0
        return gh / n, None


def rfft(x: torch.Tensor) -> torch.Tensor:
    """Half spectrum (bins 0..N/2) of real rows: torch.fft.rfft(x, dim=-1)."""
    return RFFTFunction.apply(x)


def irfft(h: torch.Tensor, n: Optional[int] = None) -> torch.Tensor:
    """1/N-scaled real inverse of a half spectrum: torch.fft.irfft(h, n, dim=-1)."""
    if n is None:
        n = 2 * (h.shape[-1] - 1)
    return IRFFTFunction.apply(h, n)


# ---------------------------------------------------------------------------
# FFT convolution over every dimension of x
# ---------------------------------------------------------------------------
def _conv_forward(x, khat, loss_w=None):
    """y = IFFTn(FFTn(x) * conj(K)); returns (y, X, loss_partials or None)."""
    shape, d, dt = tuple(x.shape), x.dim(), x.dtype
    y = torch.empty_like(x)
    spec = torch.empty_like(x)
    s = _stream()
    src = x
    for ax in range(d - 1):
        _c2c_plan(shape, ax, False, False, dt).exec(src.data_ptr(), y.data_ptr(), None, s)
        src = y
    _conv_plan(shape, d - 1, L.VDX_KOP_MUL_CONJ, dt).exec_ops(
        src.data_ptr(), y.data_ptr(), khat.data_ptr(), _ops(spec_out=spec.data_ptr()), s)
    partials = None
    for ax in range(d - 2, -1, -1):
        pl = _c2c_plan(shape, ax, True, True, dt)
        if ax == 0 and loss_w is not None:
            partials = torch.empty(pl.ctas(), dtype=torch.float32, device="cuda")
            pl.exec_ops(y.data_ptr(), y.data_ptr(), None,
                        _ops(loss_weight=loss_w.data_ptr(), loss_partials=partials.data_ptr()), s)
        else:
            pl.exec(y.data_ptr(), y.data_ptr(), None, s)
    return y, spec, partials


def _conv_backward(g, spec, khat, w=None, grad_loss=None):
    """(grad_x, grad_K) for y = IFFTn(FFTn(x) conj K); with w set, g is taken
    as y (the forward output) and the loss gradient 2 w y * grad_loss is
    formed on load."""
    shape, d, dt = tuple(g.shape), g.dim(), g.dtype
    n_total = 1
    for s_ in shape:
        n_total *= s_
    gx = torch.empty_like(g)
    gk = torch.empty_like(khat)
    s = _stream()
    src = g
    for ax in range(d - 1):
        pl = _c2c_plan(shape, ax, False, False, dt)
        if ax == 0 and w is not None:
            pl.exec_ops(src.data_ptr(), gx.data_ptr(), None,
                        _ops(in_weight=w.data_ptr(), in_weight_scale=2.0,
                             in_weight_scale_ptr=grad_loss.data_ptr()), s)
        else:
            pl.exec(src.data_ptr(), gx.data_ptr(), None, s)
        src = gx
    _conv_plan(shape, d - 1, L.VDX_KOP_MUL, dt).exec_ops(
        src.data_ptr(), gx.data_ptr(), khat.data_ptr(),
        _ops(spec_out=gk.data_ptr(), spec_aux=spec.data_ptr(), spec_scale=1.0 / n_total), s)
    for ax in range(d - 2, -1, -1):
        _c2c_plan(shape, ax, True, True, dt).exec(gx.data_ptr(), gx.data_ptr(), None, s)
    return gx, gk


class FFTConvFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, khat):
        x, khat = _raw(x), _raw(khat)
        for t, nm in ((x, "x"), (khat, "khat")):
            _check_tensor(t, nm)
        if x.dtype != torch.complex64 or khat.dtype != torch.complex64 or khat.shape != x.shape:
            raise ValueError("complex64 x and a complex64 kernel spectrum of the same shape are required")
        y, spec, _ = _conv_forward(x, khat)
        ctx.save_for_backward(spec, khat)
        return y

    @staticmethod
    def backward(ctx, g):
        spec, khat = ctx.saved_tensors
        gx, gk = _conv_backward(_raw(g), spec, khat)
        return gx, gk


def fft_convolve(x: torch.Tensor, khat: torch.Tensor) -> torch.Tensor:
    """IFFTn(FFTn(x) * conj(khat)) over every dimension, differentiable in both."""
    return FFTConvFunction.apply(x, khat)


class ConvWeightedSqnormFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, khat, w):
        x, khat, w = _raw(x), _raw(khat), _raw(w)
        for t, nm in ((x, "x"), (khat, "khat"), (w, "w")):
            _check_tensor(t, nm)
        if x.dim() < 2:
            raise ValueError("the fused loss path needs at least 2 dimensions")
        if x.dtype != torch.complex64 or khat.shape != x.shape or w.shape != x.shape or w.dtype != torch.float32:
            raise ValueError("complex64 x, complex64 khat and float32 w of one shape are required")
        y, spec, partials = _conv_forward(x, khat, loss_w=w)
        loss = _sum_f32(partials)
        ctx.save_for_backward(y, spec, khat, w)
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        y, spec, khat, w = ctx.saved_tensors
        gl = grad_loss.to(torch.float32).reshape(1).contiguous()
        gx, gk = _conv_backward(y, spec, khat, w=w, grad_loss=gl)
        return gx, gk, None


def conv_weighted_sqnorm(x: torch.Tensor, khat: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
    """sum(w * |IFFTn(FFTn(x) * conj(khat))|^2), fused, differentiable in x and khat."""
    return ConvWeightedSqnormFunction.apply(x, khat, w)


def _sum_f32(v: torch.Tensor) -> torch.Tensor:
    import ctypes

    n = v.numel()
    parts = ctypes.c_int64()
    L.check(L.lib().vdx_reduce_partial_count(n, ctypes.byref(parts)), "reduce")
    out = torch.empty(1, dtype=torch.float32, device="cuda")
    ws = torch.empty(parts.value, dtype=torch.float32, device="cuda")
    L.check(L.lib().vdx_reduce(L.VDX_RED_ADD, L.VDX_MAP_IDENTITY, L.VDX_F32, v.data_ptr(), n, 1, out.data_ptr(),
                               ws.data_ptr(), _stream()), "reduce")
    return out.reshape(())


# ---------------------------------------------------------------------------
# the unfused composition (per-axis transforms and separate element-wise ops)
# ---------------------------------------------------------------------------
def _fftn(x, inverse, dims: Sequence[int]):
    out = x
    for ax in dims:
        out = _c2c(out, ax, inverse, inverse)
    return out


class PlainConvWeightedSqnormFunction(torch.autograd.Function):
    """The same loss as conv_weighted_sqnorm built from plain per-axis FFT
    launches and separate element-wise kernels: the comparator for the fused
    path."""

    @staticmethod
    def forward(ctx, x, khat, w):
        dims = list(range(x.dim()))
        X = _fftn(x, False, dims)
        y = _fftn(X * khat.conj(), True, dims[::-1])
        loss = (w * (y.real * y.real + y.imag * y.imag)).sum()
        ctx.save_for_backward(X, y, khat, w)
        return loss

    @staticmethod
    def backward(ctx, grad_loss):
        X, y, khat, w = ctx.saved_tensors
        dims = list(range(X.dim()))
        g = (2.0 * grad_loss) * w * y
        G = _fftn(g, False, dims)
        gk = X * G.conj() / X.numel()
        gx = _fftn(G * khat, True, dims[::-1])
        return gx, gk, None


def conv_weighted_sqnorm_plain(x, khat, w):
    return PlainConvWeightedSqnormFunction.apply(x, khat, w)
