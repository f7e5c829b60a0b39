"""A torch.fft-compatible front end on libvdx kernels.

`fft, ifft, rfft, irfft, fft2, ifft2, rfft2, irfft2, fftn, ifftn, rfftn,
irfftn, hfft, ihfft` take and return torch tensors with torch.fft's argument meanings:
`n` / `s` zero-pad or trim the transformed dimensions, `dim` picks them and
`norm` is "backward" (default: forward unscaled, inverse 1/n), "forward"
(forward 1/n, inverse unscaled) or "ortho" (1/sqrt(n) both ways).  Results
are new tensors; gradients flow through the hand-written adjoints of
`vkdispatch_gb300.autograd`.  Inputs may have any strides (they are made
contiguous first) but must live on the GPU: there is no CPU path.  Real
inputs of the complex transforms are promoted to complex64 (float32 and
narrower) or complex128 (float64).  Lengths with prime factors above 13 run
as Bluestein transforms (up to 2^23 points in complex64, 4096 in
complex128); their real transforms go through the complex ones.  `hfft` /
`ihfft` are the Hermitian pair (irfft / rfft of the conjugate with the
opposite normalisation), `fftshift` / `ifftshift` roll the dimensions, and
`fftfreq` / `rfftfreq` are torch's own generators.

The reference's own interop is the contiguous CAI buffer
(vkdispatch/base/buffer.py:353-362); this module is the torch-side entry to
the same kernels.
"""

from __future__ import annotations

import math
from typing import Optional, Sequence, Tuple

import torch

from . import autograd as ag

_NORMS = ("backward", "forward", "ortho")


def _norm_code(norm: Optional[str], inverse: bool) -> int:
    """libvdx normalize code of one direction: 0 = none, 1 = 1/n, 2 = 1/sqrt(n)."""
    norm = "backward" if norm is None else norm
    if norm not in _NORMS:
        raise ValueError(f'norm must be one of "backward", "forward", "ortho" (got {norm!r})')
    if norm == "ortho":
        return 2
    return 1 if (norm == "backward") == inverse else 0


def _scale(code: int, n: int) -> float:
    return (1.0, 1.0 / n, 1.0 / math.sqrt(n))[code]


def _cuda(x: torch.Tensor) -> torch.Tensor:
    if not isinstance(x, torch.Tensor) or not x.is_cuda:
        raise ValueError("input must be a CUDA tensor (there is no CPU path)")
    return x


def _complex(x: torch.Tensor) -> torch.Tensor:
    if x.dtype in (torch.complex64, torch.complex128):
        return x
    if x.dtype == torch.complex32:
        return x.to(torch.complex64)
    if x.dtype == torch.float64:
        return x.to(torch.complex128)
    if x.is_floating_point():
        return x.to(torch.float32).to(torch.complex64)
    raise ValueError(f"unsupported input dtype {x.dtype}")


def _real(x: torch.Tensor) -> torch.Tensor:
    if x.dtype == torch.float64:
        return x
    if x.is_floating_point():
        return x.to(torch.float32)
    raise ValueError(f"real transforms need a real floating-point input (got {x.dtype})")


def _resize(x: torch.Tensor, dim: int, n: Optional[int]) -> torch.Tensor:
    """Zero-pads or trims dimension `dim` to n (torch.fft's n / s)."""
    if n is None or n == x.shape[dim]:
        return x
    if n < 1:
        raise ValueError(f"invalid number of data points ({n}) specified")
    if n < x.shape[dim]:
        return x.narrow(dim, 0, n)
    pad = [0, 0] * (x.dim() - 1 - dim) + [0, n - x.shape[dim]]
    return torch.nn.functional.pad(x, pad)


def _dims(x: torch.Tensor, s: Optional[Sequence[int]], dim) -> Tuple[Tuple[int, ...], Tuple[Optional[int], ...]]:
    if dim is None:
        dims = tuple(range(x.dim())) if s is None else tuple(range(x.dim() - len(s), x.dim()))
    elif isinstance(dim, int):
        dims = (dim,)
    else:
        dims = tuple(dim)
    dims = tuple(d % x.dim() for d in dims)
    if len(set(dims)) != len(dims):
        raise ValueError("dims must be unique")
    if s is not None and len(s) != len(dims):
        raise ValueError("s and dim must have the same length")
    sizes = tuple(s) if s is not None else (None,) * len(dims)
    return dims, sizes


def _c2c(x: torch.Tensor, dim: int, inverse: bool, code: int) -> torch.Tensor:
    return ag.FFTFunction.apply(x, dim, inverse, code)


# ---------------------------------------------------------------------------
# one dimension
# ---------------------------------------------------------------------------
def fft(input: torch.Tensor, n: Optional[int] = None, dim: int = -1, norm: Optional[str] = None) -> torch.Tensor:
    x = _complex(_cuda(input))
    d = dim % x.dim()
    return _c2c(_resize(x, d, n), d, False, _norm_code(norm, False))


def ifft(input: torch.Tensor, n: Optional[int] = None, dim: int = -1, norm: Optional[str] = None) -> torch.Tensor:
    x = _complex(_cuda(input))
    d = dim % x.dim()
    return _c2c(_resize(x, d, n), d, True, _norm_code(norm, True))


def rfft(input: torch.Tensor, n: Optional[int] = None, dim: int = -1, norm: Optional[str] = None) -> torch.Tensor:
    x = _real(_cuda(input))
    d = dim % x.dim()
    x = _resize(x, d, n)
    code = _norm_code(norm, False)
    n = x.shape[d]
    if not ag.smooth13(n if n % 2 else n // 2):
        # no radix kernel for this length: the complex transform, cropped
        return _c2c(_complex(x), d, False, code).narrow(d, 0, n // 2 + 1)
    last = d == x.dim() - 1
    y = ag.rfft((x if last else x.movedim(d, -1)).contiguous())
    if code:
        y = y * _scale(code, n)
    return y if last else y.movedim(-1, d)


def irfft(input: torch.Tensor, n: Optional[int] = None, dim: int = -1, norm: Optional[str] = None) -> torch.Tensor:
    h = _complex(_cuda(input))
    d = dim % h.dim()
    nout = 2 * (h.shape[d] - 1) if n is None else int(n)
    if nout < 1:
        raise ValueError(f"invalid number of data points ({nout}) specified")
    h = _resize(h, d, nout // 2 + 1)
    code = _norm_code(norm, True)
    if not ag.smooth13(nout if nout % 2 else nout // 2):
        # no radix kernel for this length: Hermitian extension, complex
        # inverse, real part (the imaginary parts of bins 0 and n/2 drop out)
        tail = h.narrow(d, 1, (nout - 1) // 2).flip(d).conj()
        return _c2c(torch.cat([h, tail], dim=d), d, True, code).real
    last = d == h.dim() - 1
    y = ag.irfft((h if last else h.movedim(d, -1)).contiguous(), nout)  # 1/n scaled
    if code != 1:
        y = y * (_scale(code, nout) * nout)
    return y if last else y.movedim(-1, d)


# ---------------------------------------------------------------------------
# several dimensions
# ---------------------------------------------------------------------------
def fftn(input: torch.Tensor, s: Optional[Sequence[int]] = None, dim=None, norm: Optional[str] = None):
    x = _complex(_cuda(input))
    dims, sizes = _dims(x, s, dim)
    code = _norm_code(norm, False)
    for d, n in zip(dims, sizes):
        x = _c2c(_resize(x, d, n), d, False, code)
    return x


def ifftn(input: torch.Tensor, s: Optional[Sequence[int]] = None, dim=None, norm: Optional[str] = None):
    x = _complex(_cuda(input))
    dims, sizes = _dims(x, s, dim)
    code = _norm_code(norm, True)
    for d, n in zip(dims, sizes):
        x = _c2c(_resize(x, d, n), d, True, code)
    return x


def rfftn(input: torch.Tensor, s: Optional[Sequence[int]] = None, dim=None, norm: Optional[str] = None):
    x = _real(_cuda(input))
    dims, sizes = _dims(x, s, dim)
    y = rfft(x, sizes[-1], dims[-1], norm)
    code = _norm_code(norm, False)
    for d, n in zip(dims[:-1], sizes[:-1]):
        y = _c2c(_resize(y, d, n), d, False, code)
    return y


def irfftn(input: torch.Tensor, s: Optional[Sequence[int]] = None, dim=None, norm: Optional[str] = None):
    h = _complex(_cuda(input))
    dims, sizes = _dims(h, s, dim)
    code = _norm_code(norm, True)
    for d, n in zip(dims[:-1], sizes[:-1]):
        h = _c2c(_resize(h, d, n), d, True, code)
    return irfft(h, sizes[-1], dims[-1], norm)


def fft2(input, s=None, dim=(-2, -1), norm=None):
    return fftn(input, s, dim, norm)


def ifft2(input, s=None, dim=(-2, -1), norm=None):
    return ifftn(input, s, dim, norm)


def rfft2(input, s=None, dim=(-2, -1), norm=None):
    return rfftn(input, s, dim, norm)


def irfft2(input, s=None, dim=(-2, -1), norm=None):
    return irfftn(input, s, dim, norm)


# ---------------------------------------------------------------------------
# Hermitian transforms, shifts and sample frequencies
# ---------------------------------------------------------------------------
_SWAP = {None: "forward", "backward": "forward", "forward": "backward", "ortho": "ortho"}


def _swap(norm: Optional[str]) -> str:
    if norm not in _SWAP:
        raise ValueError(f'norm must be one of "backward", "forward", "ortho" (got {norm!r})')
    return _SWAP[norm]


def hfft(input: torch.Tensor, n: Optional[int] = None, dim: int = -1, norm: Optional[str] = None) -> torch.Tensor:
    """The one-sided half of a Hermitian signal to its real spectrum:
    irfft of the conjugate with the opposite normalisation (torch.fft.hfft)."""
    return irfft(_complex(_cuda(input)).conj(), n=n, dim=dim, norm=_swap(norm))


def ihfft(input: torch.Tensor, n: Optional[int] = None, dim: int = -1, norm: Optional[str] = None) -> torch.Tensor:
    """A real signal to the one-sided half of its Hermitian inverse
    spectrum: the conjugate of rfft with the opposite normalisation
    (torch.fft.ihfft)."""
    return rfft(input, n=n, dim=dim, norm=_swap(norm)).conj()


def _shift_dims(x: torch.Tensor, dim):
    if dim is None:
        return tuple(range(x.dim()))
    return (dim,) if isinstance(dim, int) else tuple(dim)


def fftshift(input: torch.Tensor, dim=None) -> torch.Tensor:
    """Moves the zero-frequency bin to the centre (torch.fft.fftshift)."""
    dims = _shift_dims(input, dim)
    return torch.roll(input, shifts=[input.shape[d] // 2 for d in dims], dims=dims)


def ifftshift(input: torch.Tensor, dim=None) -> torch.Tensor:
    """The inverse of fftshift (torch.fft.ifftshift)."""
    dims = _shift_dims(input, dim)
    return torch.roll(input, shifts=[-(input.shape[d] // 2) for d in dims], dims=dims)


fftfreq = torch.fft.fftfreq  # sample frequencies: tensor generators, no transform
rfftfreq = torch.fft.rfftfreq

__all__ = ["fft", "ifft", "rfft", "irfft", "fft2", "ifft2", "rfft2", "irfft2", "fftn", "ifftn", "rfftn", "irfftn",
           "hfft", "ihfft", "fftshift", "ifftshift", "fftfreq", "rfftfreq"]
