"""Tensor-core DFT stages (csrc/fft_tc.cu, VDX_FFT_FLAG_TENSOR_CORE) against
FP64 numpy.fft and against the fp32-butterfly four-step path.

Tolerance.  Each 128-point short transform is two BF16 GEMM stages with the
three-product split: an operand's hi + lo pair carries 16 significant bits,
so a product's neglected terms are ~2^-17 of its size, about 8e-6, and the
rounding of the FP32 accumulators and twiddles adds the usual fp32 terms.
One 16384-point axis is four such stages plus two fp32 twiddle
multiplications; the neglected lo*lo terms and the accumulator rounding are
independent between elements, so they add in quadrature.  The tests hold
complex64 storage to the benchmark spec's 1e-5 relative L2 per 16384-point axis
(the bench measures 7.9e-6 for the full 16384 x 16384 FFT2, both axes on the
tensor cores).  For bf16 / fp16 storage the rounding of the stored workspace
and outputs dominates, exactly as on the fp32-butterfly path.
"""

import numpy as np
import pytest
import torch

import vkdispatch_gb300 as vd
from vkdispatch_gb300 import _lib as L
from vkdispatch_gb300.fft import plan as P

from helpers import crandn, rel_l2

pytestmark = pytest.mark.gpu

TC_AXIS_TOL = 1e-5  # complex64 storage, one 16384-point axis


def _desc(shape, axis, inverse=False, normalize=0, io=L.VDX_C64, flags=L.VDX_FFT_FLAG_TENSOR_CORE):
    d = L.FftDesc()
    d.ndim = len(shape)
    for i, s in enumerate(shape):
        d.shape[i] = int(s)
    d.axis = axis
    d.kind = L.VDX_KIND_C2C
    d.inverse = int(inverse)
    d.normalize = int(normalize)
    d.io_type = io
    d.compute_type = L.VDX_C128 if io == L.VDX_C128 else L.VDX_C64
    d.signal_lo, d.signal_hi = -1, -1
    d.kernel_op = L.VDX_KOP_MUL_CONJ
    d.kernel_type = io
    d.flags = flags
    return d


def _plan(*args, **kw):
    return P.Plan(_desc(*args, **kw))


def _run(plan, t):
    plan.exec(t.data_ptr(), t.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()


@pytest.mark.parametrize("shape,axis", [((4, 16384), 1), ((16384, 48), 0), ((2, 16384, 20), 1)])
def test_complex64_forward_and_inverse(shape, axis):
    rng = np.random.default_rng(4 + axis)
    x = crandn(rng, shape)
    t = torch.from_numpy(x).cuda()
    p = _plan(shape, axis)
    assert p.describe()["tensor_core"] is True
    _run(p, t)
    ref = np.fft.fft(x.astype(np.complex128), axis=axis)
    assert rel_l2(t.cpu().numpy(), ref) <= TC_AXIS_TOL
    pi = _plan(shape, axis, inverse=True, normalize=1)
    _run(pi, t)
    assert rel_l2(t.cpu().numpy(), x) <= 2 * TC_AXIS_TOL
    assert p.status() == 0 and pi.status() == 0


def test_matches_fp32_butterfly_path():
    rng = np.random.default_rng(7)
    x = crandn(rng, (16384, 32))
    a = torch.from_numpy(x).cuda()
    b = a.clone()
    _run(_plan((16384, 32), 0), a)
    _run(_plan((16384, 32), 0, flags=0), b)
    assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) <= TC_AXIS_TOL


def test_orthonormal_scaling():
    rng = np.random.default_rng(8)
    x = crandn(rng, (2, 16384))
    t = torch.from_numpy(x).cuda()
    _run(_plan((2, 16384), 1, normalize=2), t)
    ref = np.fft.fft(x.astype(np.complex128), axis=1, norm="ortho")
    assert rel_l2(t.cpu().numpy(), ref) <= TC_AXIS_TOL


@pytest.mark.parametrize("vt,tol", [(vd.complexbf16, 5e-3), (vd.complex32, 1.2e-3)])
def test_half_storage_fft2_through_the_api(vt, tol):
    rng = np.random.default_rng(4)
    x = crandn(rng, (16384, 64)) * 0.25
    buf = vd.Buffer(x.shape, vt)
    buf.write(x)
    q = buf.read(0).astype(np.complex128)
    with vd.fft.tensor_core_stages():
        vd.fft.fft2(buf)  # axis 0 (16384) on the tensor cores, axis 1 (64) on fp32 butterflies
    assert rel_l2(buf.read(0), np.fft.fft2(q)) < tol


def test_context_only_flags_eligible_plans():
    with vd.fft.tensor_core_stages():
        p = P.get_plan((2, 16384), 1, L.VDX_KIND_C2C, False, False, L.VDX_C64, L.VDX_C64)
        q = P.get_plan((2, 8192), 1, L.VDX_KIND_C2C, False, False, L.VDX_C64, L.VDX_C64)
    assert p.describe()["tensor_core"] is True
    assert q.describe().get("tensor_core", False) is False
    r = P.get_plan((2, 16384), 1, L.VDX_KIND_C2C, False, False, L.VDX_C64, L.VDX_C64)
    assert r.describe()["tensor_core"] is False


@pytest.mark.parametrize("shape,axis,io", [((2, 8192), 1, L.VDX_C64), ((16384, 8), 0, L.VDX_C64),
                                           ((2, 16384), 1, L.VDX_C128)])
def test_ineligible_requests_are_refused(shape, axis, io):
    with pytest.raises(ValueError):
        P.Plan(_desc(shape, axis, io=io))
