"""GPU tests of buffers over non-contiguous CUDA arrays
(from_cuda_array(..., require_contiguous=False)).  The reference requires C
order (vkdispatch/base/buffer.py:353-362); here C2C transforms and
convolutions address such buffers through their strides with no copy, and
reductions read a C-order copy.  Checked against FP64 numpy on the same
logical arrays."""

import numpy as np
import pytest

from helpers import rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
vd = pytest.importorskip("vkdispatch_gb300")


def _crandn(shape, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(shape, dtype=torch.complex64, device="cuda", generator=g)


def test_contiguous_required_by_default():
    t = _crandn((16, 8), 1).t()
    with pytest.raises(ValueError, match="contiguous"):
        vd.from_cuda_array(t)
    b = vd.from_cuda_array(t, require_contiguous=False)
    assert b.strides == (1, 8) and not b.contiguous


@pytest.mark.parametrize("axis", [0, 1])
def test_transposed_view_fft(axis):
    base = _crandn((48, 40), 2)
    view = base.t()  # (40, 48), strides (1, 40)
    x = view.cpu().numpy().astype(np.complex128)
    b = vd.from_cuda_array(view, require_contiguous=False)
    vd.fft.fft(b, axis=axis)
    assert rel_l2(view.cpu().numpy(), np.fft.fft(x, axis=axis)) <= tol_fp32(x.shape[axis])
    vd.fft.ifft(b, axis=axis)
    assert rel_l2(view.cpu().numpy(), x) <= 2 * tol_fp32(x.shape[axis])


def test_pitched_rows_leave_the_padding_untouched():
    base = _crandn((12, 130), 3)
    before = base.cpu().numpy()
    view = base[:, 1:129]  # rows of 128 points, pitch 130
    b = vd.from_cuda_array(view, require_contiguous=False)
    vd.fft.fft(b)
    after = base.cpu().numpy()
    assert rel_l2(after[:, 1:129], np.fft.fft(before[:, 1:129].astype(np.complex128), axis=1)) <= tol_fp32(128)
    assert np.array_equal(after[:, 0], before[:, 0]) and np.array_equal(after[:, 129], before[:, 129])


def test_fft2_and_fft3_on_permuted_views():
    base = _crandn((8, 20, 6), 4)
    view = base.permute(2, 0, 1)  # (6, 8, 20)
    x = view.cpu().numpy().astype(np.complex128)
    b = vd.from_cuda_array(view, require_contiguous=False)
    vd.fft.fft3(b)
    assert rel_l2(view.cpu().numpy(), np.fft.fftn(x)) <= tol_fp32(6, 8, 20)


def test_convolution_with_strided_signal_and_kernel():
    sig = _crandn((64, 10), 5).t()  # (10, 64)
    ker = _crandn((64, 10), 6).t()
    x, k = (t.cpu().numpy().astype(np.complex128) for t in (sig, ker))
    vd.fft.convolve(vd.from_cuda_array(sig, require_contiguous=False),
                    vd.from_cuda_array(ker, require_contiguous=False))
    want = np.fft.ifft(np.fft.fft(x, axis=1) * np.conj(k), axis=1)
    assert rel_l2(sig.cpu().numpy(), want) <= tol_fp32(64, 64)


def test_reduction_over_a_strided_view():
    base = torch.rand((300, 70), device="cuda")
    view = base[:, 3:67]
    b = vd.from_cuda_array(view, require_contiguous=False)

    @vd.reduce.reduce(0)
    def total(a: vd.float32, c: vd.float32) -> vd.float32:
        return a + c

    got = float(total(b).read(0)[0])
    want = view.double().sum().item()
    assert abs(got - want) <= 1e-5 * abs(want)


def test_real_transforms_refuse_strided_buffers():
    view = _crandn((8, 33), 7)[:, :17]
    b = vd.from_cuda_array(view, require_contiguous=False)
    with pytest.raises(ValueError):
        vd.fft.fft(b, buffer_shape=(8, 32), r2c=True)
