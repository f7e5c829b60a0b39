"""vdx_conv2d_groups_plan and vdx_group_plan through the C ABI alone
(ctypes on include/vdx.h, no Python FFT layer): the image groups' chains of
transforms on the plans' own streams give the FP64 result, the same result
as one group, for uneven groups, broadcast kernels, non-square images,
four-step rows, CUDA-graph capture of the caller's stream, and the fft2 /
ifft2 / rfft2 / convolve2D chains."""

import ctypes
import json

import numpy as np
import pytest
import torch

from vkdispatch_gb300 import _lib as L

from helpers import rel_l2, tol_fp32

pytestmark = pytest.mark.gpu


def _desc(n, H, W, broadcast, normalize=1):
    d = L.FftDesc()
    d.ndim = 3
    d.shape[0], d.shape[1], d.shape[2] = n, H, W
    d.axis = 1
    d.kind = L.VDX_KIND_CONV2D_REAL
    d.normalize = normalize
    d.io_type = d.compute_type = L.VDX_C64
    d.signal_lo = d.signal_hi = -1
    d.kernel_op = L.VDX_KOP_MUL_CONJ
    d.kernel_type = L.VDX_C64
    d.kernel_broadcast = int(broadcast)
    return d


class _Plan:
    def __init__(self, n, H, W, groups, broadcast=False, normalize=1):
        self.h = ctypes.c_void_p()
        d = _desc(n, H, W, broadcast, normalize)
        L.check(L.lib().vdx_conv2d_groups_plan_create(ctypes.byref(d), groups, ctypes.byref(self.h)), "create")

    def describe(self):
        buf = ctypes.create_string_buffer(1024)
        L.check(L.lib().vdx_conv2d_groups_plan_describe(self.h, buf, len(buf)), "describe")
        return json.loads(buf.value.decode())

    def exec(self, data, ker, stream=None):
        s = torch.cuda.current_stream() if stream is None else stream
        L.check(L.lib().vdx_conv2d_groups_exec(self.h, data.data_ptr(), ker.data_ptr(), s.cuda_stream), "exec")

    def __del__(self):
        L.lib().vdx_conv2d_groups_plan_destroy(self.h)


def _case(n, H, W, seed, broadcast=False):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, H, W)).astype(np.float32)
    kn = 1 if broadcast else n
    K = ((rng.standard_normal((kn, H, W // 2 + 1)) + 1j * rng.standard_normal((kn, H, W // 2 + 1))) * 0.01
         ).astype(np.complex64)
    return x, K


def _packed(x):
    n, H, W = x.shape
    t = torch.zeros((n, H, W // 2 + 1), dtype=torch.complex64, device="cuda")
    t.view(torch.float32).view(n, H, W + 2)[..., :W].copy_(torch.from_numpy(x))
    return t


def _real(t, W):
    n, H, _ = t.shape
    return t.view(torch.float32).view(n, H, W + 2)[..., :W].cpu().numpy()


def _ref(x, K, normalize=True):
    S = np.fft.rfft(x.astype(np.float64), axis=-1)
    T = np.fft.ifft(np.fft.fft(S, axis=-2) * np.conj(K.astype(np.complex128)), axis=-2)
    out = np.fft.irfft(T, n=x.shape[-1], axis=-1)
    if not normalize:
        out = out * x.shape[-2] * x.shape[-1]
    return out


@pytest.mark.parametrize(
    "n,H,W,groups,broadcast",
    [(8, 512, 512, 2, False), (10, 256, 512, 3, False), (12, 512, 256, 4, True), (5, 128, 128, 8, False),
     (16, 384, 320, 2, True), (1, 64, 64, 1, False)],
)
def test_groups_match_fp64_and_one_group(n, H, W, groups, broadcast):
    x, K = _case(n, H, W, n * 7 + groups, broadcast)
    ker = torch.from_numpy(K).cuda()
    tol = 4 * tol_fp32(max(H, W))
    p = _Plan(n, H, W, groups, broadcast)
    info = p.describe()
    assert info["groups"] == min(groups, n)
    assert sum(info["group_images"]) == n
    data = _packed(x)
    p.exec(data, ker)
    torch.cuda.synchronize()
    got = _real(data, W)
    assert rel_l2(got, _ref(x, K)) <= tol
    one = _Plan(n, H, W, 1, broadcast)
    data = _packed(x)
    one.exec(data, ker)
    torch.cuda.synchronize()
    assert rel_l2(got, _real(data, W)) <= tol


def test_without_normalization():
    x, K = _case(8, 256, 256, 3)
    p = _Plan(8, 256, 256, 2, normalize=0)
    data = _packed(x)
    p.exec(data, torch.from_numpy(K).cuda())
    torch.cuda.synchronize()
    assert rel_l2(_real(data, 256), _ref(x, K, normalize=False)) <= 4 * tol_fp32(256)


def test_side_stream_caller_and_graph_capture():
    """The fork and join events order the groups after earlier work on the
    caller's (non-default) stream and before later work on it, and the whole
    fork / groups / join pattern captures into a CUDA graph."""
    x, K = _case(16, 512, 512, 11)
    ker = torch.from_numpy(K).cuda()
    p = _Plan(16, 512, 512, 2)
    data = _packed(x)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        data.copy_(_packed(x))  # earlier work on the caller's stream
        p.exec(data, ker, s)
        after = data.clone()  # later work on the caller's stream
    s.synchronize()
    ref = _ref(x, K)
    assert rel_l2(_real(after, 512), ref) <= 4 * tol_fp32(512)
    g = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    cap.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cap):
        with torch.cuda.graph(g, stream=cap):
            p.exec(data, ker, cap)
    torch.cuda.current_stream().wait_stream(cap)
    data.copy_(_packed(x))
    g.replay()
    torch.cuda.synchronize()
    assert rel_l2(_real(data, 512), ref) <= 4 * tol_fp32(512)


def test_odd_width_refused_on_device():
    d = _desc(8, 64, 63, False)
    h = ctypes.c_void_p()
    assert L.lib().vdx_conv2d_groups_plan_create(ctypes.byref(d), 2, ctypes.byref(h)) == L.VDX_ERR_INVALID
    assert not h.value


def _steps(specs):
    arr = (L.FftDesc * len(specs))()
    for d, (shape, axis, kind, inverse, normalize, broadcast) in zip(arr, specs):
        d.ndim = 3
        for i, x in enumerate(shape):
            d.shape[i] = x
        d.axis, d.kind, d.inverse, d.normalize = axis, kind, int(inverse), int(normalize)
        d.io_type = d.compute_type = L.VDX_C64
        d.signal_lo = d.signal_hi = -1
        d.kernel_op = L.VDX_KOP_MUL_CONJ
        d.kernel_type = L.VDX_C64
        d.kernel_broadcast = int(broadcast)
    return arr


class _Chain:
    def __init__(self, specs, groups):
        self.h = ctypes.c_void_p()
        arr = _steps(specs)
        L.check(L.lib().vdx_group_plan_create(arr, len(specs), groups, ctypes.byref(self.h)), "create")

    def describe(self):
        buf = ctypes.create_string_buffer(1024)
        L.check(L.lib().vdx_group_plan_describe(self.h, buf, len(buf)), "describe")
        return json.loads(buf.value.decode())

    def exec(self, data, ker=None):
        L.check(L.lib().vdx_group_exec(self.h, data.data_ptr(), None if ker is None else ker.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream), "exec")

    def __del__(self):
        L.lib().vdx_group_plan_destroy(self.h)


def _crand(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)


@pytest.mark.parametrize("n,H,W,groups", [(8, 256, 512, 2), (11, 128, 384, 3), (8, 64, 16384, 2)])
def test_group_chain_fft2_ifft2(n, H, W, groups):
    """fft2 then ifft2 as two chains; the 16384-point rows are four-step plans
    with a workspace per group."""
    rng = np.random.default_rng(n + W)
    x = _crand(rng, (n, H, W))
    data = torch.from_numpy(x).cuda()
    C2C = L.VDX_KIND_C2C
    fwd = _Chain([((n, H, W), 1, C2C, 0, 0, 0), ((n, H, W), 2, C2C, 0, 0, 0)], groups)
    inv = _Chain([((n, H, W), 1, C2C, 1, 1, 0), ((n, H, W), 2, C2C, 1, 1, 0)], groups)
    assert fwd.describe()["group_images"] == [n * (g + 1) // groups - n * g // groups for g in range(groups)]
    fwd.exec(data)
    torch.cuda.synchronize()
    assert rel_l2(data.cpu().numpy(), np.fft.fft2(x.astype(np.complex128))) <= 2 * tol_fp32(H, W)
    inv.exec(data)
    torch.cuda.synchronize()
    assert rel_l2(data.cpu().numpy(), x) <= 4 * tol_fp32(H, W)


def test_group_chain_rfft2_and_convolve2d():
    rng = np.random.default_rng(5)
    n, H, W = 9, 256, 256
    x = rng.uniform(-1, 1, (n, H, W)).astype(np.float32)
    data = _packed(x)
    R = (n, H, W)
    HC = W // 2 + 1
    rfft2 = _Chain([(R, 2, L.VDX_KIND_R2C, 0, 0, 0), ((n, H, HC), 1, L.VDX_KIND_C2C, 0, 0, 0)], 2)
    rfft2.exec(data)
    torch.cuda.synchronize()
    assert rel_l2(data.cpu().numpy(), np.fft.rfft2(x.astype(np.float64))) <= 2 * tol_fp32(H, W)
    # convolve2D of a complex batch with one broadcast kernel spectrum
    z = _crand(rng, (n, H, W))
    K = _crand(rng, (H, W)) * 0.05
    zt = torch.from_numpy(z).cuda()
    conv = _Chain([((n, H, W), 2, L.VDX_KIND_C2C, 0, 0, 0), ((n, H, W), 1, L.VDX_KIND_CONV, 0, 1, 1),
                   ((n, H, W), 2, L.VDX_KIND_C2C, 1, 1, 0)], 3)
    conv.exec(zt, torch.from_numpy(K).cuda())
    torch.cuda.synchronize()
    z64 = z.astype(np.complex128)
    S = np.fft.fft(z64, axis=2)
    ref = np.fft.ifft(np.fft.ifft(np.fft.fft(S, axis=1) * np.conj(K), axis=1), axis=2)
    assert rel_l2(zt.cpu().numpy(), ref) <= 4 * tol_fp32(H, W)


def test_group_chain_needs_kernel_for_convolution():
    n, H, W = 8, 64, 64
    conv = _Chain([((n, H, W), 1, L.VDX_KIND_CONV, 0, 1, 0)], 2)
    data = torch.zeros((n, H, W), dtype=torch.complex64, device="cuda")
    rc = L.lib().vdx_group_exec(conv.h, data.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    assert rc == L.VDX_ERR_INVALID and "kernel" in L.last_error()
