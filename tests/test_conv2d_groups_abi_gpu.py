"""vdx_conv2d_groups_plan through the C ABI alone (ctypes on include/vdx.h,
no Python FFT layer): the image groups' rfft -> column convolution -> irfft
chains on the plan's own streams give the FP64 result, the same result as
one group, for uneven groups, broadcast kernels, non-square images and
CUDA-graph capture of the caller's stream."""

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
