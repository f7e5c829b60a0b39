"""GPU test of vdx_reduce_noalloc, the reduction entry point that allocates
nothing (for callers that cannot call cudaMalloc: applications whose device
memory belongs to their own pool allocator, and latency-critical loops that
cannot take cudaMalloc's device-wide synchronisation).

Its results must equal those of vdx_reduce, the entry point that takes a
caller-provided workspace, on two calls in a row (the second call reuses the
static scratch the first call left behind).  This file sorts last so that a
run stopping at the first failure has already run every other test; it also
passes alone in a fresh process.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from vkdispatch_gb300 import _lib as L  # noqa: E402


def _parts(n):
    p = ctypes.c_int64()
    L.check(L.lib().vdx_reduce_partial_count(n, ctypes.byref(p)), "partial count")
    return int(p.value)


def _both(op, mp, in_type, x, n, batch, out_dtype):
    """Runs vdx_reduce (workspace) and vdx_reduce_noalloc on the same input."""
    lib = L.lib()
    stream = torch.cuda.current_stream().cuda_stream
    out_ws = torch.empty(batch, dtype=out_dtype, device="cuda")
    ws = torch.empty(_parts(n) * batch, dtype=out_dtype, device="cuda")
    L.check(lib.vdx_reduce(op, mp, in_type, x.data_ptr(), n, batch, out_ws.data_ptr(), ws.data_ptr(), stream),
            "vdx_reduce")
    out_na = torch.empty(batch, dtype=out_dtype, device="cuda")
    L.check(lib.vdx_reduce_noalloc(op, mp, in_type, x.data_ptr(), n, batch, out_na.data_ptr(), stream),
            "vdx_reduce_noalloc")
    torch.cuda.synchronize()
    return out_ws.cpu().numpy(), out_na.cpu().numpy()


def test_noalloc_matches_workspace_entry_point_on_two_calls():
    torch.cuda.set_device(0)
    rng = np.random.default_rng(17)
    # call 1: float sum over 3 rows; call 2: complex magnitude sum over 5 rows
    cases = [
        (L.VDX_RED_ADD, L.VDX_MAP_IDENTITY, L.VDX_F32, rng.random((3, 300001)).astype(np.float32)),
        (L.VDX_RED_ADD, L.VDX_MAP_ABS, L.VDX_C64,
         (rng.standard_normal((5, 262144)) + 1j * rng.standard_normal((5, 262144))).astype(np.complex64)),
    ]
    for op, mp, in_type, data in cases:
        x = torch.from_numpy(data).cuda()
        batch, n = data.shape
        ws, na = _both(op, mp, in_type, x, n, batch, torch.float32)
        ref = np.abs(data.astype(np.complex128)).sum(axis=1) if in_type == L.VDX_C64 else data.astype(
            np.float64).sum(axis=1)
        # same kernels, same partial count and a fixed fold order: bit-identical
        # to the workspace entry point, and within the float-sum tolerance of
        # the FP64 result
        assert np.array_equal(na, ws)
        assert np.all(np.abs(na - ref) <= 1e-5 * np.abs(ref))


def test_noalloc_integer_bit_exact():
    torch.cuda.set_device(0)
    rng = np.random.default_rng(23)
    data = rng.integers(0, 2**31 - 1, size=(4, 123457), dtype=np.int32)
    x = torch.from_numpy(data).cuda()
    for _ in range(2):
        ws, na = _both(L.VDX_RED_XOR, L.VDX_MAP_IDENTITY, L.VDX_I32, x, data.shape[1], 4, torch.int32)
        assert np.array_equal(na, ws)
        assert np.array_equal(na, np.bitwise_xor.reduce(data, axis=1))
