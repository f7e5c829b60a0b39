"""Multi-kernel convolution (kernel_num > 1, vkdispatch/fft/shader_factories.py:
166-193): one signal against a bank of kernel spectra, the kernel map and the
output map indexing their buffers with ``io_index + mapped_kernel_index() * C``.
Checked against FP64 numpy per kernel, within the fused convolution's
tolerance (forward + inverse pass)."""

import numpy as np
import pytest

from helpers import crandn, rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

vd = pytest.importorskip("vkdispatch_gb300")
import vkdispatch_gb300.codegen as vc  # noqa: E402


def _maps(slab, conj=True):
    def kernel_map(kernels: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        kv = vc.new_register(vd.complex64)
        op.read_from_buffer(kernels, register=kv, io_index=op.io_index + vd.fft.mapped_kernel_index() * slab)
        op.register[:] = vc.mult_complex(op.register, kv.conjugate() if conj else kv)

    def output_map(out: vc.Buffer[vd.complex64]):
        op = vd.fft.write_op()
        op.write_to_buffer(out, io_index=op.io_index + slab * vd.fft.mapped_kernel_index())

    return vd.map(kernel_map), vd.map(output_map)


@pytest.mark.parametrize("axis", [1, 0])
def test_kernel_bank_into_output_slices(axis):
    rng = np.random.default_rng(12 + axis)
    B, N, K = 6, 256, 5
    shape = (B, N) if axis == 1 else (N, B)
    x = crandn(rng, shape)
    bank = crandn(rng, (K,) + shape) * 0.1
    slab = B * N
    km, om = _maps(slab)
    sig, kb = vd.asbuffer(x), vd.asbuffer(bank.reshape((K * shape[0],) + shape[1:]))
    out = vd.Buffer((K * shape[0],) + shape[1:], vd.complex64)
    vd.fft.convolve(out, sig, kb, kernel_map=km, output_map=om, kernel_num=K, buffer_shape=shape, axis=axis)
    got = out.read(0).reshape((K,) + shape)
    s = np.fft.fft(x.astype(np.complex128), axis=axis)
    for k in range(K):
        ref = np.fft.ifft(s * np.conj(bank[k]), axis=axis)
        assert rel_l2(got[k], ref) <= 2 * tol_fp32(N)
    assert rel_l2(sig.read(0), x) == 0.0  # the signal is not modified


def test_in_place_bank_reads_the_original_signal():
    # the output map writes slice k over a buffer whose slice 0 is the signal:
    # every kernel must still see the original signal
    rng = np.random.default_rng(21)
    B, N, K = 4, 128, 3
    x = crandn(rng, (B, N))
    bank = crandn(rng, (K, B, N)) * 0.1
    slab = B * N
    km, om = _maps(slab, conj=False)
    buf = vd.Buffer((K * B, N), vd.complex64)
    init = np.zeros((K * B, N), np.complex64)
    init[:B] = x
    buf.write(init)
    kb = vd.asbuffer(bank.reshape(K * B, N))
    vd.fft.convolve(buf, buf, kb, kernel_map=km, output_map=om, kernel_num=K, buffer_shape=(B, N), axis=1)
    got = buf.read(0).reshape(K, B, N)
    s = np.fft.fft(x.astype(np.complex128), axis=1)
    for k in range(K):
        assert rel_l2(got[k], np.fft.ifft(s * bank[k], axis=1)) <= 2 * tol_fp32(N)


def test_default_maps_repeat_the_single_convolution():
    # without maps every kernel index reads the same kernel and writes the same
    # output, as in the reference: the result is the single convolution
    rng = np.random.default_rng(22)
    x = crandn(rng, (3, 64))
    k = crandn(rng, (3, 64))
    a, b = vd.asbuffer(x), vd.asbuffer(x)
    vd.fft.convolve(a, vd.asbuffer(k), kernel_num=3)
    vd.fft.convolve(b, vd.asbuffer(k))
    assert rel_l2(a.read(0), b.read(0)) <= 2 * tol_fp32(64)


def test_index_expression_outside_the_menu_is_compiled():
    """A kernel map reading at io_index * 2 is outside the menu: it runs
    through the run-time compiler, one launch per kernel index, with the
    signal read from a copy because the output overwrites it."""

    def strided_map(kernels: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        kv = vc.new_register(vd.complex64)
        op.read_from_buffer(kernels, register=kv, io_index=op.io_index * 2)
        op.register[:] = vc.mult_complex(op.register, kv.conjugate())

    from vkdispatch_gb300.fft import jit

    rng = np.random.default_rng(21)
    x = (rng.standard_normal((2, 32)) + 1j * rng.standard_normal((2, 32))).astype(np.complex64)
    k = (rng.standard_normal((4, 32)) + 1j * rng.standard_normal((4, 32))).astype(np.complex64)
    b = vd.asbuffer(x)
    jit.out_of_range(reset=True)
    # no input or output map: the output buffer, then the kernel map's buffer
    vd.fft.convolve(b, vd.asbuffer(k), kernel_map=vd.map(strided_map), kernel_num=2)
    assert not jit.out_of_range()
    k2 = k.reshape(-1)[::2].reshape(2, 32).astype(np.complex128)
    want = np.fft.ifft(np.fft.fft(x.astype(np.complex128), axis=1) * np.conj(k2), axis=1)
    assert np.linalg.norm(b.read(0) - want) / np.linalg.norm(want) <= 2 * 5e-7 * 5


@pytest.mark.parametrize("dtype,axis,N", [("complex64", 1, 384), ("complex64", 0, 384), ("complex128", 1, 384),
                                          ("complex64", 1, 1024), ("complex64", 0, 512)])
def test_fused_multi_kernel_launch(dtype, axis, N):
    """One launch for all kernels (vdx_conv_exec_multi; runtime-radix and
    compile-time plans) against one convolution launch per kernel and FP64
    numpy."""
    import torch

    from vkdispatch_gb300 import _lib as L
    from vkdispatch_gb300.fft import plan as P

    rng = np.random.default_rng(30 + axis)
    B, K = 8, 4
    shape = (B, N) if axis == 1 else (N, B)
    tdt = getattr(torch, dtype)
    code = L.VDX_C64 if dtype == "complex64" else L.VDX_C128
    x = crandn(rng, shape).astype(dtype)
    bank = (crandn(rng, (K,) + shape) * 0.1).astype(dtype)
    xt, kt = torch.from_numpy(x).cuda(), torch.from_numpy(bank).cuda()
    slab = B * N
    plan = P.get_plan(shape, axis, L.VDX_KIND_CONV, False, True, code, code, None, L.VDX_KOP_MUL_CONJ, code)
    s = torch.cuda.current_stream().cuda_stream
    fused = torch.empty((K,) + shape, dtype=tdt, device="cuda")
    assert plan.exec_multi(xt.data_ptr(), fused.data_ptr(), kt.data_ptr(), K, slab, slab, s)
    loop = torch.empty_like(fused)
    for k in range(K):
        plan.exec(xt.data_ptr(), loop[k].data_ptr(), kt[k].data_ptr(), s)
    torch.cuda.synchronize()
    assert rel_l2(fused.cpu().numpy(), loop.cpu().numpy()) <= (1e-6 if dtype == "complex64" else 1e-14)
    spec = np.fft.fft(x.astype(np.complex128), axis=axis)
    tol = 2 * tol_fp32(N) if dtype == "complex64" else 1e-12
    for k in range(K):
        ref = np.fft.ifft(spec * np.conj(bank[k]), axis=axis)
        assert rel_l2(fused[k].cpu().numpy(), ref) <= tol
    assert rel_l2(xt.cpu().numpy(), x) == 0.0  # the signal is not modified


def test_fused_multi_kernel_refuses_plans_without_a_fused_kernel():
    import torch

    from vkdispatch_gb300 import _lib as L
    from vkdispatch_gb300.fft import plan as P

    c = L.VDX_C32
    plan = P.get_plan((4, 256), 1, L.VDX_KIND_CONV, False, True, c, L.VDX_C64, None, L.VDX_KOP_MUL_CONJ, c)
    buf = torch.zeros((2, 4, 256, 2), dtype=torch.float16, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert plan.exec_multi(buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), 2, 0, 1024, s) is False


@pytest.mark.parametrize("shape,axis", [((8, 1024), 1), ((512, 8), 0)])
def test_fused_multi_kernel_on_two_pass_plans(monkeypatch, shape, axis):
    import torch

    from vkdispatch_gb300 import _lib as L
    from vkdispatch_gb300.fft import plan as P

    monkeypatch.setenv("VDX_POINTS_PER_THREAD", "32")
    P.cache_clear()
    rng = np.random.default_rng(40 + axis)
    K = 3
    x = crandn(rng, shape)
    bank = crandn(rng, (K,) + shape) * 0.1
    xt, kt = torch.from_numpy(x).cuda(), torch.from_numpy(bank).cuda()
    c = L.VDX_C64
    plan = P.get_plan(shape, axis, L.VDX_KIND_CONV, False, True, c, c, None, L.VDX_KOP_MUL, c)
    assert plan.describe()["threads_per_transform"] == shape[axis] // 32
    out = torch.empty((K,) + shape, dtype=torch.complex64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert plan.exec_multi(xt.data_ptr(), out.data_ptr(), kt.data_ptr(), K, x.size, x.size, s)
    torch.cuda.synchronize()
    spec = np.fft.fft(x.astype(np.complex128), axis=axis)
    for k in range(K):
        assert rel_l2(out[k].cpu().numpy(), np.fft.ifft(spec * bank[k], axis=axis)) <= 2 * tol_fp32(shape[axis])
    P.cache_clear()


@pytest.mark.parametrize("N", [96, 256])
def test_kernel_bank_broadcast_over_batches(N):
    """kernel_num kernels, each one slab broadcast over the signal's batches
    (kernel_inner_only), through vd.fft.convolve's fused multi-kernel launch."""
    rng = np.random.default_rng(50 + N)
    B, K = 5, 3
    x = crandn(rng, (B, N))
    bank = crandn(rng, (K, N)) * 0.1
    km, _ = _maps(N)  # kernel k at k * N, its slab broadcast over the batches
    _, om = _maps(B * N)  # output slice k at k * B * N
    sig, kb = vd.asbuffer(x), vd.asbuffer(bank)
    out = vd.Buffer((K * B, N), vd.complex64)
    vd.fft.convolve(out, sig, kb, kernel_map=km, output_map=om, kernel_num=K, buffer_shape=(B, N), axis=1,
                    kernel_inner_only=True)
    got = out.read(0).reshape(K, B, N)
    s = np.fft.fft(x.astype(np.complex128), axis=1)
    for k in range(K):
        assert rel_l2(got[k], np.fft.ifft(s * np.conj(bank[k])[None, :], axis=1)) <= 2 * tol_fp32(N)


def test_out_of_range_map_index_is_caught():
    """A kernel map indexing past its buffer (io_index * 2 into a buffer of
    the signal's size) never touches memory outside it: the bounds check of
    the compiled hooks loads zero there and reports through the plan's
    status word."""
    from vkdispatch_gb300.fft import jit

    def strided_map(kernels: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        kv = vc.new_register(vd.complex64)
        op.read_from_buffer(kernels, register=kv, io_index=op.io_index * 2)
        op.register[:] = vc.mult_complex(op.register, kv.conjugate())

    rng = np.random.default_rng(22)
    x = (rng.standard_normal((2, 32)) + 1j * rng.standard_normal((2, 32))).astype(np.complex64)
    k = (rng.standard_normal((2, 32)) + 1j * rng.standard_normal((2, 32))).astype(np.complex64)
    b = vd.asbuffer(x)
    jit.out_of_range(reset=True)
    vd.fft.convolve(b, vd.asbuffer(k), kernel_map=vd.map(strided_map))
    assert jit.out_of_range()
    kk = np.zeros(64, np.complex128)
    kk[:32] = k.reshape(-1)[::2]  # indices 64.. read as zero
    want = np.fft.ifft(np.fft.fft(x.astype(np.complex128), axis=1) * np.conj(kk.reshape(2, 32)), axis=1)
    assert np.linalg.norm(b.read(0) - want) / np.linalg.norm(want) <= 2 * 5e-7 * 5
    assert not jit.out_of_range()  # the check above reset it

