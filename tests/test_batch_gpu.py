"""GPU tests of the batched uneven-length persistent launch against FP64
numpy.fft, item by item, including lengths above 16384 (four-step)."""

import numpy as np
import pytest

from helpers import rel_l2, tol_fp32

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from vkdispatch_gb300.batch import BatchPlan, pack_items  # noqa: E402


def _run(lengths_counts, inverse=False, normalize=True, seed=0):
    items, total = pack_items(lengths_counts)
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    d = torch.from_numpy(x).cuda()
    plan = BatchPlan(items, inverse=inverse, normalize=normalize)
    ws = plan.make_workspace()
    plan(d, ws)
    torch.cuda.synchronize()
    assert plan.status() == 0
    got = d.cpu().numpy()
    for off, n, c in items:
        xi = x[off: off + n * c].reshape(c, n).astype(np.complex128)
        if inverse:
            ref = np.fft.ifft(xi, axis=-1) * (1.0 if normalize else n)
        else:
            ref = np.fft.fft(xi, axis=-1)
        gi = got[off: off + n * c].reshape(c, n)
        assert rel_l2(gi, ref) <= 2 * tol_fp32(n), (n, c)
    return plan


def test_mixed_short_lengths():
    p = _run([(16, 300), (1024, 7), (81, 13), (1000, 3), (16384, 2), (2, 5), (4096, 1), (13 * 16, 9)])
    d = p.describe()
    # lengths needing more threads per transform than one CTA has run as four-step pairs
    assert d["long_items"] <= 3 and d["units"] >= 8


def test_long_lengths_four_step():
    p = _run([(32768, 2), (65536, 1), (20736, 1), (15625, 1), (24576, 2), (64, 100)], seed=1)
    d = p.describe()
    assert d["long_items"] >= 4 and d["workspace_bytes"] > 0


@pytest.mark.parametrize("cta", [256, 512, 1024])
@pytest.mark.parametrize("stage,stage_t", [("0", "2"), ("3", "2"), ("7", "16")])
def test_cta_sizes_and_staged_row_tiles(cta, stage, stage_t, monkeypatch):
    """Every CTA size, with row tiles staged through shared memory or not:
    narrow rows (fewer than 16 threads per transform, partial last tiles),
    odd radices, and four-step items whose second pass stores transposed."""
    monkeypatch.setenv("VDX_BATCH_THREADS", str(cta))
    monkeypatch.setenv("VDX_BATCH_STAGE", stage)
    monkeypatch.setenv("VDX_BATCH_STAGE_T", stage_t)
    _run([(16, 257), (21, 100), (2, 9), (39, 41), (100, 33), (243, 7), (4096, 3), (12005, 1), (50421, 1),
          (65536, 1), (8, 3)], seed=cta + int(stage))


def test_inverse_and_unnormalised():
    _run([(512, 9), (65536, 1), (45, 3)], inverse=True, seed=2)
    _run([(512, 9), (49152, 1)], inverse=True, normalize=False, seed=3)


def test_graph_capture_replay():
    items, total = pack_items([(1024, 16), (32768, 1), (343, 5)])
    rng = np.random.default_rng(4)
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    d = torch.from_numpy(x).cuda()
    plan = BatchPlan(items)
    ws = plan.make_workspace()
    plan(d, ws)  # first call outside capture (plan tables are resident already)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    import vkdispatch_gb300 as vd

    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            with vd.cuda_graph_capture(torch.cuda.current_stream()):
                plan(d, ws)
    torch.cuda.current_stream().wait_stream(s)
    d.copy_(torch.from_numpy(x))
    g.replay()
    g.replay()  # twice: forward of forward
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    for off, n, c in items:
        xi = x[off: off + n * c].reshape(c, n).astype(np.complex128)
        ref = np.fft.fft(np.fft.fft(xi, axis=-1), axis=-1)
        assert rel_l2(got[off: off + n * c].reshape(c, n), ref) <= 4 * tol_fp32(n)


def test_bad_items_rejected():
    with pytest.raises(ValueError):
        BatchPlan([(0, 17 * 4099, 1)])  # prime factor above 13
    with pytest.raises(ValueError):
        BatchPlan([(0, 0, 1)])


def test_autotuned_batch_plan_matches_numpy():
    """BatchPlan(autotune=True) picks a CTA size by timing; results stay within the bound."""
    import torch
    from vkdispatch_gb300.batch import BatchPlan, pack_items

    rng = np.random.default_rng(44)
    lengths = [16, 48, 625, 1024, 2187, 9604, 40000]
    items, total = pack_items((n, max(1, 60000 // n)) for n in lengths)
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    t = torch.from_numpy(x).cuda()
    plan = BatchPlan(items, autotune=True)
    assert plan.cta in (256, 512, 1024)
    ws = plan.make_workspace()
    plan(t, ws)
    torch.cuda.synchronize()
    got = t.cpu().numpy()
    for off, n, c in items:
        ref = np.fft.fft(x[off:off + n * c].reshape(c, n).astype(np.complex128), axis=1)
        err = np.linalg.norm(got[off:off + n * c].reshape(c, n) - ref) / np.linalg.norm(ref)
        assert err <= 5e-7 * max(1.0, np.log2(n)) * 2
    assert plan.status() == 0


def test_bounded_wait_runs_out_and_reports():
    """A dependency that can never complete (injected on the host) makes every
    second-pass wait run out at a short poll limit: the launch returns, the
    status word reads 1, and the same plan and another plan on the same
    stream then run clean."""
    items, total = pack_items([(32768, 3), (256, 4)])
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    d = torch.from_numpy(x).cuda()
    plan = BatchPlan(items)
    assert plan.describe()["long_items"] == 1
    ws = plan.make_workspace()
    plan.set_wait(wait_limit=1000, extra_dependency=1)  # about 0.1 ms per wait
    plan(d, ws)
    torch.cuda.synchronize()
    assert plan.status() == 1
    # the short item has no dependency and is still transformed
    off, n, c = items[1]
    ref = np.fft.fft(x[off: off + n * c].reshape(c, n).astype(np.complex128), axis=-1)
    assert rel_l2(d.cpu().numpy()[off: off + n * c].reshape(c, n), ref) <= 2 * tol_fp32(n)
    # restore: the same plan, then a fresh plan, run clean on the same stream
    plan.set_wait()
    assert plan.status() == 0
    d.copy_(torch.from_numpy(x))
    plan(d, ws)
    other = BatchPlan(pack_items([(65536, 1)])[0])
    y = torch.from_numpy((rng.standard_normal(65536) + 1j * rng.standard_normal(65536)).astype(np.complex64)).cuda()
    y0 = y.cpu().numpy()
    other(y, other.make_workspace())
    torch.cuda.synchronize()
    assert plan.status() == 0 and other.status() == 0
    got = d.cpu().numpy()
    for off, n, c in items:
        ref = np.fft.fft(x[off: off + n * c].reshape(c, n).astype(np.complex128), axis=-1)
        assert rel_l2(got[off: off + n * c].reshape(c, n), ref) <= 2 * tol_fp32(n)
    assert rel_l2(y.cpu().numpy(), np.fft.fft(y0.astype(np.complex128))) <= 2 * tol_fp32(65536)


def test_set_wait_validation():
    plan = BatchPlan([(0, 64, 1)])
    with pytest.raises(ValueError):
        plan.set_wait(wait_limit=0)
    with pytest.raises(ValueError):
        plan.set_wait(extra_dependency=-1)
