"""The multi-GPU form is replicas only (one process per GPU, no collective on
the data path).  These tests run the host logic of that form as two gloo
ranks on the CPU: the benchmark's max-over-ranks step time and whole-job
aggregate, and the reference arm's rank-0-only rule."""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        local_ms = 0.1 * (rank + 1)  # rank 1 is the slower replica
        ms = bench.max_over_ranks(local_ms, dist, device="cpu")
        q.put((rank, ms, bench.whole_job_gbps(world, bench.STEP_BYTES, ms), bench.reference_arm_runs_here(rank)))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_take_the_slowest_step():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, v0, ref0), (r1, ms1, v1, ref1) = results
    assert ms0 == ms1 == pytest.approx(0.2)
    assert v0 == v1 == pytest.approx(2 * 471072768 / 0.2e-3 / 1e9)
    assert ref0 and not ref1


def test_reference_arm_is_a_no_op_off_rank_0(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("RANK", "1")
    assert bench.run_reference(None) is None  # returns before touching the workload
