"""Generates the golden fixtures under tests/golden/ by importing the
reference (sharhar/vkdispatch) from a local checkout.

Run where a reference checkout exists, naming it with the
VKDISPATCH_REFERENCE environment variable:

    VKDISPATCH_REFERENCE=<checkout> python tests/golden/make_golden.py [plans|vectors|config|all]

plans   -> plans.json: the reference's own FFT plan (prime groups per stage,
           register count, threads per transform) for every 13-smooth length
           up to 16384, built by vkdispatch.fft.FFTConfig with the device
           limits its CUDA backend reports on a GB300 (1024 threads per block,
           48 KiB shared memory, 32-wide subgroups).
vectors -> vectors.npz: inputs and outputs of the reference's own generated
           FFT / convolution / R2C / C2R kernels, emitted by its CUDA code
           generator and executed on the host through oracle/shim/
           (see oracle/run_reference_kernels.py).
config  -> config_vectors.npz: the same at the benchmark configurations'
           lengths and stride classes (1024-point rows forward and inverse,
           512-point R2C / C2R rows, the 512 x 257 strided convolution, a
           32^3 FFT3) plus the reference's two-stage reductions (magnitude
           sum, uint32 xor, int32 and, float sum); inputs come from
           oracle/inputs.py and large outputs are kept at sampled indices.

Only the fixtures are committed; the reference and its generated sources are
not.  Nothing at test time reads the reference.
"""

from __future__ import annotations

import json
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = os.environ.get("VKDISPATCH_REFERENCE")

GB300_LIMITS = dict(
    subgroup_size=32,
    max_workgroup_size=(1024, 1024, 64),
    max_workgroup_invocations=1024,
    max_workgroup_count=(2**31 - 1, 65535, 65535),
    max_shared_memory=48 * 1024,
)


def _import_reference():
    sys.path.insert(0, REF)
    import vkdispatch as vd
    import vkdispatch.codegen as vc

    vd.initialize(backend="dummy")
    vc.set_codegen_backend("cuda")
    vd.set_dummy_context_params(**GB300_LIMITS)
    return vd, vc


def smooth(limit):
    out = set()

    def rec(v, i, primes=(2, 3, 5, 7, 11, 13)):
        if v > limit:
            return
        out.add(v)
        for j in range(i, len(primes)):
            rec(v * primes[j], j)

    rec(1, 0)
    return sorted(x for x in out if x >= 2)


def make_plans():
    vd, _ = _import_reference()
    from vkdispatch.fft.config import FFTConfig

    plans = {}
    for n in smooth(16384):
        for inner in (1, 4):
            shape = (n,) if inner == 1 else (n, inner)
            try:
                cfg = FFTConfig(shape, 0)
                plans[f"{n}/{inner}"] = {
                    "groups": [list(s.primes) for s in cfg.stages],
                    "register_count": cfg.register_count,
                    "batch_threads": cfg.batch_threads,
                    "thread_counts": list(cfg.thread_counts),
                }
            except ValueError as e:
                plans[f"{n}/{inner}"] = {"error": str(e).split(":")[0]}
    (HERE / "plans.json").write_text(json.dumps(plans, indent=0, sort_keys=True))
    print(f"wrote {len(plans)} plans")


if __name__ == "__main__":
    if not REF:
        sys.exit("set VKDISPATCH_REFERENCE to the reference checkout")
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("plans", "all"):
        make_plans()
    if what in ("vectors", "all"):
        sys.path.insert(0, str(HERE.parent.parent))
        from oracle import run_reference_kernels

        run_reference_kernels.make_vectors(REF, HERE / "vectors.npz", GB300_LIMITS)
    if what in ("config", "all"):
        sys.path.insert(0, str(HERE.parent.parent))
        from oracle import run_reference_kernels

        run_reference_kernels.make_config_vectors(REF, HERE / "config_vectors.npz", GB300_LIMITS)
