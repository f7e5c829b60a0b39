"""Builds the oracle's C restatement into oracle/liboracle.so (test
infrastructure only).  gcc with OpenMP; -ffp-contract=off keeps every fp32
operation rounded as written (explicit fmaf where the reference uses fma),
so x86-64 and aarch64 hosts produce identical results."""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "vdx_ref.c"
LIB = HERE / "liboracle.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp), str(SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
