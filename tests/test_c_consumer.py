"""include/vdx.h from plain C (tests/c_consumer/vdx_c_consumer.c): the
header compiles as C, the program links against the in-tree libvdx.so with
no Python or torch in the process, and its checks pass -- argument
validation on the CPU, and on the GPU a runtime-radix C2C, the convolve2DR
image groups, a reduction and a persistent batch of uneven lengths against
double-precision DFTs computed in C, with the three-step vdx_group_plan
bit-equal to vdx_conv2d_groups."""

import subprocess
from pathlib import Path

import pytest

from vkdispatch_gb300 import _build
from vkdispatch_gb300 import _lib as L

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "c_consumer" / "vdx_c_consumer.c"


@pytest.fixture(scope="module")
def consumer(tmp_path_factory):
    L.lib()  # the in-tree build must exist
    exe = tmp_path_factory.mktemp("c_consumer") / "vdx_c_consumer"
    cmd = [_build.nvcc_path(), "-O2", "-I", str(ROOT / "include"), str(SRC), str(L.LIB_PATH), "-o", str(exe), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_c_consumer_validates_without_gpu(consumer):
    r = subprocess.run([str(consumer), "validate"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "validate: ok" in r.stdout


@pytest.mark.gpu
def test_c_consumer_runs_on_gpu(consumer):
    r = subprocess.run([str(consumer), "run"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "run: ok" in r.stdout
    assert "chain_bit_equal=1" in r.stdout
