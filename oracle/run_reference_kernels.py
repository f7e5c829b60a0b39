"""Runs the reference's own generated FFT kernels on the host to produce the
golden vectors of tests/golden/vectors.npz (test infrastructure only).

For each case the reference (imported from a local checkout, dummy backend,
CUDA code generator, GB300 limits) builds its kernel exactly as
vd.fft.fft / convolve would (vkdispatch/fft/shader_factories.py:11-60,
107-195); the emitted CUDA source is compiled with g++ against
oracle/shim/cuda_runtime.h into oracle/_ref/ (git-ignored) and launched over
its own grid on seeded inputs.  Only inputs and outputs are kept.
"""

from __future__ import annotations

import ctypes
import json
import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SHIM = HERE / "shim"
OUT_DIR = HERE / "_ref"


def _cases():
    # name, kind, shape, axis, extra
    return [
        ("c2c_fwd_7x1024", "fft", (7, 1024), None, {}),
        ("c2c_inv_7x1024", "ifft", (7, 1024), None, {}),
        ("c2c_fwd_3x162", "fft", (3, 162), None, {}),
        ("c2c_fwd_4x243", "fft", (4, 243), None, {}),
        ("c2c_fwd_2x1000", "fft", (2, 1000), None, {}),
        ("c2c_fwd_5x13", "fft", (5, 13), None, {}),
        ("c2c_fwd_2x2048", "fft", (2, 2048), None, {}),
        ("c2c_fwd_6x48x7_ax1", "fft", (6, 48, 7), 1, {}),
        ("c2c_fwd_13x11_ax0", "fft", (13, 11), 0, {}),
        ("c2c_inv_4x8x26_ax1", "ifft", (4, 8, 26), 1, {}),
        ("c2c_sig_5x64", "fft", (5, 64), None, {"signal_range": (3, 40)}),
        ("r2c_5x64", "rfft", (5, 64), None, {}),
        ("r2c_3x45", "rfft", (3, 45), None, {}),
        ("r2c_sig_4x100", "rfft", (4, 100), None, {"signal_range": (10, 77)}),
        ("c2r_5x64", "irfft", (5, 64), None, {}),
        ("c2r_3x45", "irfft", (3, 45), None, {}),
        ("conv_6x48x7_ax1", "conv", (6, 48, 7), 1, {}),
        ("conv_4x64", "conv", (4, 64), None, {}),
        ("conv_2x12x33_ax1", "conv", (2, 12, 33), 1, {}),
    ]


def _import_reference(ref_root, limits):
    sys.path.insert(0, str(ref_root))
    import vkdispatch as vd
    import vkdispatch.codegen as vc

    vd.initialize(backend="dummy")
    vc.set_codegen_backend("cuda")
    vd.set_dummy_context_params(**limits)
    return vd


def _compile(name: str, src: str, nbuf: int) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    args = ", ".join(f"(vkdispatch_float2*)bufs[{i}]" for i in range(nbuf))
    driver = (
        src
        + '\n#include "launch.h"\n'
        + 'extern "C" void vdx_run(void** bufs, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by, '
        + "unsigned bz) {\n"
        + f"  vdx_shim::run_grid(dim3{{gx, gy, gz}}, dim3{{bx, by, bz}}, [&] {{ vkdispatch_main({args}); }});\n"
        + "}\n"
    )
    cpp = OUT_DIR / f"{name}.cpp"
    so = OUT_DIR / f"{name}.so"
    cpp.write_text(driver)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    cmd = [cxx, "-std=c++20", "-O1", "-ffp-contract=off", "-fPIC", "-shared", f"-I{SHIM}", "-o", str(so), str(cpp),
           "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on {name}:\n{r.stderr[:4000]}")
    return so


def _run(so: Path, arrays, local, exec_size):
    lib = ctypes.CDLL(str(so))
    lib.vdx_run.argtypes = [ctypes.POINTER(ctypes.c_void_p)] + [ctypes.c_uint] * 6
    ptrs = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
    grid = [exec_size[i] // local[i] for i in range(3)]
    for i in range(3):
        assert grid[i] * local[i] == exec_size[i], (exec_size, local)
    lib.vdx_run(ptrs, *grid, *local)


def make_vectors(ref_root, out_path, limits) -> None:
    vd = _import_reference(ref_root, limits)
    from vkdispatch.fft.shader_factories import make_convolution_shader, make_fft_shader

    store = {}
    meta = {}
    for idx, (name, kind, shape, axis, extra) in enumerate(_cases()):
        rng = np.random.default_rng(1000 + idx)
        sr = extra.get("signal_range")
        if kind in ("fft", "ifft"):
            sh = make_fft_shader(tuple(shape), axis, inverse=(kind == "ifft"), normalize_inverse=True,
                                 output_type=vd.complex64, input_type=vd.complex64, compute_type=vd.complex64,
                                 input_signal_range=sr)
            x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
            bufs = [x.copy()]
        elif kind in ("rfft", "irfft"):
            sh = make_fft_shader(tuple(shape), None, inverse=(kind == "irfft"), normalize_inverse=True, r2c=True,
                                 output_type=vd.complex64, input_type=vd.complex64, compute_type=vd.complex64,
                                 input_signal_range=sr)
            n = shape[-1]
            h = n // 2 + 1
            if kind == "rfft":
                xr = rng.uniform(-1, 1, shape).astype(np.float32)
                packed = np.zeros(shape[:-1] + (2 * h,), dtype=np.float32)
                packed[..., :n] = xr
                x = packed.view(np.complex64)
            else:
                x = (rng.standard_normal(shape[:-1] + (h,)) + 1j * rng.standard_normal(shape[:-1] + (h,))).astype(
                    np.complex64)
            bufs = [np.ascontiguousarray(x).copy()]
        else:  # conv
            sh = make_convolution_shader(tuple(shape), None, 1, axis, output_type=vd.complex64,
                                         input_type=vd.complex64, kernel_type=vd.complex64,
                                         compute_type=vd.complex64)
            x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
            k = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
            bufs = [x.copy(), k]
        src = str(sh)
        m = re.search(r"vkdispatch_main\(([^)]*)\)", src)
        nbuf = m.group(1).count("vkdispatch_binding_")
        assert nbuf == len(bufs), (name, nbuf, len(bufs))
        so = _compile(name, src, nbuf)
        _run(so, bufs, tuple(sh.local_size), tuple(sh.exec_size))
        store[f"{name}__in"] = x
        store[f"{name}__out"] = bufs[0]
        if kind == "conv":
            store[f"{name}__kernel"] = bufs[1]
        meta[name] = {"kind": kind, "shape": list(shape), "axis": axis, "signal_range": sr,
                      "local_size": list(sh.local_size), "exec_size": list(sh.exec_size)}
        print(f"{name}: local {sh.local_size} exec {sh.exec_size}", flush=True)
    store["__meta__"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(out_path, **store)
    print(f"wrote {out_path}")
