"""Runs the reference's own generated FFT kernels on the host to produce the
golden vectors of tests/golden/vectors.npz (test infrastructure only).

For each case the reference (imported from a local checkout, dummy backend,
CUDA code generator, GB300 limits) builds its kernel exactly as
vd.fft.fft / convolve would (vkdispatch/fft/shader_factories.py:11-60,
107-195); the emitted CUDA source is compiled with g++ against
oracle/shim/cuda_runtime.h into oracle/_ref/ (git-ignored) and launched over
its own grid on seeded inputs.  Only inputs and outputs are kept.
"""


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


def _params(src: str):
    """The generated kernel's parameters: ("ubo", None) for the uniform
    struct, ("buf", type) for each buffer pointer, in order."""
    m = re.search(r"vkdispatch_main\(([^)]*)\)", src)
    out = []
    for p in m.group(1).split(","):
        p = p.strip()
        if "UniformObjectBuffer" in p:
            out.append(("ubo", None))
        else:
            out.append(("buf", p.rsplit(" ", 1)[0].strip()))
    return out


def _compile(name: str, src: str, nbuf: int) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    params = _params(src)
    args, b = [], 0
    for kind, typ in params:
        if kind == "ubo":
            args.append("u")
        else:
            args.append(f"({typ})bufs[{b}]")
            b += 1
    assert b == nbuf, (name, b, nbuf)
    has_ubo = any(k == "ubo" for k, _ in params)
    ubo = "  UniformObjectBuffer u;\n  std::memcpy(&u, ubo, sizeof(u));\n" if has_ubo else "  (void)ubo;\n"
    driver = (
        src
        + '\n#include "launch.h"\n'
        + 'extern "C" void vdx_run(void** bufs, const void* ubo, unsigned gx, unsigned gy, unsigned gz, unsigned bx, '
        + "unsigned by, unsigned bz) {\n"
        + ubo
        + f"  vdx_shim::run_grid(dim3{{gx, gy, gz}}, dim3{{bx, by, bz}}, [&] {{ vkdispatch_main({', '.join(args)}); }});\n"
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


def _run(so: Path, arrays, local, exec_size, ubo: bytes = b""):
    """Launches over the reference's own grid: ceil(exec_size / local) CTAs."""
    lib = ctypes.CDLL(str(so))
    lib.vdx_run.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p] + [ctypes.c_uint] * 6
    ptrs = (ctypes.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
    grid = [(exec_size[i] + local[i] - 1) // local[i] for i in range(3)]
    lib.vdx_run(ptrs, ubo or b"\0" * 64, *grid, *local)


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


# ---------------------------------------------------------------------------
# Config-shape cases: the benchmark configurations' lengths and stride
# classes.  Inputs come from oracle/inputs.py (regenerated at test time, not
# stored); large outputs are kept at sampled flat indices only.
# ---------------------------------------------------------------------------
def _fft_shader(vd, shape, axis, kind, sr=None):
    from vkdispatch.fft.shader_factories import make_fft_shader

    r2c = kind in ("rfft", "irfft")
    return make_fft_shader(tuple(shape), axis, inverse=kind in ("ifft", "irfft"), normalize_inverse=True, r2c=r2c,
                           output_type=vd.complex64, input_type=vd.complex64, compute_type=vd.complex64,
                           input_signal_range=sr)


def _launch(vd, name, sh, bufs, ubo=b""):
    src = str(sh)
    nbuf = sum(1 for k, _ in _params(src) if k == "buf")
    so = _compile(name, src, nbuf)
    _run(so, bufs, tuple(sh.local_size), tuple(sh.exec_size), ubo)


def _reduce_stage_ubo(exec_limits, fields):
    """UniformObjectBuffer of a reduction stage: exec_count (uvec4: the exec
    limits and 0) then the nine ReductionParams fields in declaration order
    (vkdispatch/reduce/stage.py:9-20)."""
    import struct

    return struct.pack("<4I9I", exec_limits[0], exec_limits[1], exec_limits[2], 0, *fields) + b"\0" * 12


def _reference_reduce(vd, name, rf, data, batch, out_dtype):
    """Runs a reference ReduceFunction's two generated stages the way
    ReduceFunction.__call__ launches them (reduce_function.py:73-162); returns
    its output buffer (results first, then the stage-1 partials)."""
    rf.make_stages()
    group = rf.group_size
    n = data.size // batch
    wx = min(-(-n // group), group)
    out = np.zeros((wx + 1) * batch, dtype=out_dtype)
    src1, src2 = rf.get_src()
    p1 = (0, n, 1, n, 0, batch, 1, wx, 0)
    so1 = _compile(name + "_s1", str(src1), 2)
    _run(so1, [out, data], (group, 1, 1), (wx * group, batch, 1), _reduce_stage_ubo((wx * group, batch, 1), p1))
    p2 = (batch, wx, 1, wx, 0, 0, 1, 1, 0)
    so2 = _compile(name + "_s2", str(src2), 1)
    _run(so2, [out], (group, 1, 1), (group, batch, 1), _reduce_stage_ubo((group, batch, 1), p2))
    return out


def make_config_vectors(ref_root, out_path, limits) -> None:
    vd = _import_reference(ref_root, limits)
    import vkdispatch.codegen as vc
    from vkdispatch.fft.shader_factories import make_convolution_shader

    from . import inputs

    store, meta = {}, {}

    def keep(name, arr, seed):
        flat = np.ascontiguousarray(arr).reshape(-1)
        if flat.size <= 8192:
            store[name] = flat.copy()
            meta[name] = {"full": True}
        else:
            idx = inputs.sample_indices(seed, flat.size)
            store[name + "__idx"] = idx
            store[name] = flat[idx].copy()
            meta[name] = {"full": False, "size": int(flat.size), "norm": float(np.linalg.norm(flat.astype(
                np.complex128 if np.iscomplexobj(flat) else np.float64)))}

    # Cfg1: 256 x 1024 complex64, forward then inverse, then the magnitude sum
    x = inputs.complex_uniform(101, (256, 1024))
    buf = x.copy()
    _launch(vd, "cfg1_fwd", _fft_shader(vd, (256, 1024), None, "fft"), [buf])
    keep("cfg1_fwd", buf, 1)
    _launch(vd, "cfg1_inv", _fft_shader(vd, (256, 1024), None, "ifft"), [buf])
    keep("cfg1_inv", buf, 2)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def mag(b: vc.Buffer[vd.complex64]) -> vd.float32:
        v = b[vd.reduce.mapped_io_index()]
        return vc.sqrt(v.real * v.real + v.imag * v.imag)

    store["cfg1_magsum"] = _reference_reduce(vd, "cfg1_magsum", mag, buf.reshape(-1), 1, np.float32)
    meta["cfg1_magsum"] = {"full": True, "input": "cfg1_inv output (full, in the reference's own bits)"}

    # 512-point R2C / C2R rows (Cfg2's row passes), 8 rows
    xr = inputs.uniform(102, (8, 512))
    packed = np.zeros((8, 2 * 257), dtype=np.float32)
    packed[:, :512] = xr
    pk = packed.view(np.complex64).copy()
    _launch(vd, "r2c_8x512", _fft_shader(vd, (8, 512), None, "rfft"), [pk])
    keep("r2c_8x512", pk, 3)
    spec = inputs.complex_uniform(103, (8, 257))
    sp = spec.copy()
    _launch(vd, "c2r_8x512", _fft_shader(vd, (8, 512), None, "irfft"), [sp])
    keep("c2r_8x512", sp.view(np.float32)[:, :512], 4)

    # Cfg2's strided convolution: 2 x 512 x 257 complex64 along axis 1
    xs = inputs.complex_uniform(104, (2, 512, 257))
    ks = inputs.complex_uniform(105, (2, 512, 257))
    cb = xs.copy()
    sh = make_convolution_shader((2, 512, 257), None, 1, 1, output_type=vd.complex64, input_type=vd.complex64,
                                 kernel_type=vd.complex64, compute_type=vd.complex64)
    _launch(vd, "conv_2x512x257_ax1", sh, [cb, ks])
    keep("conv_2x512x257_ax1", cb, 5)

    # a 3-D transform: 32^3, axes 0, 1, 2 (vkdispatch/fft/functions.py fft3 order)
    x3 = inputs.complex_uniform(106, (32, 32, 32))
    b3 = x3.copy()
    for ax in (0, 1, 2):
        _launch(vd, f"fft3_32_ax{ax}", _fft_shader(vd, (32, 32, 32), ax, "fft"), [b3])
    keep("fft3_32", b3, 6)

    # integer reductions: xor over uint32, and over int32 (3 rows of 100003)
    u = inputs.uint32(107, (3 * 100003,))

    @vd.reduce.reduce(0, axes=[1])
    def xor_u(a: vd.uint32, b: vd.uint32) -> vd.uint32:
        return a ^ b

    # a ReduceFunction over axes [1] of a (3, 100003) buffer: 3 rows
    store["xor_u32_3x100003"] = _reference_reduce(vd, "xor_u32", xor_u, u, 3, np.uint32)
    meta["xor_u32_3x100003"] = {"full": True}
    i = inputs.uint32(109, (3 * 100003,)).view(np.int32) | np.int32(0x10204081)  # keep some bits set

    @vd.reduce.reduce(-1, axes=[1])
    def and_i(a: vd.int32, b: vd.int32) -> vd.int32:
        return a & b

    # (the reference's vc.min returns float32 for int32 operands, so an
    # integer min reduction cannot be written against it; AND is pinned)
    store["and_i32_3x100003"] = _reference_reduce(vd, "and_i32", and_i, i, 3, np.int32)
    meta["and_i32_3x100003"] = {"full": True}

    # a float sum over 3 rows (order-dependent: pins the restatement's order)
    f = inputs.uniform(108, (3 * 300001,))

    @vd.reduce.reduce(0, axes=[1])
    def sum_f(a: vd.float32, b: vd.float32) -> vd.float32:
        return a + b

    store["sum_f32_3x300001"] = _reference_reduce(vd, "sum_f32", sum_f, f, 3, np.float32)
    meta["sum_f32_3x300001"] = {"full": True}

    store["__meta__"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(out_path, **store)
    print(f"wrote {out_path}")
