"""Generates the reference's own CUDA kernels for the benchmark workloads, as
its CUDA backend would build and launch them, so that a GB300 run can time
them beside libvdx (a comparator only: nothing here enters the product).

The reference (sharhar/vkdispatch, imported from a checkout named by the
VKDISPATCH_REFERENCE environment variable; dummy backend, CUDA code
generator, the device limits its CUDA backend reports on a GB300) emits each
kernel exactly as vd.fft.* / vd.reduce would (vkdispatch/fft/
shader_factories.py:11-60, 107-195; vkdispatch/reduce/stage.py:147-186).
Each source is written to baseline/_ref_kernels/<name>.cu (git-ignored)
with an extern "C" launcher appended, and kernels.json records its launch
(the reference's local size and exec size; grid = ceil(exec / local), as in
vkdispatch/shader/shader_function.py:106-121).  build() compiles every
source with nvcc for sm_103, the architecture option the reference's NVRTC
call passes (vkdispatch/backends/cuda_backend/api_compute.py:17-27).

    VKDISPATCH_REFERENCE=<checkout> python baseline/make_reference_kernels.py
"""

import json
import os
import re
import shutil
import struct
import subprocess
import sys
from concurrent import futures
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref_kernels"

GB300_LIMITS = dict(
    subgroup_size=32,
    max_workgroup_size=(1024, 1024, 64),
    max_workgroup_invocations=1024,
    max_workgroup_count=(2**31 - 1, 65535, 65535),
    max_shared_memory=48 * 1024,
)


def _params(src):
    m = re.search(r"vkdispatch_main\(([^)]*)\)", src)
    out = []
    for p in m.group(1).split(","):
        p = p.strip()
        out.append(("ubo", None) if "UniformObjectBuffer" in p else ("buf", p.rsplit(" ", 1)[0].strip()))
    return out


def _launcher(name, src):
    params = _params(src)
    args, b = [], 0
    for kind, typ in params:
        if kind == "ubo":
            args.append("u")
        else:
            args.append(f"({typ})bufs[{b}]")
            b += 1
    ubo = any(k == "ubo" for k, _ in params)
    body = ("  UniformObjectBuffer u;\n  memcpy(&u, ubo, sizeof(u));\n" if ubo else "  (void)ubo;\n")
    return b, ubo, (
        src
        + "\n#include <string.h>\n"
        + f'extern "C" int vdref_launch(void** bufs, const void* ubo, unsigned gx, unsigned gy, unsigned gz, '
        + "unsigned bx, unsigned by, unsigned bz, void* stream) {\n"
        + body
        + f"  vkdispatch_main<<<dim3(gx, gy, gz), dim3(bx, by, bz), 0, (cudaStream_t)stream>>>({', '.join(args)});\n"
        + "  return (int)cudaGetLastError();\n}\n"
    )


def _reduce_ubo(exec_limits, fields):
    """exec_count (the exec limits and 0) then the nine ReductionParams
    fields in declaration order (vkdispatch/reduce/stage.py:9-20)."""
    return list(struct.pack("<4I9I", exec_limits[0], exec_limits[1], exec_limits[2], 0, *fields) + b"\0" * 12)


def generate(ref_root):
    sys.path.insert(0, str(ref_root))
    import vkdispatch as vd
    import vkdispatch.codegen as vc
    from vkdispatch.fft.shader_factories import make_convolution_shader, make_fft_shader

    vd.initialize(backend="dummy")
    vc.set_codegen_backend("cuda")
    vd.set_dummy_context_params(**GB300_LIMITS)
    OUT.mkdir(exist_ok=True)
    table = {}

    def add(name, src, local, exec_size, ubo_bytes=None, note=""):
        nbuf, has_ubo, text = _launcher(name, str(src))
        (OUT / f"{name}.cu").write_text(text)
        grid = [(exec_size[i] + local[i] - 1) // local[i] for i in range(3)]
        table[name] = {"local": list(local), "exec": list(exec_size), "grid": grid, "nbuf": nbuf,
                       "ubo": ubo_bytes if has_ubo else None, "note": note}

    def fft(name, shape, axis, inverse=False, r2c=False):
        try:
            sh = make_fft_shader(tuple(shape), axis, inverse=inverse, normalize_inverse=True, r2c=r2c,
                                 output_type=vd.complex64, input_type=vd.complex64, compute_type=vd.complex64)
        except Exception as e:  # noqa: BLE001 - the reference's planner rejects the length
            table[name] = {"unavailable": f"plan error: {str(e).splitlines()[0][:160]}"}
            return
        add(name, sh, tuple(sh.local_size), tuple(sh.exec_size))

    def conv(name, shape, axis):
        sh = make_convolution_shader(tuple(shape), None, 1, axis, output_type=vd.complex64,
                                     input_type=vd.complex64, kernel_type=vd.complex64,
                                     compute_type=vd.complex64)
        add(name, sh, tuple(sh.local_size), tuple(sh.exec_size))

    # the 2-D convolution workload (convolve2DR on 64 x 512 x 512 real images)
    fft("cfg2_rfft", (64, 512, 512), None, r2c=True)
    conv("cfg2_conv", (64, 512, 257), 1)
    fft("cfg2_irfft", (64, 512, 512), None, inverse=True, r2c=True)
    # the plain C2C workload, as specified and at HBM scale
    fft("cfg1_fft", (256, 1024), None)
    fft("cfg1_ifft", (256, 1024), None, inverse=True)
    fft("cfg1_hbm_fft", (262144, 1024), None)
    fft("cfg1_hbm_ifft", (262144, 1024), None, inverse=True)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def mag(b: vc.Buffer[vd.complex64]) -> vd.float32:
        v = b[vd.reduce.mapped_io_index()]
        return vc.sqrt(v.real * v.real + v.imag * v.imag)

    mag.make_stages()
    src1, src2 = mag.get_src()
    n, g = 256 * 1024, mag.group_size
    wx = min(-(-n // g), g)
    add("cfg1_magsum_s1", src1, (g, 1, 1), (wx * g, 1, 1), _reduce_ubo((wx * g, 1, 1), (0, n, 1, n, 0, 1, 1, wx, 0)))
    add("cfg1_magsum_s2", src2, (g, 1, 1), (g, 1, 1), _reduce_ubo((g, 1, 1), (1, wx, 1, wx, 0, 0, 1, 1, 0)))
    # the 3-D convolution workload's forward pass (256^3, reference schedule)
    fft("cfg3_fft_ax0", (256, 256, 256), 0)
    fft("cfg3_fft_ax1", (256, 256, 256), 1)
    conv("cfg3_conv_ax2", (256, 256, 256), 2)
    fft("cfg3_ifft_ax1", (256, 256, 256), 1, inverse=True)
    fft("cfg3_ifft_ax0", (256, 256, 256), 0, inverse=True)
    # the mixed-precision workload's 16384-point axes (complex64 storage)
    fft("cfg5_fft_ax0", (16384, 16384), 0)
    fft("cfg5_fft_ax1", (16384, 16384), 1)
    (OUT / "kernels.json").write_text(json.dumps(table, indent=1))
    print(f"wrote {len(table)} kernels to {OUT}")


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def build():
    """Compiles every generated source into baseline/_ref_kernels/<name>.so;
    a source that does not compile (e.g. more static shared memory than a
    CTA may declare) is recorded as unavailable in built.json."""
    table_path = OUT / "kernels.json"
    if not table_path.exists():
        return None
    table = json.loads(table_path.read_text())
    nvcc = _nvcc()

    def one(name):
        src, so = OUT / f"{name}.cu", OUT / f"{name}.so"
        if so.exists() and so.stat().st_mtime >= src.stat().st_mtime:
            return name, None
        cmd = [nvcc, "-arch=sm_103", "-w", "-O3", "-Xcompiler", "-fPIC", "-shared", "-o", str(so), str(src)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return name, (r.stderr.strip().splitlines() or ["nvcc failed"])[-1][:200]
        return name, None

    names = [k for k, v in table.items() if "unavailable" not in v]
    status = {}
    with futures.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for name, err in ex.map(one, names):
            status[name] = err
    (OUT / "built.json").write_text(json.dumps(status, indent=1))
    return status


if __name__ == "__main__":
    ref = os.environ.get("VKDISPATCH_REFERENCE")
    if not ref:
        sys.exit("set VKDISPATCH_REFERENCE to the reference checkout")
    generate(ref)
    if "--build" in sys.argv:
        print(build())
