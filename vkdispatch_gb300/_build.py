"""Builds libvdx.so in-tree from csrc/*.cu with nvcc for sm_103a.

Translation units compile in parallel into ``_build/`` and link into
``vkdispatch_gb300/libvdx.so`` (both git-ignored).  Objects are rebuilt when
their source or any header is newer.  The kernel headers that the run-time
compiled map kernels include (JIT_HEADERS) are embedded into
``_build/jit_headers.inc`` as string literals for jit.cu.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
INCLUDE = REPO_DIR / "include"
BUILD_DIR = REPO_DIR / "_build"
LIB_PATH = PKG_DIR / "libvdx.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC",
    f"-I{INCLUDE}",
    f"-I{CSRC}",
    f"-I{BUILD_DIR}",
]

# headers NVRTC compiles the map kernels from (csrc/jit.cu), in include order
JIT_HEADERS = ("vdx_common.cuh", "fft_kernels.cuh", "fft_mapped.cuh", "reduce_mapped.cuh")


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvdx")


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(nvcc: str, src: Path, obj: Path, verbose: bool) -> None:
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")


def _write_jit_headers() -> None:
    """_build/jit_headers.inc: the JIT_HEADERS as C++ raw string literals
    (rewritten only when their text changes)."""
    names, bodies = [], []
    for h in JIT_HEADERS:
        text = (CSRC / h).read_text()
        delim = "VDXJIT"
        assert f"){delim}\"" not in text
        names.append(f'"{h}"')
        bodies.append(f'R"{delim}({text}){delim}"')
    inc = ("// generated by vkdispatch_gb300/_build.py from csrc/" + ", ".join(JIT_HEADERS) + "\n"
           f"static const int kJitHeaderCount = {len(JIT_HEADERS)};\n"
           "static const char* const kJitHeaderNames[] = {" + ", ".join(names) + "};\n"
           "static const char* const kJitHeaderSources[] = {\n" + ",\n".join(bodies) + "};\n")
    out = BUILD_DIR / "jit_headers.inc"
    if not out.exists() or out.read_text() != inc:
        out.write_text(inc)


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    _write_jit_headers()
    srcs = sorted(CSRC.glob("*.cu"))
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for src in srcs:
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr):
            jobs.append((src, obj))
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = [ex.submit(_compile, nvcc, s, o, verbose) for s, o in jobs]
            for f in futs:
                f.result()
    newest = max(o.stat().st_mtime for o in objs)
    if force or jobs or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < newest:
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs), "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libvdx.so failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
