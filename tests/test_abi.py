"""CPU tests of the C ABI boundary: libvdx.so loads, exports every entry
point include/vdx.h declares, constants and struct layout agree with the
Python binding, and host-side validation rejects bad arguments before any
CUDA call."""

import ctypes
import re
from pathlib import Path

import pytest

from vkdispatch_gb300 import _lib as L

HEADER = Path(__file__).resolve().parent.parent / "include" / "vdx.h"


def _declared():
    src = HEADER.read_text()
    return sorted(set(re.findall(r"^int\s+(vdx_\w+)\s*\(", src, flags=re.M)))


def _defines():
    src = HEADER.read_text()
    return {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(VDX_\w+)\s+(\d+)", src)}


def test_library_exports_every_declared_symbol():
    lib = L.lib()
    names = _declared()
    assert len(names) >= 9
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(L.EXPORTED) | {n for n in names if hasattr(lib, n)}


def test_constants_match_header():
    d = _defines()
    for k, v in d.items():
        if hasattr(L, k):
            assert getattr(L, k) == v, k


def test_desc_struct_layout():
    # int32 ndim, int64 shape[4], int32 axis..compute_type, int64 lo, hi, 4 x int32
    assert ctypes.sizeof(L.FftDesc) == 8 + 32 + 5 * 4 + 4 + 16 + 16
    assert L.FftDesc.shape.offset == 8
    assert L.FftDesc.signal_lo.offset == 64


def test_version_and_last_error():
    lib = L.lib()
    assert lib.vdx_version() >= 100
    rc = lib.vdx_fft_plan_create(None, None)
    assert rc == L.VDX_ERR_INVALID
    assert "non-NULL" in L.last_error()


@pytest.mark.parametrize(
    "field,value",
    [("ndim", 0), ("ndim", 5), ("axis", 3), ("kind", 9), ("io_type", 7), ("compute_type", 4)],
)
def test_plan_validation_without_gpu(field, value):
    d = L.FftDesc()
    d.ndim = 2
    d.shape[0], d.shape[1] = 4, 64
    d.axis = 1
    d.io_type = L.VDX_C64
    d.compute_type = L.VDX_C64
    d.signal_lo = d.signal_hi = -1
    setattr(d, field, value)
    h = ctypes.c_void_p()
    rc = L.lib().vdx_fft_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == L.VDX_ERR_INVALID
    assert not h.value
    with pytest.raises(ValueError):
        L.check(rc, "plan")


def test_real_transform_needs_last_axis():
    d = L.FftDesc()
    d.ndim = 2
    d.shape[0], d.shape[1] = 4, 64
    d.axis = 0
    d.kind = L.VDX_KIND_R2C
    d.io_type = d.compute_type = L.VDX_C64
    h = ctypes.c_void_p()
    assert L.lib().vdx_fft_plan_create(ctypes.byref(d), ctypes.byref(h)) == L.VDX_ERR_INVALID
    assert "last" in L.last_error()


def test_reduce_validation_without_gpu():
    lib = L.lib()
    parts = ctypes.c_int64()
    assert lib.vdx_reduce_partial_count(300000, ctypes.byref(parts)) == 0
    assert 1 <= parts.value <= 1024
    # bitwise op on floats is rejected before any launch
    rc = lib.vdx_reduce(L.VDX_RED_XOR, 0, L.VDX_F32, 1, 10, 1, 1, 1, None)
    assert rc == L.VDX_ERR_INVALID
    rc = lib.vdx_reduce(L.VDX_RED_ADD, L.VDX_MAP_IDENTITY, L.VDX_C64, 1, 10, 1, 1, 1, None)
    assert rc == L.VDX_ERR_INVALID and "map" in L.last_error()


def test_reduce_noalloc_size_limit_without_gpu():
    """A request whose stage-1 partials exceed the static scratch array is
    refused before any CUDA call: dummy non-null pointers never reach a
    device."""
    lib = L.lib()
    parts = ctypes.c_int64()
    n = 4096 * 1024
    assert lib.vdx_reduce_partial_count(n, ctypes.byref(parts)) == 0
    batch = L.VDX_REDUCE_NOALLOC_SCRATCH_BYTES // (4 * parts.value) + 1
    rc = lib.vdx_reduce_noalloc(L.VDX_RED_ADD, L.VDX_MAP_IDENTITY, L.VDX_F32, 1, n, batch, 1, None)
    assert rc == L.VDX_ERR_UNSUPPORTED
    assert "static scratch" in L.last_error()
    # argument checks come first as well
    assert lib.vdx_reduce_noalloc(L.VDX_RED_XOR, 0, L.VDX_F32, 1, 10, 1, 1, None) == L.VDX_ERR_INVALID


def test_multi_kernel_and_batch_validation_without_gpu():
    """Host-side argument checks of the newer entry points return a status
    before touching the device."""
    lib = L.lib()
    assert lib.vdx_conv_exec_multi(None, None, None, None, 2, 0, 0, None) == L.VDX_ERR_INVALID
    assert "plan" in L.last_error()
    assert lib.vdx_batch_plan_create(None, 0, 0, 1, None) == L.VDX_ERR_INVALID
    ws = ctypes.c_size_t()
    assert lib.vdx_batch_workspace_bytes(None, ctypes.byref(ws)) == L.VDX_ERR_INVALID


def _conv2d_groups_desc(shape=(8, 64, 64)):
    d = L.FftDesc()
    d.ndim = 3
    for i, x in enumerate(shape):
        d.shape[i] = x
    d.axis = 1
    d.kind = L.VDX_KIND_CONV2D_REAL
    d.normalize = 1
    d.io_type = d.compute_type = L.VDX_C64
    d.signal_lo = d.signal_hi = -1
    return d


@pytest.mark.parametrize(
    "field,value,groups",
    [("kind", 3, 2), ("ndim", 2, 2), ("axis", 2, 2), ("io_type", 2, 2), ("flags", 1, 2), (None, None, 0),
     (None, None, 9), ("shape", (8, 64, 63), 2), ("shape", (0, 64, 64), 2)],
)
def test_conv2d_groups_validation_without_gpu(field, value, groups):
    """vdx_conv2d_groups_plan_create checks the descriptor and group count
    before any CUDA call and leaves the handle NULL."""
    d = _conv2d_groups_desc(value if field == "shape" else (8, 64, 64))
    if field not in (None, "shape"):
        setattr(d, field, value)
    h = ctypes.c_void_p()
    rc = L.lib().vdx_conv2d_groups_plan_create(ctypes.byref(d), groups, ctypes.byref(h))
    assert rc in (L.VDX_ERR_INVALID, L.VDX_ERR_UNSUPPORTED), L.last_error()
    assert not h.value
    lib = L.lib()
    assert lib.vdx_conv2d_groups_exec(None, None, None, None) == L.VDX_ERR_INVALID
    assert lib.vdx_conv2d_groups_plan_describe(None, None, 0) == L.VDX_ERR_INVALID
    assert lib.vdx_conv2d_groups_plan_destroy(None) == L.VDX_OK


def _group_steps(specs):
    arr = (L.FftDesc * len(specs))()
    for d, (shape, axis, kind) in zip(arr, specs):
        d.ndim = len(shape)
        for i, x in enumerate(shape):
            d.shape[i] = x
        d.axis = axis
        d.kind = kind
        d.io_type = d.compute_type = L.VDX_C64
        d.signal_lo = d.signal_hi = -1
    return arr


@pytest.mark.parametrize(
    "specs,groups",
    [
        ([], 2),  # no steps
        ([((8, 64, 64), 1, L.VDX_KIND_C2C)] * 5, 2),  # more than 4 steps
        ([((8, 64, 64), 1, L.VDX_KIND_C2C)], 0),  # group count
        ([((8, 64, 64), 0, L.VDX_KIND_C2C)], 2),  # axis 0 runs across images
        ([((8, 64, 64), 1, L.VDX_KIND_CONV2D_REAL)], 2),  # not a per-image step
        ([((8, 64, 64), 2, L.VDX_KIND_R2C), ((8, 64, 64), 1, L.VDX_KIND_C2C)], 2),  # 33 vs 64 columns
        ([((8, 64, 64), 1, L.VDX_KIND_C2C), ((4, 64, 64), 2, L.VDX_KIND_C2C)], 2),  # image counts differ
        ([((8, 64, 63), 2, L.VDX_KIND_R2C)], 2),  # odd real width
        ([((64, 64), 1, L.VDX_KIND_C2C)], 2),  # not a batch of images
    ],
)
def test_group_plan_validation_without_gpu(specs, groups):
    """vdx_group_plan_create refuses malformed chains before any CUDA call."""
    arr = _group_steps(specs) if specs else None
    h = ctypes.c_void_p()
    rc = L.lib().vdx_group_plan_create(arr, len(specs), groups, ctypes.byref(h))
    assert rc == L.VDX_ERR_INVALID, L.last_error()
    assert not h.value
    assert L.lib().vdx_group_exec(None, None, None, None) == L.VDX_ERR_INVALID
    assert L.lib().vdx_group_plan_describe(None, None, 0) == L.VDX_ERR_INVALID
    assert L.lib().vdx_group_plan_destroy(None) == L.VDX_OK


def test_every_entry_point_cites_the_reference():
    """Each declaration of include/vdx.h sits under a comment that names the
    reference interface it replaces (a vkdispatch/ file) or says it has no
    counterpart there."""
    src = HEADER.read_text()
    last = ""
    missing = []
    for part in re.split(r"(/\*.*?\*/)", src, flags=re.S):
        if part.startswith("/*"):
            last = part
            continue
        for m in re.finditer(r"^int\s+(vdx_\w+)\s*\(", part, flags=re.M):
            if "vkdispatch/" not in last and "counterpart" not in last.lower():
                missing.append(m.group(1))
    assert not missing, missing


@pytest.mark.parametrize("lang", ["c99", "c++11"])
def test_header_compiles_as_strict_c_and_cpp(tmp_path, lang):
    """A cgo, JNI or C++ host includes include/vdx.h as is: it compiles as
    C99 and as C++11 with every warning an error."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c99" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / "t.c"
    src.write_text('#include "vdx.h"\nint main(void) { vdx_fft_desc d; vdx_batch_item b; (void)d; (void)b; '
                   'return 0; }\n')
    cmd = [cc, f"-std={lang}", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", str(HEADER.parent), "-c", str(src),
           "-o", str(tmp_path / "t.o")]
    if lang != "c99":
        cmd[1:1] = ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
