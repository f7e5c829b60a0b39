"""ctypes binding of libvdx.so (declared in include/vdx.h).

The library is required: there is no CPU or PyTorch fallback.  Loading fails
with an explicit error when the in-tree build is missing.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libvdx.so"

VDX_OK = 0
VDX_ERR_INVALID = 1
VDX_ERR_UNSUPPORTED = 2
VDX_ERR_CUDA = 3
VDX_ERR_NOMEM = 4

# element types
VDX_C64, VDX_C32, VDX_C128, VDX_BF16X2, VDX_F32, VDX_F64, VDX_I32, VDX_U32, VDX_V2F32 = range(9)


def convert(src_ptr: int, src_type: int, dst_ptr: int, dst_type: int, count: int, stream: int) -> None:
    check(lib().vdx_convert(src_ptr, src_type, dst_ptr, dst_type, count, stream), "convert")

# transform kinds
VDX_KIND_C2C, VDX_KIND_R2C, VDX_KIND_C2R, VDX_KIND_CONV, VDX_KIND_CONV2D_REAL = range(5)
VDX_KOP_MUL_CONJ, VDX_KOP_MUL = range(2)
VDX_FFT_FLAG_TENSOR_CORE = 1
VDX_FFT_FLAG_AUTOTUNE = 2
VDX_FFT_FLAG_BLUESTEIN = 4

# reductions and maps
VDX_RED_ADD, VDX_RED_MUL, VDX_RED_MIN, VDX_RED_MAX, VDX_RED_AND, VDX_RED_OR, VDX_RED_XOR = range(7)
VDX_MAP_IDENTITY, VDX_MAP_ABS, VDX_MAP_SQUARE, VDX_MAP_REAL, VDX_MAP_IMAG, VDX_MAP_SIN = range(6)

EXPORTED = (
    "vdx_version",
    "vdx_last_error",
    "vdx_device_count",
    "vdx_fft_plan_create",
    "vdx_fft_plan_destroy",
    "vdx_fft_plan_describe",
    "vdx_fft_exec",
    "vdx_reduce_partial_count",
    "vdx_reduce",
    "vdx_reduce_noalloc",
    "vdx_fft_exec_ops",
    "vdx_fft_plan_ctas",
    "vdx_convert",
    "vdx_conv_exec_multi",
    "vdx_batch_plan_create",
    "vdx_batch_plan_destroy",
    "vdx_batch_plan_describe",
    "vdx_batch_workspace_bytes",
    "vdx_batch_exec",
    "vdx_batch_status",
    "vdx_batch_plan_set_wait",
    "vdx_map_plan_create",
    "vdx_map_plan_destroy",
    "vdx_map_exec",
    "vdx_map_plan_source",
    "vdx_map_plan_status",
    "vdx_reduce_map_plan_create",
    "vdx_reduce_map_plan_destroy",
    "vdx_reduce_map_exec",
    "vdx_reduce_map_plan_status",
    "vdx_reduce_map_plan_source",
    "vdx_conv2d_groups_plan_create",
    "vdx_conv2d_groups_plan_destroy",
    "vdx_conv2d_groups_plan_describe",
    "vdx_conv2d_groups_exec",
    "vdx_group_plan_create",
    "vdx_group_plan_destroy",
    "vdx_group_plan_describe",
    "vdx_group_exec",
)
VDX_REDUCE_NOALLOC_SCRATCH_BYTES = 1048576


class FftDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("shape", ctypes.c_int64 * 4),
        ("axis", ctypes.c_int32),
        ("kind", ctypes.c_int32),
        ("inverse", ctypes.c_int32),
        ("normalize", ctypes.c_int32),
        ("io_type", ctypes.c_int32),
        ("compute_type", ctypes.c_int32),
        ("signal_lo", ctypes.c_int64),
        ("signal_hi", ctypes.c_int64),
        ("kernel_op", ctypes.c_int32),
        ("kernel_type", ctypes.c_int32),
        ("kernel_broadcast", ctypes.c_int32),
        ("flags", ctypes.c_int32),
    ]


class ExecOps(ctypes.Structure):
    _fields_ = [
        ("in_weight", ctypes.c_void_p),
        ("in_weight_scale_ptr", ctypes.c_void_p),
        ("in_weight_scale", ctypes.c_float),
        ("spec_scale", ctypes.c_float),
        ("spec_out", ctypes.c_void_p),
        ("spec_aux", ctypes.c_void_p),
        ("loss_weight", ctypes.c_void_p),
        ("loss_partials", ctypes.c_void_p),
    ]


class MapArgs(ctypes.Structure):
    """vdx_map_args: the buffers and scalars a run-time compiled map reads."""

    _fields_ = [
        ("buffers", ctypes.c_void_p * 8),
        ("counts", ctypes.c_int64 * 8),
        ("fscalars", ctypes.c_double * 8),
        ("iscalars", ctypes.c_int64 * 8),
        ("kernel_index", ctypes.c_int64),
    ]


class BatchItem(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_int64), ("length", ctypes.c_int32), ("count", ctypes.c_int32)]


class VdxError(RuntimeError):
    """Raised for CUDA-side failures reported by libvdx."""


_lib = None
_lock = threading.Lock()


def _declare(lib: ctypes.CDLL) -> None:
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
    lib.vdx_version.restype = i32
    lib.vdx_version.argtypes = []
    lib.vdx_last_error.restype = i32
    lib.vdx_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    lib.vdx_device_count.restype = i32
    lib.vdx_device_count.argtypes = [ctypes.POINTER(ctypes.c_int)]
    lib.vdx_fft_plan_create.restype = i32
    lib.vdx_fft_plan_create.argtypes = [ctypes.POINTER(FftDesc), ctypes.POINTER(vp)]
    lib.vdx_fft_plan_destroy.restype = i32
    lib.vdx_fft_plan_destroy.argtypes = [vp]
    lib.vdx_fft_plan_describe.restype = i32
    lib.vdx_fft_plan_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.vdx_fft_exec.restype = i32
    lib.vdx_fft_exec.argtypes = [vp, vp, vp, vp, vp]
    lib.vdx_reduce_partial_count.restype = i32
    lib.vdx_reduce_partial_count.argtypes = [i64, ctypes.POINTER(i64)]
    lib.vdx_reduce.restype = i32
    lib.vdx_reduce.argtypes = [i32, i32, i32, vp, i64, i64, vp, vp, vp]
    lib.vdx_fft_exec_ops.restype = i32
    lib.vdx_fft_exec_ops.argtypes = [vp, vp, vp, vp, ctypes.POINTER(ExecOps), vp]
    lib.vdx_fft_plan_ctas.restype = i32
    lib.vdx_fft_plan_ctas.argtypes = [vp, ctypes.POINTER(i64)]
    lib.vdx_autotune_entries.restype = i32
    lib.vdx_autotune_entries.argtypes = [ctypes.POINTER(i64), ctypes.POINTER(i64)]
    lib.vdx_autotune_save.restype = i32
    lib.vdx_autotune_save.argtypes = [ctypes.c_char_p]
    lib.vdx_autotune_load.restype = i32
    lib.vdx_autotune_load.argtypes = [ctypes.c_char_p]
    lib.vdx_fft_plan_status.restype = i32
    lib.vdx_fft_plan_status.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    lib.vdx_convert.restype = i32
    lib.vdx_convert.argtypes = [vp, i32, vp, i32, i64, vp]
    lib.vdx_conv_exec_multi.restype = i32
    lib.vdx_conv_exec_multi.argtypes = [vp, vp, vp, vp, i32, i64, i64, vp]
    lib.vdx_conv2d_groups_plan_create.restype = i32
    lib.vdx_conv2d_groups_plan_create.argtypes = [ctypes.POINTER(FftDesc), i32, ctypes.POINTER(vp)]
    lib.vdx_conv2d_groups_plan_destroy.restype = i32
    lib.vdx_conv2d_groups_plan_destroy.argtypes = [vp]
    lib.vdx_conv2d_groups_plan_describe.restype = i32
    lib.vdx_conv2d_groups_plan_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.vdx_conv2d_groups_exec.restype = i32
    lib.vdx_conv2d_groups_exec.argtypes = [vp, vp, vp, vp]
    lib.vdx_group_plan_create.restype = i32
    lib.vdx_group_plan_create.argtypes = [ctypes.POINTER(FftDesc), i32, i32, ctypes.POINTER(vp)]
    lib.vdx_group_plan_destroy.restype = i32
    lib.vdx_group_plan_destroy.argtypes = [vp]
    lib.vdx_group_plan_describe.restype = i32
    lib.vdx_group_plan_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.vdx_group_exec.restype = i32
    lib.vdx_group_exec.argtypes = [vp, vp, vp, vp]
    lib.vdx_batch_plan_create.restype = i32
    lib.vdx_batch_plan_create.argtypes = [ctypes.POINTER(BatchItem), i32, i32, i32, ctypes.POINTER(vp)]
    lib.vdx_batch_plan_destroy.restype = i32
    lib.vdx_batch_plan_destroy.argtypes = [vp]
    lib.vdx_batch_plan_describe.restype = i32
    lib.vdx_batch_plan_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.vdx_batch_workspace_bytes.restype = i32
    lib.vdx_batch_workspace_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
    lib.vdx_batch_exec.restype = i32
    lib.vdx_batch_exec.argtypes = [vp, vp, vp, vp]
    lib.vdx_batch_status.restype = i32
    lib.vdx_batch_status.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    lib.vdx_batch_plan_set_wait.restype = i32
    lib.vdx_batch_plan_set_wait.argtypes = [vp, i64, i32]
    lib.vdx_map_plan_create.restype = i32
    lib.vdx_map_plan_create.argtypes = [ctypes.POINTER(FftDesc), ctypes.c_char_p, ctypes.POINTER(vp)]
    lib.vdx_map_plan_destroy.restype = i32
    lib.vdx_map_plan_destroy.argtypes = [vp]
    lib.vdx_map_exec.restype = i32
    lib.vdx_map_exec.argtypes = [vp, ctypes.POINTER(MapArgs), vp]
    lib.vdx_map_plan_status.restype = i32
    lib.vdx_map_plan_status.argtypes = [vp, ctypes.POINTER(ctypes.c_int), i32]
    lib.vdx_map_plan_source.restype = i32
    lib.vdx_map_plan_source.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    lib.vdx_reduce_noalloc.restype = i32
    lib.vdx_reduce_noalloc.argtypes = [i32, i32, i32, vp, i64, i64, vp, vp]
    lib.vdx_reduce_map_plan_create.restype = i32
    lib.vdx_reduce_map_plan_create.argtypes = [ctypes.c_char_p, i32, i32, ctypes.POINTER(vp)]
    lib.vdx_reduce_map_plan_destroy.restype = i32
    lib.vdx_reduce_map_plan_destroy.argtypes = [vp]
    lib.vdx_reduce_map_exec.restype = i32
    lib.vdx_reduce_map_exec.argtypes = [vp, ctypes.POINTER(MapArgs), i64, i64, vp, vp, vp]
    lib.vdx_reduce_map_plan_status.restype = i32
    lib.vdx_reduce_map_plan_status.argtypes = [vp, ctypes.POINTER(ctypes.c_int), i32]
    lib.vdx_reduce_map_plan_source.restype = i32
    lib.vdx_reduce_map_plan_source.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]


def lib() -> ctypes.CDLL:
    """Loads libvdx.so once; raises when the in-tree build is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"libvdx.so not found at {LIB_PATH}; build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` or "
                    "`python -m vkdispatch_gb300._build` (requires nvcc)"
                )
            handle = ctypes.CDLL(str(LIB_PATH))
            _declare(handle)
            _lib = handle
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(4096)
    lib().vdx_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "libvdx") -> None:
    """Maps a libvdx status to the reference's exception types."""
    if rc == VDX_OK:
        return
    msg = f"{what}: {last_error()}"
    if rc in (VDX_ERR_INVALID, VDX_ERR_UNSUPPORTED):
        raise ValueError(msg)
    raise VdxError(msg)
