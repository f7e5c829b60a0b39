"""Runtime helpers of the reference's top-level API that scripts around the
FFT path call: device listing, state queries, logging and the typed buffer
allocators (vkdispatch/base/init.py:103-175, 366-380, 622-760;
vkdispatch/base/context.py:431-439; vkdispatch/base/buffer_allocators.py).
There is one backend (CUDA through libvdx), so the backend queries answer
for it."""

from __future__ import annotations

import enum
import inspect
import logging
import os
from typing import List, Tuple

from . import dtypes as dt
from .buffer import Buffer


class LogLevel(enum.IntEnum):
    """The reference's vd.LogLevel."""

    VERBOSE = 0
    INFO = 1
    WARNING = 2
    ERROR = 3


_logger = logging.getLogger("vkdispatch_gb300")
_PY_LEVEL = {LogLevel.VERBOSE: logging.DEBUG, LogLevel.INFO: logging.INFO, LogLevel.WARNING: logging.WARNING,
             LogLevel.ERROR: logging.ERROR}
_initialized = False


def _mark_initialized() -> None:
    global _initialized
    _initialized = True


def is_initialized() -> bool:
    """Whether vd.initialize / vd.make_context (or any call that loads the
    kernel library through them) has run."""
    return _initialized


def is_context_initialized() -> bool:
    from . import _context_made

    return _context_made()


def is_dummy() -> bool:
    return False


def is_opencl() -> bool:
    return False


class DeviceInfo:
    """One CUDA device as the reference's DeviceInfo describes a device: the
    fields scripts read (index, name, vendor, limits, subgroup size), filled
    from the CUDA device properties."""

    def __init__(self, dev_index: int):
        import torch

        p = torch.cuda.get_device_properties(dev_index)
        self.dev_index = dev_index
        self.device_name = p.name
        self.vendor_id = 0x10DE
        self.device_id = 0
        self.device_type = 2  # discrete GPU
        self.version_major, self.version_minor = p.major, p.minor
        self.version_variant = self.version_patch = 0
        self.driver_version = 0
        self.float_64_support = self.float_16_support = 1
        self.int_64_support = self.int_16_support = 1
        self.shader_buffer_float32_atomics = self.shader_buffer_float32_atomic_add = 1
        self.sub_group_size = 32
        self.max_workgroup_size: Tuple[int, int, int] = (1024, 1024, 64)
        self.max_workgroup_invocations = 1024
        self.max_workgroup_count: Tuple[int, int, int] = (2 ** 31 - 1, 65535, 65535)
        self.max_compute_shared_memory_size = int(getattr(p, "shared_memory_per_block_optin", 232448))
        self.total_memory = p.total_memory
        self.multiprocessor_count = p.multi_processor_count

    def get_info_string(self, verbose: bool = False) -> str:
        s = (f"Device {self.dev_index}: {self.device_name} (compute capability "
             f"{self.version_major}.{self.version_minor}, {self.multiprocessor_count} SMs, "
             f"{self.total_memory / 2**30:.1f} GiB)")
        if verbose:
            s += (f"\n  subgroup size {self.sub_group_size}, max workgroup size {self.max_workgroup_size}, "
                  f"max shared memory {self.max_compute_shared_memory_size} B")
        return s

    def __repr__(self) -> str:
        return self.get_info_string()


def get_devices() -> List[DeviceInfo]:
    """Every visible CUDA device (an empty list without a CUDA driver)."""
    import torch

    if not torch.cuda.is_available():
        return []
    return [DeviceInfo(i) for i in range(torch.cuda.device_count())]


def set_log_level(level: LogLevel) -> None:
    _logger.setLevel(_PY_LEVEL[LogLevel(level)])


def log(text: str, end: str = "\n", level: LogLevel = LogLevel.ERROR, stack_offset: int = 1) -> None:
    """Logs `text` at `level` with the caller's file and line, through the
    Python logger "vkdispatch_gb300"."""
    frame = inspect.stack()[stack_offset]
    where = f"{os.path.relpath(frame.filename, os.getcwd())}:{frame.lineno}"
    _logger.log(_PY_LEVEL[LogLevel(level)], "[%s] %s", where, (text + end).rstrip("\n"))


def log_error(text: str, end: str = "\n") -> None:
    log(text, end, LogLevel.ERROR, 2)


def log_warning(text: str, end: str = "\n") -> None:
    log(text, end, LogLevel.WARNING, 2)


def log_info(text: str, end: str = "\n") -> None:
    log(text, end, LogLevel.INFO, 2)


def log_verbose(text: str, end: str = "\n") -> None:
    log(text, end, LogLevel.VERBOSE, 2)


def buffer_f32(shape: Tuple[int, ...]) -> Buffer:
    return Buffer(shape, dt.float32)


def buffer_f64(shape: Tuple[int, ...]) -> Buffer:
    return Buffer(shape, dt.float64)


def buffer_i32(shape: Tuple[int, ...]) -> Buffer:
    return Buffer(shape, dt.int32)


def buffer_u32(shape: Tuple[int, ...]) -> Buffer:
    return Buffer(shape, dt.uint32)


def buffer_v2(shape: Tuple[int, ...]) -> Buffer:
    return Buffer(shape, dt.vec2)


def buffer_c64(shape: Tuple[int, ...]) -> Buffer:
    return Buffer(shape, dt.complex64)
