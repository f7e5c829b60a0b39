"""vkdispatch_gb300: GB300-native (sm_103a) FFT, FFT-convolution and
reduction path with vkdispatch's call surface.

    import vkdispatch_gb300 as vd
    buf = vd.asbuffer(x)            # or vd.from_cuda_array(torch_tensor)
    vd.fft.fft(buf); vd.fft.ifft(buf)
    res = vd.reduce.map_reduce(vd.reduce.SubgroupAdd)(f)(buf)

Kernels live in libvdx.so (include/vdx.h), called through ctypes; PyTorch
provides device memory and streams.  There is no CPU fallback.
"""

from . import codegen  # noqa: F401
from . import fft  # noqa: F401
from . import reduce  # noqa: F401
from . import torch_fft  # noqa: F401
from ._lib import lib as _load_lib  # noqa: F401
from .buffer import Buffer, RFFTBuffer, asbuffer, asrfftbuffer, from_cuda_array  # noqa: F401
from .dtypes import (  # noqa: F401
    bfloat16,
    complex32,
    complex64,
    complex128,
    complexbf16,
    dtype,
    float16,
    float32,
    float64,
    int32,
    uint32,
    vec2,
)
from .graph import (  # noqa: F401
    CommandGraph,
    CUDAGraphCapture,
    cuda_graph_capture,
    default_graph,
    get_cuda_capture,
    global_graph,
    queue_wait_idle,
    set_global_graph,
    suspend_cuda_capture,
)
from .fft.shader_factories import ShaderFunction  # noqa: F401
from .fft.src_functions import ShaderSource  # noqa: F401
from .reduce import MappingFunction, map  # noqa: F401
from .runtime import (  # noqa: F401
    DeviceInfo,
    LogLevel,
    buffer_c64,
    buffer_f32,
    buffer_f64,
    buffer_i32,
    buffer_u32,
    buffer_v2,
    get_devices,
    is_context_initialized,
    is_dummy,
    is_initialized,
    is_opencl,
    log,
    log_error,
    log_info,
    log_verbose,
    log_warning,
    set_log_level,
)
from . import runtime as _runtime

__version__ = "0.1.0"

# `from vkdispatch_gb300.codegen.abbreviations import *`, as user code writes
# it for the reference (codegen is a module here, not a package)
import sys as _sys  # noqa: E402

from . import _abbreviations  # noqa: E402

_sys.modules[__name__ + ".codegen.abbreviations"] = _abbreviations
codegen.abbreviations = _abbreviations


class Context:
    """The device a process computes on (the reference's vd.Context,
    made by vd.make_context): here the current CUDA device."""

    def __init__(self, device: int):
        import torch

        self.device = device
        props = torch.cuda.get_device_properties(device)
        self.device_name = props.name
        self.multiprocessor_count = props.multi_processor_count
        self.total_memory = props.total_memory

    def __repr__(self):
        return f"Context(device={self.device}, {self.device_name})"


_context = None


def make_context(devices=None, use_cpu: bool = False, **kwargs) -> Context:
    """Selects the GPU to compute on (the reference's vd.make_context,
    which picks Vulkan or CUDA devices).  One CUDA device: `devices` may name
    it (its first entry); `use_cpu` and the queue settings have no meaning
    here and are accepted so that calls written for the reference run."""
    import torch

    global _context
    if devices is not None:
        dev = int(devices[0] if isinstance(devices, (list, tuple)) else devices)
        torch.cuda.set_device(dev)
    _load_lib()
    _runtime._mark_initialized()
    _context = Context(torch.cuda.current_device())
    return _context


def get_context() -> Context:
    return _context if _context is not None else make_context()


def initialize(*args, **kwargs) -> None:
    """Loads libvdx (there is a single CUDA backend; arguments are ignored)."""
    _load_lib()
    _runtime._mark_initialized()


def is_cuda() -> bool:
    return True


def get_backend() -> str:
    return "cuda"


def is_vulkan() -> bool:
    return False


def _context_made() -> bool:
    return _context is not None
