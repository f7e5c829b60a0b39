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
    cuda_graph_capture,
    default_graph,
    global_graph,
    queue_wait_idle,
    set_global_graph,
    suspend_cuda_capture,
)
from .reduce import MappingFunction, map  # noqa: F401

__version__ = "0.1.0"


def initialize(*args, **kwargs) -> None:
    """Loads libvdx (there is a single CUDA backend; arguments are ignored)."""
    _load_lib()


def is_cuda() -> bool:
    return True


def get_backend() -> str:
    return "cuda"
