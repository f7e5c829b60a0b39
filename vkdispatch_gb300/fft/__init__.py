"""vd.fft-compatible FFT, real FFT and FFT-convolution API."""

from .functions import (  # noqa: F401
    cache_clear,
    convolve,
    convolve2D,
    convolve2DR,
    fft,
    fft2,
    fft3,
    get_transposed_size,
    ifft,
    ifft2,
    ifft3,
    irfft,
    irfft2,
    irfft3,
    resolve_compute_precision,
    rfft,
    rfft2,
    rfft3,
    transpose,
)
from .maps import mapped_kernel_index, read_op, write_op  # noqa: F401
from .plan import (  # noqa: F401
    autotune,
    autotune_load,
    autotune_save,
    autotune_stats,
    bluestein,
    get_plan,
    tensor_core_stages,
)
