"""The reference's public kernel factories (vkdispatch/fft/shader_factories.py:
11-195): make_fft_shader, make_convolution_shader and make_transpose_shader
return a callable bound to one transform's arguments, which the caller runs
on buffers as often as it likes (``shader(*buffers, graph=None)``), prints
(its source) or asks for ``get_src()``.  Here the callable runs the same
libvdx plans as vd.fft.fft / convolve / transpose with those arguments; the
factories are cached per argument tuple, as the reference's lru_cache'd
factories are."""

from __future__ import annotations

from functools import lru_cache
from typing import Callable, Optional, Tuple

from .. import dtypes as dt
from . import functions as F
from . import src_functions as S


class ShaderFunction:
    """A transform bound to its arguments (the reference's ShaderFunction as
    the FFT factories return it, vkdispatch/shader/shader_function.py:
    162-300): call it on buffers, print it for its source."""

    def __init__(self, name: str, run: Callable, src: Callable[[bool], S.ShaderSource]):
        self.name = name
        self._run = run
        self._src = src

    def __call__(self, *buffers, graph=None):
        self._run(*buffers, graph=graph)

    def get_src(self, line_numbers: bool = None, build: bool = True) -> S.ShaderSource:
        return self._src(bool(line_numbers))

    def print_src(self, line_numbers: bool = None) -> None:
        print(self.get_src(line_numbers))

    def __repr__(self) -> str:
        return repr(self.get_src())


@lru_cache(maxsize=None)
def make_fft_shader(buffer_shape: Tuple, axis: int = None, inverse: bool = False, normalize_inverse: bool = True,
                    r2c: bool = False, input_map=None, output_map=None, input_type: dt.dtype = None,
                    output_type: dt.dtype = None, compute_type: dt.dtype = None,
                    input_signal_range: Optional[Tuple[Optional[int], Optional[int]]] = None) -> ShaderFunction:
    shape = tuple(buffer_shape)

    def run(*buffers, graph=None):
        F.fft(*buffers, buffer_shape=shape, graph=graph, axis=axis, inverse=inverse,
              normalize_inverse=normalize_inverse, r2c=r2c, input_map=input_map, output_map=output_map,
              output_type=output_type, input_type=input_type, compute_type=compute_type,
              input_signal_range=input_signal_range)

    def src(line_numbers):
        return S.fft_src(shape, axis=axis, inverse=inverse, normalize_inverse=normalize_inverse, r2c=r2c,
                         input_map=input_map, output_map=output_map, input_signal_range=input_signal_range,
                         line_numbers=line_numbers)

    return ShaderFunction(f"fft_shader_{shape}_{axis}_{inverse}_{normalize_inverse}_{r2c}", run, src)


@lru_cache(maxsize=None)
def make_convolution_shader(buffer_shape: Tuple, kernel_map=None, kernel_num: int = 1, axis: int = None,
                            normalize: bool = True, transposed_kernel: bool = False, kernel_inner_only: bool = False,
                            input_map=None, output_map=None, input_type: dt.dtype = None,
                            output_type: dt.dtype = None, kernel_type: dt.dtype = None,
                            compute_type: dt.dtype = None,
                            input_signal_range: Optional[Tuple[Optional[int], Optional[int]]] = None
                            ) -> ShaderFunction:
    if kernel_num < 1:
        raise ValueError("kernel_num must be >= 1")
    shape = tuple(buffer_shape)

    def run(*buffers, graph=None):
        F.convolve(*buffers, kernel_map=kernel_map, kernel_num=kernel_num, buffer_shape=shape, graph=graph,
                   axis=axis, normalize=normalize, transposed_kernel=transposed_kernel,
                   kernel_inner_only=kernel_inner_only, input_map=input_map, output_map=output_map,
                   output_type=output_type, input_type=input_type, kernel_type=kernel_type,
                   compute_type=compute_type, input_signal_range=input_signal_range)

    def src(line_numbers):
        return S.convolve_src(shape, kernel_map=kernel_map, kernel_num=kernel_num, axis=axis, normalize=normalize,
                              transposed_kernel=transposed_kernel, kernel_inner_only=kernel_inner_only,
                              input_map=input_map, output_map=output_map, input_signal_range=input_signal_range,
                              line_numbers=line_numbers)

    return ShaderFunction(f"convolution_shader_{shape}_{axis}_{kernel_num}", run, src)


@lru_cache(maxsize=None)
def make_transpose_shader(buffer_shape: Tuple, axis: int = None, kernel_inner_only: bool = False,
                          input_type: dt.dtype = dt.complex64, output_type: dt.dtype = dt.complex64,
                          compute_type: dt.dtype = dt.complex64) -> ShaderFunction:
    """Called as shader(out_buffer, in_buffer), like the reference's
    transpose shader (vkdispatch/fft/functions.py:709)."""
    shape = tuple(buffer_shape)

    def run(out_buffer, in_buffer, graph=None):
        F.transpose(in_buffer, conv_shape=shape, axis=axis, out_buffer=out_buffer, graph=graph,
                    kernel_inner_only=kernel_inner_only, input_type=input_type, output_type=output_type,
                    compute_type=compute_type)

    def src(line_numbers):
        return S.transpose_src(shape, axis=axis, kernel_inner_only=kernel_inner_only, line_numbers=line_numbers)

    return ShaderFunction(f"transpose_shader_{shape}_{axis}", run, src)


def cache_clear() -> None:
    """Forgets the bound factories (the reference clears its factory caches
    in vd.fft.cache_clear, shader_factories.py:207-209)."""
    make_fft_shader.cache_clear()
    make_convolution_shader.cache_clear()
    make_transpose_shader.cache_clear()
