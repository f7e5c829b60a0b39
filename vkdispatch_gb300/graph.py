"""Deferred recording and stream selection: the reference's CommandGraph
(vkdispatch/execution_pipeline/command_graph.py:38-348) and
cuda_graph_capture (vkdispatch/execution_pipeline/cuda_graph_capture.py:24-52).

Every operation of this package becomes one host closure that enqueues its
kernels on a stream.  The thread-local default graph runs closures as they
are recorded (the reference's immediate mode); an explicit ``CommandGraph``
stores them until ``submit()``.  Inside ``cuda_graph_capture(stream)``
closures enqueue on that stream, so a ``torch.cuda.graph`` capture records
them into a CUDA graph.
"""

from __future__ import annotations

import contextlib
import threading
from typing import Callable, List, Optional

import torch

_tls = threading.local()


_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)
_get_device = getattr(torch._C, "_cuda_getDevice", None)


def current_stream_handle() -> int:
    """The cudaStream_t (as int) launches go to: the capture override, else
    the current torch stream of the current device (read directly, without
    the device-index resolution of torch.cuda.current_stream())."""
    override = getattr(_tls, "stream", None)
    if override is not None:
        return override
    if _raw_stream is not None and _get_device is not None:
        return int(_raw_stream(_get_device()))
    return int(torch.cuda.current_stream().cuda_stream)


class CommandGraph:
    """Records launch closures; ``submit()`` enqueues them in order."""

    def __init__(self, reset_on_submit: bool = False, submit_on_record: bool = False):
        self.records: List[tuple] = []
        self.reset_on_submit = reset_on_submit
        self.submit_on_record = submit_on_record

    def record(self, launch: Callable[[int], None], keepalive=()) -> None:
        if self.submit_on_record:
            launch(current_stream_handle())
            return
        self.records.append((launch, keepalive))

    def submit(self, instance_count: int = 1, stream=None) -> None:
        handle = current_stream_handle() if stream is None else _as_handle(stream)
        for _ in range(instance_count):
            for launch, _keep in self.records:
                launch(handle)
        if self.reset_on_submit:
            self.reset()

    def reset(self) -> None:
        self.records = []

    def __len__(self):
        return len(self.records)


def _as_handle(stream) -> int:
    if stream is None:
        return current_stream_handle()
    if isinstance(stream, int):
        return stream
    if hasattr(stream, "cuda_stream"):
        return int(stream.cuda_stream)
    raise TypeError("stream must be a torch.cuda.Stream, an int handle or None")


def default_graph() -> CommandGraph:
    g = getattr(_tls, "default", None)
    if g is None:
        g = CommandGraph(submit_on_record=True)
        _tls.default = g
    return g


def global_graph() -> CommandGraph:
    g = getattr(_tls, "global_graph", None)
    return g if g is not None else default_graph()


def set_global_graph(graph: Optional[CommandGraph] = None) -> CommandGraph:
    old = global_graph()
    _tls.global_graph = graph
    return old


def resolve(graph: Optional[CommandGraph]) -> CommandGraph:
    return graph if graph is not None else global_graph()


@contextlib.contextmanager
def cuda_graph_capture(stream=None):
    """Routes every launch in the block to ``stream`` (default: torch's
    current stream), e.g. inside ``torch.cuda.graph(g)``; yields the
    capture state (vkdispatch/execution_pipeline/cuda_graph_capture.py:9-41)."""
    prev, prev_cap = getattr(_tls, "stream", None), getattr(_tls, "capture", None)
    _tls.stream = _as_handle(stream) if stream is not None else int(torch.cuda.current_stream().cuda_stream)
    cap = CUDAGraphCapture(stream if stream is not None else torch.cuda.current_stream())
    _tls.capture = cap
    try:
        yield cap
    finally:
        _tls.stream, _tls.capture = prev, prev_cap


@contextlib.contextmanager
def suspend_cuda_capture():
    prev, prev_cap = getattr(_tls, "stream", None), getattr(_tls, "capture", None)
    _tls.stream = _tls.capture = None
    try:
        yield
    finally:
        _tls.stream, _tls.capture = prev, prev_cap


class CUDAGraphCapture:
    """The state of one cuda_graph_capture block: the stream launches go to,
    and the buffers the capture keeps alive (none are needed here: libvdx
    launches take their arguments by value)."""

    def __init__(self, cuda_stream):
        self.cuda_stream = cuda_stream
        self.uniform_buffers: List = []

    def add_uniform_buffer(self, buffer) -> None:
        self.uniform_buffers.append(buffer)


def get_cuda_capture():
    """The calling thread's active CUDAGraphCapture, or None."""
    return getattr(_tls, "capture", None)


def queue_wait_idle() -> None:
    torch.cuda.synchronize()
