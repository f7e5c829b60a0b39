"""Batched FFTs of uneven lengths in one persistent launch (libvdx
vdx_batch_*).  Many transforms of different lengths and batch counts, laid
out back to back in one complex64 buffer, run in a single kernel launch that
claims work units from a device queue; capture `BatchPlan.__call__` inside
``torch.cuda.graph`` (or record it in a CommandGraph) to replay the whole set
as one graph node group.  The reference runs one generated kernel per length
(vkdispatch/fft/shader_factories.py:11-60), launched separately.
"""

from __future__ import annotations

import ctypes
import hashlib
import json
import os
import statistics
from typing import Dict, Iterable, Optional, Sequence, Tuple

import torch

from . import _lib as L
from . import graph as G


_CTA_CHOICES = (256, 512, 1024)
_tuned_cta: Dict[str, int] = {}  # item-list digest -> threads per CTA


def _create(arr, nitems, inverse, normalize, cta=None):
    """A libvdx batch plan; `cta` (threads per CTA) is passed through the
    planner's VDX_BATCH_THREADS setting for the duration of the call."""
    old = os.environ.get("VDX_BATCH_THREADS")
    if cta is not None:
        os.environ["VDX_BATCH_THREADS"] = str(cta)
    try:
        h = ctypes.c_void_p()
        L.check(L.lib().vdx_batch_plan_create(arr, nitems, int(bool(inverse)), int(bool(normalize)), ctypes.byref(h)),
                "batch plan")
        return h
    finally:
        if cta is not None:
            if old is None:
                os.environ.pop("VDX_BATCH_THREADS", None)
            else:
                os.environ["VDX_BATCH_THREADS"] = old


class BatchPlan:
    """items: (offset, length, count) per item, offsets in complex elements.

    autotune=True times the plan at each CTA size (256, 512 and 1024 threads:
    how many transforms or columns a work unit holds, and how many CTAs share
    an SM) on scratch buffers of the same items, keeps the fastest and caches
    the choice per item list.  The timing allocates and synchronises: create
    such plans outside stream capture."""

    def __init__(self, items: Sequence[Tuple[int, int, int]], inverse: bool = False, normalize: bool = True,
                 autotune: bool = False):
        arr = (L.BatchItem * len(items))()
        for i, (off, n, c) in enumerate(items):
            arr[i].offset, arr[i].length, arr[i].count = int(off), int(n), int(c)
        self.cta = None
        if autotune:
            key = hashlib.sha1(repr((list(items), bool(inverse), bool(normalize))).encode()).hexdigest()
            if key not in _tuned_cta:
                _tuned_cta[key] = _tune_cta(arr, items, inverse, normalize)
            self.cta = _tuned_cta[key]
        h = _create(arr, len(items), inverse, normalize, self.cta)
        self.handle = h
        self.items = [tuple(int(v) for v in it) for it in items]
        self.total_points = max(off + n * c for off, n, c in self.items)
        ws = ctypes.c_size_t()
        L.check(L.lib().vdx_batch_workspace_bytes(h, ctypes.byref(ws)), "batch workspace")
        self.workspace_bytes = int(ws.value)

    def describe(self) -> dict:
        buf = ctypes.create_string_buffer(1024)
        L.check(L.lib().vdx_batch_plan_describe(self.handle, buf, len(buf)), "batch describe")
        return json.loads(buf.value.decode())

    def make_workspace(self) -> Optional[torch.Tensor]:
        if self.workspace_bytes == 0:
            return None
        return torch.empty(self.workspace_bytes // 8, dtype=torch.complex64, device="cuda")

    def __call__(self, data: torch.Tensor, workspace: Optional[torch.Tensor] = None, graph=None) -> None:
        if data.dtype != torch.complex64 or not data.is_cuda or not data.is_contiguous():
            raise ValueError("data must be a contiguous complex64 CUDA tensor")
        if data.numel() < self.total_points:
            raise ValueError(f"data holds {data.numel()} points, the items need {self.total_points}")
        if self.workspace_bytes and (workspace is None or workspace.numel() * workspace.element_size()
                                     < self.workspace_bytes):
            raise ValueError(f"this batch needs a workspace of {self.workspace_bytes} bytes")
        dptr = data.data_ptr()
        wptr = workspace.data_ptr() if workspace is not None else None
        h = self.handle
        G.resolve(graph).record(lambda s: L.check(L.lib().vdx_batch_exec(h, dptr, wptr, s), "batch exec"),
                                (data, workspace))

    def set_wait(self, wait_limit: int = 1 << 22, extra_dependency: int = 0) -> None:
        """Poll limit of the launch's dependency waits, and an optional
        injected unmet dependency (see vdx_batch_plan_set_wait); clears the
        status word.  Synchronous."""
        L.check(L.lib().vdx_batch_plan_set_wait(self.handle, int(wait_limit), int(extra_dependency)),
                "batch set_wait")

    def status(self) -> int:
        """0, or 1 when a dependency wait inside a launch gave up (synchronous)."""
        st = ctypes.c_int()
        L.check(L.lib().vdx_batch_status(self.handle, ctypes.byref(st)), "batch status")
        return int(st.value)

    def __del__(self):
        try:
            if self.handle:
                L.lib().vdx_batch_plan_destroy(self.handle)
        except Exception:
            pass


def _tune_cta(arr, items, inverse, normalize, reps: int = 5) -> int:
    total = max(int(off) + int(n) * int(c) for off, n, c in items)
    data = torch.zeros(total, dtype=torch.complex64, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    best, best_ms = None, None
    for cta in _CTA_CHOICES:
        try:
            h = _create(arr, len(items), inverse, normalize, cta)
        except ValueError:
            continue  # some length does not fit this CTA size
        try:
            wsb = ctypes.c_size_t()
            L.check(L.lib().vdx_batch_workspace_bytes(h, ctypes.byref(wsb)), "batch workspace")
            ws = torch.empty(max(1, int(wsb.value) // 8), dtype=torch.complex64, device="cuda")
            s = G.current_stream_handle()
            ts = []
            for r in range(reps + 1):
                ev[0].record()
                L.check(L.lib().vdx_batch_exec(h, data.data_ptr(), ws.data_ptr(), s), "batch exec")
                ev[1].record()
                torch.cuda.synchronize()
                if r:
                    ts.append(ev[0].elapsed_time(ev[1]))
            ms = statistics.median(ts)
            if best_ms is None or ms < best_ms:
                best, best_ms = cta, ms
        finally:
            L.lib().vdx_batch_plan_destroy(h)
    del data
    return best if best is not None else 512


def pack_items(lengths_counts: Iterable[Tuple[int, int]]):
    """Lays (length, count) pairs out back to back: [(offset, length, count)]."""
    items, off = [], 0
    for n, c in lengths_counts:
        items.append((off, int(n), int(c)))
        off += int(n) * int(c)
    return items, off
