"""CPU tests of host-side logic: map and reduction tracing against the
functor menu, precision resolution, graph recording."""

import pytest

import vkdispatch_gb300 as vd
from vkdispatch_gb300 import _lib as L
from vkdispatch_gb300 import codegen as vc
from vkdispatch_gb300.codegen import Buff, c64, f32, i32
from vkdispatch_gb300.reduce import _trace_map, _trace_reduction


def test_reduction_tracing():
    def add(a: f32, b: f32) -> f32:
        return a + b

    def mn(a: f32, b: f32) -> f32:
        return vc.min(a, b)

    def x(a: i32, b: i32) -> i32:
        return a ^ b

    assert _trace_reduction(add).code == L.VDX_RED_ADD
    assert _trace_reduction(mn).code == L.VDX_RED_MIN
    assert _trace_reduction(x).code == L.VDX_RED_XOR

    def weird(a: f32, b: f32) -> f32:
        return a + b + a

    with pytest.raises(NotImplementedError):
        _trace_reduction(weird)


def test_map_tracing_menu():
    idx = vd.reduce.mapped_io_index

    def ident(b: Buff[f32]) -> f32:
        return b[idx()]

    def sn(b: Buff[f32]) -> f32:
        return vc.sin(b[idx()])

    def mag(b: Buff[c64]) -> f32:
        v = b[idx()]
        return vc.sqrt(v.real * v.real + v.imag * v.imag)

    def mag2(b: Buff[c64]) -> f32:
        v = b[idx()]
        return v.real * v.real + v.imag * v.imag

    def two(b: Buff[f32], c: Buff[f32]) -> f32:
        return b[idx()] + c[idx()]

    assert _trace_map(ident, [f32]) == L.VDX_MAP_IDENTITY
    assert _trace_map(sn, [f32]) == L.VDX_MAP_SIN
    assert _trace_map(mag, [c64]) == L.VDX_MAP_ABS
    assert _trace_map(mag2, [c64]) == L.VDX_MAP_SQUARE
    with pytest.raises(NotImplementedError):
        _trace_map(two, [f32, f32])


def test_reduce_decorator_needs_annotation():
    with pytest.raises(ValueError):

        @vd.reduce.reduce(0)
        def f(a, b):
            return a + b


def test_precision_resolution():
    r = vd.fft.resolve_compute_precision
    assert r([vd.complex32], None) == vd.complex64
    assert r([vd.complex64, vd.complex32], None) == vd.complex64
    assert r([vd.complex128, vd.complex64], None) == vd.complex128
    assert r([vd.complex64], vd.complex128) == vd.complex128
    with pytest.raises(ValueError):
        r([vd.float32], None)


def test_command_graph_records_and_replays_in_order():
    g = vd.CommandGraph()
    seen = []
    g.record(lambda s: seen.append(("a", s)))
    g.record(lambda s: seen.append(("b", s)))
    g.submit(stream=123)
    g.submit(instance_count=2, stream=7)
    assert seen == [("a", 123), ("b", 123), ("a", 7), ("b", 7), ("a", 7), ("b", 7)]


def test_cuda_graph_capture_routes_stream():
    from vkdispatch_gb300 import graph as G

    with G.cuda_graph_capture(stream=4242):
        assert G.current_stream_handle() == 4242
        with G.suspend_cuda_capture():
            assert G._tls.stream is None


def test_global_graph_swap():
    g = vd.CommandGraph()
    old = vd.set_global_graph(g)
    try:
        assert vd.global_graph() is g
    finally:
        vd.set_global_graph(old)


def test_string_annotations_resolve():
    ns = {}
    exec(
        "from __future__ import annotations\n"
        "import vkdispatch_gb300 as vd\n"
        "def m(b: vd.codegen.Buff[vd.complex64]) -> vd.float32:\n"
        "    v = b[vd.reduce.mapped_io_index()]\n"
        "    return vd.codegen.sqrt(v.real * v.real + v.imag * v.imag)\n",
        ns,
    )
    mf = vd.reduce.MappingFunction(ns["m"])
    assert mf.input_dtypes() == [vd.complex64]
    assert mf.return_type == vd.float32


def test_string_annotations_of_enclosing_locals_resolve_by_name():
    ns = {}
    exec(
        "from __future__ import annotations\n"
        "def outer():\n"
        "    import vkdispatch_gb300 as vdl\n"
        "    def m(b: vdl.codegen.Buff[vdl.complex64]) -> vdl.float32:\n"
        "        return b[0]\n"
        "    return m\n",
        ns,
    )
    mf = vd.reduce.MappingFunction(ns["outer"]())
    assert mf.input_dtypes() == [vd.complex64]
    assert mf.return_type == vd.float32


def test_output_map_requires_input_buffer_after_map_args():
    from vkdispatch_gb300.fft.functions import _split_buffers

    class Fake:
        def __init__(self, t):
            self.var_type = t

    om = vd.map(lambda b: None, input_types=[vc.Buffer[vd.complex64], vc.Buffer[vd.float32]])
    outs, ins, _ = _split_buffers((Fake(vd.complex64), Fake(vd.float32), Fake(vd.complex128)), None, om)
    assert len(outs) == 2 and ins[0].var_type == vd.complex128
    om1 = vd.map(lambda b: None, input_types=[vc.Buffer[vd.complex64]])
    with pytest.raises(ValueError, match="input buffer argument must be provided"):
        _split_buffers((Fake(vd.complex64),), None, om1)


def test_map_classification_menu():
    from vkdispatch_gb300.fft import maps as M

    def rin(buffer: vc.Buffer[vd.float32]):
        op = vd.fft.read_op()
        op.register.real = vc.to_dtype(vd.float32, buffer[op.io_index])
        op.register.imag = vc.to_dtype(vd.float32, 0)

    def cout(buffer: vc.Buffer[vd.complex128]):
        vd.fft.write_op().write_to_buffer(buffer)

    def nothing():
        return

    assert M.classify_input(vd.map(rin)).kind == "real"
    assert M.classify_output(vd.map(cout)).var_type == vd.complex128
    assert M.classify_kernel(vd.map(nothing)).kind == "identity"
    with pytest.raises(ValueError):
        vd.fft.read_op()  # only valid while a map function is traced


def test_multi_kernel_map_strides_are_recognised():
    """Kernel and output maps of a multi-kernel convolution index their buffers
    with io_index + mapped_kernel_index() * C (either operand order); other
    index expressions are refused."""
    import vkdispatch_gb300 as vd
    import vkdispatch_gb300.codegen as vc
    from vkdispatch_gb300.fft import maps as M

    def kmap(kernels: vc.Buffer[vd.complex64]):
        op = vd.fft.read_op()
        kv = vc.new_register(vd.complex64)
        op.read_from_buffer(kernels, register=kv, io_index=vd.fft.mapped_kernel_index() * 96 + op.io_index)
        op.register[:] = vc.mult_complex(op.register, kv.conjugate())

    def omap(out: vc.Buffer[vd.complex64]):
        op = vd.fft.write_op()
        op.write_to_buffer(out, io_index=op.io_index + 40 * vd.fft.mapped_kernel_index())

    def bad(out: vc.Buffer[vd.complex64]):
        op = vd.fft.write_op()
        op.write_to_buffer(out, io_index=op.io_index * 2)

    assert M.classify_kernel(vd.map(kmap)).stride == 96
    assert M.classify_output(vd.map(omap)).stride == 40
    assert vd.fft.mapped_kernel_index() is None
    with pytest.raises(NotImplementedError):
        M.classify_output(vd.map(bad))


def test_torch_fft_front_end_norm_codes_and_cpu_refusal():
    """torch.fft norm modes map to libvdx normalize codes (0 none, 1 1/n,
    2 1/sqrt(n)) per direction; CPU tensors are refused, with no fallback."""
    import torch

    import vkdispatch_gb300.torch_fft as tf

    assert tf._norm_code(None, False) == 0 and tf._norm_code(None, True) == 1
    assert tf._norm_code("backward", False) == 0 and tf._norm_code("backward", True) == 1
    assert tf._norm_code("forward", False) == 1 and tf._norm_code("forward", True) == 0
    assert tf._norm_code("ortho", False) == 2 and tf._norm_code("ortho", True) == 2
    with pytest.raises(ValueError):
        tf._norm_code("none", False)
    with pytest.raises(ValueError):
        tf.fft(torch.zeros(8, dtype=torch.complex64))
    dims, sizes = tf._dims(torch.zeros(2, 3, 4), (5, 6), None)
    assert dims == (1, 2) and sizes == (5, 6)


def test_thread_local_state():
    """Per-thread state, as the reference keeps its graph, builder and map op
    thread-local (vkdispatch/base/command_graph.py:321-348, fft/io_manager.py:
    14-15, tests/test_threading.py): graphs, plan-option contexts and map
    tracing in one thread do not leak into another."""
    import threading

    from vkdispatch_gb300 import graph as G
    from vkdispatch_gb300.fft import plan as P

    idx = vd.reduce.mapped_io_index

    def sn(b: Buff[f32]) -> f32:
        return vc.sin(b[idx()])

    def mag(b: Buff[c64]) -> f32:
        v = b[idx()]
        return vc.sqrt(v.real * v.real + v.imag * v.imag)

    entered, release = threading.Event(), threading.Event()
    seen = {}

    def holder():
        g = G.CommandGraph()
        G.set_global_graph(g)
        with vd.fft.autotune(), vd.fft.bluestein(False):
            seen["holder_graph"] = G.global_graph() is g
            entered.set()
            release.wait(10)
        G.set_global_graph(None)

    def other():
        entered.wait(10)
        seen["other_graph_is_default"] = G.global_graph() is G.default_graph()
        seen["other_tune"] = getattr(P._tls, "tune", False)
        seen["other_bluestein"] = P.bluestein_enabled()
        # concurrent tracing of different maps gives each its own result
        seen["traces"] = [_trace_map(sn, [f32]) for _ in range(50)]
        release.set()

    results = []

    def tracer():
        results.extend(_trace_map(mag, [c64]) for _ in range(50))

    th = [threading.Thread(target=holder), threading.Thread(target=other), threading.Thread(target=tracer)]
    for t in th:
        t.start()
    for t in th:
        t.join(20)
    assert seen["holder_graph"] and seen["other_graph_is_default"]
    assert seen["other_tune"] is False and seen["other_bluestein"] is True  # the holder's False stays its own
    assert seen["traces"] == [L.VDX_MAP_SIN] * 50
    assert results == [L.VDX_MAP_ABS] * 50


def test_torch_fft_front_end_resize():
    """torch.fft's n / s: zero-pad or trim one dimension (host-side helper)."""
    import torch

    import vkdispatch_gb300.torch_fft as tf

    x = torch.arange(12.0).reshape(3, 4)
    assert tf._resize(x, 1, None) is x and tf._resize(x, 1, 4) is x
    assert torch.equal(tf._resize(x, 1, 2), x[:, :2])
    p = tf._resize(x, 0, 5)
    assert p.shape == (5, 4) and torch.equal(p[:3], x) and torch.all(p[3:] == 0)
    q = tf._resize(x, 1, 6)
    assert q.shape == (3, 6) and torch.equal(q[:, :4], x) and torch.all(q[:, 4:] == 0)
    with pytest.raises(ValueError):
        tf._resize(x, 1, 0)


@pytest.mark.parametrize("value,parts", [(None, 2), ("3", 3), ("1", 1), ("0", 1), ("20", 8), ("x", 2)])
def test_image_group_count_setting(monkeypatch, value, parts):
    """VDX_CONV2D_STREAMS: image groups of the batched 2-D transforms, 1-8."""
    from vkdispatch_gb300.fft import functions as F

    if value is None:
        monkeypatch.delenv("VDX_CONV2D_STREAMS", raising=False)
    else:
        monkeypatch.setenv("VDX_CONV2D_STREAMS", value)
    assert F._conv2d_split_parts() == parts


def test_image_groups_refuse_small_batches_without_gpu(monkeypatch):
    """Batches of fewer than 8 images, or under 16 MiB, or one group: nothing
    is recorded and the caller runs the whole batch itself."""
    from vkdispatch_gb300.fft import functions as F

    class FakeBuf:
        def __init__(self, shape):
            self.shape = shape
            n = 8
            for d in shape:
                n *= d
            self.mem_size = n

    def no_plan(*a, **k):
        raise AssertionError("no plan may be built for a refused batch")

    monkeypatch.setattr(F.P, "get_group_plan", no_plan)
    steps = [((4, 512, 257), 2, 0, False, False, False)]
    monkeypatch.setenv("VDX_CONV2D_STREAMS", "2")
    assert not F._image_groups(FakeBuf((4, 512, 257)), None, (), steps)  # 4 images
    assert not F._image_groups(FakeBuf((8, 64, 64)), None, (), steps)  # 256 KiB
    assert not F._image_groups(FakeBuf((512, 257)), None, (), steps)  # not a batch
    monkeypatch.setenv("VDX_CONV2D_STREAMS", "1")
    assert not F._image_groups(FakeBuf((64, 512, 257)), None, (), steps)


def test_codegen_abbreviations_module():
    """`from vkdispatch_gb300.codegen.abbreviations import *` gives the
    reference's short names (vkdispatch/codegen/abbreviations.py)."""
    ns = {}
    exec("from vkdispatch_gb300.codegen.abbreviations import *", ns)
    assert ns["f32"] is vd.float32 and ns["v2"] is vd.vec2 and ns["c64"] is vd.complex64
    assert ns["Buff"][vd.float32].var_type is vd.float32
    assert callable(vd.make_context) and callable(vd.get_context)


class _FakeImages:
    """Stands in for a contiguous complex64 Buffer / RFFTBuffer of a batch
    of images on the host: enough for the image-group dispatch, which only
    reads shapes, sizes and the data pointer before recording a launch."""

    def __init__(self, shape, real_shape=None, ptr=4096):
        from vkdispatch_gb300 import dtypes as dt

        self.shape = tuple(shape)
        if real_shape is not None:
            self.real_shape = tuple(real_shape)
        self.size = 1
        for d in shape:
            self.size *= d
        self.mem_size = 8 * self.size
        self.var_type = dt.complex64
        self.contiguous = True
        self.ptr = ptr


def _capture_chains(monkeypatch):
    from vkdispatch_gb300.fft import functions as F

    seen = []

    class FakePlan:
        def exec(self, *a):
            raise AssertionError("a deferred CommandGraph must not launch")

        def describe(self):
            return {}

    def fake(steps, groups):
        seen.append((tuple(steps), groups))
        return FakePlan()

    monkeypatch.setattr(F.P, "get_group_plan", fake)
    monkeypatch.setenv("VDX_CONV2D_STREAMS", "2")
    return F, seen


def test_image_group_chains_of_the_2d_functions(monkeypatch):
    """Each batched 2-D function hands the group plan the reference's own
    composition (vkdispatch/fft/functions.py:164-300, 373-448, 549-646):
    transform kinds, axes, direction, normalisation and kernel broadcast."""
    import vkdispatch_gb300 as vd
    from vkdispatch_gb300 import _lib as L

    F, seen = _capture_chains(monkeypatch)
    C2C, R2C, C2R, CONV = L.VDX_KIND_C2C, L.VDX_KIND_R2C, L.VDX_KIND_C2R, L.VDX_KIND_CONV
    img = _FakeImages((16, 512, 512))
    rimg = _FakeImages((16, 512, 257), real_shape=(16, 512, 512))
    g = vd.CommandGraph()

    F.fft2(img, graph=g)
    F.ifft2(img, graph=g, normalize=False)
    F.rfft2(rimg, graph=g)
    F.irfft2(rimg, graph=g)
    F.convolve2D(img, _FakeImages((16, 512, 512), ptr=8192), graph=g)
    F.convolve2DR(rimg, _FakeImages((1, 512, 257), ptr=8192), graph=g)  # one kernel for every image
    F.convolve2DR(rimg, _FakeImages((16, 512, 257), ptr=8192), graph=g, normalize=False)
    assert len(g) == 7
    full, half, real = (16, 512, 512), (16, 512, 257), (16, 512, 512)
    want = [
        ((full, 1, C2C, False, False, False), (full, 2, C2C, False, False, False)),
        ((full, 1, C2C, True, False, False), (full, 2, C2C, True, False, False)),
        ((real, 2, R2C, False, False, False), (half, 1, C2C, False, False, False)),
        ((half, 1, C2C, True, True, False), (real, 2, C2R, True, True, False)),
        ((full, 2, C2C, False, False, False), (full, 1, CONV, False, True, False), (full, 2, C2C, True, True, False)),
        ((real, 2, R2C, False, False, False), (half, 1, CONV, False, True, True), (real, 2, C2R, True, True, False)),
        ((real, 2, R2C, False, False, False), (half, 1, CONV, False, False, False), (real, 2, C2R, True, False, False)),
    ]
    got = [tuple((tuple(s[0]), s[1], s[2], bool(s[3]), bool(s[4]), bool(s[5])) for s in steps) for steps, _ in seen]
    assert got == want
    assert all(groups == 2 for _, groups in seen)


def test_image_groups_keep_a_small_kernel_refused(monkeypatch):
    """A kernel buffer smaller than one image is refused with ValueError, as
    the ungrouped convolution refuses it."""
    import vkdispatch_gb300 as vd

    F, seen = _capture_chains(monkeypatch)
    rimg = _FakeImages((16, 512, 257), real_shape=(16, 512, 512))
    with pytest.raises(ValueError):
        F.convolve2DR(rimg, _FakeImages((1, 256, 257), ptr=8192), graph=vd.CommandGraph())
    assert not seen


def test_runtime_helpers_without_gpu(caplog):
    """Top-level runtime helpers of the reference (vkdispatch/base/init.py:
    366-380, 622-760): backend queries, logging through the Python logger
    with the caller's location, and the log-level filter."""
    import logging

    import vkdispatch_gb300 as vd

    assert vd.is_cuda() and not vd.is_vulkan() and not vd.is_dummy() and not vd.is_opencl()
    vd.initialize()
    assert vd.is_initialized()
    with caplog.at_level(logging.DEBUG, logger="vkdispatch_gb300"):
        vd.set_log_level(vd.LogLevel.WARNING)
        vd.log_info("not shown")
        vd.log_warning("shown")
        vd.log_error("also shown")
    msgs = [r.getMessage() for r in caplog.records if r.name == "vkdispatch_gb300"]
    assert any("shown" in m and "test_host_logic.py" in m for m in msgs)
    assert not any("not shown" in m for m in msgs)
    vd.set_log_level(vd.LogLevel.INFO)
    assert vd.get_cuda_capture() is None
