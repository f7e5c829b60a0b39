"""GPU tests of compiled map-reduce: mapping functions outside vdx_reduce's
fixed maps (several buffers, scalars, vec2 results, integer expressions,
strided buffers), against numpy; the reference's own cases
(tests/test_reductions.py: test_listed_reductions, batched mapped
reductions) included."""

import numpy as np
import pytest

import vkdispatch_gb300 as vd
import vkdispatch_gb300.codegen as vc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_listed_reductions_two_vec2_buffers():
    rng = np.random.default_rng(1)
    data = rng.random((1024, 2)).astype(np.float32)
    data2 = rng.random((1024, 2)).astype(np.float32)
    buf, buf2 = vd.Buffer((1024,), vd.vec2), vd.Buffer((1024,), vd.vec2)
    buf.write(data)
    buf2.write(data2)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def sum_map(buffer: vc.Buffer[vd.vec2], buffer2: vc.Buffer[vd.vec2]) -> vd.vec2:
        ind = vd.reduce.mapped_io_index()
        return vc.sin(buffer[ind] + buffer2[ind])

    graph = vd.CommandGraph()
    res = sum_map(buf, buf2, graph=graph)
    graph.submit()
    torch.cuda.synchronize()
    assert np.allclose(np.sin(data + data2).sum(axis=0), res.read(0)[0], rtol=1e-5)


@pytest.mark.parametrize("op,np_op", [(vd.reduce.SubgroupAdd, np.sum), (vd.reduce.SubgroupMin, np.min),
                                      (vd.reduce.SubgroupMax, np.max)])
def test_scalar_and_two_buffers(op, np_op):
    rng = np.random.default_rng(2)
    a = rng.standard_normal(300001).astype(np.float32)
    b = rng.standard_normal(300001).astype(np.float32)
    ba, bb = vd.asbuffer(a), vd.asbuffer(b)

    @vd.reduce.map_reduce(op)
    def weighted(x: vc.Buffer[vc.f32], y: vc.Buffer[vc.f32], w: vc.Var[vc.f32]) -> vc.f32:
        i = vd.reduce.mapped_io_index()
        return x[i] * w + vc.cos(y[i])

    got = weighted(ba, bb, 0.75).read(0)[0]
    ref = np_op(a.astype(np.float64) * 0.75 + np.cos(b.astype(np.float64)))
    assert abs(got - ref) <= 1e-5 * max(1.0, np.abs(a).sum())


def test_integer_expression_bit_exact():
    rng = np.random.default_rng(3)
    u = rng.integers(0, 2 ** 32, 70000, dtype=np.uint64).astype(np.uint32)
    bu = vd.asbuffer(u)

    @vd.reduce.map_reduce(vd.reduce.SubgroupXor)
    def mixed(x: vc.Buffer[vc.u32]) -> vc.u32:
        i = vd.reduce.mapped_io_index()
        return x[i] ^ (i * 3)

    got = int(mixed(bu).read(0)[0])
    ref = int(np.bitwise_xor.reduce(u ^ (np.arange(70000, dtype=np.uint64) * 3).astype(np.uint32)))
    assert got == ref


def test_batched_rows_and_mapping_function():
    rng = np.random.default_rng(4)
    data = rng.random((10, 30000)).astype(np.float32)
    buf = vd.asbuffer(data)

    @vd.map
    def reduction_map(inp: vc.Buffer[vc.f32]) -> vc.f32:
        i = vd.reduce.mapped_io_index()
        return vc.exp(inp[i]) - 1.0

    @vd.reduce.reduce(0, axes=[1], mapping_function=reduction_map)
    def sum_reduce(a: vc.f32, b: vc.f32) -> vc.f32:
        return a + b

    got = sum_reduce(buf).read(0)[0]
    ref = (np.exp(data.astype(np.float64)) - 1.0).sum(axis=1)
    assert np.allclose(got, ref, rtol=2e-5)


def test_strided_buffer_and_out_of_range_status():
    rng = np.random.default_rng(5)
    t = torch.from_numpy(rng.standard_normal((64, 80)).astype(np.float32)).cuda()[:, ::2]  # strided view
    b = vd.from_cuda_array(t, require_contiguous=False)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def sq(x: vc.Buffer[vc.f32]) -> vc.f32:
        i = vd.reduce.mapped_io_index()
        return x[i] * x[i] + 0.0 * x[i]

    got = sq(b).read(0)[0]
    ref = (t.cpu().numpy().astype(np.float64) ** 2).sum()
    assert abs(got - ref) <= 1e-5 * ref

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def shifted(x: vc.Buffer[vc.f32]) -> vc.f32:
        return x[vd.reduce.mapped_io_index() + 1]  # the last element reads past the buffer

    c = vd.asbuffer(np.ones(1000, np.float32))
    res = shifted(c)
    torch.cuda.synchronize()
    assert res.read(0)[0] == 999.0  # the out-of-range read loads 0
    assert shifted.last_plan.status() == 1


def test_reference_preamble_and_abbreviations():
    """The reference's test files start with vd.initialize and vd.make_context
    and annotate maps with the abbreviations module: the same lines run here."""
    from vkdispatch_gb300.codegen.abbreviations import Buff, f32

    vd.initialize(debug_mode=True)
    ctx = vd.make_context(use_cpu=True)
    assert ctx.multiprocessor_count > 0 and vd.get_context() is ctx
    data = np.random.default_rng(6).random(1536).astype(np.float32)
    buf = vd.Buffer((1536,), vd.float32)
    buf.write(data)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def sum_map(buffer: Buff[f32]) -> f32:
        return buffer[vd.reduce.mapped_io_index()]

    assert np.allclose([data.sum()], [sum_map(buf).read(0)[0]])


def test_map_with_registers_and_control_flow():
    """A mapping function with registers, in-place updates, an if / else-if /
    else chain and a bounded while loop before its return value."""
    rng = np.random.default_rng(7)
    a = (rng.standard_normal(200003) * 3).astype(np.float32)
    ba = vd.asbuffer(a)

    @vd.reduce.map_reduce(vd.reduce.SubgroupAdd)
    def clipped(buf: vc.Buffer[vc.f32], lim: vc.Var[vc.f32]) -> vc.f32:
        i = vd.reduce.mapped_io_index()
        r = vc.new_float_register(buf[i])
        with vc.if_block(r > lim):
            r[:] = lim
        with vc.else_if_block(r < -lim):
            r[:] = -lim
        with vc.else_block():
            r += 1.0
        c = vc.new_int_register(0)
        with vc.while_block(c < 3):
            c += 1
            r *= 0.5
        return r

    got = clipped(ba, 2.0).read(0)[0]
    x = a.astype(np.float64)
    ref = (np.where(x > 2.0, 2.0, np.where(x < -2.0, -2.0, x + 1.0)) * 0.125).sum()
    assert abs(got - ref) <= 1e-5 * np.abs(x).sum()
