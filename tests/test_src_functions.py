"""The reference's source-inspection surface (vd.fft.*_src, *_print_src,
pad_dim, get_cache_info; vkdispatch/fft/src_functions.py,
prime_utils.py:50-64).  Maps lower to the hooks source without a GPU; the
plan descriptions of transforms without maps need one."""

import pytest

import vkdispatch_gb300 as vd
import vkdispatch_gb300.codegen as vc


def _reference_pad(dim, limit=16):
    """Plain restatement for the check: the next length whose prime factors
    are all at most `limit`."""
    n = dim
    while True:
        m, p, ok = n, 2, True
        while m > 1:
            if m % p == 0:
                if p > limit:
                    ok = False
                    break
                m //= p
            else:
                p += 1
        if ok:
            return n
        n += 1


@pytest.mark.parametrize("dim", [1, 2, 16, 17, 31, 34, 143, 169, 1000, 8209, 16411, 65537])
def test_pad_dim(dim):
    assert vd.fft.pad_dim(dim) == _reference_pad(dim)
    assert vd.fft.pad_dim(dim, 32) == _reference_pad(dim, 32)


def test_pad_dim_rejects_non_positive():
    with pytest.raises(ValueError):
        vd.fft.pad_dim(0)


def test_map_sources_without_gpu():
    @vd.map
    def scaled(buf: vc.Buffer[vc.c64], s: vc.Var[vc.f32]):
        op = vd.fft.read_op()
        op.read_from_buffer(buf)
        op.register *= s

    src = vd.fft.fft_src((8, 1000), input_map=scaled)
    assert isinstance(src, vd.fft.ShaderSource)
    assert "struct VdxHooks" in src.code and "m.fs[0]" in src.code
    numbered = vd.fft.fft_src((8, 1000), input_map=scaled, line_numbers=True)
    assert numbered.code.splitlines()[0].lstrip().startswith("1 ")
    conv = vd.fft.convolve_src((8, 1000), kernel_map=None, input_map=scaled)
    assert "cmulc" in conv.code  # the default kernel hook: * conj(K)


def test_print_src_prints_each_stage(capsys):
    @vd.map
    def copy_in(buf: vc.Buffer[vc.c64]):
        op = vd.fft.read_op()
        op.read_from_buffer(buf)

    vd.fft.fft_print_src((4, 64), input_map=copy_in)
    assert "VdxHooks" in capsys.readouterr().out


def test_cache_info_fields():
    info = vd.fft.get_cache_info()
    assert info.maxsize is None and info.currsize >= 0 and info.hits >= 0 and info.misses >= 0


@pytest.mark.gpu
def test_plan_sources():
    s = vd.fft.fft_src((256, 1024))
    assert s.name == "vdx::k_c2c" and '"radices"' in s.code and s.local_size[0] > 0
    assert len(vd.fft.fft2_src((64, 128, 256))) == 2
    assert len(vd.fft.rfft3_src((8, 32, 64))) == 3
    r = vd.fft.convolve2DR_src((4, 512, 512))
    assert [x.name for x in r] == ["vdx::k_r2c_even", "vdx::k_conv", "vdx::k_c2r_even"]
    assert "fourstep" in vd.fft.fft_src((2, 65536)).code
    assert vd.fft.transpose_src((4, 512, 257)).name == "ordered copy"
    before = vd.fft.get_cache_info()
    vd.fft.fft_src((256, 1024))
    assert vd.fft.get_cache_info().hits == before.hits + 1


def test_shader_factories_are_cached_callables():
    """vd.fft.make_fft_shader / make_convolution_shader / make_transpose_shader
    (vkdispatch/fft/shader_factories.py:11-195): cached per argument tuple,
    cleared by vd.fft.cache_clear, argument errors raised at creation."""
    import pytest

    import vkdispatch_gb300 as vd

    a = vd.fft.make_fft_shader((8, 1024), 1, inverse=True)
    assert a is vd.fft.make_fft_shader((8, 1024), 1, inverse=True)
    assert a is not vd.fft.make_fft_shader((8, 1024), 1)
    assert isinstance(a, vd.fft.ShaderFunction) and callable(a)
    c = vd.fft.make_convolution_shader((8, 1024), kernel_num=2)
    t = vd.fft.make_transpose_shader((8, 1024), axis=1)
    assert "convolution" in c.name and "transpose" in t.name
    with pytest.raises(ValueError):
        vd.fft.make_convolution_shader((8, 1024), kernel_num=0)
    vd.fft.cache_clear()
    assert vd.fft.make_fft_shader((8, 1024), 1, inverse=True) is not a
