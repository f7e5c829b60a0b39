"""The plan autotuner (VDX_FFT_FLAG_AUTOTUNE, vd.fft.autotune): tuned plans
give the same results as default plans (against FP64 numpy.fft, within the
per-pass tolerance), the choice is cached per (kind, N, stride class, batch
class, dtype, direction), and the cache survives a save / load round trip."""

import numpy as np
import pytest
import torch

import vkdispatch_gb300 as vd
from vkdispatch_gb300 import _lib as L
from vkdispatch_gb300.fft import plan as P

from helpers import crandn, rel_l2, tol_fp32

pytestmark = pytest.mark.gpu


def _tuned(shape, axis, kind=L.VDX_KIND_C2C, inverse=False, normalize=False, broadcast=False):
    return P.get_plan(shape, axis, kind, inverse, normalize, L.VDX_C64, L.VDX_C64, None, L.VDX_KOP_MUL_CONJ,
                      L.VDX_C64, broadcast, flags=L.VDX_FFT_FLAG_AUTOTUNE)


@pytest.mark.parametrize("shape,axis", [((512, 1024), 1), ((64, 768, 24), 1), ((300, 40), 0), ((2, 8192), 1),
                                        ((4096, 16), 0)])
def test_tuned_c2c_matches_numpy(shape, axis):
    rng = np.random.default_rng(sum(shape))
    x = crandn(rng, shape)
    t = torch.from_numpy(x).cuda()
    p = _tuned(shape, axis)
    d = p.describe()
    assert d["autotuned"] is True
    p.exec(t.data_ptr(), t.data_ptr(), None, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rel_l2(t.cpu().numpy(), np.fft.fft(x.astype(np.complex128), axis=axis)) <= tol_fp32(shape[axis])


def test_tuned_convolution_and_real_transforms():
    rng = np.random.default_rng(9)
    x = crandn(rng, (8, 256, 96))
    k = crandn(rng, (8, 256, 96))
    with vd.fft.autotune():
        buf = vd.asbuffer(x)
        kb = vd.asbuffer(k)
        vd.fft.convolve(buf, kb, axis=1)
        r = rng.standard_normal((16, 1000)).astype(np.float32)
        rb = vd.asrfftbuffer(r)
        vd.fft.rfft(rb)
    ref = np.fft.ifft(np.fft.fft(x.astype(np.complex128), axis=1) * np.conj(k), axis=1)
    assert rel_l2(buf.read(0), ref) <= 2 * tol_fp32(256)
    assert rel_l2(rb.read_fourier(0), np.fft.rfft(r.astype(np.float64), axis=-1)) <= tol_fp32(1000)


def test_cache_hits_and_round_trip(tmp_path):
    _tuned((256, 2048), 1)
    entries, searches = vd.fft.autotune_stats()
    P.cache_clear()
    p = _tuned((256, 2048), 1)  # same key: no new search
    assert vd.fft.autotune_stats() == (entries, searches)
    assert p.describe()["autotuned"] is True
    path = tmp_path / "tune.txt"
    vd.fft.autotune_save(path)
    lines = [ln for ln in path.read_text().splitlines() if not ln.startswith("#")]
    assert len(lines) == entries and all(len(ln.split()) == 17 for ln in lines)
    vd.fft.autotune_load(path)
    assert vd.fft.autotune_stats()[0] == entries
