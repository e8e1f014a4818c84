"""Parity at the benchmarked configurations, through the C ABI, against the closed forms and the oracle.

- The white floor at its stated size (256 x 256, 16 samples, 4 bounces, PCG seed 1): floor pixels rho L = 800 cd/m^2
  to 0.1 %, sky 1000, and the oracle pixel by pixel (the reference's photometry row, lib/pathtracer/tests.js:447-509).
- The SDF room as the headline runs it (1920 x 1080, depth 8, march tolerance 1e-4 m, the step cache on with one look
  and 16 M cells): a band of 24 full rows against the oracle marching without the cache, on the same seeds and sample
  indices, per pixel within the Monte-Carlo error bars. At 1920 x 1080 a tile is a pixel, so a band of rows is a
  contiguous range of paths the oracle can trace alone.
- The photon map with the learned 128^2 emission map on (core/wavefront.js:628-711): the map's rebuild from the
  GPU's own counts equals the oracle's build of those counts bit for bit (integer counts, IEEE-rounded f32 sums in the
  same order), the counts agree with the oracle's, and the caustic agrees within the error bars.
"""
import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes
from shadytracer_gb300.renderer import create_path_tracer

pytestmark = pytest.mark.gpu

LUMA = np.array([0.2126, 0.7152, 0.0722])


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


def test_white_floor_at_its_stated_size():
    s = scenes.floor_furnace(width=256, height=256, spp=16, maxbounce=4, seed=1)
    with create_path_tracer(s) as rt:
        rt.step(16)
        rgb, V, S, cnt = rt.read_accum()
        c = rt.counters()
    # a jittered ray lands in its own pixel but where f32 rounds cx + u up to the next pixel's edge (cx + u needs more
    # bits than a float has past x = 1): a few pixels of the 65 536 take 15 or 17 samples, on both sides alike
    assert (cnt == 16).mean() > 0.999
    assert c["paths"] == 256 * 256 * 16 and c["nonfinite"] == 0
    L = rgb @ LUMA
    ref = oracle.render(s, 16)
    Lr = ref.luma()
    assert (cnt == ref.count).mean() > 0.9999
    # the closed form: every floor pixel's every sample is rho * 1000 (MIS splits the sky, half a side), the sky 1000
    floor = np.isclose(Lr, 800.0, rtol=1e-3)
    sky = np.isclose(Lr, 1000.0, rtol=1e-3)
    assert floor.mean() > 0.4 and sky.mean() > 0.05, (floor.mean(), sky.mean())
    assert abs(L[floor].mean() / 800.0 - 1) < 1e-3, L[floor].mean()
    assert abs(L[sky].mean() / 1000.0 - 1) < 1e-3, L[sky].mean()
    assert (np.abs(L[floor] - 800.0) <= 0.8).mean() > 0.995
    # the oracle, pixel by pixel: the same numbers on nearly every path
    close = np.abs(L - Lr) <= 1e-3 * np.maximum(Lr, 1.0)
    assert close.mean() > 0.99, (~close).sum()


@pytest.fixture(scope="module")
def room_1080p():
    s = scenes.sdf_room(width=1920, height=1080, spp=8, sky="physical")      # the bench's room
    s.params.step_cache = 1
    s.params.step_cache_cells = 16.0
    with create_path_tracer(s) as rt:
        rt.step(8)
        out = rt.read_accum()
        c = rt.counters()
    return s, out, c


@pytest.mark.parametrize("row0", [300, 560])
def test_room_1080p_with_the_step_cache_matches_the_oracle_on_a_band(room_1080p, row0):
    s, (rgb, V, S, cnt), c = room_1080p
    assert c["nonfinite"] == 0
    # a jittered ray lands in its own pixel but for f32 rounding at a pixel's very edge (1/1920 is inexact)
    assert (cnt == 8).mean() > 0.998
    W, rows = 1920, 24
    s0 = scenes.sdf_room(width=1920, height=1080, spp=8, sky="physical")   # the oracle marches without the cache
    ref = oracle.render(s0, 8, path_first=row0 * W, path_count=rows * W)
    band = slice(row0, row0 + rows)
    L = (rgb @ LUMA)[band]
    Lr = ref.luma()[band]
    both = (ref.count[band] == 8) & (cnt[band] == 8)
    assert both.mean() > 0.998
    sd = np.hypot(se_of(V[band], S[band]), se_of(ref.V[band], ref.S[band]))
    ok = (sd > 0) & both
    z = (L - Lr)[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.98, np.mean(np.abs(z) < 4)
    # the band's mean within its own error bar: no bias from the cache's balls or the GPU's arithmetic
    zm = (L - Lr)[ok].sum() / np.sqrt(np.sum(sd[ok] ** 2))
    assert abs(zm) < 5, zm
    exact = (np.abs(L - Lr) <= 1e-3 * np.maximum(np.abs(Lr), 1.0))[both]
    assert exact.mean() > 0.2, exact.mean()


def emission_map(rt):
    import ctypes as C
    sent = np.zeros(oracle.LT_N, np.uint32)
    stored = np.zeros(oracle.LT_N, np.uint32)
    cdf = np.zeros(oracle.LT_N + oracle.LT_G, np.float32)
    P = C.c_void_p
    rc = rt.L.st_sppm_emission_map(rt.ctx, sent.ctypes.data_as(P), stored.ctypes.data_as(P), cdf.ctypes.data_as(P))
    assert rc == 0, rt.L.st_last_error(rt.ctx)
    return sent, stored, cdf


def test_learned_emission_map_matches_the_oracle():
    s = scenes.sppm_caustic(width=64, height=64, photons=300_000, r1=0.01)
    s.params.sppm_learn = 1
    with create_path_tracer(s) as rt:
        rt.step(8)
        sent8, stored8, cdf8 = emission_map(rt)
        rt.step(1)                                   # the ninth sample starts with the third rebuild, from the counts
        sent9, stored9, cdf9 = emission_map(rt)      # the first eight left
        rgb, V, S, cnt = rt.read_accum()
    # the rebuild: a function of the integer counts alone, bit for bit
    _, _, ocdf = oracle.lt_build(sent8, stored8)
    assert np.array_equal(cdf9.view(np.uint32), ocdf.view(np.uint32)), \
        "rebuilt CDF differs in %d entries" % np.count_nonzero(cdf9 != ocdf)
    assert not np.array_equal(cdf8, cdf9)          # it learned: the map moved between the rebuilds
    # the counts after nine samples: the same photons through the same gates, up to the few f32 rounding sends
    # another way
    ref = oracle.render(s, 9)
    osent, ostored, ocdf_end = oracle.last_lt()
    assert stored9.sum() > 1000
    assert abs(int(sent9.sum()) / int(osent.sum()) - 1) < 0.01, (sent9.sum(), osent.sum())
    assert abs(int(stored9.sum()) / int(ostored.sum()) - 1) < 0.02, (stored9.sum(), ostored.sum())
    assert np.corrcoef(ostored.astype(float), stored9.astype(float))[0, 1] > 0.98
    # the picture: within the error bars, per channel on average
    for ch in range(3):
        assert abs(rgb[..., ch].mean() / ref.rgb[..., ch].mean() - 1) < 0.03, ch
    L, Lr = rgb @ LUMA, ref.luma()
    se = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    within = np.abs(L - Lr) <= 4 * se + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert within.mean() > 0.98, (~within).sum()
