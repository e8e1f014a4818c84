"""Parity of the GPU path tracer (libshadytracer.so, through the C ABI) with the oracle.

Both sides seed every path from (sample, path, event) with the reference's PCG4D, so most paths take the same
random numbers and land on the same pixel values; where f32 rounding (fused multiply-adds, sin/cos/log in other
orders) sends a path another way, the two still agree within the Monte-Carlo error bars -- the reference's own
bar (lib/pathtracer/tests.js verdicts: within 3 sigma). Sizes are small enough for the oracle to finish in seconds.
"""
import numpy as np
import pytest

from shadytracer_gb300 import scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

LUMA = np.array([0.2126, 0.7152, 0.0722])


@pytest.fixture(scope="module")
def rt_factory():
    from shadytracer_gb300.renderer import create_path_tracer
    made = []

    def make(scene):
        rt = create_path_tracer(scene, device=0)
        made.append(rt)
        return rt
    yield make
    for r in made:
        r.close()


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


def test_albedo_tables_match_the_oracle(rt_factory):
    rt = rt_factory(scenes.floor_furnace(width=16, height=16))
    ec, ecavg, e1 = rt.mf_tables()
    oec, oavg, oe1 = oracle.mf_tables(fp64=False)
    # the same 32 x 32 warped quadrature in f32 on both sides; the sums differ only in rounding
    assert np.max(np.abs(ec - oec)) < 2e-4
    assert np.max(np.abs(ecavg - oavg)) < 2e-4
    assert np.max(np.abs(e1 - oe1)) < 2e-4
    # E1 of a smooth lobe keeps everything; albedos are in [0, 1]
    assert abs(e1[0 * 32 + 31] - 1.0) < 1e-3
    assert ec.min() >= 0 and ec.max() <= 1.0001


def test_white_floor_closed_form(rt_factory):
    """The photometry floor (photometry row, tests.js:447-509): floor pixels rho * L = 800 cd/m^2, sky 1000, to 0.1 %."""
    s = scenes.floor_furnace(width=128, height=128)
    rt = rt_factory(s)
    rt.step(4)
    rgb, V, S, cnt = rt.read_accum()
    L = rgb @ LUMA
    assert (cnt == 4).all()
    # the rows whose camera rays meet the floor steeply: light sampling and the bounce split the sky by MIS, half
    # each, so every sample is 800 -- but for a bounce so near the horizon that its steps run out (maxiter)
    floor = L[:40]
    assert abs(floor.mean() / 800.0 - 1) < 1e-3, floor.mean()
    assert (np.abs(floor - 800.0) <= 0.08).mean() > 0.995
    sky = L[-3:]
    assert np.all(np.abs(sky - 1000.0) <= 1.0)


def test_white_floor_matches_the_oracle(rt_factory):
    s = scenes.floor_furnace(width=64, height=64)
    rt = rt_factory(s)
    rt.step(4)
    rgb, V, S, cnt = rt.read_accum()
    ref = oracle.render(s, 4)
    L, Lr = rgb @ LUMA, ref.luma()
    assert (cnt == ref.count).all()
    close = np.abs(L - Lr) <= 1e-3 * np.maximum(Lr, 1.0)
    assert close.mean() > 0.99, (~close).sum()
    c = rt.counters()
    assert c["paths"] == ref.counters[0]
    assert c["nonfinite"] == 0


def test_room_matches_the_oracle_within_error_bars(rt_factory):
    """The SDF room (24 smooth-unioned primitives, GGX metal and plastic, sun + sky through a window), small."""
    s = scenes.sdf_room(width=96, height=54, spp=4, maxbounce=8)
    rt = rt_factory(s)
    rt.step(4)
    rgb, V, S, cnt = rt.read_accum()
    ref = oracle.render(s, 4)
    L, Lr = rgb @ LUMA, ref.luma()
    se = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    exact = np.abs(L - Lr) <= 1e-3 * np.maximum(np.abs(Lr), 1.0)
    within = np.abs(L - Lr) <= 4 * se + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert exact.mean() > 0.5, "most paths should take the same numbers: %.3f" % exact.mean()
    assert within.mean() > 0.985, "pixels outside 4 sigma: %d of %d" % ((~within).sum(), within.size)
    assert abs(L.mean() / Lr.mean() - 1) < 0.03, (L.mean(), Lr.mean())
    c = rt.counters()
    assert c["paths"] == 96 * 54 * 4
    assert c["nonfinite"] == 0


def test_haze_furnace_conserves_energy(rt_factory):
    """The haze box's furnace (tests.js:1818-1866): an albedo-1 haze box in a uniform environment reads the
    environment exactly -- every collision scatters what it takes back in."""
    s = scenes.haze_furnace(width=48, height=48, sigma_t=1.0, g=0.7)
    rt = rt_factory(s)
    rt.step(16)
    rgb, V, S, cnt = rt.read_accum()
    L = rgb @ LUMA
    assert abs(L.mean() / 1000.0 - 1) < 2e-3, L.mean()
    ref = oracle.render(s, 4)
    assert abs(ref.luma().mean() / 1000.0 - 1) < 5e-3


@pytest.mark.parametrize("sigma_s", [0.05, 0.2, 1.0])
def test_haze_box_grid_conserves_energy(rt_factory, sigma_s):
    """The haze box at every scattering coefficient and anisotropy of its grid: an albedo-1 box in a uniform
    1000 cd/m^2 environment. Drawing the phase function alone, every path's weight is exactly one (HG drawn exactly),
    so the picture reads 1000 to 0.02 % with 64 bounces -- what the cap ends is all it may lose. With the light sample
    and its MIS weights (32 bounces), each sample is 1000 only on average: the mean within its error bar."""
    for g in (0.0, 0.7, 0.9):
        s = scenes.haze_furnace(width=64, height=64, sigma_t=sigma_s, g=g, maxbounce=64)
        s.params.nee = 0
        rt = rt_factory(s)
        rt.step(16)
        L = rt.read_accum()[0] @ LUMA
        assert abs(L.mean() / 1000.0 - 1) < 2e-4 and L.max() <= 1000.0 * (1 + 1e-5), (sigma_s, g, L.mean(), L.max())
        assert rt.counters()["nonfinite"] == 0
        s = scenes.haze_furnace(width=64, height=64, sigma_t=sigma_s, g=g, maxbounce=32)
        rt = rt_factory(s)
        rt.step(16)
        rgb, V, S, cnt = rt.read_accum()
        L = rgb @ LUMA
        se = np.sqrt(np.sum(se_of(V, S) ** 2)) / L.size
        assert abs(L.mean() - 1000.0) < 5 * se + 0.05, (sigma_s, g, L.mean(), se)


def test_invalidate_and_state(rt_factory):
    from shadytracer_gb300._lib import StError
    s = scenes.floor_furnace(width=32, height=32)
    rt = rt_factory(s)
    rt.step(2)
    assert rt.counters()["samples"] == 2
    rt.invalidate()
    rgb, V, S, cnt = rt.read_accum()
    assert cnt.max() == 0 and np.all(rgb == 0)
    # a bad scene is refused and the old one kept
    bad = scenes.floor_furnace(width=32, height=32)
    bad.prims[0].material = 99
    with pytest.raises(StError):
        rt.set_scene(bad)
    rt.step(1)
    assert rt.read_accum()[3].max() == 1
    assert rt.set(maxbounce=3, not_a_setting=1) == ["not_a_setting"]


def test_thin_lens_matches_the_oracle(rt_factory):
    """The thin lens (genrays.js:80-87, lens.js lensDisc): a 5 cm aperture focused at 2 m in the room -- the picture
    GPU and oracle agree on, pixel by pixel within the error bars, and the lens blurs (a pinhole's picture differs)."""
    s = scenes.sdf_room(width=64, height=36, spp=16)
    s.view.lens_radius = 0.05
    s.view.focus_distance = 2.0
    rt = rt_factory(s)
    rt.step(16)
    rgb, V, S, cnt = rt.read_accum()
    ref = oracle.render(s, 16)
    L, Lr = rgb @ LUMA, ref.luma()
    sd = np.hypot(se_of(V, S), se_of(ref.V, ref.S))
    ok = sd > 0
    z = (L - Lr)[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.98, np.mean(np.abs(z) < 4)
    close = np.abs(L - Lr) <= 1e-3 * np.maximum(Lr, 1.0)
    assert close.mean() > 0.5, close.mean()          # most paths take the same numbers through the lens too
    s.view.lens_radius = 0.0
    pin = oracle.render(s, 16).luma()
    assert np.mean(np.abs(pin - Lr) > 0.05 * np.maximum(Lr, 1.0)) > 0.2


@pytest.mark.parametrize("looks", [1, 2])
def test_step_cache_keeps_the_picture(rt_factory, looks):
    """The step cache (wavefront.js:67-150): balls with no surface in them, crossed with no distance evaluation. The
    room with it on reads as the oracle, marching without it, reads, pixel by pixel within the error bars, and the
    march evaluates the scene's distance fewer times."""
    s = scenes.sdf_room(width=96, height=54, spp=4)
    rt0 = rt_factory(s)
    rt0.step(16)
    steps0 = rt0.counters()["march_steps"]
    s.params.step_cache = looks
    rt = rt_factory(s)
    rt.step(16)
    rgb, V, S, cnt = rt.read_accum()
    L = rgb @ LUMA
    steps = rt.counters()["march_steps"]
    ref = oracle.render(s, 16)
    sd = np.hypot(se_of(V, S), se_of(ref.V, ref.S))
    ok = sd > 0
    z = (L - ref.luma())[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.98, np.mean(np.abs(z) < 4)
    zm = (L - ref.luma())[ok].mean() / (np.sqrt(np.sum(sd[ok] ** 2)) / ok.sum())
    assert abs(zm) < 5, zm
    assert steps < 0.9 * steps0, (steps, steps0)
    assert rt.counters()["nonfinite"] == 0
