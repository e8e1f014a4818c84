"""Scattering inside a material on the GPU (csrc/st_scene_kernels.cuh k_march's walk; the medium a ray carries, set where
it refracts, st_render.cu / st_photons.cu): an index-matched slab against the walk radiative transfer pins
(tests/slab_walk.py; the reference's core/test/volume.gpu.mjs holds its march to its mirror the same way), a lossless
milky sphere in the furnace, and milky and opal glass under the sun against the oracle pixel by pixel.
"""
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes
from shadytracer_gb300.renderer import create_path_tracer
from slab_walk import slab_walk

pytestmark = pytest.mark.gpu
LUMA = np.array([0.2126, 0.7152, 0.0722])
se = lambda p, n: math.sqrt(max(p * (1 - p), 1e-12) / n)


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


@pytest.mark.parametrize("tau,g", [(0.5, 0.0), (1.0, 0.0), (3.0, 0.8), (6.0, 0.5), (10.0, 0.0)])
def test_the_slab_is_the_walk(tau, g):
    s = scenes.volume_slab(tau, g, width=32, height=32)
    n = 32 * 32 * 64
    with create_path_tracer(s, device=0) as rt:
        rt.step(64)
        rgb, V, S, cnt = rt.read_accum()
        c = rt.counters()
    assert c["nonfinite"] == 0
    L = (rgb @ LUMA) / 1000.0
    T = slab_walk(tau, g, 400_000, seed=3)["T"]
    assert abs(L.mean() - T) < 4 * math.hypot(se(T, n), se(T, 400_000)) + 0.002, (L.mean(), T)


def test_a_milky_sphere_vanishes_in_the_furnace():
    s = scenes.milky_spheres(width=64, height=64, furnace=True)
    with create_path_tracer(s, device=0) as rt:
        rt.step(64)
        rgb, V, S, cnt = rt.read_accum()
    assert np.allclose(rgb.reshape(-1, 3).mean(0), 1000.0, rtol=2e-3), rgb.reshape(-1, 3).mean(0)


def test_milky_glass_matches_the_oracle():
    s = scenes.milky_spheres(width=64, height=48)
    with create_path_tracer(s, device=0) as rt:
        rt.step(8)
        rgb, V, S, cnt = rt.read_accum()
        c = rt.counters()
    assert c["nonfinite"] == 0
    ref = oracle.render(s, 8)
    for k in range(3):
        g, r = rgb[..., k], ref.rgb[..., k]
        assert abs(g.mean() / r.mean() - 1) < 0.03, (k, g.mean(), r.mean())
    L, Lr = rgb @ LUMA, ref.luma()
    sd = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    exact = np.abs(L - Lr) <= 1e-3 * np.maximum(np.abs(Lr), 1.0)
    within = np.abs(L - Lr) <= 4 * sd + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert exact.mean() > 0.3, exact.mean()
    assert within.mean() > 0.985, (~within).sum()


def test_a_clear_volume_is_the_glass_alone():
    """scatter_distance 0 reads none of the walk: the picture is the clear glass's, sample for sample, whatever g."""
    out = []
    for g in (0.0, 0.9):
        s = scenes.milky_spheres(width=32, height=24)
        for i in (2, 3):
            s.materials[i].scatter_distance = 0.0
            s.materials[i].scatter_g = g
        with create_path_tracer(s, device=0) as rt:
            rt.step(4)
            out.append(rt.read_accum()[0])
    assert np.array_equal(out[0], out[1])


def render(s, n):
    import ctypes as C
    from shadytracer_gb300 import st_types as T
    with create_path_tracer(s, device=0) as rt:
        rt.step(n)
        rgb, V, S, cnt = rt.read_accum()
        c = rt.counters()
        if s.params.sppm:
            stt = T.StSppmStats()
            assert rt.L.st_sppm_stats_read(rt.ctx, C.byref(stt)) == 0
            c["stored"], c["dropped"] = stt.stored, stt.cut
        return rgb @ LUMA, V, S, c


def test_the_map_in_the_volume_matches_the_oracle():
    """The photons' records where they collide in the slab, gathered at the camera's first collision: the GPU's picture
    against the oracle's, band by band within their error bars, and both against the camera's own paths."""
    s = scenes.milky_slab(sppm=True)
    L, V, S, c = render(s, 16)
    assert c["nonfinite"] == 0
    # records where the photons collided in the slab too, none dropped
    assert c["stored"] > s.params.sppm_photons and c["dropped"] == 0, (c["stored"], c["dropped"])
    ref = oracle.render(s, 16)
    Lr = ref.luma()
    sd = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    for r0 in range(0, 48, 8):
        band = slice(r0, r0 + 8)
        e = np.sqrt(np.sum(sd[band] ** 2)) / sd[band].size
        assert abs(L[band].mean() - Lr[band].mean()) < 4 * e + 0.01 * Lr[band].mean(), (r0, L[band].mean(), Lr[band].mean())
    P, Vp, Sp, _ = render(scenes.milky_slab(sppm=False), 512)
    e = math.hypot(np.sqrt(np.sum(se_of(V, S) ** 2)) / V.size, np.sqrt(np.sum(se_of(Vp, Sp) ** 2)) / Vp.size)
    assert abs(L.mean() - P.mean()) < 4 * e + 0.01 * P.mean(), (L.mean(), P.mean())
