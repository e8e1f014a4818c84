"""Scattering inside a material on the CPU (materials.js scatterDistance, haze.js:574-650 THE MEDIUM'S WALK): the
walk in numpy (tests/slab_walk.py) against what radiative transfer says of a slab -- the reference's own checks of its
mirror, core/test/volume.test.mjs -- and the oracle's march walking an index-matched slab against that walk, as the
reference holds its march to its mirror (core/test/volume.gpu.mjs); a lossless milky sphere vanishes in the furnace.
"""
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes
from slab_walk import hg_cos, slab_walk

LUMA = np.array([0.2126, 0.7152, 0.0722])
se = lambda p, n: math.sqrt(max(p * (1 - p), 1e-12) / n)


@pytest.mark.parametrize("tau,g", [(0.3, 0.0), (1.0, 0.0), (2.0, 0.8), (3.0, -0.4)])
def test_the_ballistic_part_and_nothing_lost(tau, g):
    N = 200_000
    r = slab_walk(tau, g, N, seed=11)
    assert abs(r["ballistic"] - math.exp(-tau)) < 4 * se(math.exp(-tau), N)
    assert abs(r["T"] + r["R"] - 1.0) < 1e-12


def test_the_diffusion_regime():
    """T(tau) -> C / (tau + 2 q) for isotropic scattering, q = 0.7104 the Milne problem's extrapolation length: T (tau
    + 2 q) stops depending on the depth; and the collisions a ray takes grow with it."""
    q = 0.7104
    rows = []
    for tau, N in ((10, 100_000), (20, 100_000), (40, 60_000)):
        r = slab_walk(tau, 0.0, N, seed=12)
        rows.append((tau, r["T"] * (tau + 2 * q), se(r["T"], N) * (tau + 2 * q), r["steps"]))
    ref = rows[1][1]
    for tau, c, e, _ in rows:
        assert abs(c - ref) < 4 * math.hypot(e, rows[1][2]) + 0.01 * ref, rows
    assert rows[2][3] > 1.5 * rows[1][3] and rows[1][3] > 1.5 * rows[0][3], rows


def test_forward_scattering_and_the_phase_functions_mean():
    a, b = slab_walk(3.0, 0.0, 100_000, 13), slab_walk(3.0, 0.8, 100_000, 13)
    assert b["T"] > a["T"] + 0.1
    r = np.random.default_rng(7)
    for g in (0.7, -0.3):
        assert abs(hg_cos(g, r.random(400_000)).mean() - g) < 0.005


@pytest.mark.parametrize("tau,g", [(0.5, 0.0), (1.0, 0.0), (3.0, 0.8), (6.0, 0.5)])
def test_the_oracles_slab_is_the_walk(tau, g):
    """An index-matched slab seen head-on in front of a glowing plane: each pixel reads le x T(tau, g)."""
    s = scenes.volume_slab(tau, g, width=16, height=16)
    n = 16 * 16 * 16
    L = oracle.render(s, 16).luma() / 1000.0
    T = slab_walk(tau, g, 400_000, seed=3)["T"]
    assert abs(L.mean() - T) < 4 * math.hypot(se(T, n), se(T, 400_000)) + 0.003, (L.mean(), T)


def test_a_milky_sphere_vanishes_in_the_furnace():
    s = scenes.milky_spheres(width=48, height=48, furnace=True)
    r = oracle.render(s, 16)
    assert np.allclose(r.rgb.reshape(-1, 3).mean(0), 1000.0, rtol=2e-3), r.rgb.reshape(-1, 3).mean(0)


def test_a_clear_volume_is_the_glass_alone():
    """scatter_distance 0: the walk is not there -- the picture is the clear glass's, path for path."""
    s = scenes.milky_spheres(width=32, height=24)
    a = oracle.render(s, 2).rgb
    for i in (2, 3):
        s.materials[i].scatter_distance = 0.0
    b = oracle.render(s, 2).rgb
    s2 = scenes.milky_spheres(width=32, height=24)
    for i in (2, 3):
        s2.materials[i].scatter_distance = 0.0
        s2.materials[i].scatter_g = 0.9
    c = oracle.render(s2, 2).rgb
    assert np.array_equal(b, c) and not np.allclose(a, b)


def test_the_map_in_the_volume_agrees_with_the_camera_alone():
    """The photon map in the volume (sppm.js sppmGatherVolume, haze.js mediumStore): a milky slab lit by the sun only;
    with the map on, the sun's photons store where they collide in it and a camera ray that came in through its face
    gathers them at its first collision (and the floor under it, what the slab let through); with it off, the camera's
    paths find the sun through the walk by chance (its disc made 5 degrees wide). The same picture on average."""
    a = oracle.render(scenes.milky_slab(sppm=True), 16)
    b = oracle.render(scenes.milky_slab(sppm=False), 512)
    A, B = a.luma(), b.luma()
    se_b = np.sqrt(np.sum(np.nan_to_num(b.se()) ** 2)) / B.size
    se_a = np.sqrt(np.sum(np.nan_to_num(a.se()) ** 2)) / A.size
    assert abs(A.mean() - B.mean()) < 4 * math.hypot(se_a, se_b) + 0.01 * B.mean(), (A.mean(), B.mean(), se_a, se_b)


def test_the_slab_glows_from_the_map_alone():
    """With the sun's true disc (0.53 degrees) the camera's own paths almost never find it through the walk; the map's
    photons carry its light into the slab, which glows."""
    a = oracle.render(scenes.milky_slab(sppm=True, sun_diameter=0.53), 8).luma()
    b = oracle.render(scenes.milky_slab(sppm=False, sun_diameter=0.53), 8).luma()
    rows = slice(8, 32)                                        # the slab's face and the floor it shades
    assert a[rows].mean() > 1.15 * b[rows].mean(), (a[rows].mean(), b[rows].mean())
