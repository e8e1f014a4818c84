"""The detector map on the host (shadytracer_gb300/optics.py detector_map, a restatement of optics/detmap.js:104-213):
hits recorded on a detector as an illuminance map in FP64. Checked on hits of a known illuminance: a uniform square
patch of flux on a tilted plane, and a Gaussian spot."""
import math

import numpy as np
import pytest

from shadytracer_gb300.optics import detector_map, map_frame


def plane_hits(n, seed, tilt=0.3, half=0.05, aspect=0.5):
    """A rectangle 2 half by 2 half aspect on a tilted plane (unequal sides, so the fitted frame is the rectangle's)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(-half, half, n)
    b = rng.uniform(-half * aspect, half * aspect, n)
    u = np.array([math.cos(tilt), 0.0, math.sin(tilt)])
    v = np.array([0.0, 1.0, 0.0])
    return np.outer(a, u) + np.outer(b, v) + np.array([0.1, 0.2, 0.3])


def test_the_frame_is_the_hits_plane():
    p = plane_hits(5000, 1)
    F = map_frame(p)
    n = np.array([-math.sin(0.3), 0.0, math.cos(0.3)])
    assert abs(abs(F["normal"] @ n) - 1) < 1e-9
    assert F["flatness"] < 1e-6


def test_a_floor_is_squared_up_to_the_world():
    rng = np.random.default_rng(2)
    p = np.stack([rng.uniform(-1, 1, 3000), rng.uniform(-1, 1, 3000), np.full(3000, 0.5)], 1)
    F = map_frame(p)
    assert np.allclose(np.abs(F["normal"]), [0, 0, 1])
    assert np.allclose(np.abs(F["u"]) + np.abs(F["v"]), [1, 1, 0])


@pytest.mark.parametrize("smooth", ["none", "gauss", "epan"])
def test_a_uniform_patch_reads_its_illuminance_and_keeps_its_flux(smooth):
    n, half = 400_000, 0.05
    p = plane_hits(n, 3, half=half)
    flux = np.full(n, 1e-3)                              # 400 lm over 0.005 m^2: 80 000 lx
    m = detector_map(p, flux, cells=32, smooth=smooth, bandwidth=1.5)
    E0 = flux.sum() / ((2 * half) * (2 * half * 0.5))
    cell_area = m["cell_m"] ** 2
    assert (m["E"] * cell_area).sum() == pytest.approx(flux.sum(), rel=1e-8)
    # the cells a whole cell (the histogram) or a kernel's reach (the estimates) inside the patch's bounds
    F = m["frame"]
    margin = 1 if smooth == "none" else 5
    ys, xs = np.mgrid[0:F["ny"], 0:F["nx"]]
    lo_a, hi_a = F["a0"] + (xs - margin) * F["size"], F["a0"] + (xs + 1 + margin) * F["size"]
    lo_b, hi_b = F["b0"] + (ys - margin) * F["size"], F["b0"] + (ys + 1 + margin) * F["size"]
    inner = (lo_a >= F["a0"]) & (hi_a <= F["a1"]) & (lo_b >= F["b0"]) & (hi_b <= F["b1"])
    assert inner.sum() >= 60
    assert abs(m["E"][inner].mean() / E0 - 1) < 0.01, (m["E"][inner].mean(), E0)
    assert m["relNoise"] is not None and m["hitsPerLitCell"] > 100


def test_knn_reads_a_gaussian_spot():
    rng = np.random.default_rng(4)
    n, s = 100_000, 0.01
    ab = rng.normal(scale=s, size=(n, 2))
    p = np.stack([ab[:, 0], ab[:, 1], np.zeros(n)], 1)
    flux = np.full(n, 1.0 / n)
    m = detector_map(p, flux, cells=32, smooth="knn", k=64)
    F = m["frame"]
    size = F["size"]
    ca = F["a0"] + (np.arange(F["nx"]) + 0.5) * size
    cb = F["b0"] + (np.arange(F["ny"]) + 0.5) * size
    A, B = np.meshgrid(ca, cb)
    # the map's frame is the world's (a floor): a and b are x and y up to a sign
    E = np.exp(-(A ** 2 + B ** 2) / (2 * s * s)) / (2 * math.pi * s * s)
    centre = (A ** 2 + B ** 2) < (1.5 * s) ** 2
    assert abs(np.median(m["E"][centre] / E[centre]) - 1) < 0.1
