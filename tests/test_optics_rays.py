"""Ray-set sources (optics/sources.js rayset, optics/kernels.js:320-336) and Zemax source files (optics/zemax.js),
on the CPU: the parser against files written here (the header's length unit and placement applied, the spectral
format's wavelength, the refusals), the placement's weights, and the oracle's trace of a ray set through an empty
scene, whose far field is the set's own directions; on the GPU (marked) the same trace against the oracle.
"""
import ctypes as C
import math
import struct

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import optics, scenes
from shadytracer_gb300.st_types import ST_PRIM_SPHERE


def zemax_bytes(rays, units=4, loc=(0.0, 0.0, 0.0), rot=(0.0, 0.0, 0.0), fmt=2, wavelength=0.0, flux_type=1):
    """A source file as OpticStudio writes one (little endian, 208-byte header)."""
    nf = 7 if fmt == 0 else 8
    h = struct.pack("<iI", 8675309, len(rays)) + b"test".ljust(100, b"\0")
    h += struct.pack("<7f", 1000.0, 999.0, wavelength, 0.0, 90.0, 0.0, 360.0)
    h += struct.pack("<i", units) + struct.pack("<3f", *loc) + struct.pack("<3f", *rot)
    h += struct.pack("<7f", 1, 1, 1, 0, 0, 0, 0) + struct.pack("<ii", fmt, flux_type) + struct.pack("<ii", 0, 0)
    assert len(h) == 208
    return h + np.asarray(rays, "<f4").reshape(-1)[: len(rays) * nf].tobytes()


def test_parse_spectral_mm_file():
    rays = [[1.0, 2.0, 3.0, 0.0, 0.0, 2.0, 0.5, 0.55], [0.0, 0.0, 0.0, 3.0, 4.0, 0.0, 1.5, 0.45]]
    head, r = optics.parse_zemax(zemax_bytes(rays, units=4, loc=(10.0, 0.0, 0.0)))
    assert head["count"] == 2 and head["units"] == "mm" and head["flux_type"] == "lm" and not head["rotated"]
    assert np.allclose(r[0, 0:3], [0.011, 0.002, 0.003]) and np.allclose(r[1, 0:3], [0.010, 0.0, 0.0])
    assert np.allclose(r[0, 4:7], [0, 0, 1]) and np.allclose(r[1, 4:7], [0.6, 0.8, 0.0])
    assert np.allclose(r[:, 3], [0.5, 1.5]) and np.allclose(r[:, 7], [550.0, 450.0])


def test_parse_flux_only_and_rotation():
    rays = [[0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 2.0]]
    head, r = optics.parse_zemax(zemax_bytes(rays, units=0, fmt=0, wavelength=0.6, rot=(math.pi / 2, 0.0, 0.0)))
    assert head["rotated"] and np.allclose(r[0, 4:7], [0.0, -1.0, 0.0], atol=1e-6)   # +z about x by 90: -y
    assert r[0, 7] == pytest.approx(600.0)


def test_parse_refuses():
    good = zemax_bytes([[0, 0, 0, 0, 0, 1, 1, 0.5]])
    with pytest.raises(ValueError):
        optics.parse_zemax(good[:-4])                      # a length that disagrees with the count
    with pytest.raises(ValueError):
        optics.parse_zemax(good[:100])                     # shorter than the header
    with pytest.raises(ValueError):
        optics.parse_zemax(zemax_bytes([[0, 0, 0, 0, 0, 1, 1, 0.5]], units=9))
    with pytest.raises(ValueError):
        optics.parse_zemax(zemax_bytes([[0, 0, 0, 0, 0, 1, 1, 0.5]], fmt=1))


def test_placement_weights():
    r = np.zeros((4, 8), np.float32)
    r[:, 3] = [1, 2, 3, 6]
    r[:, 6] = 1
    p = optics.ray_set_rays(r, origin=(0, 0, 1))
    assert np.allclose(p[:, 3].mean(), 1.0) and np.allclose(p[:, 2], 1.0)


def lamp_set(n=2000, seed=3):
    """A small ray set: a cone of directions about +z from points near the origin, weights uneven."""
    rng = np.random.default_rng(seed)
    th = np.arccos(1 - rng.random(n) * (1 - math.cos(math.radians(40))))
    ph = rng.random(n) * 2 * math.pi
    r = np.zeros((n, 8), np.float32)
    r[:, 0:2] = rng.normal(scale=1e-3, size=(n, 2))
    r[:, 3] = rng.uniform(0.2, 2.0, n)
    r[:, 4] = np.sin(th) * np.cos(ph)
    r[:, 5] = np.sin(th) * np.sin(ph)
    r[:, 6] = np.cos(th)
    return optics.ray_set_rays(r)


def empty_bench():
    """One instance whose only primitive is a small sphere well below the source (nothing in the rays' way)."""
    s = scenes.Scene([scenes.prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, -3.0), params=(0.05,), material=1, flags=0)],
                     [scenes.air(), scenes.diffuse((0.5, 0.5, 0.5))], env_radius=10.0, name="empty")
    s.params = scenes.default_params(width=8, height=8, maxbounce=8)
    s.view = scenes.look_at((0, -3, 0), (0, 0, 0), 40.0, 1.0)
    return s


def test_oracle_ray_set_far_field():
    """Through an empty scene every traced ray escapes along its set ray's direction: the far field holds the set's
    weights by direction (sampled), and what escapes is what was emitted, exactly."""
    rays = lamp_set()
    s = empty_bench()
    s.info = {"sources": [optics.ray_set_source(0, len(rays), 1000.0)]}
    try:
        oracle.optics_set_rays(rays)
        out = oracle.optics_run(s, [200000], nC=36, nG=19)
    finally:
        oracle.optics_set_rays(None)
    t = out["totals"][0]
    assert abs(t["escaped"] / t["emitted"] - 1) < 1e-9 and abs(t["emitted"] / 200000 - 1) < 0.01
    far = out["far"][0]
    # the set's own weights binned the same way (gamma from +z, C from +x), scaled to the emitted weight
    d = rays[:, 4:7].astype(np.float64)
    g = np.arccos(np.clip(d[:, 2], -1, 1))
    c = np.mod(np.arctan2(d[:, 1], d[:, 0]), 2 * math.pi)
    ig = np.minimum((g / math.pi * 18 + 0.5).astype(int), 18)
    ic = (c / (2 * math.pi) * 36 + 0.5).astype(int) % 36
    exp = np.zeros((19, 36))
    np.add.at(exp, (ig, ic), rays[:, 3])
    exp *= t["emitted"] / exp.sum()
    big = exp > 200
    rel = np.abs(far[big] - exp[big]) / exp[big]
    assert np.median(rel) < 0.05, np.median(rel)


@pytest.mark.gpu
def test_gpu_ray_set_matches_the_oracle():
    from shadytracer_gb300.renderer import create_path_tracer
    rays = lamp_set()
    s = empty_bench()
    src = optics.ray_set_source(0, len(rays), 1000.0)
    with create_path_tracer(s, device=0) as rt:
        O = optics.Optics(rt)
        O.set_rays(rays)
        O.set_sources([src])
        O.set_far(nC=36, nG=19)
        r = O.run([400000], lux_cells=8)
    s.info = {"sources": [src]}
    try:
        oracle.optics_set_rays(rays)
        ref = oracle.optics_run(s, [400000], nC=36, nG=19)
    finally:
        oracle.optics_set_rays(None)
    t, tr = r["totals"][0], ref["totals"][0]
    assert abs(t["escaped"] / t["emitted"] - 1) < 1e-6
    assert abs(t["emitted"] / tr["emitted"] - 1) < 0.01
    a, b = r["far"][0], ref["far"][0]
    big = b > 500                       # bins of a few hundred rays or more: within 10 %, as sampling allows
    assert np.mean(np.abs(a[big] - b[big]) / b[big] < 0.1) > 0.9
