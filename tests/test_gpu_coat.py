"""Coatings on the GPU (st_device.cuh coat_edge_rgb, make_lobes, coat_pick; csrc/st_optics.cu, st_render.cu,
st_photons.cu): the optics trace of a coated slab against the incoherent series of the reference's optics-coating
test (optics/fresnel.js coatedSlabT; lib/pathtracer/tests.js:1257-1330), a lossless coating in the white furnace,
and a render of coated glass, a coated metal and a coated dispersive glass against the oracle.
"""
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import optics, scenes as S
from shadytracer_gb300.renderer import create_path_tracer

from test_oracle_coat import CASES, LUMA, slab_expected

pytestmark = pytest.mark.gpu


def se_of(V, Sm):
    ok = (Sm > 0) & (Sm < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(Sm[ok] * V[ok] / (1 - Sm[ok]))
    return out


def gpu_slab(s, n):
    with create_path_tracer(s, device=0) as rt:
        O = optics.Optics(rt)
        O.set_sources(s.info["sources"])
        O.set_far(nC=36, nG=19)
        return O.run([n], lux_cells=8)["totals"][0]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_the_coated_slab(case):
    label, where, lo, hi, deg = case
    n = 400_000
    t = gpu_slab(S.coated_slab(where, lo, hi, deg=deg, rays=n), n)
    share = t["detected"] / t["emitted"]
    exp = slab_expected(where, lo, hi, deg)
    assert abs(share - exp) < 4 * math.sqrt(max(exp * (1 - exp), 0.01) / n) * 1.5 + 1e-9, (label, share, exp)


def test_the_bare_slab_is_the_glass_alone():
    n = 400_000
    t = gpu_slab(S.coated_slab(S.COAT_NONE, rays=n), n)
    F = 0.04
    assert t["detected"] / t["emitted"] == pytest.approx((1 - F) / (1 + F), abs=4 * math.sqrt(0.08 / n))


@pytest.mark.parametrize("where", [S.COAT_AR_BACK, S.COAT_BARE_BACK, S.COAT_EVERY_FACE])
def test_a_lossless_coating_in_the_furnace(where):
    """R + T = 1 in every channel and the glass absorbs nothing: every pixel reads the environment on average, each
    channel alone -- the pick by the ray's own channels (coat_pick) keeps the weights unbiased."""
    s = S.coated_spheres(width=64, height=64, furnace=True, where=where, maxbounce=64)
    with create_path_tracer(s, device=0) as rt:
        rt.step(64)
        rgb, V, Sm, cnt = rt.read_accum()
        c = rt.counters()
    assert c["nonfinite"] == 0
    assert np.allclose(rgb.reshape(-1, 3).mean(0), 1000.0, rtol=1e-2), rgb.reshape(-1, 3).mean(0)


def test_coated_spheres_match_the_oracle():
    s = S.coated_spheres(width=64, height=48)
    with create_path_tracer(s, device=0) as rt:
        rt.step(8)
        rgb, V, Sm, cnt = rt.read_accum()
    ref = oracle.render(s, 8)
    for c in range(3):                                  # per channel: a dichroic is colour
        g, r = rgb[..., c], ref.rgb[..., c]
        assert abs(g.mean() / r.mean() - 1) < 0.03, (c, g.mean(), r.mean())
    L, Lr = rgb @ LUMA, ref.luma()
    se = np.sqrt(se_of(V, Sm) ** 2 + np.nan_to_num(ref.se()) ** 2)
    exact = np.abs(L - Lr) <= 1e-3 * np.maximum(np.abs(Lr), 1.0)
    within = np.abs(L - Lr) <= 4 * se + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert exact.mean() > 0.5, exact.mean()
    assert within.mean() > 0.985, (~within).sum()


def test_no_coating_is_the_bare_material():
    """coat 0 reads none of the coating's fields: the picture is the bare glass's, sample for sample."""
    out = []
    for junk in (False, True):
        s = S.dispersive_furnace(width=48, height=32, abbe=0.0, floor=True)
        if junk:
            m = s.materials[1]                      # the table the scene hands the library, changed in place
            m.coat, m.coat_lo, m.coat_hi, m.coat_edge, m.coat_width = 0, 0.9, 0.9, 500.0, 5.0
        with create_path_tracer(s, device=0) as rt:
            rt.step(4)
            out.append(rt.read_accum()[0])
    assert np.array_equal(out[0], out[1])
