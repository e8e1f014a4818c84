"""The side beyond on the GPU (st_device.cuh: the translucent base, rough refraction's value and density below the
surface, the sky's draw from the far hemisphere; st_render.cu shade_surface's area mix with haze and its light samples
through a face), through the C ABI: GPU against the oracle's restatement (oracle/st_oracle_render.h) in the white
furnace and under the sun, and light sampling through the faces unbiased against the BSDF's draw alone.
"""
import math

import numpy as np
import pytest

from shadytracer_gb300 import scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

LUMA = np.array([0.2126, 0.7152, 0.0722])


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


def render(s, n):
    from shadytracer_gb300.renderer import create_path_tracer
    with create_path_tracer(s, device=0) as r:
        r.step(n)
        rgb, V, S, cnt = r.read_accum()
        ctr = r.counters()
    return rgb @ LUMA, se_of(V, S), ctr


def z_parity(L, se, ref):
    sd = np.hypot(se, se_of(ref.V, ref.S))
    ok = sd > 0
    z = (L - ref.luma())[ok] / sd[ok]
    zm = (L - ref.luma())[ok].mean() / (np.sqrt(np.sum(sd[ok] ** 2)) / ok.sum())
    return np.mean(np.abs(z) < 4), zm


@pytest.mark.parametrize("kind", ["opal", "hazy", "rough", "frosted"])
def test_translucent_furnace_matches_the_oracle(kind):
    s = scenes.translucent_furnace(kind, width=32, height=32)
    L, se, ctr = render(s, 128)
    ref = oracle.render(s, 128)
    frac, zm = z_parity(L, se, ref)
    assert frac > 0.98 and abs(zm) < 5, (frac, zm)
    c = L[10:22, 10:22]
    if kind != "rough":
        assert abs(c.mean() / 1000.0 - 1) < 0.01, c.mean()
    assert ctr["nonfinite"] == 0


@pytest.mark.parametrize("kind", ["opal", "frosted"])
def test_translucent_sun_matches_the_oracle(kind):
    s = scenes.translucent_sun(kind, width=48, height=36)
    L, se, _ = render(s, 128)
    ref = oracle.render(s, 128)
    frac, zm = z_parity(L, se, ref)
    assert frac > 0.98 and abs(zm) < 5, (frac, zm)


def test_light_through_the_face_is_unbiased():
    """The opal sphere under the sun, light sampling on and off: the same picture in the mean, far less noise on."""
    out = {}
    for nee, n in ((1, 128), (0, 1024)):
        s = scenes.translucent_sun("opal", width=48, height=36)
        s.params.nee = nee
        L, se, _ = render(s, n)
        out[nee] = (L.mean(), math.sqrt(np.sum(se ** 2)) / L.size)
    (m1, e1), (m0, e0) = out[1], out[0]
    assert abs(m1 - m0) < 5 * math.hypot(e1, e0) + 1e-3 * m0, out
    assert e0 * math.sqrt(1024 / 128) > 2 * e1, out


@pytest.mark.parametrize("furnace", [False, True])
def test_anisotropic_gloss_matches_the_oracle(furnace):
    """Anisotropic metal and plastic spheres (microfacet.js mfAnisoAlpha), under the sun and in the furnace: GPU
    against the oracle's restatement, pixel by pixel."""
    s = scenes.aniso_spheres(0.8, width=48, height=36, furnace=furnace)
    L, se, ctr = render(s, 128)
    ref = oracle.render(s, 128)
    frac, zm = z_parity(L, se, ref)
    assert frac > 0.98 and abs(zm) < 5, (frac, zm)
    assert ctr["nonfinite"] == 0


def test_absorption_inside_closed_form():
    """Beer-Lambert inside a material (absorbAlong): every ray through the 1 m cube reads the sky times base^(1 / d),
    each channel, on the GPU as in the oracle."""
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.absorbing_box()
    with create_path_tracer(s, device=0) as r:
        r.step(4)
        rgb = r.read_accum()[0]
    assert np.allclose(rgb.reshape(-1, 3), s.info["expected"], rtol=5e-5)
