"""Dispersion on the GPU (csrc/st_render.cu shade_surface; st_device.cuh cauchy_n, spec_draw; st_spectral.h's
table) against its closed form and the oracle (oracle/st_oracle_spectral.h).

A clear dispersive glass sphere in a uniform environment must read the environment on average: the glass absorbs
nothing and the wavelength a refraction draws weighs each channel by exactly 1 on average. On a floor, its
per-pixel picture -- the coloured fringes Cauchy's index puts in the refraction -- must match the oracle's within
the error bars, most pixels to the last digit (both sides draw the wavelength from the same random number).
"""
import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes

pytestmark = pytest.mark.gpu
LUMA = np.array([0.2126, 0.7152, 0.0722])


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


def test_dispersive_furnace():
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.dispersive_furnace(width=64, height=64, abbe=30.0)
    with create_path_tracer(s, device=0) as rt:
        rt.step(64)
        rgb, V, S, cnt = rt.read_accum()
    L = rgb @ LUMA
    assert abs(L.mean() / 1000.0 - 1) < 5e-3, L.mean()
    # every channel, not only the luminance
    assert np.allclose(rgb.reshape(-1, 3).mean(0), 1000.0, rtol=1e-2)


def test_dispersion_matches_the_oracle():
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.dispersive_furnace(width=64, height=48, abbe=25.0, floor=True)
    with create_path_tracer(s, device=0) as rt:
        rt.step(8)
        rgb, V, S, cnt = rt.read_accum()
    ref = oracle.render(s, 8)
    for c in range(3):                                # per channel: the fringes are colour
        g, r = rgb[..., c], ref.rgb[..., c]
        assert abs(g.mean() / r.mean() - 1) < 0.03, (c, g.mean(), r.mean())
    L, Lr = rgb @ LUMA, ref.luma()
    se = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    exact = np.abs(L - Lr) <= 1e-3 * np.maximum(np.abs(Lr), 1.0)
    within = np.abs(L - Lr) <= 4 * se + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert exact.mean() > 0.5, exact.mean()
    assert within.mean() > 0.985, (~within).sum()


def test_no_abbe_is_no_dispersion():
    """Abbe 0 takes no wavelength: the picture is the same as the glass's without dispersion, sample for sample."""
    from shadytracer_gb300.renderer import create_path_tracer
    out = []
    for abbe in (0.0, -1.0):
        s = scenes.dispersive_furnace(width=32, height=32, abbe=abbe, floor=True)
        with create_path_tracer(s, device=0) as rt:
            rt.step(2)
            out.append(rt.read_accum()[0])
    assert np.array_equal(out[0], out[1])
