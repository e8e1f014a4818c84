"""The photon map inside the wavefront on the GPU (csrc/st_photons.cu: the sun's photons, their store, the grid, the
camera's gather; st_render.cu's lens field and the disc the map owns) against its closed form and the oracle.

The pane (scenes.sppm_pane): a floor lit only through a clear glass pane, seen through it; its radiance is
T(view) rho / pi E_sun sin(elevation) T(sun), all of it the map's light (light sampling from the floor is blocked by
the glass). The caustic (scenes.sppm_caustic, small): a dispersive glass sphere on a floor under the sun and
a sky; the GPU's picture and the oracle's, photons and camera paths seeded alike, agree within the error bars.
"""
import math

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


def pane_closed_form(ior=1.5, elevation=60.0):
    Fv = oracle.fresnel_dielectric(1.0, 1 / ior)
    Fs = oracle.fresnel_dielectric(math.cos(math.radians(90 - elevation)), 1 / ior)
    return (1 - Fv) / (1 + Fv) * 0.7 / math.pi * 1e5 * math.sin(math.radians(elevation)) * (1 - Fs) / (1 + Fs)


def test_pane_closed_form():
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.sppm_pane(width=64, height=64, photons=1_000_000, r1=0.03)
    with create_path_tracer(s, device=0) as rt:
        rt.step(16)
        rgb, V, S, cnt = rt.read_accum()
        st = rt.L
    L = rgb @ LUMA
    cf = pane_closed_form()
    assert abs(L.mean() / cf - 1) < 0.02, (L.mean(), cf)
    assert np.all(cnt == 16)


def test_pane_needs_the_map():
    """Off, nothing reaches the floor under the glass but what light sampling cannot (the map owns it)."""
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.sppm_pane(width=32, height=32)
    s.params.sppm = 0
    with create_path_tracer(s, device=0) as rt:
        rt.step(4)
        L = rt.read_accum()[0] @ LUMA
    assert L.mean() < 0.01 * pane_closed_form()


def test_caustic_matches_the_oracle():
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.sppm_caustic(width=64, height=64, photons=300_000, r1=0.01)
    with create_path_tracer(s, device=0) as rt:
        rt.step(6)
        rgb, V, S, cnt = rt.read_accum()
        import ctypes as C
        from shadytracer_gb300.st_types import StSppmStats
        stt = StSppmStats()
        assert rt.L.st_sppm_stats_read(rt.ctx, C.byref(stt)) == 0
    ref = oracle.render(s, 6)
    for c in range(3):
        assert abs(rgb[..., c].mean() / ref.rgb[..., c].mean() - 1) < 0.03, c
    L, Lr = rgb @ LUMA, ref.luma()
    se = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    within = np.abs(L - Lr) <= 4 * se + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert within.mean() > 0.98, (~within).sum()
    # the last sample's photon pass stored as many records as the oracle's (the same photons, the same gates)
    n_ref, _ = oracle.sppm_photons(s, 5)
    assert stt.stored > 0 and abs(stt.stored / n_ref - 1) < 0.01, (stt.stored, n_ref)
    assert stt.cut == 0
