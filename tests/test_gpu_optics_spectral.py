"""The optics trace by wavelength on the GPU (csrc/st_optics.cu: the source's three wavelengths and weights, a
material and a coating at each, the tallies' Y, the hits' XYZ; st_spectral.h's tables and spectra), held to the closed
forms the reference's optics-spectral rows are (lib/pathtracer/tests.js:1469-1531; tests/spectral_forms.py): a light by
its spectrum through clear glass reads its own chromaticity and passes the slab's Fresnel; a light by its colour is a
stand-in spectrum of exactly that colour; the dichroic of the coated slab by wavelength passes the spectrum times y-bar
times the slab's transmission at each wavelength. (The reference's LED preset is a published table; a blackbody of its
4100 K stands in for it here.) And the colour trace's coloured light: a red light through the dichroic passes 1 - R_red.
"""
import math

import numpy as np
import pytest

from shadytracer_gb300 import optics, scenes as S
from shadytracer_gb300.renderer import create_path_tracer
import spectral_forms as F

pytestmark = pytest.mark.gpu
LUMA = np.array([0.2126, 0.7152, 0.0722])


def run(s, n, spectral=1, spectra=None):
    with create_path_tracer(s, device=0) as rt:
        O = optics.Optics(rt)
        if spectra is not None:
            O.set_spectra(spectra)
        O.set_sources(s.info["sources"])
        O.set_far(nC=36, nG=19)
        O.set_detail(det_cap=1 << 21)
        r = O.run([n], lux_cells=8, spectral=spectral)
        hits, nh = O.hits()
    t = r["totals"][0]
    X = np.array([hits[:, 9].sum(), hits[:, 3].sum(), hits[:, 10].sum()])
    return t["detected"] / t["emitted"], F.xy(X), nh


def slab(where=S.COAT_NONE, deg=0.0, n=400_000, colour=None, cct=0.0, spectrum=0):
    s = S.coated_slab(where, 0.0, 1.0, deg=deg, rays=n)
    src = s.info["sources"][0]
    if colour is not None:
        for k in range(3):
            src.colour[k] = colour[k]
    src.cct, src.spectrum = cct, spectrum
    return s


CLEAR = (1 - 0.04) / (1 + 0.04)


@pytest.mark.parametrize("cct", [2700.0, 4100.0, 6500.0])
def test_a_blackbody_through_clear_glass(cct):
    n = 400_000
    share, c, nh = run(slab(cct=cct, n=n), n)
    assert nh > 0.9 * n
    assert abs(share - CLEAR) < 4 * math.sqrt(CLEAR * (1 - CLEAR) / n) + 2e-3, share
    target = F.xy(np.array([np.sum(F.planck(cct) * F.CMF[k]) for k in range(3)]))
    assert F.duv(c, target) < 1e-3, (c, target)


def test_a_light_by_its_colour_is_that_colour():
    n = 400_000
    rgb = (1.0, 0.55, 0.25)
    share, c, _ = run(slab(colour=rgb, n=n), n)
    assert abs(share - CLEAR) < 4 * math.sqrt(CLEAR * (1 - CLEAR) / n) + 2e-3, share
    assert F.duv(c, F.xy(F.RGB_TO_XYZ @ np.array(rgb))) < 1e-3


def test_a_light_by_its_spectrum():
    """A spectrum of the table: two peaks at 450 and 600 nm."""
    n = 400_000
    sp = np.exp(-0.5 * ((F.L - 450) / 12) ** 2) + 0.6 * np.exp(-0.5 * ((F.L - 600) / 20) ** 2)
    share, c, _ = run(slab(spectrum=1, n=n), n, spectra=sp[None, :].astype(np.float32))
    assert abs(share - CLEAR) < 4 * math.sqrt(CLEAR * (1 - CLEAR) / n) + 2e-3, share
    assert F.duv(c, F.xy(F.CMF @ sp)) < 1.5e-3


@pytest.mark.parametrize("where,deg", [(S.COAT_AR_BACK, 0.0), (S.COAT_AR_BACK, 45.0), (S.COAT_EVERY_FACE, 0.0)])
def test_the_dichroic_by_wavelength(where, deg):
    n = 400_000
    edge = S.coat_edge_at(600.0, math.sin(math.radians(deg)), 1.8)
    s20 = 20.0 / (2 * math.log(9))
    R = 1.0 / (1.0 + np.exp(-(F.L - edge) / s20))
    T = (1 - R) / (1 + R) if where == S.COAT_EVERY_FACE else 1 - R
    share_e, c_e = F.through(F.planck(4100.0), T)
    share, c, _ = run(slab(where=where, deg=deg, cct=4100.0, n=n), n)
    assert abs(share - share_e) < 4 * math.sqrt(max(share_e * (1 - share_e), 0.01) / n) * 1.5 + 3e-3, (share, share_e)
    assert F.duv(c, c_e) < 2e-3, (c, c_e)


def test_a_red_light_through_the_dichroic_in_colour():
    """The colour trace (optics-coating's last row): a red light's rays pick reflection by what they carry, so it passes
    1 - R_red exactly, its rays not split into heavy and empty ones."""
    n = 400_000
    R = S.coat_edge_rgb(0.0, 1.0, 600.0, 20.0)
    share, c, _ = run(slab(where=S.COAT_AR_BACK, colour=(1.0, 0.0, 0.0), n=n), n, spectral=0)
    assert abs(share - (1 - R[0])) < 4 * math.sqrt((1 - R[0]) * R[0] / n) + 2e-3, (share, 1 - R[0])


def channel_weights():
    """The camera's wavelength table as the draw reads it (st_spectral.h spectral_table): per 1 nm cell from 380 nm,
    each channel's clipped Rec.709 colour-matching function averaged over the cell (8 midpoints), normalised."""
    l = 380.0 + (np.arange(400 * 8) + 0.5) / 8.0
    rgb = np.maximum(F.XYZ_TO_RGB @ F.cmf(l), 0.0).reshape(3, 400, 8).mean(axis=2)
    return rgb / rgb.sum(axis=1, keepdims=True), 380.0 + np.arange(400) + 0.5


def cauchy(nd, vd, l):
    B = (nd - 1) / (vd * (1 / 486.13 ** 2 - 1 / 656.27 ** 2))
    return nd + B * (1 / l ** 2 - 1 / 587.56 ** 2)


@pytest.mark.parametrize("abbe", [0.0, 28.0])
def test_a_dispersive_wedge_fans_the_beam(abbe):
    """optics-dispersion (lib/pathtracer/tests.js:1331-1390): a collimated white beam through a 30 degree wedge of n_d
    1.75; each ray refracted into the glass takes a wavelength and refracts at n(l), so each channel's mean exit angle
    over the detector hits is Snell's at each wavelength averaged with that channel's weights; Abbe 0, one angle."""
    n = 200_000
    s = S.dispersive_wedge(abbe=abbe, rays=n)
    with create_path_tracer(s, device=0) as rt:
        O = optics.Optics(rt)
        O.set_sources(s.info["sources"])
        O.set_far(nC=36, nG=19)
        O.set_detail(det_cap=1 << 20)
        O.run([n], lux_cells=8)
        hits, nh = O.hits()
    ang = np.degrees(np.arctan2(hits[:, 4], -hits[:, 6]))
    ok = (ang > -30.0) & (ang < -18.0)
    assert ok.mean() > 0.8, ok.mean()
    rgb = (F.XYZ_TO_RGB @ np.stack([hits[ok, 9], hits[ok, 3], hits[ok, 10]])).astype(np.float64)
    got = (rgb * ang[ok]).sum(axis=1) / rgb.sum(axis=1)
    if abbe == 0.0:
        assert np.allclose(got, S.wedge_exit_deg(30.0, 1.75), atol=2e-3), got
        return
    W, lc = channel_weights()
    a = np.array([S.wedge_exit_deg(30.0, cauchy(1.75, abbe, x)) for x in lc])
    expect = W @ a
    assert np.all(np.diff(got) < 0), got                       # blue bent most, red least
    assert np.allclose(got, expect, atol=0.01), (got, expect)
