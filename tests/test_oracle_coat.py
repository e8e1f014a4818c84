"""Coatings on the CPU (core/materials.js coat, core/spectral.js edgeRGB / edgeAt / edgeAt1, materials_pbr.js
coatFresnel / coatPick / coatOverMetal): the reflectance per channel against its own definition, the oracle's
coated lobes, and the oracle's optics trace of a coated slab against the incoherent series the reference's
optics-coating test holds it to (optics/fresnel.js coatedSlabT; lib/pathtracer/tests.js:1257-1330).
"""
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes as S

LUMA = np.array([0.2126, 0.7152, 0.0722])


def test_a_constant_coating_is_its_reflectance_in_every_channel():
    """Each channel's weights sum to 1, so a coating with no edge (lo = hi: a beam splitter) reflects R exactly."""
    for R in (0.0, 0.37, 0.5, 1.0):
        assert np.allclose(oracle.coat_rgb(R, R, 600.0, 20.0), R, atol=1e-12)
        assert np.allclose(S.coat_edge_rgb(R, R, 600.0, 20.0), R, atol=1e-12)
    # an edge far below the visible is hi everywhere, far above it lo
    assert np.allclose(oracle.coat_rgb(0.1, 0.9, 200.0, 20.0), 0.9, atol=1e-9)
    assert np.allclose(oracle.coat_rgb(0.1, 0.9, 1100.0, 20.0), 0.1, atol=1e-9)


def test_the_bins_mean_of_the_edge_is_exact():
    """A bin's mean of the logistic is a softplus difference: the same as integrating the logistic across the bin."""
    for edge, width in ((600.0, 20.0), (551.8, 5.0), (483.0, 0.0), (620.0, 80.0)):
        got = oracle.coat_rgb(0.0, 1.0, edge, width)
        assert np.allclose(got, S.coat_edge_rgb(0.0, 1.0, edge, width), atol=1e-10)
        # brute force: the logistic at 0.001 nm against each bin's weight
        s = max(width, 0.01) / (2 * math.log(9))
        l = 380.0 + (np.arange(400000) + 0.5) * 0.001
        R = 1.0 / (1.0 + np.exp(-np.clip((l - edge) / s, -700, 700)))
        mean = R.reshape(40, 10000).mean(axis=1)
        # the weights themselves: a step at each bin boundary picks them out
        bins = np.array([S.coat_edge_rgb(0, 1, 380.0 + 10 * k, 0.0) - S.coat_edge_rgb(0, 1, 390.0 + 10 * k, 0.0)
                         for k in range(40)])
        assert np.allclose(bins.sum(axis=0), 1.0, atol=1e-6)
        assert np.allclose(bins.T @ mean, got, atol=2e-5), (edge, width)


def test_a_step_at_600_reflects_each_channels_share_above_it():
    r = oracle.coat_rgb(0.0, 1.0, 600.0, 0.0)
    assert r[0] > 0.5 and r[1] < 0.05 and r[2] < 1e-6          # red mostly above 600 nm, blue none of it
    assert np.all(np.diff([oracle.coat_rgb(0, 1, e, 20.0)[1] for e in (650, 600, 550, 500)]) > 0)


def test_the_edge_moves_with_the_angle():
    # 600 nm at normal incidence through an effective index of 1.8, at 45 degrees: 551.8 nm (the reference's note)
    assert S.coat_edge_at(600.0, math.sin(math.radians(45)), 1.8) == pytest.approx(551.8, abs=0.05)
    # past what the stack's index can carry, every wavelength is on the long side
    assert S.coat_edge_at(600.0, 2.0, 1.8) == 0.0


def test_one_wavelength_takes_the_logistic_itself():
    assert oracle.coat_at_lambda(0.0, 1.0, 600.0, 20.0, 600.0) == pytest.approx(0.5)
    s = 20.0 / (2 * math.log(9))
    assert oracle.coat_at_lambda(0.0, 1.0, 600.0, 20.0, 610.0) == pytest.approx(1 / (1 + math.exp(-10 / s)))
    # the 10-90 % width: 10 % at edge - w/2, 90 % at edge + w/2
    assert oracle.coat_at_lambda(0.0, 1.0, 600.0, 20.0, 590.0) == pytest.approx(0.1, abs=1e-12)
    assert oracle.coat_at_lambda(0.0, 1.0, 600.0, 20.0, 610.0) == pytest.approx(0.9, abs=1e-12)


def coated_glass(where, lo, hi, edge=600.0, width=20.0):
    return S.coated(S.material(base=(1, 1, 1), roughness=0.0, specular=0.5, transmission=1.0, ior=1.5),
                    where, lo, hi, edge, width, 1.8)


def test_a_coloured_ray_picks_reflection_by_what_it_carries():
    """coatPick: a red ray at a dichroic reflects as often as red does, with weight 1 -- no heavy and empty rays -- and a
    white one splits by the channels' mean; either way each channel's reflected and passed weights average R_c, 1 - R_c."""
    m = coated_glass(S.COAT_AR_BACK, 0.0, 1.0)
    R = oracle.coat_rgb(0.0, 1.0, 600.0, 20.0)
    v = (0.0, 0.0, 1.0)
    n = 200_000
    d, w = oracle.lobes_sample_coat(m, v, 1 / 1.5, 1.0, False, 0.0, (1.0, 0.0, 0.0), 3, n)
    refl = d[:, 2] > 0
    assert refl.mean() == pytest.approx(R[0], abs=4 * math.sqrt(R[0] * (1 - R[0]) / n))
    assert np.allclose(w[refl, 0], 1.0) and np.allclose(w[~refl, 0], 1.0)
    d, w = oracle.lobes_sample_coat(m, v, 1 / 1.5, 1.0, False, 0.0, (1.0, 1.0, 1.0), 3, n)
    refl = d[:, 2] > 0
    ps = R.mean()
    assert refl.mean() == pytest.approx(ps, abs=4 * math.sqrt(ps * (1 - ps) / n))
    for c in range(3):
        assert (w[refl, c].sum() / n) == pytest.approx(R[c], abs=0.01)
        assert (w[~refl, c].sum() / n) == pytest.approx(1 - R[c], abs=0.01)


def test_coatings_by_face():
    """Seen from inside (the face light leaves by): coat 1 reflects nothing but total internal reflection, coat 2 the
    glass's own Fresnel, coat 3 the coating again."""
    v = (0.0, 0.0, 1.0)
    n = 100_000
    for where, expect in ((S.COAT_AR_BACK, 0.0), (S.COAT_BARE_BACK, 0.04), (S.COAT_EVERY_FACE, 0.5)):
        m = coated_glass(where, 0.5, 0.5)
        d, w = oracle.lobes_sample_coat(m, v, 1.5, 1.5, True, 0.0, (1.0, 1.0, 1.0), 5, n)
        refl = (d[:, 2] > 0)
        got = (w[refl, 1]).sum() / n
        assert got == pytest.approx(expect, abs=0.01), (where, got)
    # and past the critical angle every coating reflects it all
    m = coated_glass(S.COAT_AR_BACK, 0.0, 0.0)
    c = 0.3                                                      # sin 0.954 > 1 / 1.5
    d, w = oracle.lobes_sample_coat(m, (math.sqrt(1 - c * c), 0.0, c), 1.5, 1.5, True, 0.0, (1, 1, 1), 5, 1000)
    assert np.all(d[:, 2] > 0) and np.allclose(w, 1.0)


def test_a_coating_over_a_metal():
    """1 - (1 - R)(1 - F) / (1 - R F): never below either alone; a white metal stays white, no coating changes a
    black one's R, an AR layer (R 0) changes nothing."""
    m = S.coated(S.metal((0.9, 0.6, 0.3), 0.0), S.COAT_AR_BACK, 0.3, 0.3, 600.0, 20.0)
    d, w = oracle.lobes_sample_coat(m, (0, 0, 1), 1.0, 1.0, False, 0.0, (1, 1, 1), 1, 16)
    F = np.array([0.9, 0.6, 0.3])
    assert np.allclose(w[0], 1 - 0.7 * (1 - F) / (1 - 0.3 * F), atol=1e-9)
    m = S.coated(S.metal((0.9, 0.6, 0.3), 0.0), S.COAT_AR_BACK, 0.0, 0.0, 600.0, 20.0)
    d, w = oracle.lobes_sample_coat(m, (0, 0, 1), 1.0, 1.0, False, 0.0, (1, 1, 1), 1, 16)
    assert np.allclose(w[0], F, atol=1e-9)


CASES = [  # (label, where, R below the edge, R above it, the beam's tilt in degrees); the edge at 600 nm, 20 nm wide
    ("beam splitter 50/50, AR back, 0 deg", S.COAT_AR_BACK, 0.5, 0.5, 0.0),
    ("beam splitter 50/50, AR back, 45 deg", S.COAT_AR_BACK, 0.5, 0.5, 45.0),
    ("beam splitter 50/50, bare back, 0 deg", S.COAT_BARE_BACK, 0.5, 0.5, 0.0),
    ("beam splitter 50/50, every face, 0 deg", S.COAT_EVERY_FACE, 0.5, 0.5, 0.0),
    ("anti-reflective (R 0), 45 deg", S.COAT_AR_BACK, 0.0, 0.0, 45.0),
    ("dichroic > 600 nm, AR back, 0 deg", S.COAT_AR_BACK, 0.0, 1.0, 0.0),
    ("dichroic > 600 nm, AR back, 45 deg", S.COAT_AR_BACK, 0.0, 1.0, 45.0),
    ("dichroic > 600 nm, every face, 0 deg", S.COAT_EVERY_FACE, 0.0, 1.0, 0.0),
]


def slab_expected(where, lo, hi, deg):
    """The share of a white beam's luminous flux the coated slab passes: per channel the incoherent series at R_c,
    weighed by luminance (the trace tallies a ray by its luminance)."""
    R = S.coat_edge_rgb(lo, hi, S.coat_edge_at(600.0, math.sin(math.radians(deg)), 1.8), 20.0)
    return float(LUMA @ np.array([S.coated_slab_t(deg, 1.5, r, where) for r in R]))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_the_oracles_coated_slab(case):
    label, where, lo, hi, deg = case
    n = 100_000
    s = S.coated_slab(where, lo, hi, deg=deg, rays=n)
    t = oracle.optics_run(s, [n], nC=36, nG=19)["totals"][0]
    share = t["detected"] / t["emitted"]
    exp = slab_expected(where, lo, hi, deg)
    # a ray carries weight up to 1 / min(ps, 1 - ps): 4 sigma of a binomial share with room for that
    assert abs(share - exp) < 4 * math.sqrt(max(exp * (1 - exp), 0.01) / n) * 1.5 + 1e-9, (label, share, exp)


def test_the_bare_slab_is_the_glass_alone():
    n = 100_000
    s = S.coated_slab(S.COAT_NONE, deg=0.0, rays=n)
    t = oracle.optics_run(s, [n], nC=36, nG=19)["totals"][0]
    F = ((1.5 - 1) / (1.5 + 1)) ** 2
    assert t["detected"] / t["emitted"] == pytest.approx((1 - F) / (1 + F), abs=4 * math.sqrt(0.08 / n))
