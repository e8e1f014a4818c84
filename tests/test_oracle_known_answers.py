"""The oracle pinned to the reference's own known answers, on the CPU.

Each block restates assertions from the reference's unit tests (lib/pathtracer/core/test/*.test.mjs and
lib/pathtracer/optics/test/*.test.mjs) against the oracle's entry points: the photometry of the sun's disc, the error
bar's algebra, the photon map's hash, grid, keep, sub-lists and radius schedule, the haze box's span and the
Henyey-Greenstein lobe, the dielectric Fresnel term, and the far field's bins and intensity. The GPU path is then
held to the oracle by the gpu-marked tests.
"""
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes
from shadytracer_gb300.st_types import default_params

LUMA = (0.2126, 0.7152, 0.0722)


def derive(**kw):
    s = scenes.Scene([scenes.prim(scenes.ST_PRIM_PLANE)], [scenes.air(), scenes.diffuse((0.5, 0.5, 0.5))])
    s.params = default_params(**kw)
    return oracle.derive(s)


# ---- photometry (core/test/photometry.test.mjs:24-90) ----
@pytest.mark.parametrize("deg", [0.53, 5.0, 20.0, 60.0])
def test_disc_integrates_back_to_its_illuminance(deg):
    d = derive(sun_diameter=deg, sun_illuminance=100000.0)
    half, L = d["sun_half"], d["disc_lum"]
    n = 20000
    h = half / n
    t = (np.arange(n) + 0.5) * h
    E = 2 * math.pi * float(np.sum(L * np.cos(t) * np.sin(t) * h))
    assert E == pytest.approx(100000.0, rel=1e-6)
    assert d["sun_omega"] == pytest.approx(2 * math.pi * (1 - math.cos(half)), rel=1e-6)
    assert d["sun_sin2"] == pytest.approx(math.sin(half) ** 2, rel=1e-12)


def test_real_sun():
    d = derive(sun_diameter=0.53, sun_illuminance=100000.0)
    assert 1.4e9 < d["disc_lum"] < 1.8e9
    assert 1.0e-5 < d["sun_omc"] < 1.1e-5
    tint = (d["tint_r"], d["tint_g"], d["tint_b"])
    assert sum(a * b for a, b in zip(tint, LUMA)) == pytest.approx(1.0, abs=1e-12)


def test_sun_on_and_pick():
    assert derive(sun_diameter=0.53, sun_elevation=-0.3)["sun_on"] == 0
    assert derive(sun_diameter=0.53, sun_elevation=-0.2)["sun_on"] == 1
    d = derive(sun_hint=0)
    assert d["sun_on"] == 0 and d["nee_sun_pick"] == 0
    d = derive(env_sun_gain=0.0, sun_elevation=45.0)
    assert d["sun_on"] == 1 and d["nee_sun_pick"] == 0
    d = derive(sun_elevation=45.0, nee_sun_pick=0.5)
    assert d["sun_on"] == 1 and d["nee_sun_pick"] == 0.5


def test_tolerance_and_radius_defaults():
    d = derive(eps=0.0)
    assert d["tol_setting"] == pytest.approx(1e-3)
    assert d["env_radius"] == 400.0 or d["env_radius"] > 0


# ---- the error bar (core/test/measure.test.mjs:36-77) ----
def _spread(window, steps, trials, seed=12345):
    rng = np.random.default_rng(seed)
    xs = -np.log(1 - rng.random((trials, steps)))          # exponential, mean 1, sd 1: a long bright tail
    est, se2 = np.zeros(trials), np.zeros(trials)
    for t in range(trials):
        st = np.zeros(4)
        for k in range(steps):
            oracle.step_moments(st, float(xs[t, k]), window)
        est[t] = st[0]
        se2[t] = oracle.standard_error(st[1], st[2]) ** 2
    return math.sqrt(se2.mean()) / est.std(ddof=1)


@pytest.mark.parametrize("window,steps", [(math.inf, 32), (10.0, 32), (1.0, 50)])
def test_reported_error_is_the_real_spread(window, steps):
    ratio = _spread(window, steps, 6000)
    assert abs(ratio - 1) < 0.05, ratio


def test_moment_algebra():
    rng = np.random.default_rng(1)
    st = np.zeros(4)
    for _ in range(16):
        oracle.step_moments(st, float(rng.exponential()))
    assert abs(st[2] - 1 / 16) < 1e-12                     # a true mean of 16: S = 1/16
    st = np.zeros(4)
    for _ in range(2000):
        oracle.step_moments(st, float(rng.exponential()), 10.0)
    assert abs(1 / st[2] - 21) < 1e-6                      # an EMA window of 10 is worth 21 samples
    st = np.zeros(4)
    for _ in range(50):
        oracle.step_moments(st, float(rng.exponential()))
    st[0] = 1e20
    oracle.step_moments(st, 3.0, 0.0)                      # a reset leaves one sample
    assert st[2] == 1 and st[1] == 0 and st[0] == 3
    assert oracle.standard_error(st[1], st[2]) is None
    assert oracle.standard_error(400.0, 0.2) == pytest.approx(math.sqrt(0.2 * 400 / 0.8), abs=1e-12)


# ---- the photon map (core/test/sppm.test.mjs:201-281) ----
def test_hash_wraps_at_32_bits():
    assert oracle.sppm_hash(-1, 2, 3) == oracle.sppm_hash(np.int32(np.uint32(2 ** 32 - 1).view(np.int32)), 2, 3)
    # the three 32-bit wrapping multiplies XORed, masked to the 2^20 lists (sppm.js:197-198 hashCell)
    for i, j, k in ((1, 0, 0), (0, 1, 0), (0, 0, 1), (-7, 123, -99999), (2 ** 31 - 1, -2 ** 31, 5)):
        h = ((i * 73856093) ^ (j * 19349663) ^ (k * 83492791)) & 0xFFFFFFFF
        assert oracle.sppm_hash(i, j, k) == h & ((1 << 20) - 1)


def test_keep_and_sub_lists():
    assert oracle.sppm_keep(1000, 800) == 1
    assert abs(oracle.sppm_keep(1000, 2000) - 0.85 / 2) < 1e-15
    assert oracle.sppm_keep(0, 5) == 1 and oracle.sppm_keep(1000, 0) == 1
    assert oracle.sppm_subs_of(64, 64) == 32
    assert oracle.sppm_subs_of(65, 64) == math.floor(32 * 64 / 65)
    assert oracle.sppm_subs_of(1000000, 8) == 1


def test_radius_schedule():
    r = lambda k: oracle.sppm_radius(1.0, k, 2.0 / 3.0)
    assert r(1) == 1
    assert all(r(k) < r(k - 1) for k in (2, 3, 10, 100, 1000))
    c = lambda k: r(k) ** 2 * k ** (1 - 2.0 / 3.0)
    assert abs(c(4000) / c(2000) - 1) < 0.001


def test_oct_round_trip():
    rng = np.random.default_rng(3)
    v = rng.normal(size=(200, 3)).astype(np.float32)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for a in v:
        b = oracle.sppm_unoct(oracle.sppm_oct(a))
        assert np.abs(a - b).max() < 1e-4
    assert np.array_equal(oracle.sppm_unoct(oracle.sppm_oct(np.array([0, 0, 1], np.float32))), [0, 0, 1])


def _grid_case(seed=2):
    rng = np.random.default_rng(seed)
    n = 4000
    pos = np.stack([(rng.random(n) - 0.5) * 0.4, (rng.random(n) - 0.5) * 0.4, (rng.random(n) - 0.5) * 0.04], 1)
    pos = pos.astype(np.float32)
    up = rng.random(n) < 0.9
    nv = np.where(up[:, None], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]).astype(np.float32)
    nrm = np.array([oracle.sppm_oct(a) for a in nv], np.uint32)
    power = np.tile(np.array([1.0, 0.0, 0.0], np.float32), (n, 1))
    flags = np.zeros(n, np.uint32)
    return pos, power, nrm, flags, up


def test_grid_finds_every_photon_once():
    r = np.float32(0.013)
    pos, power, nrm, flags, up = _grid_case()
    key, cnt = oracle.sppm_build(pos, power, nrm, flags, np.float32(2 * r))
    assert int(cnt.sum()) == len(flags)
    rng = np.random.default_rng(5)
    m = 2000
    q = np.stack([(rng.random(m) - 0.5) * 0.4, (rng.random(m) - 0.5) * 0.4, (rng.random(m) - 0.5) * 0.04], 1)
    q = q.astype(np.float32)
    qn = np.tile(np.array([0, 0, 1], np.float32), (m, 1))
    qa = np.full((m, 3), np.float32(math.pi), np.float32)   # f = albedo / pi = 1: the sum counts the records
    out, visits, cut = oracle.sppm_gather(q, qn, qa, np.zeros(m, np.uint32), r, 10, 0, 1)
    # brute force, each distance in f32 with each product and sum rounded as the gather rounds it
    d = pos[None, :, :] - q[:, None, :]
    dd = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    brute = ((dd <= r * r) & up[None, :]).sum(1)
    assert brute.sum() > 1000
    assert np.array_equal(np.rint(out[:, 0]).astype(np.int64), brute)
    assert not cut.any()


def test_bounce_cap():
    pos = np.zeros((1, 3), np.float32)
    nrm = np.array([oracle.sppm_oct(np.array([0, 0, 1], np.float32))], np.uint32)
    oracle.sppm_build(pos, np.array([[1, 0, 0]], np.float32), nrm, np.array([5], np.uint32), np.float32(0.1))
    qa = np.full((1, 3), np.float32(math.pi), np.float32)
    qn = np.array([[0, 0, 1]], np.float32)
    got = lambda bc: oracle.sppm_gather(pos, qn, qa, np.array([bc - 1], np.uint32), np.float32(0.05), 9, 0, 1)[0][0, 0]
    assert got(5) == pytest.approx(1, rel=1e-6) and got(6) == 0                    # b_c + b_p <= maxbounce + 1


def test_sub_lists_are_unbiased():
    rng = np.random.default_rng(7)
    n = 6000
    pos = np.stack([(rng.random(n) - 0.5) * 0.01, (rng.random(n) - 0.5) * 0.01, np.zeros(n)], 1).astype(np.float32)
    nrm = np.full(n, oracle.sppm_oct(np.array([0, 0, 1], np.float32)), np.uint32)
    power = np.ones((n, 3), np.float32)
    q = np.zeros((1, 3), np.float32)
    qn = np.array([[0, 0, 1]], np.float32)
    qa = np.full((1, 3), np.float32(math.pi), np.float32)
    full = None
    vals, walked = [], []
    for t in range(300):
        flags = (rng.integers(0, 32, n) << 16).astype(np.uint32)
        oracle.sppm_build(pos, power, nrm, flags, np.float32(0.02))
        if full is None:
            full = oracle.sppm_gather(q, qn, qa, np.zeros(1, np.uint32), np.float32(0.006), 10, 0, 1)[0][0, 0]
        o, v, c = oracle.sppm_gather(q, qn, qa, np.zeros(1, np.uint32), np.float32(0.006), 10, 64, 100 + t)
        vals.append(o[0, 0])
        walked.append(int(v[0]))
    vals = np.array(vals)
    se = vals.std(ddof=1) / math.sqrt(len(vals))
    assert se > 0 and abs(vals.mean() - full) < 3 * se
    assert max(walked) < 8 * 64 and max(walked) < 2000
    o, v, c = oracle.sppm_gather(q, qn, qa, np.zeros(1, np.uint32), np.float32(0.006), 10, 1, 9)
    assert c[0] == 1 and v[0] == 8                         # the hard cap stops a gather and says so


# ---- haze (core/test/haze.test.mjs:43-128) ----
def test_haze_span_matches_stepping():
    s = scenes.Scene([scenes.prim(scenes.ST_PRIM_PLANE)], [scenes.air(), scenes.diffuse((1, 1, 1))],
                     haze={"centre": (0.3, -0.2, 1.0), "half": (1.0, 2.0, 0.5), "sigma_t": 0.5})
    rng = np.random.default_rng(4)
    for _ in range(200):
        A = rng.uniform(-3, 3, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        L = 8.0
        t0, t1 = oracle.haze_span(s, A, d, L, 100.0)
        ts = np.linspace(0, L, 80001)
        p = A[None, :] + ts[:, None] * d[None, :] - np.array([0.3, -0.2, 1.0])
        inside = (np.abs(p) <= np.array([1.0, 2.0, 0.5])).all(1)
        if not inside.any():
            assert not (t1 > t0 + 1e-3)
        else:
            assert abs(t0 - ts[inside][0]) < 2e-4 and abs(t1 - ts[inside][-1]) < 2e-4


@pytest.mark.parametrize("g", [0.0, 0.3, -0.6, 0.9])
def test_hg_lobe(g):
    c = np.linspace(-1, 1, 200001)
    p = np.array([oracle.hg_eval(float(x), g) for x in c[::50]])
    integral = 2 * math.pi * np.trapezoid(p, c[::50])
    assert integral == pytest.approx(1.0, rel=2e-3 if abs(g) < 0.8 else 2e-2)
    d = np.array([0.0, 0.6, 0.8])
    w = oracle.hg_sample(g, d, 11, 40000)
    assert np.allclose(np.linalg.norm(w, axis=1), 1, atol=1e-9)
    assert (w @ d).mean() == pytest.approx(g, abs=0.012)


# ---- the dielectric Fresnel term (materials_pbr.js) ----
def test_fresnel_dielectric():
    assert oracle.fresnel_dielectric(1.0, 1.5) == pytest.approx(0.04, abs=1e-12)
    assert oracle.fresnel_dielectric(1e-9, 1.5) == pytest.approx(1.0, abs=1e-6)
    # eta = n_incident / n_transmitted: from inside glass past the critical angle, total internal reflection
    assert oracle.fresnel_dielectric(0.5, 1.5) == 1.0
    assert 0 < oracle.fresnel_dielectric(0.5, 1 / 1.5) < 1
    assert oracle.fresnel_dielectric(1.0, 1 / 1.5) == pytest.approx(0.04, abs=1e-12)


# ---- the far field (optics/test/farfield.test.mjs) ----
def test_far_geometry_tiles_the_sphere():
    for nC, nG in ((360, 181), (90, 46), (4, 3)):
        om = oracle.far_geometry(nC, nG)
        assert om.sum() * nC == pytest.approx(4 * math.pi, rel=1e-12)


def test_lambertian_intensity():
    nC, nG, flux = 360, 181, 1000.0
    dG = math.radians(180.0 / (nG - 1))
    F = np.zeros((nG, nC))
    for j in range(nG):
        lo, hi = max(0.0, (j - 0.5) * dG), min(math.pi / 2, (j + 0.5) * dG)
        if hi > lo:
            F[j, :] = flux * (math.sin(hi) ** 2 - math.sin(lo) ** 2) / nC
    assert F.sum() == pytest.approx(flux, rel=1e-12)
    I = oracle.far_intensity(F, nC, nG)
    assert I[0, 0] == pytest.approx(flux / math.pi, rel=1e-4)                  # I(0) = flux / pi
    assert I[60, 7] == pytest.approx(flux / math.pi * math.cos(math.radians(60)), rel=1e-3)


def test_far_bins():
    ax, c0 = (0, 0, 1), (1, 0, 0)
    assert oracle.far_bin((0, 0, 1), ax, c0, 360, 181) == 0
    assert oracle.far_bin((0, 0, -1), ax, c0, 360, 181) // 360 == 180
    assert oracle.far_bin((1, 0, 0), ax, c0, 360, 181) == 90 * 360
    assert oracle.far_bin((0, 1, 0), ax, c0, 360, 181) == 90 * 360 + 90
    assert oracle.far_bin((0, -1, 0), ax, c0, 360, 181) == 90 * 360 + 270


# ---- dispersion (core/test/spectral.test.mjs:138-151, lightspectra.js's table) ----
def test_cauchy_index():
    LD, LF, LC = 587.56, 486.13, 656.27
    assert oracle.cauchy_n(1.5168, 64.17, LD) == pytest.approx(1.5168, abs=1e-15)
    assert (1.75 - 1) / (oracle.cauchy_n(1.75, 28, LF) - oracle.cauchy_n(1.75, 28, LC)) == pytest.approx(28, abs=1e-9)
    assert oracle.cauchy_n(1.5168, 64.17, LF) == pytest.approx(1.52238, abs=1e-4)          # Schott N-BK7
    assert oracle.cauchy_n(1.5168, 64.17, LC) == pytest.approx(1.51432, abs=1e-4)
    ns = [oracle.cauchy_n(1.6, 40, l) for l in (400, 450, 500, 600, 700, 780)]
    assert all(b < a for a, b in zip(ns, ns[1:]))                                      # blue bends more
    assert all(oracle.cauchy_n(1.5, 0, l) == 1.5 for l in (380, 587.56, 780))            # Abbe 0: no dispersion


def test_lambda_code():
    for l in (380, 412.345, 550, 699.999, 780):
        assert abs(oracle.lambda_of(oracle.lambda_code(l)) - l) <= 400 / 32766 / 2 + 1e-9
    assert oracle.lambda_of(0) == 0
    assert oracle.lambda_code(380) == 1 and oracle.lambda_code(780) == 32767
    assert oracle.lambda_code(200) == 1 and oracle.lambda_code(900) == 32767


def test_camera_wavelength_table():
    cdf, col = oracle.spec_table()
    q = np.diff(np.concatenate([[0.0], cdf.astype(np.float64)]))
    assert np.all(q >= 0) and cdf[-1] == 1.0
    assert np.allclose((q[:, None] * col).sum(0), 1.0, atol=1e-5)       # each channel's mean weight is 1
    assert col.max() <= 3.0 + 1e-6 and col.min() >= 0
    # a draw lands in its cell, uniform inside it, its colour the cell's
    for u in (0.0, 0.1, 0.5, 0.9, 0.999999):
        lam, w = oracle.spec_draw(u)
        i = int(np.searchsorted(cdf, u, side="right"))
        assert 380 + i <= lam <= 381 + i
        assert np.allclose(w, col[i])
    # blue early, red late
    assert oracle.spec_draw(0.05)[1][2] > oracle.spec_draw(0.05)[1][0]
    assert oracle.spec_draw(0.95)[1][0] > oracle.spec_draw(0.95)[1][2]


def test_dispersive_furnace_on_the_oracle():
    s = scenes.dispersive_furnace(width=24, height=24)
    a = oracle.render(s, 8)
    L = a.luma()
    assert abs(L.mean() / 1000.0 - 1) < 0.02
