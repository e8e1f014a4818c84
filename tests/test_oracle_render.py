"""The oracle's render against closed forms, on the CPU (the reference's own on-GPU answers, lib/pathtracer/tests.js:
the photometry floor and the haze furnace, restated here for the CPU restatement the GPU path is held to).

A Lambertian floor of albedo a under a uniform sky L reads a L wherever it is seen (every path that leaves it sees the
sky); an albedo-1 haze box in a uniform sky reads L everywhere (what it scatters out of a ray it scatters back in).
The microfacet albedo tables and the scene distance function are checked for their defining properties.
"""
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes


def test_floor_closed_form():
    s = scenes.floor_furnace(width=64, height=64, maxbounce=4)
    a = oracle.render(s, 2)
    L = a.luma()
    # the rows that meet the floor steeply read 800 in every sample; nearer the horizon a bounce so shallow that its
    # march steps run out (maxiter) ends dark, as the reference's does
    floor = L[:20]
    assert abs(floor.mean() / 800.0 - 1) < 1e-3, floor.mean()
    assert np.mean(np.abs(floor - 800.0) < 0.08) > 0.99
    assert np.allclose(L[-3:], 1000.0, rtol=1e-6)


def test_haze_furnace_closed_form():
    s = scenes.haze_furnace(width=24, height=24, sigma_t=0.5, g=0.3)
    a = oracle.render(s, 4)
    assert abs(a.luma().mean() - 1000.0) < 1000.0 * 2e-3


def test_counts_and_moments():
    s = scenes.floor_furnace(width=16, height=16, maxbounce=4)
    a = oracle.render(s, 3)
    assert np.all(a.count == 3)
    assert np.allclose(a.S, 1.0 / 3.0)
    a = oracle.render(s, 1, accum=a)
    assert np.all(a.count == 4) and a.next_sample == 4


def test_microfacet_tables():
    ec, ecavg, e1 = oracle.mf_tables()
    assert np.all(ec >= 0) and np.all(ec <= 1.0 + 1e-5)
    assert np.all(e1 >= 0) and np.all(e1 <= 1.0 + 1e-5)
    e1 = e1.reshape(32, 32)                 # rows: roughness, smoothest first
    assert np.all(e1[0] > 0.99)             # the smoothest lobe reflects next to everything in one bounce
    assert np.all(np.diff(e1[:, -1]) <= 1e-3) and e1[-1, -1] < 0.5     # rougher loses more to multiple scattering
    ec64, ecavg64, e164 = oracle.mf_tables(fp64=True)
    assert np.abs(e164 - e1.reshape(-1)).max() < 2e-3 and np.abs(ec64 - ec).max() < 2e-3


def test_scene_distance_is_a_distance():
    s = scenes.sdf_room(width=32, height=18, n_prims=24)
    rng = np.random.default_rng(0)
    p = rng.uniform([-3, -2, 0], [3, 2, 3], (2000, 3)).astype(np.float32)
    d, m, _ = oracle.scene_sdf(s, p)
    # 1-Lipschitz (up to the smooth unions' slack): no two points' distances differ by more than their separation
    q = p + rng.normal(scale=0.05, size=p.shape).astype(np.float32)
    dq, _, _ = oracle.scene_sdf(s, q)
    sep = np.linalg.norm(p - q, axis=1)
    assert np.all(np.abs(d - dq) <= sep * 1.05 + 1e-5)
    assert np.any(d < 0) and np.any(d > 0)


def test_photon_map_pane_closed_form():
    """The oracle's photon map (per sample: sun photons, stores past glass, the grid, the camera's gather) against the
    pane's closed form T(view) rho / pi E_sun sin(elevation) T(sun)."""
    import math
    s = scenes.sppm_pane(width=32, height=32, photons=400_000, r1=0.03)
    a = oracle.render(s, 4)
    Fv = oracle.fresnel_dielectric(1.0, 1 / 1.5)
    Fs = oracle.fresnel_dielectric(math.cos(math.radians(30)), 1 / 1.5)
    cf = (1 - Fv) / (1 + Fv) * 0.7 / math.pi * 1e5 * math.sin(math.radians(60)) * (1 - Fs) / (1 + Fs)
    assert abs(a.luma().mean() / cf - 1) < 0.03
    # the stored photons' power over a patch of the floor is the slab's transmitted irradiance
    n, pw = oracle.sppm_photons(s, 0, lo=(-0.3, -0.3, -0.01), hi=(0.3, 0.3, 0.01))
    E = (pw @ np.array([0.2126, 0.7152, 0.0722])) / 0.36
    assert abs(E / (1e5 * math.sin(math.radians(60)) * (1 - Fs) / (1 + Fs)) - 1) < 0.01


def test_light_tracing_pane_closed_form():
    """The oracle's light tracing (materials_pbr.js ltConnect: the sun's photons past the pane connected to the camera
    where they land on the floor, shadow-tested, splatted, added to the pixel as they are) against the floor seen
    directly under the pane: rho / pi E_sun sin(elevation) (1 - F)^2; the connections reach every floor pixel."""
    s = scenes.lt_pane(width=48, height=36, photons=300_000)
    a = oracle.render(s, 8)
    m = np.array(scenes.floor_mask(s))
    cf = scenes.lt_pane_closed_form(s, oracle.fresnel_dielectric)
    assert m.sum() > 300
    assert abs(a.luma()[m].mean() / cf - 1) < 0.01, (a.luma()[m].mean(), cf)
    counts = oracle.last_lt_counts(48, 36)
    assert np.all(counts[m] > 0)
    # off: the floor under the glass is dark (the class is light tracing's; the sun's disc through the pane is rare)
    s.params.lt = 0
    b = oracle.render(s, 2)
    assert b.luma()[m].mean() < 0.05 * cf


def test_light_tracing_emitter_photons_closed_form():
    """The oracle's emitter photons (wavefront.js:552-588 probes; THE PROBE: a random line through a listed box's
    sphere followed back to the first emissive surface seen from outside, the photon's flux the emission over the
    probes and the line density there) connected to the camera: a lamp's light on a floor through a pane, which the
    camera's paths leave to them once the lamp is listed (from the third sample on: the first two are taken out)."""
    s = scenes.lt_lamp(width=48, height=36, photons=100_000)
    cf = scenes.lt_lamp_closed_form(s, oracle.fresnel_dielectric)
    m = cf > 0.5 * np.median(cf[cf > 0])
    L2 = oracle.render(s, 2).luma()
    L = oracle.render(s, 128).luma()
    X = (128 * L - 2 * L2) / 126
    assert m.sum() > 300
    # (the camera's paths keep the lamp's points no listed sphere covers: their rare hits converge slowly)
    assert abs(X[m].mean() / cf[m].mean() - 1) < 0.025, X[m].mean() / cf[m].mean()
    assert oracle.last_lt_counts(48, 36)[m].min() > 0


def inner_pixels(hit):
    inner = hit.copy()
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            inner &= np.roll(np.roll(hit, dy, 0), dx, 1)
    return inner


def test_light_tracing_in_the_haze_closed_form():
    """The oracle's photons scattered in a haze box (haze.js ltConnectMedium: the phase function, dist / z^3, the haze
    on the connection) against the sun's single scattering through a pane, by quadrature along each pixel's ray."""
    s = scenes.lt_haze(width=48, height=36)
    cf = scenes.lt_haze_single_scatter(s, oracle.fresnel_dielectric)
    a = oracle.render(s, 32)
    m = inner_pixels(cf > 0)
    assert m.sum() > 300
    assert abs(a.luma()[m].sum() / cf[m].sum() - 1) < 0.015, a.luma()[m].sum() / cf[m].sum()


def test_lamp_floor_closed_form():
    """The oracle's emitter discovery, list and light sample (materials_pbr.js:887-960, wavefront.js:715-815): the
    floor under a sphere lamp in the dark reads albedo Le a^2 h / D^3, and the list is the lamp's voxels."""
    s = scenes.lamp_floor(width=48, height=32)
    ref = oracle.render(s, 256)
    L = ref.luma()
    W, H = s.params.width, s.params.height
    v = s.view
    fwd, right, up, eye = [np.array(list(x), np.float64) for x in (v.fwd, v.right, v.up, v.cam_pos)]
    X, Y = np.meshgrid((np.arange(W) + 0.5) / W * 2 - 1, (np.arange(H) + 0.5) / H * 2 - 1)
    d = -fwd + right * (X[..., None] * v.fx) + up * (Y[..., None] * v.fy)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    t = -eye[2] / d[..., 2]
    pts = eye + d * t[..., None]
    oc = eye - np.array([0.0, 0.0, 1.0])
    b = np.sum(d * oc, -1)
    ok = (t > 0) & ((b * b - (oc @ oc - 0.15 ** 2)) <= 0) & (np.linalg.norm(pts[..., :2], axis=-1) < 8.0)
    cf = scenes.lamp_floor_closed_form(s, pts)
    assert abs(L[ok].sum() / cf[ok].sum() - 1) < 0.02, L[ok].sum() / cf[ok].sum()
    assert abs(np.median(L[ok] / cf[ok]) - 1) < 0.02


def spot_floor_points(s):
    """The floor point under each pixel centre of the spot-floor's orthographic camera, and each point's angle (deg)
    off the beam's axis, seen from the centre of the lamp's lower face."""
    W, H = s.params.width, s.params.height
    X, Y = np.meshgrid((np.arange(W) + 0.5) / W * 2 - 1, (np.arange(H) + 0.5) / H * 2 - 1)
    pts = np.stack([X, Y, np.zeros_like(X)], -1)
    axis = np.array([1.0, 0.0, -1.0]) / math.sqrt(2.0)
    face = np.array([-1.0, 0.0, 1.0]) + axis * 0.0005
    d = pts - face
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    return pts, np.degrees(np.arccos(np.clip(d @ axis, -1, 1)))


def test_spot_floor_flux():
    """A 10-degree spot of 1000 lm (a beam emitter: a thin lamp whose face emits only within 10 degrees of its normal)
    on a Lambertian floor: pi / albedo times the floor's luminance summed over its area is the lamp's flux, and the
    floor is dark outside the cone."""
    s = scenes.spot_floor(width=64, height=64)
    ref = oracle.render(s, 256)
    L = ref.luma()
    flux = L.sum() * s.info["pixel_area"] * math.pi / s.info["albedo"]
    assert abs(flux / s.info["flux"] - 1) < 0.04, flux
    # the 20 cm lamp blurs the cone's edge by about 7 degrees either way; past that only the rims of the lamp's faces,
    # where the distance field's normal turns from one face to the next, send a little light
    _, ang = spot_floor_points(s)
    out = ang > 18.0
    assert np.mean(L[out] == 0.0) > 0.99 and L[out].sum() < 0.005 * L.sum()
    assert np.all(L[ang < 3.0] > 0.0)


@pytest.mark.parametrize("side", [0.2, 0.05])
def test_spot_face_flux(side):
    """The spot as a light's face (builder/lights.js: one-sided, 1000 lm through its beam by fluxFactor; light sampling
    aims at a point of it, scene_api.js lightFaceDensity): pi / albedo times the floor's luminance summed over its area
    is the flux, and nothing lands past the cone's blurred edge."""
    s = scenes.spot_floor(width=64, height=64, side=side, light="face")
    ref = oracle.render(s, 64)
    L = ref.luma()
    k = s.info["pixel_area"] * math.pi / s.info["albedo"]
    flux, err = L.sum() * k, math.sqrt(np.sum(ref.V / 64)) * k
    assert abs(flux - 1000.0) < max(5 * err, 10.0), (flux, err)
    _, ang = spot_floor_points(s)
    assert np.all(L[ang > 18.0] == 0.0)


def test_face_light_sample_is_unbiased():
    """A BSDF's hits of a face weighed against the face's light sample (codegen.js:826-834) and the light sample
    itself: the floor lit through both agrees with the floor lit by the BSDF's hits alone (light sampling off)."""
    s = scenes.spot_floor(width=32, height=32, side=0.4, light="face")
    s.params.maxbounce = 2
    on = oracle.render(s, 256)
    s.params.nee = 0
    off = oracle.render(s, 2048)
    k = s.info["pixel_area"] * math.pi / s.info["albedo"]
    f_on, f_off = on.luma().sum() * k, off.luma().sum() * k
    e_on, e_off = math.sqrt(np.sum(on.V / 256)) * k, math.sqrt(np.sum(off.V / 2048)) * k
    assert abs(f_on - f_off) < 5 * math.hypot(e_on, e_off), (f_on, e_on, f_off, e_off)
    assert abs(f_on - 1000.0) < 5 * e_on + 10.0


@pytest.mark.parametrize("kind", ["opal", "hazy", "rough", "frosted"])
def test_translucent_furnace(kind):
    """The side beyond (materials_pbr.js THE SIDE BEYOND): a translucent, hazy, rough or frosted sphere in the white
    furnace. The light sample through its faces from inside and the BSDF's draw below them are one estimator: with and
    without light sampling the sphere reads the same; where the model keeps energy (a diffused or smooth transmission)
    it reads the furnace, and rough glass loses only what single-scattering GGX loses."""
    out = []
    for nee in (1, 0):
        s = scenes.translucent_furnace(kind, width=24, height=24)
        s.params.nee = nee
        r = oracle.render(s, 128)
        c = r.luma()[8:16, 8:16]
        out.append((c.mean(), math.sqrt(np.nansum(r.se()[8:16, 8:16] ** 2)) / c.size))
    (m1, e1), (m0, e0) = out
    assert abs(m1 - m0) < 5 * math.hypot(e1, e0) + 1.0, out
    if kind != "rough":
        assert abs(m0 / 1000.0 - 1) < 0.01 + 5 * e0 / 1000.0, out
    else:
        assert 0.8 < m0 / 1000.0 < 0.95, out


def test_anisotropic_gloss_light_sampling_is_unbiased():
    """Anisotropic lobes (microfacet.js mfAnisoAlpha): the light sample's MIS weights and the BSDF's draw agree on the
    stretched lobes' density -- the same picture with light sampling on and off -- and the stretch changes it."""
    out = []
    for nee, n in ((1, 128), (0, 512)):
        s = scenes.aniso_spheres(0.8, width=32, height=24)
        s.params.nee = nee
        r = oracle.render(s, n)
        out.append((r.luma().mean(), math.sqrt(np.nansum(r.se() ** 2)) / r.luma().size))
    (m1, e1), (m0, e0) = out
    assert abs(m1 - m0) < 5 * math.hypot(e1, e0) + 1e-3 * m0, out
    iso = oracle.render(scenes.aniso_spheres(0.0, width=32, height=24), 128).luma()
    an = oracle.render(scenes.aniso_spheres(0.8, width=32, height=24), 128).luma()
    assert np.abs(an - iso).max() > 0.05 * iso.max()


def test_absorption_inside_closed_form():
    """Beer-Lambert inside a material (absorbAlong): every ray through the 1 m cube reads the sky times base^(1 / d)."""
    s = scenes.absorbing_box()
    r = oracle.render(s, 4)
    # the march stops within its tolerance (1e-5 m) of each face
    assert np.allclose(r.rgb.reshape(-1, 3), s.info["expected"], rtol=5e-5)


def clusters_scene(width=48, height=32):
    """Four separate smooth-unioned pairs over a floor: groups whose boxes the reference's root cull skips wherever a
    point is farther from them than ten surface tolerances."""
    from shadytracer_gb300.scenes import Scene, prim, air, diffuse, plastic, look_at, default_params
    from shadytracer_gb300.st_types import ST_PRIM_PLANE, ST_PRIM_SPHERE, ST_PRIM_BOX, ST_OP_SMOOTH
    mats = [air(), diffuse((0.7, 0.7, 0.7)), plastic((0.8, 0.3, 0.2), 0.3)]
    prims = [prim(ST_PRIM_PLANE, material=1)]
    for i, (x, y) in enumerate([(-1.5, -1.5), (1.5, -1.5), (-1.5, 1.5), (1.5, 1.5)]):
        prims.append(prim(ST_PRIM_SPHERE, pos=(x, y, 0.4), params=(0.35,), material=2))
        prims.append(prim(ST_PRIM_BOX, pos=(x + 0.3, y, 0.3), params=(0.25, 0.25, 0.3), material=2, op=ST_OP_SMOOTH,
                          k=0.08))
    s = Scene(prims, mats, env_radius=30.0, name="clusters")
    s.params = default_params(width=width, height=height, maxbounce=4, sun_elevation=40.0, sun_azimuth=30.0,
                              sun_illuminance=100000.0, sky_luminance=3000.0, ground_luminance=500.0, eps=1e-4, seed=3)
    s.view = look_at((-4.0, -5.0, 3.0), (0.0, 0.0, 0.3), 50.0, width / height)
    s.info = {"spp": 4}
    return s


@pytest.mark.parametrize("make", [clusters_scene, lambda: scenes.sdf_room(width=48, height=27)])
def test_the_references_root_cull_keeps_the_picture(make):
    """The oracle's timing mode with the reference's bounding-box culling at the root (builder/codegen.js:2141-2193,
    scene_api.js cullDist): a culled group's box distance stands in for it, so the march takes different steps
    but meets the same surfaces -- the picture within the error bars of the unculled one, most pixels equal."""
    s = make()
    a = oracle.render(s, 4)
    b = oracle.render(make(), 4, cull=True)
    La, Lb = a.luma(), b.luma()
    sd = np.hypot(np.nan_to_num(a.se()), np.nan_to_num(b.se()))
    ok = sd > 0
    assert np.mean(np.abs((La - Lb)[ok]) <= 4 * sd[ok] + 1e-3 * np.maximum(La[ok], 1.0)) > 0.98
    assert np.mean(np.abs(La - Lb) <= 1e-3 * np.maximum(La, 1.0)) > 0.5
