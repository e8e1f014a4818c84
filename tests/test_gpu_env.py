"""The environment image and its map on the GPU (st_device.cuh env_image, env_map_sample / env_map_pdf and the three-way
environment draw; st_render.cu k_env_bake; st_capi.cu st_set_env_image), through the C ABI: the image as the camera sees
it against a numpy restatement of envimage.js envImageAt, a floor under a panorama against its closed form, the map's
light samples unbiased against the cosine lobe alone and far less noisy, and GPU against the oracle, on a surface and
in the haze.
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


def render(s, n, img, lum=179.0, turn=0.0):
    from shadytracer_gb300.renderer import create_path_tracer
    with create_path_tracer(s, device=0) as r:
        r.set_env_image(img, lum, turn)
        r.step(n)
        rgb, V, S, cnt = r.read_accum()
        ctr = r.counters()
    return rgb @ LUMA, se_of(V, S), ctr


def test_camera_sees_the_image():
    """A pinhole of a 0.2-degree field looking out in several directions at nothing: each picture is the image
    there, turned as asked (a smooth panorama, periodic across the seam, so the field's width does not matter)."""
    hh, ww = 64, 128
    col = np.arange(ww)[None, :, None] / ww
    row = np.arange(hh)[:, None, None] / hh
    img = (1.5 + np.sin(2 * np.pi * col + np.array([0.0, 2.0, 4.0])) * np.cos(np.pi * row)).astype(np.float32)
    img = np.broadcast_to(img, (hh, ww, 3)).copy()
    rng = np.random.default_rng(2)
    for k in range(6):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        s = scenes.env_floor(width=4, height=4)
        s.prim_list[0].pos[2] = -1000.0               # the floor far below, out of sight
        s.prims[0].pos[2] = -1000.0
        s.view = scenes.look_at((0.0, 0.0, 0.0), tuple(d), 0.2, 1.0, up=(0.0, 0.0, 1.0) if abs(d[2]) < 0.9 else (1.0, 0.0, 0.0))
        L, _, _ = render(s, 4, img, 179.0, 25.0)
        ref = float(scenes.env_image_lookup(img, d[None], 179.0, 25.0)[0] @ LUMA)
        assert abs(L.mean() - ref) <= 0.02 * ref + 1.0, (k, L.mean(), ref)


def test_env_floor_closed_form():
    img = scenes.env_patch_image()
    cf = 0.8 / math.pi * scenes.env_level_illuminance(img)
    s = scenes.env_floor(width=64, height=64)
    L, se, ctr = render(s, 256, img)
    err = math.sqrt(np.sum(se ** 2)) / L.size
    assert abs(L.mean() - cf) < 5 * err + 5e-4 * cf, (L.mean(), cf, err)
    assert ctr["nonfinite"] == 0


def test_map_is_unbiased_and_pays():
    """With the map off the environment's light samples are the cosine lobe's alone: the same floor, far noisier
    where a small bright patch lights it."""
    img = scenes.env_patch_image(patch=20000.0, size=3)
    cf = 0.8 / math.pi * scenes.env_level_illuminance(img)
    out = {}
    for off in (0, 1):
        s = scenes.env_floor(width=64, height=64)
        s.params.env_map_off = off
        L, se, _ = render(s, 128, img)
        out[off] = (L.mean(), math.sqrt(np.sum(se ** 2)) / L.size, float(np.sqrt(np.mean((L - cf) ** 2)) / cf))
    (m0, e0, r0), (m1, e1, r1) = out[0], out[1]
    assert abs(m0 - cf) < 5 * e0 + 5e-4 * cf and abs(m1 - cf) < 5 * e1 + 5e-4 * cf, out
    assert r1 > 3 * r0, out                           # relative RMSE: the lobe alone over with the map


def z_parity(L, se, ref):
    sd = np.hypot(se, se_of(ref.V, ref.S))
    ok = sd > 0
    z = (L - ref.luma())[ok] / sd[ok]
    zm = (L - ref.luma())[ok].mean() / (np.sqrt(np.sum(sd[ok] ** 2)) / ok.sum())
    return ok, np.mean(np.abs(z) < 4), zm


@pytest.mark.parametrize("haze", [False, True])
def test_env_image_matches_the_oracle(haze):
    """The room's primitives under a panorama (and in a haze box): GPU against oracle, pixel by pixel."""
    img = scenes.env_patch_image(patch=5000.0, size=8)
    s = scenes.sdf_room(width=48, height=27, spp=16, maxbounce=4)
    if haze:
        s = scenes.Scene(s.prim_list, s.material_list, env_radius=20.0, name="room-haze",
                         haze={"centre": (0.0, 0.0, 1.5), "half": (3.0, 2.0, 1.5), "sigma_t": 0.3, "g": 0.5})
        s.params = scenes.sdf_room(width=48, height=27, spp=16, maxbounce=4).params
        s.view = scenes.sdf_room(width=48, height=27).view
    L, se, ctr = render(s, 64, img, 179.0, 40.0)
    try:
        oracle.set_env_image(img, 179.0, 40.0)
        ref = oracle.render(s, 64)
    finally:
        oracle.set_env_image(None)
    ok, frac, zm = z_parity(L, se, ref)
    assert frac > 0.98 and abs(zm) < 5, (frac, zm)
    assert ctr["nonfinite"] == 0


def test_clearing_goes_back_to_the_sky():
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.floor_furnace(width=16, height=16)
    with create_path_tracer(s, device=0) as r:
        r.set_env_image(np.zeros((8, 16, 3), np.float32))
        r.step(4)
        dark = (r.read_accum()[0] @ LUMA).mean()
        r.set_env_image(None)
        r.step(4)
        lit = (r.read_accum()[0] @ LUMA)
    assert dark == 0.0
    assert abs(lit[:4].mean() / 800.0 - 1) < 0.01


# ---- the presets (core/environment.js): the physical sun and sky, the studio ----
def render_preset(s, n):
    from shadytracer_gb300.renderer import create_path_tracer
    with create_path_tracer(s, device=0) as r:
        r.step(n)
        rgb, V, S, cnt = r.read_accum()
        ctr = r.counters()
    return rgb, V, S, ctr


@pytest.mark.parametrize("elevation, turbidity", [(45.0, 0.7), (12.0, 3.0)])
def test_sun_and_sky_floor_closed_form_and_oracle(elevation, turbidity):
    """The floor under the physical sun and sky: albedo / pi times the sun's and the sky's illuminance on it (the
    oracle's radiance integrated), and the oracle's picture pixel by pixel; the sky seen above the horizon is the
    oracle's radiance there."""
    mk = lambda w: scenes.floor_sky(width=w, height=w, env_mode=1, sun_elevation=elevation, turbidity=turbidity)
    s = mk(64)
    rgb, V, S, ctr = render_preset(s, 64)
    e_sun, e_sun_level, e_sky = scenes.sky_illuminance(lambda d: oracle.env_radiance(s, d), elevation)
    L = rgb @ LUMA
    cf = 0.8 / math.pi * (e_sun_level + e_sky)
    assert abs(L[:24].mean() / cf - 1) < 0.01, (L[:24].mean(), cf)
    assert ctr["nonfinite"] == 0
    small = mk(32)
    g = render_preset(small, 16)
    ref = oracle.render(mk(32), 16)
    Lg, Lr = g[0] @ LUMA, ref.luma()
    se = np.sqrt(se_of(g[1], g[2]) ** 2 + np.nan_to_num(ref.se()) ** 2)
    within = np.abs(Lg - Lr) <= 4 * se + 2e-3 * np.maximum(np.abs(Lr), 1.0)
    assert within.mean() > 0.98, (~within).sum()


def test_studio_floor_closed_form():
    """The studio puts exactly studio_illuminance lux on a level surface, whatever its top: the floor reads
    albedo / pi times it."""
    for top in (0.0, 1.0):
        s = scenes.floor_sky(width=48, height=48, env_mode=2, studio_illuminance=10000.0, studio_top=top)
        rgb, V, S, ctr = render_preset(s, 32)
        L = (rgb @ LUMA)[:18]
        assert abs(L.mean() / (0.8 / math.pi * 10000.0) - 1) < 0.01, (top, L.mean())
