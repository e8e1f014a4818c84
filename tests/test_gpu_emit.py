"""Emissive surfaces on the GPU (csrc/st_emit.cu, st_emit.cuh; st_render.cu's light sample and emitter hits; the
occlusion pass's hand-off), through the C ABI: the lamp over a floor against its closed form and against the oracle
(oracle/st_oracle.cpp's restatement of discovery, the list and the emitter light sample), the list the discovery
builds, and the light sample's gain over finding the lamp by the BSDF alone.
"""
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


def floor_pixels(s):
    return scenes.lamp_floor_pixels(s)


def render(s, n):
    from shadytracer_gb300.renderer import create_path_tracer
    with create_path_tracer(s, device=0) as r:
        r.step(n)
        rgb, V, S, cnt = r.read_accum()
        lst = r.emit_list()
    return rgb @ LUMA, se_of(V, S), lst


def test_lamp_floor_closed_form():
    """The floor under a sphere lamp in the dark reads albedo Le a^2 h / D^3 (the sphere as a point source), with the
    lamp found by the camera paths and light sampling aimed at it from the third sample on."""
    s = scenes.lamp_floor(width=96, height=64)
    L, se, lst = render(s, 512)
    cf, ok = floor_pixels(s)
    r = L[ok] / cf[ok]
    assert abs(np.median(r) - 1) < 0.01 and abs(L[ok].sum() / cf[ok].sum() - 1) < 0.01, (np.median(r), L[ok].sum() / cf[ok].sum())
    # the pixels' footprints average L over about 4 cm of floor: second order, well under the error bars' share
    z = (L - cf)[ok] / np.maximum(se[ok], 1e-3 * cf[ok])
    assert np.mean(np.abs(z) < 4) > 0.97, np.mean(np.abs(z) < 4)
    # the list: the lamp sits on a corner of four voxels (the grid's 1.875 m cells meet at x = y = 0), so four boxes,
    # each the bounding sphere of its quarter of the lamp, a quarter of the probability each
    assert len(lst) == 4
    assert np.all(np.linalg.norm(lst[:, :3] - np.array([0.0, 0.0, 1.0]), axis=1) < 0.1)
    assert np.all((lst[:, 3] > 0.07) & (lst[:, 3] < 0.15))
    assert np.allclose(lst[:, 4], 0.25, atol=0.01) and abs(lst[-1, 5] - 1) < 1e-6


def test_lamp_floor_matches_the_oracle():
    s = scenes.lamp_floor(width=48, height=32)
    s.params.samples_per_wave = 1                # a list built between every two samples, as the oracle's
    L, se, _ = render(s, 64)
    ref = oracle.render(s, 64)
    Lr = ref.luma()
    ser = se_of(ref.V, ref.S)
    sd = np.hypot(se, ser)
    ok = sd > 0
    z = (L - Lr)[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.98, np.mean(np.abs(z) < 4)
    zm = (L - Lr)[ok].mean() / (np.sqrt(np.sum(sd[ok] ** 2)) / ok.sum())
    assert abs(zm) < 5, zm


def test_light_sampling_the_lamp_is_unbiased_and_pays():
    """With the emitter light sample off, the floor is lit only by the BSDF's hits of the lamp: the same mean, a far
    larger error against the closed form."""
    out = {}
    for off in (0, 1):
        s = scenes.lamp_floor(width=96, height=64)
        s.params.emit_off = off
        L, se, _ = render(s, 256)
        cf, ok = floor_pixels(s)
        out[off] = (L[ok].mean(), np.sqrt(np.sum(se[ok] ** 2)) / ok.sum(),
                    float(np.sqrt(np.mean((L[ok] - cf[ok]) ** 2)) / cf[ok].mean()))
    (m0, s0, e0), (m1, s1, e1) = out[0], out[1]
    assert abs(m0 - m1) < 5 * np.hypot(s0, s1) + 0.01 * m0, out
    assert e1 > 4 * e0, out                       # relative RMSE: the BSDF alone over with the light sample


def test_lamp_in_haze_matches_the_oracle():
    """The lamp in a haze box: the air's light sample aims at the list too (haze.js:324-370); GPU and oracle agree
    pixel by pixel within the error bars, and the light sample is unbiased against the phase function's hits alone."""
    s = scenes.lamp_floor(width=48, height=32, haze_sigma_t=0.5, haze_g=0.5, maxbounce=6)
    s.params.samples_per_wave = 1
    L, se, _ = render(s, 64)
    ref = oracle.render(s, 64)
    sd = np.hypot(se, se_of(ref.V, ref.S))
    ok = sd > 0
    z = (L - ref.luma())[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.98, np.mean(np.abs(z) < 4)
    s.params.emit_off = 1
    L1, se1, _ = render(s, 256)
    s.params.emit_off = 0
    L0, se0, _ = render(s, 256)
    m0, m1 = L0.mean(), L1.mean()
    e0, e1 = np.sqrt(np.sum(se0 ** 2)) / se0.size, np.sqrt(np.sum(se1 ** 2)) / se1.size
    assert abs(m0 - m1) < 5 * np.hypot(e0, e1) + 0.01 * m0, (m0, m1, e0, e1)


def spot_angles(s):
    """Each pixel's floor point's angle (deg) off the spot's axis, from the centre of the lamp's lower face."""
    W, H = s.params.width, s.params.height
    X, Y = np.meshgrid((np.arange(W) + 0.5) / W * 2 - 1, (np.arange(H) + 0.5) / H * 2 - 1)
    pts = np.stack([X, Y, np.zeros_like(X)], -1)
    axis = np.array([1.0, 0.0, -1.0]) / np.sqrt(2.0)
    d = pts - (np.array([-1.0, 0.0, 1.0]) + axis * 0.0005)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    return np.degrees(np.arccos(np.clip(d @ axis, -1, 1)))


def test_spot_floor_flux():
    """A 10-degree spot of 1000 lm (a beam emitter: its faces emit only within 10 degrees of their normals) on a
    Lambertian floor: pi / albedo times the floor's luminance summed over its area is the lamp's flux, to 1 %, and the
    floor is dark outside the cone, at the BSDF's hits of the lamp and at the light sample's alike."""
    s = scenes.spot_floor(width=128, height=128)
    L, se, lst = render(s, 512)
    k = s.info["pixel_area"] * np.pi / s.info["albedo"]
    flux, err = L.sum() * k, np.sqrt(np.sum(se ** 2)) * k
    assert abs(flux - s.info["flux"]) < max(5 * err, 0.01 * s.info["flux"]), (flux, err)
    ang = spot_angles(s)
    out = ang > 18.0
    assert np.mean(L[out] == 0.0) > 0.99 and L[out].sum() < 0.005 * L.sum()
    assert np.all(L[ang < 3.0] > 0.0)
    assert len(lst) >= 1


def test_spot_floor_matches_the_oracle():
    s = scenes.spot_floor(width=48, height=48)
    s.params.samples_per_wave = 1
    L, se, _ = render(s, 128)
    ref = oracle.render(s, 128)
    sd = np.hypot(se, se_of(ref.V, ref.S))
    ok = sd > 0
    z = (L - ref.luma())[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.98, np.mean(np.abs(z) < 4)
    zm = (L - ref.luma())[ok].mean() / (np.sqrt(np.sum(sd[ok] ** 2)) / ok.sum())
    assert abs(zm) < 5, zm
    assert np.all(L[~ok] == 0.0) and np.all(ref.luma()[~ok] == 0.0)

