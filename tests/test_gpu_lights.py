"""The lights' faces on the GPU (csrc/st_light.cuh; st_render.cu's light sample at a surface and in the air, a face's
hit and its MIS weight; the occlusion pass's arrival at a face; st_capi.cu's table and the sheets that draw the faces),
through the C ABI: the spot's flux against its closed form, GPU against the oracle (oracle/st_oracle_light.h) on the
spot over a floor and on the haze-box beam, the light sample against the BSDF's hits alone, and the table's checks.
"""
import ctypes as C
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


def spot_angles(s):
    W, H = s.params.width, s.params.height
    X, Y = np.meshgrid((np.arange(W) + 0.5) / W * 2 - 1, (np.arange(H) + 0.5) / H * 2 - 1)
    pts = np.stack([X, Y, np.zeros_like(X)], -1)
    axis = np.array([1.0, 0.0, -1.0]) / np.sqrt(2.0)
    d = pts - np.array([-1.0, 0.0, 1.0])
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    return np.degrees(np.arccos(np.clip(d @ axis, -1, 1)))


@pytest.mark.parametrize("side", [0.2, 0.05])
def test_spot_face_flux(side):
    """A 10-degree spot of 1000 lm as a light's face over a Lambertian floor: pi / albedo times the floor's luminance
    summed over its area is the flux, to 1 %, and the floor past the cone's blurred edge is dark."""
    s = scenes.spot_floor(width=128, height=128, side=side, light="face")
    L, se, ctr = render(s, 256)
    k = s.info["pixel_area"] * math.pi / s.info["albedo"]
    flux, err = L.sum() * k, math.sqrt(np.sum(se ** 2)) * k
    assert abs(flux - 1000.0) < max(5 * err, 10.0), (flux, err)
    assert np.all(L[spot_angles(s) > 18.0] == 0.0)
    assert ctr["nonfinite"] == 0


def z_parity(L, se, ref):
    sd = np.hypot(se, se_of(ref.V, ref.S))
    ok = sd > 0
    z = (L - ref.luma())[ok] / sd[ok]
    zm = (L - ref.luma())[ok].mean() / (np.sqrt(np.sum(sd[ok] ** 2)) / ok.sum())
    return ok, np.mean(np.abs(z) < 4), zm


def test_spot_face_matches_the_oracle():
    s = scenes.spot_floor(width=48, height=48, side=0.2, light="face")
    L, se, _ = render(s, 128)
    ref = oracle.render(s, 128)
    ok, frac, zm = z_parity(L, se, ref)
    assert frac > 0.98 and abs(zm) < 5, (frac, zm)
    assert np.all(L[~ok] == 0.0) and np.all(ref.luma()[~ok] == 0.0)


def test_haze_beam_matches_the_oracle():
    """The haze-box beam, small: a 5 cm spot below an albedo-1 haze box lights it; what the air scatters toward the
    camera (the faces' light sample from every medium vertex, the phase function's hits of the face weighed against
    it), GPU against oracle, pixel by pixel within the error bars."""
    s = scenes.haze_beam(width=48, height=27, sigma_s=0.2, g=0.7, maxbounce=8)
    L, se, ctr = render(s, 256)
    ref = oracle.render(s, 256)
    ok, frac, zm = z_parity(L, se, ref)
    assert ok.sum() > 60
    assert frac > 0.97 and abs(zm) < 5, (frac, zm)
    assert ctr["nonfinite"] == 0


def test_face_light_sample_is_unbiased():
    """With light sampling off the floor is lit only by the BSDF's hits of the face: the same flux."""
    out = {}
    for nee, n in ((1, 256), (0, 2048)):
        s = scenes.spot_floor(width=64, height=64, side=0.4, light="face")
        s.params.nee = nee
        L, se, _ = render(s, n)
        k = s.info["pixel_area"] * math.pi / s.info["albedo"]
        out[nee] = (L.sum() * k, math.sqrt(np.sum(se ** 2)) * k)
    (f1, e1), (f0, e0) = out[1], out[0]
    assert abs(f1 - f0) < 5 * math.hypot(e1, e0), out
    assert e0 * math.sqrt(2048 / 256) > 3 * e1, out  # the light sample's gain at equal samples


def test_face_table_is_checked():
    from shadytracer_gb300.renderer import create_path_tracer
    from shadytracer_gb300._lib import StError
    s = scenes.spot_floor(width=16, height=16, light="face")
    s.lights[0].material = 0                      # the air draws nothing
    with pytest.raises(StError):
        create_path_tracer(s, device=0)
    s = scenes.spot_floor(width=16, height=16, light="face")
    s.lights[0].half_w = 0.0
    with pytest.raises(StError):
        create_path_tracer(s, device=0)
