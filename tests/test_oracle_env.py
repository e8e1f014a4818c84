"""The environment image and its map, on the CPU: the library's tabulation of the map (st_env_map_tables, host code
of csrc/st_capi.cu, callable without a GPU) against the oracle's restatement of envmap.js envSampling, the tables'
defining properties (a density that integrates to one, CDFs that end at one, a texel's weight its luminance plus a
floor), the oracle's image lookup against a numpy restatement of envimage.js envImageAt, and the oracle's floor under
an image against its closed form.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes

W, H = 512, 256


def lib_tables(lum):
    from shadytracer_gb300._lib import load
    L = load()
    lum = np.ascontiguousarray(lum, np.float32).reshape(-1)
    tex = np.zeros(lum.size * 4, np.float32)
    assert L.st_env_map_tables(lum.ctypes.data_as(C.c_void_p), tex.ctypes.data_as(C.c_void_p)) == 0
    return tex.reshape(H, W, 4)


def test_map_tables_library_equals_oracle():
    rng = np.random.default_rng(3)
    lum = rng.exponential(1.0, (H, W)).astype(np.float32)
    lum[77, 300] = 5e4
    lum[120] = 200.0
    a, b = lib_tables(lum), oracle.env_map_tables(lum)
    assert np.allclose(a, b, rtol=1e-6, atol=1e-7)


def test_map_tables_are_a_density():
    lum = np.ones((H, W), np.float32)
    lum[77, 300] = 5e4
    t = oracle.env_map_tables(lum)
    assert abs(t[..., 1].sum() * 4 * math.pi / (W * H) - 1) < 1e-4           # the density integrates to one
    assert np.all(t[:, -1, 0] == 1.0) and t[-1, 0, 2] == 1.0                   # every CDF ends at one
    assert np.all(np.diff(t[:, :, 0], axis=1) >= 0) and np.all(np.diff(t[:, 0, 2]) >= 0)
    fl = 1e-3 * lum.mean()
    assert abs(t[77, 300, 1] / t[0, 0, 1] - (5e4 + fl) / (1 + fl)) < 1e-3 * (5e4 / 1)
    black = oracle.env_map_tables(np.zeros((H, W), np.float32))                # a black environment: uniform
    assert np.allclose(black[..., 1] * 4 * math.pi, 1.0, rtol=1e-6)


def test_image_lookup_matches_numpy():
    img = scenes.env_patch_image()
    rng = np.random.default_rng(5)
    d = rng.normal(size=(4000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    s = scenes.env_floor()
    try:
        oracle.set_env_image(img, 179.0, 30.0)
        got = oracle.env_radiance(s, d)
    finally:
        oracle.set_env_image(None)
    ref = scenes.env_image_lookup(img, d, 179.0, 30.0)
    assert np.allclose(got, ref, rtol=1e-9, atol=1e-9)


def test_env_floor_closed_form():
    """A Lambertian floor under a panorama with one bright patch: albedo / pi times the illuminance of the upper half,
    through the map's light samples, the cosine lobe's and the BSDF's hits alike."""
    img = scenes.env_patch_image()
    E = scenes.env_level_illuminance(img)
    s = scenes.env_floor(width=24, height=24)
    try:
        oracle.set_env_image(img)
        ref = oracle.render(s, 128)
    finally:
        oracle.set_env_image(None)
    L = ref.luma()
    se = math.sqrt(np.nansum(ref.se() ** 2)) / L.size
    cf = 0.8 / math.pi * E
    assert abs(L.mean() - cf) < 5 * se + 1e-3 * cf, (L.mean(), cf, se)
