"""The scene's distance on the GPU (st_eval_sdf, through the C ABI) against the oracle's (oracle/st_oracle_render.h
scene_eval: f32 without contractions, every primitive evaluated -- the reference's fold, scene_api.js FOLD_DIST).

The device fold skips a primitive where its bounding sphere shows it cannot change the running value, and computes
in f32 with fused multiply-adds and the hardware's division and square root; the two agree to f32 rounding at
random points of the scene's box, near every primitive (where the skipping decides most), and outside it.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes

pytestmark = pytest.mark.gpu
P = C.c_void_p


def ptr(a):
    return a.ctypes.data_as(P)


def points(scene, n, seed):
    rng = np.random.default_rng(seed)
    c = np.array([list(p.pos) for p in scene.prim_list], np.float64)
    lo, hi = c.min(0) - 3.0, c.max(0) + 3.0
    a = rng.uniform(lo, hi, (n // 2, 3))
    pick = rng.integers(0, len(c), n - n // 2)
    b = c[pick] + rng.normal(scale=0.25, size=(n - n // 2, 3))
    return np.concatenate([a, b]).astype(np.float32)


def eval_sdf(rt, pts):
    out = np.zeros(len(pts), np.float32)
    rc = rt.L.st_eval_sdf(rt.ctx, ptr(pts), len(pts), ptr(out))
    assert rc == 0, rt.L.st_last_error(rt.ctx)
    return out


@pytest.mark.parametrize("seed", [1, 2])
def test_room_distance_matches_the_oracle(seed):
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.sdf_room(width=64, height=36, prim_seed=seed + 1)
    rt = create_path_tracer(s, device=0)
    pts = points(s, 200000, seed)
    d = eval_sdf(rt, pts)
    rt.close()
    ref, _, _ = oracle.scene_sdf(s, pts)
    np.testing.assert_allclose(d, ref, rtol=1e-4, atol=2e-5)


def test_optics_lens_distance_matches_the_oracle():
    from shadytracer_gb300.renderer import create_path_tracer
    b = scenes.optics_bench(n_instances=2, seed=5)
    rt = create_path_tracer(b, device=0)
    rng = np.random.default_rng(4)
    pts = rng.uniform([-0.004, -0.004, -0.001], [0.004, 0.004, 0.004], (100000, 3)).astype(np.float32)
    d = eval_sdf(rt, pts)
    rt.close()
    ref, _, _ = oracle.scene_sdf(b, pts)
    np.testing.assert_allclose(d, ref, rtol=1e-3, atol=1e-7)


def test_floor_distance_is_its_height():
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.floor_furnace(width=16, height=16)
    rt = create_path_tracer(s, device=0)
    pts = points(s, 1000, 3)
    d = eval_sdf(rt, pts)
    rt.close()
    assert np.array_equal(d, pts[:, 2])
