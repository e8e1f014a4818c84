"""The scene as code on the GPU (st_set_scene with the emitter's CUDA, compiled by NVRTC for sm_103a): the same
distances, pictures and tallies as the scene as data (the primitive table), and as the oracle.

The code folds the scene as the table path does, with the same exact culls; only f32 rounding differs (constants
folded by the compiler, a sphere's distance without its rotation, a prism's sector from its edge normals rather
than an arctangent). So the scene's distance agrees to f32 rounding, and a picture agrees pixel by pixel on nearly
every path (both sides seed every path alike) and within the Monte-Carlo error bars everywhere -- through each
kernel that asks the scene: the march (with and without the haze), the surface, the occlusion pass (with a light's
face), the emitter rays' resolve, the step cache's fill, the photon map's photons and the counting pass.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import codegen, scenes, st_types as T
from shadytracer_gb300.renderer import create_path_tracer

pytestmark = pytest.mark.gpu
LUMA = np.array([0.2126, 0.7152, 0.0722])
P = C.c_void_p


def eval_sdf(rt, pts):
    out = np.zeros(len(pts), np.float32)
    rc = rt.L.st_eval_sdf(rt.ctx, pts.ctypes.data_as(P), len(pts), out.ctypes.data_as(P))
    assert rc == 0, rt.L.st_last_error(rt.ctx)
    return out


def room_points(scene, n, seed):
    rng = np.random.default_rng(seed)
    c = np.array([list(p.pos) for p in scene.prim_list], np.float64)
    lo, hi = c.min(0) - 3.0, c.max(0) + 3.0
    a = rng.uniform(lo, hi, (n // 2, 3))
    pick = rng.integers(0, len(c), n - n // 2)
    b = c[pick] + rng.normal(scale=0.25, size=(n - n // 2, 3))
    return np.concatenate([a, b]).astype(np.float32)


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


@pytest.mark.parametrize("seed", [1, 2])
def test_code_distance_matches_the_table_and_the_oracle(seed):
    s = scenes.sdf_room(width=64, height=36, prim_seed=seed + 1)
    pts = room_points(s, 200000, seed)
    with create_path_tracer(s) as rt:
        table = eval_sdf(rt, pts)
        ms = rt.set_scene(s, code=True)
        info = rt.scene_code_info()
        assert info["code"] and info["cubin_bytes"] > 0
        code = eval_sdf(rt, pts)
    np.testing.assert_allclose(code, table, rtol=1e-5, atol=2e-6)
    ref, _, _ = oracle.scene_sdf(s, pts)
    np.testing.assert_allclose(code, ref, rtol=1e-4, atol=2e-5)


def test_code_distance_of_the_lenses():
    b = scenes.optics_bench(n_instances=2, seed=5)
    rng = np.random.default_rng(4)
    pts = rng.uniform([-0.004, -0.004, -0.001], [0.004, 0.004, 0.004], (100000, 3)).astype(np.float32)
    with create_path_tracer(b, code=True) as rt:
        d = eval_sdf(rt, pts)
    ref, _, _ = oracle.scene_sdf(b, pts)
    np.testing.assert_allclose(d, ref, rtol=1e-3, atol=1e-7)


def render(s, n, code, **params):
    for k, v in params.items():
        setattr(s.params, k, v)
    with create_path_tracer(s, code=code) as rt:
        rt.step(n)
        out = rt.read_accum()
        c = rt.counters()
    return out, c


def same_picture(a, b, min_exact=0.9):
    (rgb, V, S, cnt), (rgb2, V2, S2, cnt2) = a, b
    assert np.array_equal(cnt, cnt2)
    L, L2 = rgb @ LUMA, rgb2 @ LUMA
    exact = np.abs(L - L2) <= 1e-3 * np.maximum(np.abs(L2), 1.0)
    assert exact.mean() > min_exact, exact.mean()
    sd = np.hypot(se_of(V, S), se_of(V2, S2))
    ok = sd > 0
    z = (L - L2)[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.99, np.mean(np.abs(z) < 4)


def test_room_as_code_renders_the_tables_picture():
    s = scenes.sdf_room(width=96, height=54, spp=4)
    table, c0 = render(s, 4, None)
    s = scenes.sdf_room(width=96, height=54, spp=4)
    code, c1 = render(s, 4, True)
    same_picture(code, table)
    assert c1["nonfinite"] == 0 and c1["paths"] == c0["paths"]
    # and the oracle's, within the error bars
    ref = oracle.render(scenes.sdf_room(width=96, height=54, spp=4), 4)
    rgb, V, S, cnt = code
    L, Lr = rgb @ LUMA, ref.luma()
    se = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    within = np.abs(L - Lr) <= 4 * se + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert within.mean() > 0.985, (~within).sum()


def test_room_as_code_with_the_step_cache():
    s = scenes.sdf_room(width=96, height=54, spp=4)
    table, _ = render(s, 8, None, step_cache=1, step_cache_cells=4.0)
    s = scenes.sdf_room(width=96, height=54, spp=4)
    code, c = render(s, 8, True, step_cache=1, step_cache_cells=4.0)
    same_picture(code, table, min_exact=0.5)
    assert c["nonfinite"] == 0


def test_haze_beam_as_code():
    """The spot's light face through the haze box: the march's haze variant, the occlusion pass's face rays."""
    mk = lambda: scenes.haze_beam(width=64, height=36, spp=16, sigma_s=0.2, g=0.7)
    table, _ = render(mk(), 16, None)
    code, c = render(mk(), 16, True)
    same_picture(code, table, min_exact=0.5)
    assert c["nonfinite"] == 0


def test_lamp_as_code():
    """An emissive sphere: discovery, the emitter list, its rays resolved by the code's full answer."""
    mk = lambda: scenes.lamp_floor(width=48, height=32, spp=16)
    table, _ = render(mk(), 16, None)
    code, c = render(mk(), 16, True)
    same_picture(code, table, min_exact=0.5)
    assert c["nonfinite"] == 0


def test_caustic_as_code():
    """The photon map: the sun's photons marched and met through the code's answers."""
    mk = lambda: scenes.sppm_caustic(width=48, height=48, photons=200_000, r1=0.01)
    table, _ = render(mk(), 4, None)
    code, c = render(mk(), 4, True)
    same_picture(code, table, min_exact=0.5)


def test_counting_pass_counts_the_same_fold():
    s = scenes.sdf_room(width=96, height=54, spp=2)
    counts = []
    for code in (None, True):
        with create_path_tracer(scenes.sdf_room(width=96, height=54, spp=2), code=code) as rt:
            rt.enable_kernel_times(True, count_work=True)
            rt.step(2)
            c = rt.counters()
        counts.append(c)
    a, b = counts
    for k in ("prim_evals", "bound_tests"):
        x, y = np.sum(a[k]), np.sum(b[k])
        assert x > 0 and abs(x / y - 1) < 0.01, (k, x, y)


def test_a_bad_scene_keeps_the_old_one():
    s = scenes.floor_furnace(width=32, height=32)
    with create_path_tracer(s, code=True) as rt:
        rt.step(1)
        src = codegen.generate(s).replace("out = q.z;", "out = q.z + not_a_name;")
        from shadytracer_gb300._lib import StError
        with pytest.raises(StError) as e:
            rt.set_scene(s, code=src)
        assert e.value.code == T.ST_ERR_COMPILE and "at scene line" in str(e.value)
        assert rt.scene_code_info()["code"]                 # the old scene, still code, still renders
        rt.invalidate()
        rt.step(2)
        L = rt.read_accum()[0] @ LUMA
        assert abs(np.median(L[:8]) / 800.0 - 1) < 1e-3


HAND_WRITTEN = r"""
// a sphere of glass 0.3 m over a floor, written by hand (no table)
__device__ float st_scene_dist(st::f3 p) {
    const float ds = sqrtf(p.x * p.x + p.y * p.y + (p.z - 0.3f) * (p.z - 0.3f)) - 0.3f;
    const float df = p.z;
    return fabsf(ds) < fabsf(df) ? ds : df;
}
__device__ st::SceneHit st_scene_full(st::f3 p) {
    st::SceneHit h;
    const float ds = sqrtf(p.x * p.x + p.y * p.y + (p.z - 0.3f) * (p.z - 0.3f)) - 0.3f;
    const float df = p.z;
    h.d = fabsf(ds) < fabsf(df) ? ds : df;
    h.m = fabsf(ds) < fabsf(df) ? 1u : 2u;
    h.a = ds < 0.f ? 1u : (df < 0.f ? 2u : 0u);
    return h;
}
"""


def test_a_hand_written_scene_with_no_table():
    """The contract alone: code that is no emitter's, and a scene description with no primitives, against the same
    scene as a table."""
    ref_scene = scenes.sppm_caustic(width=48, height=48, photons=100_000)
    ref_scene.params.sppm = 0
    table, _ = render(ref_scene, 4, None)
    s = scenes.sppm_caustic(width=48, height=48, photons=100_000)
    s.params.sppm = 0
    s.desc.n_prims = 0
    code, c = render(s, 4, HAND_WRITTEN)
    rgb, V, S, cnt = code
    L, L2 = rgb @ LUMA, table[0] @ LUMA
    sd = np.hypot(se_of(V, S), se_of(table[1], table[2]))
    ok = sd > 0
    assert np.mean(np.abs((L - L2)[ok] / sd[ok]) < 4) > 0.98
    assert c["nonfinite"] == 0
