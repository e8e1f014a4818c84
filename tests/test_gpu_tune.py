"""The autotuner (st_autotune, st_optics_autotune): the march's and the occlusion pass's queue tile and march chunk,
timed on the workload itself, the fastest kept. What it picks changes which rays share a warp and where a ray's march
is cut between iterations -- never a ray's own random numbers, which are seeded by the path. A path the wavefront's
last iteration still finds going is ended there (the flush), and how many iterations a long march spends depends on
the chunk, so a few paths end differently: the picture is the defaults' pixel for pixel on nearly every pixel and
within the error bars on all. The optics tallies are integers and its rays run to their ends: the same bits."""
import numpy as np
import pytest

from shadytracer_gb300 import scenes
from shadytracer_gb300.renderer import create_path_tracer

pytestmark = pytest.mark.gpu
LUMA = np.array([0.2126, 0.7152, 0.0722])


def test_the_tuned_render_is_the_defaults_picture():
    s = scenes.sdf_room(width=160, height=90, spp=4)
    with create_path_tracer(s, code=True) as rt:
        rt.step(4)
        ref = rt.read_accum()
        t = rt.autotune(2)
        assert t["claim"] in (32, 64, 128) and 24 <= t["chunk"] <= 160
        assert 0 < t["ms"] <= t["ms_default"] * 1.0001
        rt.step(4)
        got = rt.read_accum()
    assert np.array_equal(got[3], ref[3])
    same_within_error(got, ref)


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


def same_within_error(got, ref):
    L, Lr = got[0] @ LUMA, ref[0] @ LUMA
    exact = np.abs(L - Lr) <= 1e-4 * np.maximum(np.abs(Lr), 1.0)
    assert exact.mean() > 0.98, exact.mean()
    sd = np.hypot(se_of(got[1], got[2]), se_of(ref[1], ref[2]))
    ok = sd > 0
    assert np.mean(np.abs((L - Lr)[ok]) <= 4 * sd[ok] + 1e-4 * np.abs(Lr[ok])) > 0.995
    assert abs(L.mean() / Lr.mean() - 1) < 0.01


def test_a_set_tune_of_extremes_keeps_the_picture():
    """The smallest tile and chunk the tuner tries, against the defaults: the same paths, cut differently."""
    from shadytracer_gb300 import st_types as T
    import ctypes as C
    s = scenes.sdf_room(width=96, height=54, spp=2)
    with create_path_tracer(s) as rt:
        rt.step(2)
        ref = rt.read_accum()
        tn = T.StTune()
        tn.claim, tn.chunk = 32, 24
        assert rt.L.st_set_tune(rt.ctx, C.byref(tn)) == 0
        rt.invalidate()
        rt.step(2)
        got = rt.read_accum()
    same_within_error(got, ref)


def test_the_tuned_optics_batch_keeps_its_tallies():
    from shadytracer_gb300.optics import Optics
    b = scenes.optics_bench(n_instances=4, seed=5)
    rays = [200_000, 50_000, 120_000, 80_000]
    with create_path_tracer(b, device=0) as rt:
        O = Optics(rt)
        O.set_sources(b.info["sources"])
        O.set_far(nC=90, nG=46)
        a = O.run(rays, lux_cells=32, seed=3)
        t = O.autotune(rays, lux_cells=32, seed=3)
        assert t["claim"] in (32, 64, 128) and 0 < t["ms"] <= t["ms_default"] * 1.0001
        g = O.run(rays, lux_cells=32, seed=3)
    # integer tallies: the same rays, the same bits, whatever the cut
    assert np.array_equal(a["far"], g["far"]) and np.array_equal(a["lux"], g["lux"])
    assert a["totals"] == g["totals"]
