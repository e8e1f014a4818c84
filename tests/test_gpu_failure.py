"""The failure path, on the GPU, with no fault: a device-side wait that runs out, and a host-side wait that runs out.

Every kernel that stages a table into shared memory waits on an mbarrier for its bulk copy a bounded number of times
(st_kernels.cuh stage_table). st_set_wait_limit(ctx, n, arm_only=1) makes that limit short and arms the barrier
without issuing the copy, so the wait runs out with nothing in flight: the CTA flags the error and returns, st_step
reports ST_ERR_TIMEOUT once, and the context stays usable -- the next trace, with the limit back, is right. The host's
own wait (st_sync with a timeout) on a long render reports ST_ERR_TIMEOUT and a later unbounded st_sync completes. The
reference's equivalents are host-side guards: core/wavefront.js:298-303 (a clamped indirect dispatch, "an unbounded
dispatch ... is a GPU hang") and core/raytrace_main.js:67 (a frame's submissions cut short).
"""
import numpy as np
import pytest

from shadytracer_gb300 import scenes, st_types as T
from shadytracer_gb300.renderer import create_path_tracer

pytestmark = pytest.mark.gpu

LUMA = np.array([0.2126, 0.7152, 0.0722])


def floor_ok(rt, n):
    rgb, V, S, cnt = rt.read_accum()
    assert (cnt == n).all()
    L = rgb @ LUMA
    # the bottom rows see only the floor: 0.8 x 1000 cd/m^2 every sample, but for a bounce so near the horizon that
    # its steps run out (maxiter), which takes half of that sample's light
    floor = L[:20]
    assert (np.abs(floor - 800.0) <= 0.08).mean() > 0.99, (floor.min(), floor.max())
    assert abs(floor.mean() / 800.0 - 1) < 2e-3


def test_a_device_wait_that_runs_out_reports_a_timeout_and_the_context_recovers():
    s = scenes.floor_furnace(width=64, height=64)
    with create_path_tracer(s) as rt:
        rt.step(2)
        floor_ok(rt, 2)
        assert rt.L.st_set_wait_limit(rt.ctx, 1000, 1) == 0
        rc = rt.L.st_step(rt.ctx, 1)
        assert rc == T.ST_ERR_TIMEOUT, rc
        assert b"ran out" in rt.L.st_last_error(rt.ctx)
        # the waits back to their default: the flag was reported once and cleared, the next trace is right
        assert rt.L.st_set_wait_limit(rt.ctx, 0, 0) == 0
        rt.invalidate()
        rt.step(3)
        floor_ok(rt, 3)


def test_a_short_limit_with_the_copy_issued_still_renders():
    """A limit short but enough for a real copy (the table lands in well under 10^5 polls): no error, the right
    picture -- the limit bounds the wait, it does not shorten a wait that ends."""
    s = scenes.floor_furnace(width=64, height=64)
    with create_path_tracer(s) as rt:
        assert rt.L.st_set_wait_limit(rt.ctx, 100000, 0) == 0
        rt.step(2)
        floor_ok(rt, 2)


def test_sync_with_a_short_timeout_on_a_long_render():
    s = scenes.sdf_room(width=1920, height=1080)
    with create_path_tracer(s) as rt:
        assert rt.L.st_step_async(rt.ctx, 16) == 0
        rc = rt.L.st_sync(rt.ctx, 1)
        assert rc == T.ST_ERR_TIMEOUT, rc
        assert b"in time" in rt.L.st_last_error(rt.ctx)
        # still in flight: the settings are refused until it finishes, and an unbounded wait completes it
        assert rt.L.st_set_view(rt.ctx, s.view) == T.ST_ERR_BUSY
        assert rt.L.st_sync(rt.ctx, -1) == 0
        rgb, V, S, cnt = rt.read_accum()
        assert (cnt == 16).mean() > 0.998
        assert np.isfinite(rgb).all()
