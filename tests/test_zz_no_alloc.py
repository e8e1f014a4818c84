"""st_render_noalloc: the render for hosts that may not allocate device memory, through the C ABI.

Some hosts cannot call cudaMalloc when they want a picture -- a plugin held to a device memory budget its
application fixed at start-up, a real-time thread that may not block on an allocation, code whose allocations would
land inside a stream capture it does not own. st_render_noalloc serves them from a scratch array compiled into the
library (8 MiB, pictures up to 128 x 128 pixels). Its picture must equal the regular entry point's (st_create,
st_set_*, st_step, st_read_accum) for the same scene, settings, camera and samples -- the same kernels and the same
per-path random numbers; only the order of a pixel's f32 deposits within one launch may differ -- and a second call
in a row, which finds the last call's contents in the shared array, must give the same answer as the first.

This file is collected last (its name), so a run that stops at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from shadytracer_gb300 import scenes, st_types as T

pytestmark = pytest.mark.gpu

RTOL = 1e-5          # f32 deposits summed in another order; everything else is the same arithmetic


def noalloc_fn():
    from shadytracer_gb300._lib import load
    L = load()
    f = L.st_render_noalloc
    f.argtypes = [C.c_int, C.POINTER(T.StSceneDesc), C.POINTER(T.StParams), C.POINTER(T.StView), C.c_int,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def render_noalloc(f, s, n):
    p = s.params
    rgb = np.zeros((p.height, p.width, 3), np.float64)
    V = np.zeros((p.height, p.width), np.float64)
    S = np.zeros((p.height, p.width), np.float64)
    cnt = np.zeros((p.height, p.width), np.uint32)
    P = C.c_void_p
    rc = f(0, C.byref(s.desc), C.byref(p), C.byref(s.view), n, rgb.ctypes.data_as(P), V.ctypes.data_as(P),
           S.ctypes.data_as(P), cnt.ctypes.data_as(P))
    return rc, rgb, V, S, cnt


def render_regular(s, n):
    from shadytracer_gb300.renderer import create_path_tracer
    rt = create_path_tracer(s, device=0)
    try:
        rt.step(n)
        return rt.read_accum()
    finally:
        rt.close()


def lamp_by_hits():
    s = scenes.lamp_floor(width=48, height=32, spp=4)
    s.params.emit_off = 1          # the emitter rendered by the BSDF's hits alone, on both paths
    return s


@pytest.mark.parametrize("make, n", [
    (lambda: scenes.floor_furnace(width=64, height=64), 4),
    (lambda: scenes.sdf_room(width=64, height=36, maxbounce=8), 3),
    (lambda: scenes.haze_furnace(width=32, height=32, sigma_t=0.5, g=0.7), 3),
    (lambda: scenes.dispersive_furnace(width=32, height=32, floor=True), 3),
    (lambda: scenes.absorbing_box(width=32, height=32), 3),
    (lambda: scenes.aniso_spheres(width=32, height=24), 3),
    (lamp_by_hits, 3),
])
def test_noalloc_equals_the_regular_render_twice_in_a_row(make, n):
    f = noalloc_fn()
    s = make()
    ref = render_regular(s, n)
    for call in range(2):
        rc, rgb, V, S, cnt = render_noalloc(f, s, n)
        assert rc == 0, "call %d: status %d" % (call, rc)
        assert np.array_equal(cnt, ref[3]), "call %d: sample counts differ" % call
        assert np.allclose(rgb, ref[0], rtol=RTOL, atol=1e-9 * max(1.0, np.abs(ref[0]).max())), \
            "call %d: pictures differ by %g" % (call, np.abs(rgb - ref[0]).max())
        assert np.allclose(V, ref[1], rtol=1e-4, atol=1e-6 * max(1.0, np.abs(ref[1]).max()))
        assert np.allclose(S, ref[2], rtol=1e-12, atol=1e-15)


def test_noalloc_refuses_a_picture_over_its_limit():
    f = noalloc_fn()
    s = scenes.floor_furnace(width=129, height=128)
    rc, *_ = render_noalloc(f, s, 1)
    assert rc == T.ST_ERR_ARG


def refused(make, setting=None):
    f = noalloc_fn()
    s = make()
    if setting:
        setattr(s.params, setting, 1)
    rc, *_ = render_noalloc(f, s, 1)
    from shadytracer_gb300._lib import load
    return rc, load().st_last_error(None).decode()


@pytest.mark.parametrize("make, setting, why", [
    (lambda: scenes.spot_floor(width=32, height=32, light="face"), None, "light faces"),
    (lambda: scenes.floor_furnace(width=32, height=32), "sppm", "photon map"),
    (lambda: scenes.floor_furnace(width=32, height=32), "guide", "learned proposal"),
    (lambda: scenes.floor_furnace(width=32, height=32), "lt", "light tracing"),
    (lambda: scenes.floor_sky(width=32, height=32, env_mode=1), None, "presets"),
    (lambda: scenes.floor_furnace(width=32, height=32), "step_cache", "step cache"),
    (lambda: scenes.lamp_floor(width=32, height=32), None, "emissive"),
])
def test_noalloc_refuses_what_it_does_not_render(make, setting, why):
    """Each setting this render does not carry is refused with ST_ERR_ARG and a reason, never silently dropped: its
    picture would differ from st_step's."""
    rc, msg = refused(make, setting)
    assert rc == T.ST_ERR_ARG
    assert why in msg, msg
