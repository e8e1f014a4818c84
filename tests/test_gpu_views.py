"""Many views in one wavefront (st_set_views): each camera's picture, rendered in the same waves as the others, is the
picture that camera gives alone -- its paths take the same random numbers (the sample and the pixel seed them; the
view does not), the photon map's photons are the sample's for every view -- but for the order of f32 deposits into a
pixel. Light tracing, which connects to one camera, is refused with more than one view.
"""
import numpy as np
import pytest

from shadytracer_gb300 import scenes
from shadytracer_gb300._lib import StError
from shadytracer_gb300.renderer import create_path_tracer
from shadytracer_gb300.scenes import look_at

pytestmark = pytest.mark.gpu


def room_views(W, H):
    return [look_at((-2.6, -1.6, 1.7), (0.8, 0.9, 1.1), 60.0, W / H),
            look_at((2.5, -1.7, 1.5), (-0.5, 0.8, 0.8), 55.0, W / H),
            look_at((0.0, 1.6, 2.6), (0.0, -0.5, 0.3), 70.0, W / H)]


def alone(make, view, n):
    s = make()
    s.view = view
    with create_path_tracer(s, device=0) as rt:
        rt.step(n)
        return rt.read_accum()


def together(make, views, n):
    with create_path_tracer(make(), device=0) as rt:
        rt.set_views(views)
        rt.step(n)
        return [rt.read_accum(view=i) for i in range(len(views))], rt.counters()


def same(a, b):
    (rgb, V, S, cnt), (rgb2, V2, S2, cnt2) = a, b
    assert np.array_equal(cnt, cnt2)
    close = np.isclose(rgb, rgb2, rtol=1e-4, atol=1e-3).all(axis=-1)
    assert close.mean() > 0.999, close.mean()


def test_three_views_of_the_room_are_each_alone():
    make = lambda: scenes.sdf_room(width=96, height=54, spp=8)
    views = room_views(96, 54)
    pics, c = together(make, views, 8)
    assert c["paths"] == 3 * 96 * 54 * 8 and c["nonfinite"] == 0
    for i, v in enumerate(views):
        same(pics[i], alone(make, v, 8))
    # and they are three different pictures
    assert not np.allclose(pics[0][0], pics[1][0])


def test_views_share_the_photon_map():
    """The caustic from two cameras: one photon pass a sample serves both, each picture the one its camera gives
    alone."""
    make = lambda: scenes.sppm_caustic(width=64, height=64, photons=200_000, r1=0.01)
    base = make().view
    other = look_at((-1.3, -1.2, 1.1), (0.0, 0.1, 0.15), 45.0, 1.0)
    pics, c = together(make, [base, other], 4)
    same(pics[0], alone(make, base, 4))
    same(pics[1], alone(make, other, 4))


def test_light_tracing_takes_one_view():
    s = scenes.lt_pane(width=32, height=24, photons=50_000)
    with create_path_tracer(s, device=0) as rt:
        rt.set_views([s.view, s.view])
        with pytest.raises(StError):
            rt.step(1)
        rt.set_views([s.view])
        rt.step(1)
        with pytest.raises(StError):
            rt.read_accum(view=1)
