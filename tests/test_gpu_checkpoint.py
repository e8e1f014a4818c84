"""Checkpoint and resume (st_checkpoint_save / st_checkpoint_load): a render saved at N samples and resumed, in a new
context, to N + M is the render taken to N + M at once -- the same FP64 accumulation, its counts, its error bars -- on
the room and on the photon map's caustic (whose radius and photons follow the sample index); a checkpoint of another
picture is refused."""
import numpy as np
import pytest

from shadytracer_gb300 import scenes
from shadytracer_gb300._lib import StError
from shadytracer_gb300.renderer import create_path_tracer

pytestmark = pytest.mark.gpu


def straight(make, n):
    with create_path_tracer(make(), device=0) as rt:
        rt.step(n)
        return rt.read_accum()


def resumed(make, n, m):
    with create_path_tracer(make(), device=0) as rt:
        rt.step(n)
        blob = rt.checkpoint()
    with create_path_tracer(make(), device=0) as rt:
        rt.resume(blob)
        rt.step(m)
        return rt.read_accum(), rt.counters()


def same(a, b):
    (rgb, V, S, cnt), (rgb2, V2, S2, cnt2) = a, b
    assert np.array_equal(cnt, cnt2)
    close = np.isclose(rgb, rgb2, rtol=1e-4, atol=1e-3).all(axis=-1)
    assert close.mean() > 0.999, close.mean()


@pytest.mark.parametrize("make", [lambda: scenes.sdf_room(width=96, height=54, spp=16),
                                  lambda: scenes.sppm_caustic(width=64, height=64, photons=200_000, r1=0.01)],
                         ids=["room", "caustic"])
def test_a_resumed_render_is_the_render_at_once(make):
    a = straight(make, 12)
    b, c = resumed(make, 5, 7)
    same(a, b)


def test_another_pictures_checkpoint_is_refused():
    with create_path_tracer(scenes.sdf_room(width=96, height=54, spp=4), device=0) as rt:
        rt.step(2)
        blob = rt.checkpoint()
    with create_path_tracer(scenes.sdf_room(width=64, height=54, spp=4), device=0) as rt:
        with pytest.raises(StError):
            rt.resume(blob)
