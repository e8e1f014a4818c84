"""Parity of the batched optics trace (csrc/st_optics.cu, through the C ABI) with the oracle's optics run.

Each ray is seeded as the reference seeds it (optics/kernels.js: the instance's sample seed, the ray's id, the
bounce), on both sides, so most rays take the same path; the tallies are FP64 on both sides. Totals of emitted
weight are exact; the escaped / absorbed / lost weights agree within a few binomial sigma; the far field's bins
agree up to the few rays f32 rounding sends another way.
"""
import math

import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bench_run():
    from shadytracer_gb300.renderer import create_path_tracer
    from shadytracer_gb300.optics import Optics
    b = scenes.optics_bench(n_instances=4, seed=5)
    rays = [20000, 35000, 5000, 12000]
    rt = create_path_tracer(b, device=0)
    O = Optics(rt)
    O.set_sources(b.info["sources"])
    O.set_far(nC=90, nG=46)
    g = O.run(rays, lux_cells=32, lux_half=1.0, lux_height=1.0, maxbounce=32, seed=3)
    o = oracle.optics_run(b, rays, nC=90, nG=46, cells=32, half=1.0, height=1.0, maxbounce=32, seed=3)
    rt.close()
    return rays, g, o


def test_totals(bench_run):
    rays, g, o = bench_run
    for i, n in enumerate(rays):
        G, R = g["totals"][i], o["totals"][i]
        assert G["rays"] == n
        assert G["emitted"] == pytest.approx(R["emitted"], abs=1e-9)
        s = G["escaped"] + G["lost"] + G["detected"] + G["absorbed"]
        assert s == pytest.approx(G["emitted"], rel=1e-9)
        for k in ("escaped", "absorbed"):
            p = max(R[k], 1.0) / n
            sig = math.sqrt(n * p * (1 - p)) + 1.0
            assert abs(G[k] - R[k]) <= 4 * sig + 0.003 * n, (i, k, G[k], R[k])
        assert abs(G["interactions"] - R["interactions"]) <= 0.01 * R["interactions"] + 10


def test_far_field(bench_run):
    rays, g, o = bench_run
    for i, n in enumerate(rays):
        F, R = g["far"][i], o["far"][i]
        assert F.sum() == pytest.approx(g["totals"][i]["escaped"], rel=1e-9)
        # the share of weight binned differently: the rays f32 rounding sent another way
        moved = 0.5 * np.abs(F - R).sum() / max(R.sum(), 1.0)
        assert moved < 0.03, (i, moved)


def test_lux_plane(bench_run):
    rays, g, o = bench_run
    for i, n in enumerate(rays):
        F, R = g["lux"][i], o["lux"][i]
        moved = 0.5 * np.abs(F - R).sum() / max(R.sum(), 1.0)
        assert moved < 0.03, (i, moved)


def test_far_field_and_lux_per_bin_at_a_million_rays():
    """One instance at 1.2 M rays, the full 1 x 1 degree candela grid (360 x 181) and a 128^2 lux map: every bin of
    the GPU's tallies within a binomial bound of the oracle's (4 sigma of the two counts taken as independent; the
    same seeds make them far closer), and at most 1 % of the weight in another bin."""
    from shadytracer_gb300.renderer import create_path_tracer
    from shadytracer_gb300.optics import Optics
    b = scenes.optics_bench(n_instances=1, seed=7)
    rays = [1_200_000]
    with create_path_tracer(b, device=0) as rt:
        O = Optics(rt)
        O.set_sources(b.info["sources"])
        O.set_far(nC=360, nG=181)
        g = O.run(rays, lux_cells=128, lux_half=1.0, lux_height=1.0, maxbounce=32, seed=11)
    o = oracle.optics_run(b, rays, nC=360, nG=181, cells=128, half=1.0, height=1.0, maxbounce=32, seed=11)
    for key in ("far", "lux"):
        F, R = np.asarray(g[key][0], float).ravel(), np.asarray(o[key][0], float).ravel()
        assert R.sum() > 0.1 * rays[0], (key, R.sum())
        bound = 4.0 * np.sqrt(F + R) + 1.0
        inside = np.abs(F - R) <= bound
        assert inside.all(), (key, np.count_nonzero(~inside), np.abs(F - R)[~inside][:5], bound[~inside][:5])
        moved = 0.5 * np.abs(F - R).sum() / max(R.sum(), 1.0)
        assert moved < 0.01, (key, moved)
