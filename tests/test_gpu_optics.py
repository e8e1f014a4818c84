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


@pytest.fixture(scope="module")
def detector_run():
    from shadytracer_gb300.renderer import create_path_tracer
    from shadytracer_gb300.optics import Optics
    b = scenes.optics_detector_bench(n_instances=2, rays=300_000)
    rays = b.info["rays"]
    with create_path_tracer(b, device=0) as rt:
        O = Optics(rt)
        O.set_sources(b.info["sources"])
        O.set_far(nC=90, nG=46)
        O.set_detail(det_cap=1 << 20, path_rays=16, path_verts=16, esc_len=0.05)
        g = O.run(rays, lux_cells=32, maxbounce=32, seed=3)
        tags, mats = O.tallies()
        hits, nhits = O.hits()
        verts, counts = O.paths()
        g2 = O.run(rays, lux_cells=32, maxbounce=32, seed=3)     # a replay of the batch's graph
        tags2, mats2 = O.tallies()
    o = oracle.optics_run(b, rays, nC=90, nG=46, cells=32, maxbounce=32, seed=3)
    return b, rays, g, tags, mats, hits, nhits, verts, counts, g2, tags2, mats2, o


def test_a_replayed_batch_is_the_same_to_the_bit(detector_run):
    """The tallies are integers (fixed point) summed in any order: the batch's graph replayed gives the same bits."""
    b, rays, g, tags, mats, hits, nhits, verts, counts, g2, tags2, mats2, o = detector_run
    assert np.array_equal(g["far"], g2["far"]) and np.array_equal(g["lux"], g2["lux"])
    assert np.array_equal(tags, tags2) and np.array_equal(mats, mats2)
    assert g["totals"] == g2["totals"]


def test_counts_and_tallies_by_object_and_material_match_the_oracle(detector_run):
    b, rays, g, tags, mats, hits, nhits, verts, counts, g2, tags2, mats2, o = detector_run
    first = [min(i for i, p in enumerate(b.prim_list) if (p.flags >> 8) == k) for k in range(len(rays))]
    for k, n in enumerate(rays):
        G, R, D = g["totals"][k], o["totals"][k], o["detail"][k]
        assert G["n_escaped"] + G["n_lost"] + G["n_detected"] + G["n_absorbed"] <= n
        for c in ("n_escaped", "n_detected", "n_lost"):
            x, y = G[c], D["counts"][c]
            assert abs(x - y) <= 4 * math.sqrt(max(y, 1)) + 0.003 * n, (k, c, x, y)
        assert G["detected"] == pytest.approx(R["detected"], rel=0.01, abs=5)
        # by material: incident, leaving and interactions of the die, the lens and the detector
        for m in (1, 2, 3):
            gi, ri = mats[k, m], D["mat"][m]
            assert abs(gi[2] - ri[2]) <= 4 * math.sqrt(max(ri[2], 1)) + 0.003 * ri[2], (k, m, gi, ri)
            assert gi[0] == pytest.approx(ri[0], rel=0.02, abs=5), (k, m, gi, ri)
            assert gi[1] == pytest.approx(ri[1], rel=0.02, abs=5), (k, m, gi, ri)
        # by object: the instance's items by their first primitive (the GPU's tags count from the batch's table)
        for local in range(len(D["tag"])):
            ri = D["tag"][local]
            gi = tags[first[k] + local]
            assert abs(gi[2] - ri[2]) <= 4 * math.sqrt(max(ri[2], 1)) + 0.003 * ri[2] + 1, (k, local, gi, ri)
    # every interaction is some object's and some material's
    assert tags[:, 2].sum() == sum(t["interactions"] for t in g["totals"])
    assert mats[:, :, 2].sum() == sum(t["interactions"] for t in g["totals"])


def test_detector_hits_match_the_oracle(detector_run):
    b, rays, g, tags, mats, hits, nhits, verts, counts, g2, tags2, mats2, o = detector_run
    assert nhits == len(hits) == sum(t["n_detected"] for t in g["totals"])
    for k in range(len(rays)):
        mine = hits[hits[:, 8] == k]
        ref = o["detail"][k]["hits"]
        assert abs(len(mine) - len(ref)) <= 4 * math.sqrt(len(ref)) + 0.003 * len(ref)
        assert mine[:, 3].sum() == pytest.approx(g["totals"][k]["detected"], rel=1e-6)
        # on the detector's plane, spread as the oracle's
        assert np.allclose(mine[:, 2], 0.02 - 0.0005, atol=1e-4)
        for c in (0, 1):
            assert abs(mine[:, c].mean() - ref[:, c].mean()) < 4 * ref[:, c].std() / math.sqrt(len(ref)) + 1e-5
            assert abs(mine[:, c].std() / ref[:, c].std() - 1) < 0.02
        # its colour: a white source, X and Z of the weight's
        assert np.allclose(mine[:, 9] / mine[:, 3], 0.9505, rtol=2e-3)


def test_kept_paths_start_at_the_source_and_end_past_the_last_event(detector_run):
    b, rays, g, tags, mats, hits, nhits, verts, counts, g2, tags2, mats2, o = detector_run
    assert counts.shape == (2, 16) and counts.min() >= 2
    start = verts[:, :, 0, :3]
    assert np.all(np.abs(start[..., 2]) < 1e-5)                 # the die's face, z = 0
    assert np.all(np.abs(start[..., :2]) <= 0.0005 + 1e-6)      # within its 1 x 1 mm
    opl = np.array([[verts[i, r, :counts[i, r], 4] for r in range(16)] for i in range(2)], dtype=object)
    for i in range(2):
        for r in range(16):
            o_ = verts[i, r, :counts[i, r], 4]
            assert np.all(np.diff(o_) > 0), o_                   # optical length grows along the path


def test_the_detector_map(detector_run):
    """The recorded hits as an illuminance map (optics/detmap.js): the plane fitted to them is the detector's, the
    histogram and the kernel estimates hold the hits' flux, the k-nearest estimate reads the same illuminance where
    the hits are dense."""
    from shadytracer_gb300.optics import detector_map
    b, rays, g, tags, mats, hits, nhits, verts, counts, g2, tags2, mats2, o = detector_run
    mine = hits[hits[:, 8] == 0]
    m = detector_map(mine[:, :3], mine[:, 3], cells=32)
    assert abs(abs(m["frame"]["normal"][2]) - 1) < 1e-9          # squared up to the world: a floor
    assert m["total"] == pytest.approx(float(mine[:, 3].astype(np.float64).sum()), rel=1e-9)
    cell_area = m["cell_m"] ** 2
    assert (m["E"] * cell_area).sum() == pytest.approx(m["total"], rel=1e-9)
    for sm in ("gauss", "epan"):
        mk = detector_map(mine[:, :3], mine[:, 3], cells=32, smooth=sm, bandwidth=1.5)
        assert (mk["E"] * cell_area).sum() == pytest.approx(m["total"], rel=1e-9)
    mk = detector_map(mine[:, :3], mine[:, 3], cells=32, smooth="knn", k=64)
    dense = m["count"] > 200
    assert dense.any()
    assert abs(np.median(mk["E"][dense] / m["E"][dense]) - 1) < 0.1


def test_the_plane_crossing_tally_is_the_far_fields_virtual_plane_for_a_small_luminaire():
    """Two estimators of the lux plane: the trace's own (each escaping ray's line met at the plane, FP64 tally) and the
    reference's (optics/illum.js virtualPlane: the far field's intensity, the luminaire a point, E = I cos^3 / h^2).
    They agree where the luminaire is small against the distance -- a 6 mm lens at 1 m -- up to the far field's
    binning and the noise of both."""
    from shadytracer_gb300.renderer import create_path_tracer
    from shadytracer_gb300.optics import Optics, intensity, virtual_plane, lux
    b = scenes.optics_bench(n_instances=1, seed=9)
    n = 4_000_000
    with create_path_tracer(b, device=0) as rt:
        O = Optics(rt)
        O.set_sources(b.info["sources"])
        O.set_far(nC=360, nG=181)
        g = O.run([n], lux_cells=32, lux_half=1.0, lux_height=1.0, maxbounce=32, seed=2)
    scale = 1.0 / n                                                   # a unit of weight: 1 lm over n rays (flux 1)
    E_tally = lux(g["lux"][0], 32, 1.0, scale)
    E_far = virtual_plane(intensity(g["far"][0], 360, 181, scale), 360, 181, h=1.0, half=1.0, cells=32)
    lit = E_tally > 0.05 * E_tally.max()
    assert lit.sum() > 50
    ratio = E_far[lit] / E_tally[lit]
    assert abs(np.median(ratio) - 1) < 0.03, np.median(ratio)
    assert np.mean(np.abs(ratio - 1) < 0.15) > 0.9
