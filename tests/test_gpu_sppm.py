"""Parity of the photon map (csrc/st_sppm.cu, through the C ABI) with the oracle (oracle/st_oracle_sppm.h).

The grid is integer work and must agree exactly: every record's hashed cell, every cell's count, and the sorted
permutation must hold exactly the records of each cell (grouped by sub-list inside it). The gather's FP64 sums may
differ from the oracle's only by the order of the additions (records within a bucket land in atomic order).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

HEADS = 1 << 20
SUBS = 32
P = C.c_void_p


def ptr(a):
    return a.ctypes.data_as(P)


def oct_words(n):
    return np.array([oracle.sppm_oct(v) for v in n], np.uint32)


def records(seed, n, half=0.3, far=37.3):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-half, half, (n, 3)).astype(np.float32)
    pos[n // 4: n // 3] += np.float32(far)                 # a second cluster, far off: other cells, same hashes
    power = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    nv = rng.normal(size=(n, 3)) + np.array([0.0, 0.0, 4.0])
    nv /= np.linalg.norm(nv, axis=1, keepdims=True)
    nrm = oct_words(nv.astype(np.float32))
    flags = (rng.integers(0, 6, n) | (rng.integers(0, SUBS, n) << 16)).astype(np.uint32)
    return pos, power, nrm, flags


@pytest.fixture(scope="module")
def ctx():
    from shadytracer_gb300.renderer import create_path_tracer
    rt = create_path_tracer(None, device=0)
    yield rt
    rt.close()


def build(rt, pos, power, nrm, flags, cell):
    n = len(flags)
    rc = rt.L.st_sppm_build(rt.ctx, ptr(pos), ptr(power), None, ptr(nrm), ptr(flags), n, cell)
    assert rc == 0, rt.L.st_last_error(rt.ctx)
    key = np.zeros(max(n, 1), np.uint32)
    cnt = np.zeros(HEADS, np.uint32)
    start = np.zeros(HEADS, np.uint32)
    order = np.zeros(max(n, 1), np.uint32)
    assert rt.L.st_sppm_read_grid(rt.ctx, ptr(key), ptr(cnt), ptr(start), ptr(order)) == 0
    return key[:n], cnt, start, order[:n]


@pytest.mark.parametrize("n,cell", [(200000, 0.05), (1000, 0.2), (1, 0.05)])
def test_grid_matches_the_oracle(ctx, n, cell):
    pos, power, nrm, flags = records(11 + n, n)
    key, cnt, start, order = build(ctx, pos, power, nrm, flags, np.float32(cell))
    okey, ocnt = oracle.sppm_build(pos, power, nrm, flags, np.float32(cell))
    assert np.array_equal(key, okey)
    assert np.array_equal(cnt, ocnt)
    assert int(cnt.sum()) == n
    # the permutation holds each cell's records, contiguous from its start, sub-lists in order inside it
    assert np.array_equal(np.sort(order), np.arange(n, dtype=np.uint32))
    assert np.array_equal(start[1:], np.cumsum(cnt)[:-1].astype(np.uint32))
    cell_at = np.repeat(np.arange(HEADS, dtype=np.uint32), cnt)
    assert np.array_equal(okey[order], cell_at)
    sub = (flags[order] >> 16) & (SUBS - 1)
    bucket = cell_at.astype(np.int64) * SUBS + sub
    assert np.all(np.diff(bucket) >= 0)


@pytest.mark.parametrize("budget,min_whole", [(0, 0.99), (64, 0.99), (8, 0.2)])
def test_gather_matches_the_oracle(ctx, budget, min_whole):
    n, cell = 300000, np.float32(0.05)
    pos, power, nrm, flags = records(5, n)
    build(ctx, pos, power, nrm, flags, cell)
    oracle.sppm_build(pos, power, nrm, flags, cell)
    rng = np.random.default_rng(9)
    m = 40000
    q = pos[rng.integers(0, n, m)] + rng.normal(scale=0.01, size=(m, 3)).astype(np.float32)
    qn = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (m, 1))
    qa = rng.uniform(0.2, 0.9, (m, 3)).astype(np.float32)
    qb = rng.integers(0, 4, m).astype(np.uint32)
    radius, maxbounce, seed = np.float32(0.025), 4, 77
    out = np.zeros((m, 3), np.float64)
    rc = ctx.L.st_sppm_gather(ctx.ctx, ptr(q), ptr(qn), ptr(qa), ptr(qb), m, radius, maxbounce, budget, seed, ptr(out))
    assert rc == 0, ctx.L.st_last_error(ctx.ctx)
    ref, visits, cut = oracle.sppm_gather(q, qn, qa, qb, radius, maxbounce, budget, seed)
    # a gather the hard cap stopped summed the records it met first, and the order within a bucket is the atomics';
    # whether it stopped is not (the sub-lists walked and their sizes are the same on both sides)
    ok = cut == 0
    assert ok.mean() > min_whole
    assert np.count_nonzero(ref[ok]) > 0.5 * ok.sum()
    np.testing.assert_allclose(out[ok], ref[ok], rtol=1e-12, atol=1e-12)
    from shadytracer_gb300.st_types import StSppmStats
    s = StSppmStats()
    assert ctx.L.st_sppm_stats_read(ctx.ctx, C.byref(s)) == 0
    assert s.stored == n
    if budget == 0:
        assert s.visits == int(visits.sum())


def test_gather_rejects_a_radius_past_half_the_cell(ctx):
    pos, power, nrm, flags = records(3, 1000)
    build(ctx, pos, power, nrm, flags, np.float32(0.05))
    q = np.zeros((1, 3), np.float32)
    n = np.array([[0, 0, 1]], np.float32)
    a = np.ones((1, 3), np.float32)
    b = np.zeros(1, np.uint32)
    out = np.zeros((1, 3))
    rc = ctx.L.st_sppm_gather(ctx.ctx, ptr(q), ptr(n), ptr(a), ptr(b), 1, np.float32(0.04), 4, 0, 1, ptr(out))
    assert rc != 0
