"""Batching on the CPU: the host's plan_batches / split_part hold the reference's properties
(lib/pathtracer/core/test/photons.test.mjs): every stream traced whole, no batch over the buffer, each stream's batches
tiling it in order, no fewer batches than needed and at most one more, the streams asked first only in the first
batches. The optics run splits each instance's rays over its waves by the same split.
"""
import math

import pytest

from shadytracer_gb300.batching import plan_batches, split_part

MAX_RAYS = (1 << 30) // (2 * 64 + 16)     # a 1 GiB buffer over two rays and a shade item


def _round(v):
    try:
        v = float(v)
    except (TypeError, ValueError):
        return 0
    return max(0, int(math.floor(v + 0.5))) if math.isfinite(v) else 0


def sound(budget, streams, min_batches=1):
    p = plan_batches(budget, streams, min_batches)
    K = p.batches
    for s, n in enumerate(streams):
        assert sum(p.part(s, k) for k in range(K)) == _round(n)
        assert p.first(s, 0) == 0
        for k in range(K - 1):
            assert p.first(s, k) + p.part(s, k) == p.first(s, k + 1)
    worst = max(sum(p.part(s, k) for s in range(len(streams))) for k in range(K))
    assert worst <= budget
    need = max(-(-p.total // budget), min(p.total, min_batches or 1))
    assert need <= K <= need + 1
    return p


def test_the_save_that_lost_the_light():
    px = 2048 * 2048
    p = sound(MAX_RAYS, [px, px // 2, px // 2])
    assert p.batches == -(-2 * px // MAX_RAYS) and p.batches > 1
    assert all(abs(p.part(0, k) - (p.part(1, k) + p.part(2, k))) <= 2 for k in range(p.batches))


def test_one_batch_when_it_fits():
    px = 800 * 600
    p = sound(MAX_RAYS, [px, 0, px])
    assert p.batches == 1 and p.part(0, 0) == px and p.first(0, 0) == 0 and p.part(2, 0) == px


@pytest.mark.parametrize("budget,streams", [
    (MAX_RAYS, [3840 * 2160, 3840 * 2160 // 2, 3 * 3840 * 2160 // 2, 3840 * 2160]),
    (MAX_RAYS, [1920 * 1080, 12345, 2 * 1920 * 1080 - 12345, 777777]),
    (100, [1001, 7, 333, 0, 50]),
    (MAX_RAYS, [640 * 480, 0, 0]),
])
def test_sound_plans(budget, streams):
    sound(budget, streams)


def test_nonsense_streams():
    p = plan_batches(1000, [500, float("nan"), -5, None])
    assert p.batches == 1 and p.part(1, 0) == 0 and p.part(2, 0) == 0 and p.part(3, 0) == 0


def test_min_batches():
    px = 1280 * 720
    p = sound(MAX_RAYS, [px, 0, px], 12)
    assert p.batches == 12 and plan_batches(MAX_RAYS, [px, 0, px]).batches == 1
    q = plan_batches(100, [1001, 7, 333], 2)
    assert q.batches == plan_batches(100, [1001, 7, 333]).batches and q.batches > 2
    assert plan_batches(MAX_RAYS, [3, 0, 2], 50).batches == 5 and plan_batches(MAX_RAYS, [0, 0], 8).batches == 1


def check_first(budget, streams, first, min_batches=1):
    p = plan_batches(budget, streams, min_batches, first=first)
    K, Kf = p.batches, p.first_batches or 0
    for s, n in enumerate(streams):
        assert sum(p.part(s, k) for k in range(K)) == _round(n)
        ks = [k for k in range(K) if p.part(s, k) > 0]
        for k in ks:
            assert (k < Kf) if s in first else (k >= Kf)
        for j, k in enumerate(ks):
            want = 0 if j == 0 else p.first(s, ks[j - 1]) + p.part(s, ks[j - 1])
            assert p.first(s, k) == want
    assert max(sum(p.part(s, k) for s in range(len(streams))) for k in range(K)) <= budget
    return p


def test_some_streams_first():
    px = 800 * 600
    p = check_first(MAX_RAYS, [px, px // 4, px * 3 // 4, px // 2], [1, 2, 3])
    assert p.batches == 2 and p.first_batches == 1
    assert p.part(0, 0) == 0 and p.part(0, 1) == px and p.part(2, 0) == px * 3 // 4 and p.part(2, 1) == 0
    check_first(MAX_RAYS, [3840 * 2160, 10 ** 6, 7 * 10 ** 6, 3 * 10 ** 6], [1, 2, 3])
    check_first(100, [1001, 7, 333, 0, 50], [1, 2, 3, 4])
    q = check_first(MAX_RAYS, [1000, 0, 3000], [1, 2], 8)
    assert q.batches == 8 and q.first_batches == 6
    none = plan_batches(MAX_RAYS, [px, 0, 0], 1, first=[1, 2])
    assert none.batches == 1 and none.part(0, 0) == px


def test_split_part():
    for n, K in ((10, 3), (7, 7), (0, 4), (1, 5), (1000003, 17)):
        parts = [split_part(n, K, k) for k in range(K)]
        assert sum(parts) == n and max(parts) - min(parts) <= 1
