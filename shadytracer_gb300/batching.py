"""Batching: a sample's streams split over the fewest batches that fit the buffer (core/photons.js:31-76).

`plan_batches(budget, streams, min_batches, first)` is the reference's planBatches: every stream (camera rays,
emitter probes, sun photons, each light's photons; here also each optics instance's rays) is split evenly over K
batches, K the least whose largest batch fits `budget`; with `first`, those streams run in their own batches before
the rest (the photon map's photons before the camera's rays). The optics run splits each instance's rays this way
over its waves (csrc/st_optics.cu).
"""
import math


def split_part(n, K, k):
    """Stream n split into K parts as evenly as integers allow: part k. The parts add up to n exactly."""
    return (n * (k + 1)) // K - (n * k) // K


class Plan:
    def __init__(self, batches, total, streams, part, first, first_batches=None):
        self.batches = batches
        self.total = total
        self.streams = streams
        self.part = part
        self.first = first
        self.first_batches = first_batches


def _streams(streams):
    out = []
    for s in streams:
        try:
            v = float(s)
        except (TypeError, ValueError):
            v = 0.0
        out.append(max(0, int(math.floor(v + 0.5))) if math.isfinite(v) else 0)   # Math.round
    return out


def plan_batches(budget, streams, min_batches=1, first=None):
    if first:
        return _plan_in_order(budget, streams, min_batches, first)
    try:
        budget = max(1, int(math.floor(float(budget or 0))))
    except (TypeError, ValueError):
        budget = 1
    n = _streams(streams)
    total = sum(n)

    def fits(K):
        return sum(-(-s // K) for s in n) <= budget

    batches = max(1, -(-total // budget))
    while not fits(batches) and batches < total:
        batches += 1
    try:
        mb = int(math.floor(float(min_batches or 1)))
    except (TypeError, ValueError):
        mb = 1
    batches = max(batches, min(max(1, total), mb))
    return Plan(batches, total, n, lambda s, k: split_part(n[s], batches, k), lambda s, k: (n[s] * k) // batches)


def _plan_in_order(budget, streams, min_batches, first):
    n = _streams(streams)
    in_first = [s in first for s in range(len(n))]
    only = lambda keep: [v if in_first[s] == keep else 0 for s, v in enumerate(n)]
    tf, tr = sum(only(True)), sum(only(False))
    total = tf + tr
    if not tf or not tr:
        return plan_batches(budget, n, min_batches)
    mb = float(min_batches or 1)
    mf = max(1, int(math.floor(mb * tf / total + 0.5)))                          # Math.round
    mr = max(1, int(mb) - mf)
    pf, pr = plan_batches(budget, only(True), mf), plan_batches(budget, only(False), mr)
    Kf = pf.batches

    def part(s, k):
        if in_first[s]:
            return pf.part(s, k) if k < Kf else 0
        return 0 if k < Kf else pr.part(s, k - Kf)

    def first_(s, k):
        if in_first[s]:
            return pf.first(s, k) if k < Kf else n[s]
        return 0 if k < Kf else pr.first(s, k - Kf)

    return Plan(Kf + pr.batches, total, n, part, first_, Kf)
