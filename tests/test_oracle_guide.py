"""The oracle's restatement of the learned proposal (oracle/st_oracle_guide.h), pinned by mathematics: the mixture of
von Mises-Fisher lobes is a density on the sphere and its draw has that density; the training loss's gradient
agrees with finite differences of the loss; BF16 rounding is round-to-nearest-even. The reference has no learned
proposal to compare with (it removed its path guiding), so these are the pins.
"""
import numpy as np
import pytest

from oracle import oracle

NW = oracle.GUIDE_NW
NP = oracle.GUIDE_NPARAM


def random_mixture(rng):
    raw = rng.normal(size=40)
    raw[3::5] = rng.uniform(-1.0, 6.0, 8)          # log kappa: broad to sharp lobes
    return oracle.guide_decode(raw[None, :])[0]


def fib_sphere(n):
    i = np.arange(n) + 0.5
    z = 1 - 2 * i / n
    r = np.sqrt(1 - z * z)
    ph = np.pi * (1 + 5 ** 0.5) * i
    return np.stack([r * np.cos(ph), r * np.sin(ph), z], 1)


def test_mixture_is_a_density():
    rng = np.random.default_rng(3)
    d = fib_sphere(200000)
    for _ in range(3):
        mix = random_mixture(rng)
        mix[:, 3] = np.minimum(mix[:, 3], 60.0)       # a grid of 200k points resolves lobes up to kappa ~ 60
        p = np.array([oracle.guide_mix_pdf(mix, x) for x in d[::7]])
        assert abs(p.mean() * 4 * np.pi - 1) < 0.01


def test_mixture_draw_has_the_density():
    # E over draws of 1 / p(d) is the area of the sphere when the draws have density p
    rng = np.random.default_rng(5)
    for _ in range(3):
        mix = random_mixture(rng)
        u = rng.random((100000, 3))
        d = oracle.guide_mix_sample(mix, u)
        assert np.allclose(np.linalg.norm(d, axis=1), 1, atol=1e-9)
        inv = np.array([1.0 / oracle.guide_mix_pdf(mix, x) for x in d])
        est = inv.mean()
        se = inv.std() / np.sqrt(len(inv))
        assert abs(est - 4 * np.pi) < 5 * se + 0.02 * 4 * np.pi, (est, se)


def test_bf16_rounds_to_nearest_even():
    assert oracle.bf16(1.0) == 1.0
    assert oracle.bf16(1.0 + 2 ** -8) == 1.0                  # a tie: to even (1.0)
    assert oracle.bf16(1.0 + 3 * 2 ** -8) == 1.0 + 2 ** -6    # a tie: to even (1 + 2^-6)
    assert oracle.bf16(1.0 + 2 ** -8 + 2 ** -12) == 1.0 + 2 ** -7


def small_problem(seed, n=6):
    rng = np.random.default_rng(seed)
    P = np.zeros(NP, np.float32)
    P[:NW] = rng.normal(scale=0.25, size=NW)
    P[NW:] = rng.normal(scale=0.5, size=NP - NW)
    pos = rng.uniform(0.1, 0.9, (n, 3)).astype(np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    dirs = rng.normal(size=(n, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    w = rng.uniform(0.2, 2.0, n).astype(np.float32)
    return P, pos, nrm.astype(np.float32), dirs.astype(np.float32), w, np.zeros(3, np.float32), 1.0


def test_gradient_matches_finite_differences():
    P, pos, nrm, dirs, w, lo, ie = small_problem(7)
    G, loss = oracle.guide_grad(P, pos, nrm, dirs, w, lo, ie, bf16=False)
    assert np.isfinite(loss) and np.all(np.isfinite(G))
    rng = np.random.default_rng(1)
    # weights of every layer, and the hash features the samples touch
    touched = np.nonzero(G[NW:])[0] + NW
    picks = list(rng.choice(NW, 24, replace=False)) + list(rng.choice(touched, 12, replace=False))
    for i in picks:
        h = 2e-3 * max(1.0, abs(float(P[i])))
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        hp, hm = float(Pp[i]) - float(P[i]), float(P[i]) - float(Pm[i])    # the steps as FP32 took them
        fd = (oracle.guide_loss(Pp, pos, nrm, dirs, w, lo, ie) - oracle.guide_loss(Pm, pos, nrm, dirs, w, lo, ie)) / (hp + hm)
        assert abs(fd - G[i]) <= 2e-3 * max(1.0, abs(G[i])), (i, fd, G[i])


def test_bf16_forward_is_close_to_exact():
    P, pos, nrm, dirs, w, lo, ie = small_problem(9, n=64)
    a = oracle.guide_forward(P, pos, nrm, lo, ie, bf16=True)
    b = oracle.guide_forward(P, pos, nrm, lo, ie, bf16=False)
    assert np.linalg.norm(a - b) < 0.03 * np.linalg.norm(b)


@pytest.mark.parametrize("seed", [11, 12])
def test_loss_falls_along_the_negative_gradient(seed):
    P, pos, nrm, dirs, w, lo, ie = small_problem(seed, n=32)
    G, loss = oracle.guide_grad(P, pos, nrm, dirs, w, lo, ie, bf16=False)
    step = (1e-3 / np.linalg.norm(G)) * G
    loss2 = oracle.guide_loss((P - step).astype(np.float32), pos, nrm, dirs, w, lo, ie)
    assert loss2 < loss
