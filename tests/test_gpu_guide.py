"""The learned proposal on the GPU (csrc/st_guide.cu, st_guide.cuh; st_render.cu shade_surface), through the C ABI:
the network's forward pass and its training gradient against the oracle's restatement with the same BF16 rounding
(oracle/st_oracle_guide.h), the sampler's mixture against the oracle's decode, and the estimator: guided renders that
stay on the closed form and on the plain render, and a trained network that lowers the error.
"""
import numpy as np
import pytest

from shadytracer_gb300 import scenes
from shadytracer_gb300.st_types import MLP_PARAMS
from oracle import oracle

pytestmark = pytest.mark.gpu

NW = 13824
LUMA = np.array([0.2126, 0.7152, 0.0722])
LAYERS = {"W1": (0, 3072), "W2": (3072, 7168), "W3": (7168, 11264), "W4": (11264, 13824), "hash": (13824, MLP_PARAMS)}


@pytest.fixture(scope="module")
def rt():
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.sdf_room(width=64, height=36, spp=4)
    s.params.guide = 1
    r = create_path_tracer(s, device=0)
    r.step(1)                                 # the proposal's buffers and its first weights
    yield r
    r.close()


def random_weights(seed, w_scale=0.25, h_scale=0.5):
    rng = np.random.default_rng(seed)
    P = np.zeros(MLP_PARAMS, np.float32)
    P[:NW] = rng.normal(scale=w_scale, size=NW)
    P[NW:] = rng.normal(scale=h_scale, size=MLP_PARAMS - NW)
    return P


def points(rt, n, seed):
    st = rt.mlp_stats()
    lo, ext = np.array(st["box_lo"]), 1.0 / st["box_inv_ext"]
    rng = np.random.default_rng(seed)
    pos = (lo + rng.uniform(0.02, 0.98, (n, 3)) * ext).astype(np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32)
    return pos, nrm, np.array(st["box_lo"], np.float32), np.float32(st["box_inv_ext"])


def test_weights_round_trip(rt):
    P = random_weights(1)
    rt.set_mlp_weights(P)
    assert np.array_equal(rt.mlp_weights(), P)


def test_forward_matches_the_oracle(rt):
    P = random_weights(2)
    rt.set_mlp_weights(P)
    pos, nrm, lo, ie = points(rt, 3000, 3)
    raw, mix = rt.mlp_eval(pos, nrm)
    ref = oracle.guide_forward(P, pos, nrm, lo, ie, bf16=True)
    err = np.linalg.norm(raw - ref) / np.linalg.norm(ref)
    assert err < 1e-2, err
    # per point: the sums' order and a rare BF16 rounding flip are all that may differ
    rel = np.linalg.norm(raw - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert np.quantile(rel, 0.99) < 3e-2


def test_mixture_is_the_decoded_output(rt):
    P = random_weights(4)
    rt.set_mlp_weights(P)
    pos, nrm, lo, ie = points(rt, 2000, 5)
    raw, mix = rt.mlp_eval(pos, nrm)
    ref = oracle.guide_decode(raw.astype(np.float64))
    # the sampler's numbers: the direction in 2 x 16 bits, kappa and the weight as halves
    assert np.linalg.norm(mix[..., :3] - ref[..., :3], axis=-1).max() < 2e-4
    assert np.max(np.abs(mix[..., 3] / ref[..., 3] - 1)) < 1e-3
    assert np.max(np.abs(mix[..., 4] - ref[..., 4])) < 1e-3


def test_gradient_matches_the_oracle(rt):
    P = random_weights(6)
    rt.set_mlp_weights(P)
    n = 2048
    pos, nrm, lo, ie = points(rt, n, 7)
    rng = np.random.default_rng(8)
    dirs = rng.normal(size=(n, 3))
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    w = rng.exponential(1.0, n).astype(np.float32)
    g, loss = rt.mlp_grad(pos, nrm, dirs, w)
    G, ref_loss = oracle.guide_grad(P, pos, nrm, dirs, w, lo, ie, bf16=True)
    assert abs(loss / ref_loss - 1) < 2e-3, (loss, ref_loss)
    for name, (a, b) in LAYERS.items():
        x, y = g[a:b].astype(np.float64), G[a:b]
        cos = x @ y / (np.linalg.norm(x) * np.linalg.norm(y))
        rel = np.linalg.norm(x - y) / np.linalg.norm(y)
        assert cos > 0.999 and rel < 0.05, (name, cos, rel)
    # the gradient is a training step's only input: it leaves the weights as they were
    assert np.array_equal(rt.mlp_weights(), P)


def test_guided_floor_keeps_the_closed_form():
    """The photometry floor under the uniform sky, guided and training: every floor pixel's mean is still 800 cd/m^2."""
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.floor_furnace(width=128, height=128)
    s.params.guide = 1
    with create_path_tracer(s, device=0) as r:
        r.step(64)
        rgb, V, S, cnt = r.read_accum()
        st = r.mlp_stats()
    L = rgb @ LUMA
    floor = L[:40]
    se = np.sqrt(np.maximum(np.var(floor), 1e-12) / floor.size)
    assert abs(floor.mean() - 800.0) < max(5 * se, 0.4), (floor.mean(), se)
    assert st["steps"] > 0 and st["samples"] > 0 and np.isfinite(st["loss"])


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


def test_guided_room_agrees_with_plain():
    """The room at 160 x 90, 256 samples, plain and guided (training from the first wave): the pictures agree pixel by
    pixel within their error bars, and their means within the mean's."""
    from shadytracer_gb300.renderer import create_path_tracer
    out = {}
    for guide in (0, 1):
        s = scenes.sdf_room(width=160, height=90, spp=64)
        s.params.guide = guide
        with create_path_tracer(s, device=0) as r:
            r.step(256)
            rgb, V, S, cnt = r.read_accum()
            if guide:
                st = r.mlp_stats()
        out[guide] = (rgb @ LUMA, se_of(V, S))
    (L0, e0), (L1, e1) = out[0], out[1]
    sd = np.hypot(e0, e1)
    ok = sd > 0
    z = (L1 - L0)[ok] / sd[ok]
    assert np.mean(np.abs(z) < 4) > 0.99, np.mean(np.abs(z) < 4)
    zm = (L1 - L0)[ok].mean() / (np.sqrt(np.sum(sd[ok] ** 2)) / ok.sum())
    assert abs(zm) < 5, zm
    assert st["steps"] > 0 and np.isfinite(st["loss"])


def cross_entropy(mix, nrm, dirs, w):
    """-sum w log q(d) / sum w for the mixtures (n x 8 x 5) and, with mix None, the cosine lobe cos / pi."""
    if mix is None:
        q = np.maximum(np.sum(nrm * dirs, 1), 1e-9) / np.pi
    else:
        q = np.array([oracle.guide_mix_pdf(mix[i].astype(np.float64), dirs[i].astype(np.float64))
                      for i in range(len(w))])
    return float(-(w * np.log(np.maximum(q, 1e-30))).sum() / w.sum())


def test_training_learns_the_light():
    """What the trained network gains over the method without it: on records a later wave makes (which it was not
    trained on), its mixture fits the light the paths found -- f cos L_in / p at each record's vertex -- better than
    the BSDF's own cosine lobe and far better than the untrained network. The diffuse room lit by the sun's patch
    through its window (the sky almost black), 160 x 90."""
    from shadytracer_gb300.renderer import create_path_tracer
    s = scenes.sdf_room(width=160, height=90, spp=16, finish="diffuse", sky_illuminance=10.0, ground_luminance=1.0)
    s.params.guide = 1
    s.params.guide_train = 0
    s.params.samples_per_wave = 16
    with create_path_tracer(s, device=0) as r:
        r.step(1)
        w0 = r.mlp_weights()                     # as drawn
        s.params.guide_train = 1
        r.set_params(s.params)
        r.step(512)
        wt = r.mlp_weights()
        r.step(16)                               # fresh records, made with the trained weights
        pos, nrm, dirs, w = r.mlp_batch()
        keep = np.arange(len(w))[:6000]
        pos, nrm, dirs, w = pos[keep], nrm[keep], dirs[keep], w[keep]
        out = {}
        for name, P in (("untrained", w0), ("trained", wt)):
            r.set_mlp_weights(P)
            out[name] = cross_entropy(r.mlp_eval(pos, nrm)[1], nrm, dirs, w)
    out["cosine"] = cross_entropy(None, nrm, dirs, w)
    assert w.sum() > 0
    assert out["trained"] < out["cosine"] - 0.05, out
    assert out["trained"] < out["untrained"] - 0.05, out
