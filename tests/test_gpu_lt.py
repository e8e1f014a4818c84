"""Light tracing to the camera on the GPU (csrc/st_photons.cu lt_connect and the connections' append in
k_photon_shade, the occlusion pass's connections into the splat buffer, k_resolve's unaveraged add, st_render.cu's
light-tracing class) against its closed form and the oracle.

The pane seen from the side (scenes.lt_pane): a floor lit only through a clear pane, seen directly -- the class
light -> delta+ -> D -> eye, light tracing's alone (the camera's paths keep the black sky, and light sampling from
the floor is blocked by the glass); its radiance is rho / pi E_sun sin(elevation) (1 - F)^2. The same photons and
camera paths are seeded alike on both sides, so the GPU's picture and the oracle's agree within the error bars, and
the connections that reached each pixel agree in number.
"""
import numpy as np
import pytest

from oracle import oracle
from shadytracer_gb300 import scenes
from shadytracer_gb300.renderer import create_path_tracer

pytestmark = pytest.mark.gpu
LUMA = np.array([0.2126, 0.7152, 0.0722])


def se_of(V, S):
    ok = (S > 0) & (S < 1)
    out = np.zeros_like(V)
    out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
    return out


def render(s, n):
    with create_path_tracer(s, device=0) as rt:
        rt.step(n)
        out = rt.read_accum()
        counts = rt.lt_counts()
        c = rt.counters()
    return out, counts, c


def within_error_bars(gpu, ref, frac=0.98):
    rgb, V, S, _ = gpu
    L, Lr = rgb @ LUMA, ref.luma()
    se = np.sqrt(se_of(V, S) ** 2 + np.nan_to_num(ref.se()) ** 2)
    within = np.abs(L - Lr) <= 4 * se + 1e-3 * np.maximum(np.abs(Lr), 1.0)
    assert within.mean() > frac, (~within).sum()


def test_pane_seen_directly_closed_form():
    s = scenes.lt_pane(width=64, height=48, photons=1_000_000)
    (rgb, V, S, cnt), counts, c = render(s, 16)
    L = rgb @ LUMA
    m = np.array(scenes.floor_mask(s))
    cf = scenes.lt_pane_closed_form(s, oracle.fresnel_dielectric)
    assert m.sum() > 500
    assert abs(L[m].mean() / cf - 1) < 0.01, (L[m].mean(), cf)
    assert np.all(counts[m] > 0) and c["nonfinite"] == 0
    # the sky above the floor's far edge is black: nothing but connections lights the picture
    assert np.all(cnt == 16)


def test_pane_matches_the_oracle():
    s = scenes.lt_pane(width=48, height=36, photons=300_000)
    gpu, counts, _ = render(s, 8)
    ref = oracle.render(scenes.lt_pane(width=48, height=36, photons=300_000), 8)
    ref_counts = oracle.last_lt_counts(48, 36)
    within_error_bars(gpu, ref)
    # the same photons through the same gates: the connections that arrived, in all and pixel by pixel
    assert ref_counts.sum() > 100_000
    assert abs(counts.sum() / ref_counts.sum() - 1) < 0.002, (counts.sum(), ref_counts.sum())
    m = np.array(scenes.floor_mask(s))
    rel = np.abs(counts[m].astype(np.int64) - ref_counts[m]) / np.maximum(ref_counts[m], 1)
    assert np.mean(rel < 0.01) > 0.99, np.sort(rel)[-10:]


def test_pane_through_the_thin_lens():
    """A connection to a point of the lens's disc drawn from the photon's stream, the pixel where that point's ray
    through the focus plane lands; the floor's middle in focus."""
    s = scenes.lt_pane(width=48, height=36, photons=300_000, lens_radius=0.03)
    gpu, counts, _ = render(s, 8)
    ref = oracle.render(scenes.lt_pane(width=48, height=36, photons=300_000, lens_radius=0.03), 8)
    within_error_bars(gpu, ref)
    m = np.array(scenes.floor_mask(s, margin=0.3))
    cf = scenes.lt_pane_closed_form(s, oracle.fresnel_dielectric)
    L = gpu[0] @ LUMA
    assert abs(L[m].mean() / cf - 1) < 0.02, (L[m].mean(), cf)


def test_caustic_with_the_map_matches_the_oracle():
    """Light tracing and the photon map together, as the reference splits them: the caustic seen directly is the
    connections', the map gathers only past delta events from the eye (the floor seen through the sphere)."""
    mk = lambda: scenes.sppm_caustic(width=64, height=64, photons=300_000, r1=0.01)
    s = mk()
    s.params.lt = 1
    gpu, counts, c = render(s, 6)
    r = mk()
    r.params.lt = 1
    ref = oracle.render(r, 6)
    within_error_bars(gpu, ref)
    assert counts.sum() > 0 and c["nonfinite"] == 0
    assert abs(counts.sum() / oracle.last_lt_counts(64, 64).sum() - 1) < 0.005


def test_caustic_light_tracing_agrees_with_the_map():
    """The same caustic, seen directly, counted by the connections (with the map gathering only past delta events
    from the eye) or by the map's gather at the eye's first surface too (its estimate biased by its radius, 5 mm
    here): the two pictures agree, over the whole and over the caustic."""
    mk = lambda: scenes.sppm_caustic(width=96, height=96, photons=1_000_000, r1=0.005)
    a = mk()
    a.params.lt = 1
    (rgb_a, Va, Sa, _), _, _ = render(a, 16)
    b = mk()
    (rgb_b, Vb, Sb, _), _, _ = render(b, 16)
    La, Lb = rgb_a @ LUMA, rgb_b @ LUMA
    assert abs(La.mean() / Lb.mean() - 1) < 0.02, (La.mean(), Lb.mean())
    bright = Lb > np.quantile(Lb, 0.9)
    assert abs(La[bright].mean() / Lb[bright].mean() - 1) < 0.05, (La[bright].mean(), Lb[bright].mean())


def inner_pixels(hit):
    inner = hit.copy()
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            inner &= np.roll(np.roll(hit, dy, 0), dx, 1)
    return inner


def test_haze_closed_form_and_the_oracle():
    """Photons through a pane scattered in a haze box, connected through the phase function (haze.js ltConnectMedium):
    the single scattering by quadrature along each pixel's ray, and the oracle's picture pixel by pixel."""
    s = scenes.lt_haze(width=64, height=48, photons=1_000_000)
    gpu, counts, c = render(s, 32)
    cf = scenes.lt_haze_single_scatter(s, oracle.fresnel_dielectric)
    m = inner_pixels(cf > 0)
    L = gpu[0] @ LUMA
    assert m.sum() > 500 and c["nonfinite"] == 0
    assert abs(L[m].sum() / cf[m].sum() - 1) < 0.01, L[m].sum() / cf[m].sum()
    small = scenes.lt_haze(width=48, height=36, photons=300_000)
    gpu, counts, _ = render(small, 8)
    ref = oracle.render(scenes.lt_haze(width=48, height=36, photons=300_000), 8)
    within_error_bars(gpu, ref)
    ref_counts = oracle.last_lt_counts(48, 36)
    assert abs(counts.sum() / ref_counts.sum() - 1) < 0.005, (counts.sum(), ref_counts.sum())


def test_emitter_photons_closed_form_and_the_oracle():
    """A lamp's light on a floor through a pane, the emitter photons' (the probes', from the third sample on, once the
    lamp is listed; the first two samples taken out): albedo Le a^2 h / D^3 (1 - F)^2 over the floor, and the oracle's
    picture pixel by pixel with its connections counted alike."""
    s = scenes.lt_lamp(width=64, height=48, photons=1_000_000)
    cf = scenes.lt_lamp_closed_form(s, oracle.fresnel_dielectric)
    m = cf > 0.5 * np.median(cf[cf > 0])
    with create_path_tracer(s, device=0) as rt:
        rt.step(2)
        L2 = rt.read_accum()[0] @ LUMA
        rt.step(126)
        L = rt.read_accum()[0] @ LUMA
        c = rt.counters()
    X = (128 * L - 2 * L2) / 126
    assert m.sum() > 500 and c["nonfinite"] == 0
    assert abs(X[m].mean() / cf[m].mean() - 1) < 0.025, X[m].mean() / cf[m].mean()
    small = scenes.lt_lamp(width=48, height=36, photons=200_000)
    gpu, counts, _ = render(small, 16)
    ref = oracle.render(scenes.lt_lamp(width=48, height=36, photons=200_000), 16)
    within_error_bars(gpu, ref, frac=0.97)
    ref_counts = oracle.last_lt_counts(48, 36)
    assert abs(counts.sum() / ref_counts.sum() - 1) < 0.01, (counts.sum(), ref_counts.sum())


def test_invalidate_clears_the_connections():
    s = scenes.lt_pane(width=32, height=24, photons=100_000)
    with create_path_tracer(s, device=0) as rt:
        rt.step(2)
        assert rt.lt_counts().sum() > 0
        rt.invalidate()
        assert rt.lt_counts().sum() == 0
        rt.step(1)
        one = rt.lt_counts().sum()
        assert one > 0
        rt.step(1)
        assert rt.lt_counts().sum() > one


def test_off_leaves_the_floor_dark():
    """With light tracing off (and no map) the floor under the glass gets nothing but what a path meets by hitting the
    sun's disc through the pane, which is rare: the class is light tracing's."""
    s = scenes.lt_pane(width=32, height=24, photons=100_000)
    s.params.lt = 0
    (rgb, _, _, _), counts, _ = render(s, 4)
    m = np.array(scenes.floor_mask(s))
    assert (rgb @ LUMA)[m].mean() < 0.05 * scenes.lt_pane_closed_form(s, oracle.fresnel_dielectric)
    assert counts.sum() == 0
