"""TEST INFRASTRUCTURE ONLY -- the oracle's Python face.

Builds (g++, OpenMP) and loads oracle/_build/liboracle.so, the CPU restatement of the reference's rendering hot
path (st_oracle*.h / .cpp), and wraps its entry points with numpy. Only tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg may import this module: it is the checker and the CPU baseline, never the product.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["st_oracle.cpp", "st_oracle_core.h", "st_oracle_render.h", "st_oracle_extra.h", "st_oracle_sppm.h",
           "st_oracle_optics.h", "st_oracle_spectral.h", "st_oracle_guide.h", "st_oracle_light.h",
           "../include/shadytracer.h"]

_lib = None


def build(force=False):
    """Compile the oracle if a source is newer than the library. Returns the library's path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return LIB
    cpp = [os.path.join(HERE, "st_oracle.cpp")]
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-fno-fast-math", "-ffp-contract=off",
           "-o", tmp] + cpp
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _declare(_lib)
    return _lib


def _declare(L):
    P = C.c_void_p
    L.sto_render.argtypes = [P, P, P, C.c_uint32, C.c_uint32, C.c_int, P, P, P, P, P, C.c_int, C.c_uint32, C.c_uint32]
    L.sto_render.restype = C.c_int
    L.sto_mf_tables.argtypes = [C.c_int, P, P, P]
    L.sto_scene_sdf.argtypes = [P, P, C.c_uint32, P, P, P]
    L.sto_pcg4d.argtypes = [P, P]
    L.sto_prng.argtypes = [P, P, C.c_int, C.c_int, P]
    L.sto_sample_seed.argtypes = [C.c_uint32, C.c_uint32, P]
    L.sto_derive.argtypes = [P, P, P]
    L.sto_fresnel_dielectric.argtypes = [C.c_double, C.c_double]
    L.sto_fresnel_dielectric.restype = C.c_double
    L.sto_lobes.argtypes = [P, P, P, C.c_double, P, P]
    L.sto_lobes_sample.argtypes = [P, P, C.c_double, C.c_uint32, C.c_int, P, P]
    L.sto_coat_rgb.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, P]
    L.sto_coat_at_lambda.argtypes = [C.c_double] * 5
    L.sto_coat_at_lambda.restype = C.c_double
    L.sto_lobes_sample_coat.argtypes = [P, P, C.c_double, C.c_double, C.c_int, C.c_double, P, C.c_uint32, C.c_int, P, P]
    L.sto_set_env_image.argtypes = [P, C.c_uint32, C.c_uint32, C.c_float, C.c_float]
    L.sto_env_map_tables.argtypes = [P, P]
    L.sto_env_radiance.argtypes = [P, P, P, C.c_uint32, P]
    for name, args, res in _EXTRA:
        if hasattr(L, name):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res


_EXTRA = []


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Accum:
    """The FP64 accumulation a render folds into (the prog_resolve state), continued across calls."""

    def __init__(self, w, h):
        self.w, self.h = w, h
        self.rgb = np.zeros((h, w, 3), np.float64)
        self.V = np.zeros((h, w), np.float64)
        self.S = np.zeros((h, w), np.float64)
        self.count = np.zeros((h, w), np.uint32)
        self.counters = np.zeros(8, np.uint64)
        self.next_sample = 0

    def luma(self):
        return self.rgb[..., 0] * 0.2126 + self.rgb[..., 1] * 0.7152 + self.rgb[..., 2] * 0.0722

    def se(self):
        """The standard error of each pixel's mean luminance (core/measure.js:46-51), nan where unknown."""
        S, V = self.S, self.V
        ok = (S > 0) & (S < 1) & (V >= 0)
        out = np.full(S.shape, np.nan)
        out[ok] = np.sqrt(S[ok] * V[ok] / (1 - S[ok]))
        return out


def render(scene, nsamples, accum=None, fp64=False, threads=0, sample0=None, path_first=0, path_count=0, cull=False):
    """Trace `nsamples` samples of `scene` (a shadytracer_gb300.scenes.Scene) into `accum` (made if None). cull: the
    f32 arithmetic with the reference's bounding-box culling at the root (its generated code's work a step)."""
    L = lib()
    p = scene.params
    if accum is None:
        accum = Accum(p.width, p.height)
    s0 = accum.next_sample if sample0 is None else sample0
    rc = L.sto_render(C.byref(scene.desc), C.byref(p), C.byref(scene.view), s0, nsamples, 1 if fp64 else (2 if cull else 0),
                      ptr(accum.rgb), ptr(accum.V), ptr(accum.S), ptr(accum.count), ptr(accum.counters), threads,
                      path_first, path_count)
    if rc != 0:
        raise RuntimeError("sto_render failed: %d" % rc)
    accum.next_sample = s0 + nsamples
    return accum


def set_env_image(rgb=None, luminance=0.0, turn=0.0):
    """The environment image for the renders that follow (H x W x 3 linear floats, top row first); None clears it."""
    if rgb is None:
        lib().sto_set_env_image(None, 0, 0, 0.0, 0.0)
        return
    img = np.ascontiguousarray(rgb, np.float32)
    if lib().sto_set_env_image(ptr(img), img.shape[1], img.shape[0], luminance, turn) != 0:
        raise ValueError("bad environment image")


def env_map_tables(lum):
    """The map's tables (512 x 256 x 4) from its texels' mean luminances (256 rows x 512)."""
    lum = np.ascontiguousarray(lum, np.float32).reshape(-1)
    tex = np.zeros(lum.size * 4, np.float32)
    lib().sto_env_map_tables(ptr(lum), ptr(tex))
    return tex.reshape(256, 512, 4)


def env_radiance(scene, dirs):
    """The environment's radiance (rgb) in the given directions, as the oracle has it for this scene's settings."""
    d = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    out = np.zeros_like(d)
    lib().sto_env_radiance(C.byref(scene.params), C.byref(scene.desc), ptr(d), len(d), ptr(out))
    return out


def mf_tables(fp64=False):
    ec = np.zeros(16 * 32 * 32, np.float32)
    ecavg = np.zeros(16 * 32, np.float32)
    e1 = np.zeros(32 * 32, np.float32)
    lib().sto_mf_tables(1 if fp64 else 0, ptr(ec), ptr(ecavg), ptr(e1))
    return ec, ecavg, e1


def scene_sdf(scene, pts):
    pts = np.ascontiguousarray(pts, np.float32)
    n = pts.shape[0]
    d = np.zeros(n, np.float32)
    m = np.zeros(n, np.uint32)
    a = np.zeros(n, np.uint32)
    lib().sto_scene_sdf(C.byref(scene.desc), ptr(pts), n, ptr(d), ptr(m), ptr(a))
    return d, m, a


def pcg4d(v):
    a = np.asarray(v, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().sto_pcg4d(ptr(a), ptr(o))
    return o


def prng(seed4, words, n):
    s = np.asarray(seed4, np.uint32)
    w = np.asarray(words, np.uint32)
    out = np.zeros((n, 4), np.float32)
    lib().sto_prng(ptr(s), ptr(w), len(w), n, ptr(out))
    return out


def sample_seed(base, sample):
    o = np.zeros(4, np.uint32)
    lib().sto_sample_seed(base, sample, ptr(o))
    return o


def derive(scene):
    o = np.zeros(12, np.float64)
    lib().sto_derive(C.byref(scene.params), C.byref(scene.desc), ptr(o))
    keys = ["sun_half", "sun_omc", "sun_sin2", "sun_omega", "disc_lum", "sun_on", "nee_sun_pick", "tol_setting",
            "env_radius", "tint_r", "tint_g", "tint_b"]
    return dict(zip(keys, o.tolist()))


def fresnel_dielectric(cosI, eta):
    return lib().sto_fresnel_dielectric(cosI, eta)


def lobes(mat, v, l, eta):
    f = np.zeros(3, np.float64)
    pdf = np.zeros(1, np.float64)
    lib().sto_lobes(C.byref(mat), ptr(np.asarray(v, np.float64)), ptr(np.asarray(l, np.float64)), eta, ptr(f), ptr(pdf))
    return f, float(pdf[0])


def lobes_sample(mat, v, eta, seed, n):
    d = np.zeros((n, 3), np.float64)
    w = np.zeros((n, 3), np.float64)
    lib().sto_lobes_sample(C.byref(mat), ptr(np.asarray(v, np.float64)), eta, seed, n, ptr(d), ptr(w))
    return d, w


def coat_rgb(lo, hi, edge, width):
    """A coating's reflectance per channel (spectral.js edgeRGB), as the oracle's lobes take it."""
    out = np.zeros(3, np.float64)
    lib().sto_coat_rgb(lo, hi, edge, width, ptr(out))
    return out


def coat_at_lambda(lo, hi, edge, width, lam):
    return lib().sto_coat_at_lambda(lo, hi, edge, width, lam)


def lobes_sample_coat(mat, v, eta, n0, inside, lam, beta, seed, n):
    """n draws of a coated material's lobes at normal +z, view v, seen from medium n0 (inside or not), by a ray of
    wavelength lam (0 none) carrying beta: directions and weights."""
    d = np.zeros((n, 3), np.float64)
    w = np.zeros((n, 3), np.float64)
    lib().sto_lobes_sample_coat(C.byref(mat), ptr(np.asarray(v, np.float64)), eta, n0, int(inside), lam,
                                ptr(np.asarray(beta, np.float64)), seed, n, ptr(d), ptr(w))
    return d, w


# ---- the photon map (st_oracle_sppm.h) ----
def _declare_extra(L):
    P = C.c_void_p
    sig = {
        "sto_sppm_hash": ([C.c_int32, C.c_int32, C.c_int32], C.c_uint32),
        "sto_sppm_radius": ([C.c_double, C.c_int, C.c_double], C.c_double),
        "sto_sppm_keep": ([C.c_double, C.c_double], C.c_double),
        "sto_sppm_subs_of": ([C.c_uint32, C.c_uint32], C.c_uint32),
        "sto_sppm_oct": ([P], C.c_uint32),
        "sto_sppm_unoct": ([C.c_uint32, P], None),
        "sto_sppm_build": ([P, P, P, P, C.c_uint32, C.c_float, P, P], C.c_int),
        "sto_sppm_gather": ([P, P, P, P, C.c_uint32, C.c_float, C.c_uint32, C.c_uint32, C.c_uint32, P, P, P], C.c_int),
        "sto_haze_span": ([P, P, P, C.c_double, C.c_double, P], None),
        "sto_hg_eval": ([C.c_double, C.c_double], C.c_double),
        "sto_hg_sample": ([C.c_double, P, C.c_uint32, C.c_int, P], None),
        "sto_far_bin": ([P, P, P, C.c_uint32, C.c_uint32], C.c_uint32),
        "sto_far_geometry": ([C.c_uint32, C.c_uint32, P], None),
        "sto_far_intensity": ([P, C.c_uint32, C.c_uint32, P], None),
        "sto_step_moments": ([P, C.c_double, C.c_double], None),
        "sto_cauchy_n": ([C.c_double, C.c_double, C.c_double], C.c_double),
        "sto_sppm_photons": ([P, P, C.c_uint32, P, P, P], C.c_int),
        "sto_lambda_code": ([C.c_double], C.c_uint32),
        "sto_lambda_of": ([C.c_uint32], C.c_double),
        "sto_spec_table": ([P, P], None),
        "sto_spec_draw": ([C.c_double, P], C.c_double),
        "sto_optics_set_rays": ([P, C.c_uint32], C.c_int),
        "sto_optics_run": ([P, P, P, C.c_uint32, P, C.c_uint32, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float,
                            C.c_float, C.c_uint32, C.c_uint32, C.c_int, P, P, P, C.c_int], C.c_int),
        "sto_guide_forward": ([P, C.c_uint32, P, P, P, C.c_float, C.c_int, P], None),
        "sto_guide_decode": ([P, C.c_uint32, P], None),
        "sto_guide_grad": ([P, C.c_uint32, P, P, P, P, P, C.c_float, C.c_int, P], C.c_double),
        "sto_guide_loss": ([P, C.c_uint32, P, P, P, P, P, C.c_float], C.c_double),
        "sto_guide_mix_pdf": ([P, P], C.c_double),
        "sto_guide_mix_sample": ([P, P, C.c_uint32, P], None),
        "sto_bf16": ([C.c_float], C.c_float),
        "sto_lt_build": ([P, P, P], None),
        "sto_optics_detail": ([C.c_uint32, P, P, P, P, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int),
        "sto_last_lt": ([P, P, P], C.c_int),
        "sto_last_lt_counts": ([P, C.c_uint32], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res


_extra_done = False


def xlib():
    global _extra_done
    L = lib()
    if not _extra_done:
        _declare_extra(L)
        _extra_done = True
    return L


def sppm_hash(i, j, k):
    return xlib().sto_sppm_hash(i, j, k)


def sppm_radius(r1, k, alpha=2.0 / 3.0):
    return xlib().sto_sppm_radius(r1, k, alpha)


def sppm_keep(capacity, demand):
    return xlib().sto_sppm_keep(capacity, demand)


def sppm_subs_of(count, share):
    return xlib().sto_sppm_subs_of(count, share)


def sppm_oct(v):
    return xlib().sto_sppm_oct(ptr(np.asarray(v, np.float32)))


def sppm_unoct(w):
    o = np.zeros(3, np.float32)
    xlib().sto_sppm_unoct(w, ptr(o))
    return o


LT_G = 128
LT_N = LT_G * LT_G


def lt_build(sent, stored):
    """The learned emission map's rebuild (prog_lt_build, wavefront.js:628-711) on the given counts: (sent/2,
    stored/2, the CDF: LT_N conditional row entries, then LT_G rows)."""
    e = np.array(sent, np.uint32).copy()
    h = np.array(stored, np.uint32).copy()
    cdf = np.zeros(LT_N + LT_G, np.float32)
    xlib().sto_lt_build(ptr(e), ptr(h), ptr(cdf))
    return e, h, cdf


def last_lt():
    """The emission map as the last render with it on left it: (sent, stored, CDF)."""
    e = np.zeros(LT_N, np.uint32)
    h = np.zeros(LT_N, np.uint32)
    cdf = np.zeros(LT_N + LT_G, np.float32)
    if xlib().sto_last_lt(ptr(e), ptr(h), ptr(cdf)) != 0:
        raise RuntimeError("no render with the learned emission map has run")
    return e, h, cdf


def last_lt_counts(width, height):
    """Light tracing's connections that reached each pixel over the last render call, (height, width)."""
    out = np.zeros(width * height, np.uint32)
    if xlib().sto_last_lt_counts(ptr(out), width * height) != 0:
        raise RuntimeError("no render of this size has run")
    return out.reshape(height, width)


def sppm_build(pos, power, nrm_oct, flags, cell):
    pos = np.ascontiguousarray(pos, np.float32)
    power = np.ascontiguousarray(power, np.float32)
    nrm_oct = np.ascontiguousarray(nrm_oct, np.uint32)
    flags = np.ascontiguousarray(flags, np.uint32)
    n = len(flags)
    key = np.zeros(n, np.uint32)
    cnt = np.zeros(1 << 20, np.uint32)
    xlib().sto_sppm_build(ptr(pos), ptr(power), ptr(nrm_oct), ptr(flags), n, cell, ptr(key), ptr(cnt))
    return key, cnt


def sppm_gather(qpos, qnrm, qalb, qb, radius, maxbounce, budget, seed):
    qpos = np.ascontiguousarray(qpos, np.float32)
    qnrm = np.ascontiguousarray(qnrm, np.float32)
    qalb = np.ascontiguousarray(qalb, np.float32)
    qb = np.ascontiguousarray(qb, np.uint32)
    m = len(qb)
    out = np.zeros((m, 3), np.float64)
    vis = np.zeros(m, np.uint32)
    cut = np.zeros(m, np.uint32)
    xlib().sto_sppm_gather(ptr(qpos), ptr(qnrm), ptr(qalb), ptr(qb), m, radius, maxbounce, budget, seed, ptr(out),
                           ptr(vis), ptr(cut))
    return out, vis, cut


def step_moments(state, x, window=float("inf")):
    """One resolve step of a pixel's luminance moments; state = [Y, V, S, cnt] (numpy float64, updated in place)."""
    xlib().sto_step_moments(ptr(state), x, window)
    return state


def standard_error(V, S):
    """sqrt(S V / (1 - S)), None where it is unknown (measure.js:46-51)."""
    if not (0 < S < 1) or V < 0:
        return None
    return float(np.sqrt(S * V / (1 - S)))


def sppm_photons(scene, sample=0, lo=(-1e9, -1e9, -1e9), hi=(1e9, 1e9, 1e9)):
    """One sample's photon pass alone: (records stored, their power summed over the box lo..hi)."""
    out = np.zeros(4, np.float64)
    xlib().sto_sppm_photons(C.byref(scene.desc), C.byref(scene.params), sample, ptr(np.asarray(lo, np.float32)),
                            ptr(np.asarray(hi, np.float32)), ptr(out))
    return int(out[0]), out[1:]


# ---- dispersion (st_oracle_spectral.h) ----
def cauchy_n(nd, vd, lam):
    return xlib().sto_cauchy_n(nd, vd, lam)


def lambda_code(lam):
    return xlib().sto_lambda_code(lam)


def lambda_of(code):
    return xlib().sto_lambda_of(code)


def spec_table():
    cdf = np.zeros(400, np.float32)
    col = np.zeros((400, 3), np.float32)
    xlib().sto_spec_table(ptr(cdf), ptr(col))
    return cdf, col


def spec_draw(u):
    w = np.zeros(3, np.float64)
    lam = xlib().sto_spec_draw(u, ptr(w))
    return lam, w


# ---- haze and the far field ----
def haze_span(scene, A, d, length, R):
    t = np.zeros(2, np.float64)
    xlib().sto_haze_span(C.byref(scene.desc), ptr(np.asarray(A, np.float64)), ptr(np.asarray(d, np.float64)),
                         length, R, ptr(t))
    return t


def hg_eval(c, g):
    return xlib().sto_hg_eval(c, g)


def hg_sample(g, d, seed, n):
    out = np.zeros((n, 3), np.float64)
    xlib().sto_hg_sample(g, ptr(np.asarray(d, np.float64)), seed, n, ptr(out))
    return out


def far_bin(d, axis, c0, nC, nG):
    f = lambda v: ptr(np.asarray(v, np.float32))
    return xlib().sto_far_bin(f(d), f(axis), f(c0), nC, nG)


def far_geometry(nC, nG):
    o = np.zeros(nG, np.float64)
    xlib().sto_far_geometry(nC, nG, ptr(o))
    return o


def far_intensity(flux, nC, nG):
    flux = np.ascontiguousarray(flux, np.float64).reshape(-1)
    I = np.zeros(nG * nC, np.float64)
    xlib().sto_far_intensity(ptr(flux), nC, nG, ptr(I))
    return I.reshape(nG, nC)


def optics_set_rays(rays):
    """The ray table the ray-set sources of the oracle's optics runs that follow read (N x 8); None clears it."""
    if rays is None:
        xlib().sto_optics_set_rays(None, 0)
        return
    r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    xlib().sto_optics_set_rays(ptr(r), len(r))


def optics_run(bench, ray_counts, nC=360, nG=181, cells=0, half=1.0, height=1.0, maxbounce=32, seed=1, fp64=False,
               threads=0, axis=(0, 0, 1), c0=(1, 0, 0)):
    """The optics trace on the CPU: `bench` a scenes.optics_bench scene; each instance traced against its own
    primitives (flags >> 8), its rays seeded as the GPU's are."""
    from shadytracer_gb300 import scenes as S
    n = len(ray_counts)
    per = []
    for i in range(n):
        prims = [p for p in bench.prim_list if (p.flags >> 8) == i]
        per.append(S.Scene(prims, bench.material_list, env_radius=bench.desc.env_radius,
                           tolerance=bench.desc.tolerance, name="instance"))
    ptrs = (C.c_void_p * n)(*[C.cast(C.byref(s.desc), C.c_void_p) for s in per])
    srcs = bench.info["sources"]
    from shadytracer_gb300.st_types import StOpticsSource
    sarr = (StOpticsSource * len(srcs))(*srcs)
    rc = np.ascontiguousarray(ray_counts, np.uint32)
    frames = np.zeros((n, 12), np.float32)
    for i in range(n):
        s0 = [s for s in srcs if s.instance == i][0]
        frames[i, 0:3] = list(s0.centre)
        frames[i, 3:6] = axis
        frames[i, 6:9] = c0
    far = np.zeros((n, nG, nC), np.float64)
    lux = np.zeros((n, max(cells, 1), max(cells, 1)), np.float64)
    tot = np.zeros((n, 6), np.float64)
    xlib().sto_optics_run(ptrs, C.byref(bench.params), C.cast(sarr, C.c_void_p), len(srcs), ptr(rc), n, ptr(frames),
                          nC, nG, cells, half, height, maxbounce, seed, 1 if fp64 else 0, ptr(far), ptr(lux), ptr(tot),
                          threads)
    keys = ["emitted", "escaped", "lost", "detected", "absorbed", "interactions"]
    out = {"far": far, "lux": lux, "totals": [dict(zip(keys, t.tolist())) for t in tot], "scenes": per, "detail": []}
    # per instance: the tallies by its own primitives' items (tag = the item's first primitive in the instance) and
    # by material (incident, leaving, interactions), the ray counts, the detector hits
    for i in range(n):
        npr, nm = per[i].desc.n_prims, per[i].desc.n_materials
        tag = np.zeros((npr, 3))
        mat = np.zeros((nm, 3))
        cnt = np.zeros(4, np.uint64)
        nh = C.c_uint32()
        if xlib().sto_optics_detail(i, ptr(tag), ptr(mat), ptr(cnt), None, 0, C.byref(nh)) != 0:
            out["detail"].append(None)
            continue
        hits = np.zeros((nh.value, 12), np.float32)
        xlib().sto_optics_detail(i, None, None, None, ptr(hits), nh.value, C.byref(nh))
        out["detail"].append({"tag": tag, "mat": mat, "hits": hits,
                              "counts": dict(zip(["n_escaped", "n_lost", "n_detected", "n_absorbed"],
                                                 [int(c) for c in cnt]))})
    return out


# ---- the learned proposal (st_oracle_guide.h) ----
GUIDE_NW = 13824
GUIDE_NPARAM = 13824 + 131072


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    return a if shape is None else a.reshape(shape)


def guide_forward(params, pos, nrm, box_lo, inv_ext, bf16=True):
    """The network's 40 outputs at n points (double), with BF16 rounding where the tensor cores take BF16 (bf16=True)
    or exact."""
    L = xlib()
    params, pos, nrm, lo = _f32(params), _f32(pos), _f32(nrm), _f32(box_lo)
    n = len(pos)
    raw = np.zeros((n, 40), np.float64)
    L.sto_guide_forward(ptr(params), n, ptr(pos), ptr(nrm), ptr(lo), inv_ext, int(bf16), ptr(raw))
    return raw


def guide_decode(raw):
    """Each point's mixture: 8 lobes x (mean direction xyz, kappa, weight), exact."""
    raw = np.ascontiguousarray(raw, np.float64)
    out = np.zeros((len(raw), 8, 5), np.float64)
    xlib().sto_guide_decode(ptr(raw), len(raw), ptr(out))
    return out


def guide_grad(params, pos, nrm, dirs, weight, box_lo, inv_ext, bf16=True):
    """(gradient of every parameter, summed loss) of the training loss at a batch."""
    L = xlib()
    a = [_f32(x) for x in (params, pos, nrm, dirs, weight, box_lo)]
    G = np.zeros(GUIDE_NPARAM, np.float64)
    loss = L.sto_guide_grad(ptr(a[0]), len(a[1]), ptr(a[1]), ptr(a[2]), ptr(a[3]), ptr(a[4]), ptr(a[5]), inv_ext,
                            int(bf16), ptr(G))
    return G, loss


def guide_loss(params, pos, nrm, dirs, weight, box_lo, inv_ext):
    L = xlib()
    a = [_f32(x) for x in (params, pos, nrm, dirs, weight, box_lo)]
    return L.sto_guide_loss(ptr(a[0]), len(a[1]), ptr(a[1]), ptr(a[2]), ptr(a[3]), ptr(a[4]), ptr(a[5]), inv_ext)


def guide_mix_pdf(mix, d):
    mix = np.ascontiguousarray(mix, np.float64)
    d = np.ascontiguousarray(d, np.float64)
    return xlib().sto_guide_mix_pdf(ptr(mix), ptr(d))


def guide_mix_sample(mix, u):
    mix = np.ascontiguousarray(mix, np.float64)
    u = np.ascontiguousarray(u, np.float64)
    d = np.zeros((len(u), 3), np.float64)
    xlib().sto_guide_mix_sample(ptr(mix), ptr(u), len(u), ptr(d))
    return d


def bf16(x):
    return xlib().sto_bf16(float(x))
