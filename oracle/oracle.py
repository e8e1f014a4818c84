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
           "st_oracle_optics.h", "st_oracle_api2.cpp", "../include/shadytracer.h"]

_lib = None


def build(force=False):
    """Compile the oracle if a source is newer than the library. Returns the library's path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return LIB
    cpp = [os.path.join(HERE, s) for s in ("st_oracle.cpp", "st_oracle_api2.cpp") if os.path.exists(os.path.join(HERE, s))]
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


def render(scene, nsamples, accum=None, fp64=False, threads=0, sample0=None, path_first=0, path_count=0):
    """Trace `nsamples` samples of `scene` (a shadytracer_gb300.scenes.Scene) into `accum` (made if None)."""
    L = lib()
    p = scene.params
    if accum is None:
        accum = Accum(p.width, p.height)
    s0 = accum.next_sample if sample0 is None else sample0
    rc = L.sto_render(C.byref(scene.desc), C.byref(p), C.byref(scene.view), s0, nsamples, 1 if fp64 else 0,
                      ptr(accum.rgb), ptr(accum.V), ptr(accum.S), ptr(accum.count), ptr(accum.counters), threads,
                      path_first, path_count)
    if rc != 0:
        raise RuntimeError("sto_render failed: %d" % rc)
    accum.next_sample = s0 + nsamples
    return accum


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
