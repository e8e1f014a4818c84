"""The optics bench: the reference's createOptics(RT, WG) -> O (optics/index.js:92) over the C ABI, and the host's FP64
reductions of its tallies (optics/farfield.js intensity, optics/illum.js the lux plane).

    O = Optics(rt)                      # rt: a PathTracer holding the batch's scene (every instance's primitives)
    O.set_sources([...])                # O.setSources: StOpticsSource records, each naming its instance
    O.set_far(nC=360, nG=181)           # O.setFar: the (C, gamma) grid, type C about +z from +x
    r = O.run(ray_counts, lux_cells=512, lux_half=1.0, lux_height=1.0)
    I = intensity(r["far"][i], 360, 181, flux_per_ray)        # cd per bin
    E = lux(r["lux"][i], 512, 1.0, flux_per_ray)               # lx per cell

A batch runs every instance in one launch chain on the GPU (csrc/st_optics.cu); the tallies come back in ray weight
(a ray starts at 1) and the host scales them by each instance's flux over its ray count, as the reference's host does.
"""
import ctypes as C
import math

import numpy as np

from . import st_types as T
from ._lib import check


class Optics:
    def __init__(self, rt):
        self.rt = rt
        self.L = rt.L
        self.sources = []
        self.far = None

    def set_sources(self, sources):
        arr = (T.StOpticsSource * max(1, len(sources)))(*sources)
        check(self.L.st_optics_set_sources(self.rt.ctx, arr, len(sources)), self.rt.ctx, "st_optics_set_sources")
        self.sources = list(sources)

    def set_far(self, nC=360, nG=181, axis=(0.0, 0.0, 1.0), c0=(1.0, 0.0, 0.0)):
        f = T.StOpticsFar()
        f.nC, f.nG = nC, nG
        for i in range(3):
            f.axis[i] = axis[i]
            f.c0[i] = c0[i]
        check(self.L.st_optics_set_far(self.rt.ctx, C.byref(f)), self.rt.ctx, "st_optics_set_far")
        self.far = f

    def run(self, ray_counts, lux_cells=512, lux_half=1.0, lux_height=1.0, maxbounce=32, seed=1):
        n = len(ray_counts)
        rc = (C.c_uint32 * n)(*[int(x) for x in ray_counts])
        b = T.StOpticsBatch()
        b.n_instances = n
        b.ray_count = C.cast(rc, C.POINTER(C.c_uint32))
        b.lux_cells, b.lux_half, b.lux_height = lux_cells, lux_half, lux_height
        b.maxbounce, b.seed = maxbounce, seed
        nG, nC = self.far.nG, self.far.nC
        far = np.zeros((n, nG, nC), np.float64)
        lux = np.zeros((n, lux_cells, lux_cells), np.float64)
        tot = (T.StOpticsTotals * n)()
        P = C.c_void_p
        check(self.L.st_optics_run(self.rt.ctx, C.byref(b), far.ctypes.data_as(P), lux.ctypes.data_as(P), tot),
              self.rt.ctx, "st_optics_run")
        totals = [{f: getattr(tot[i], f) for f, _ in T.StOpticsTotals._fields_} for i in range(n)]
        return {"far": far, "lux": lux, "totals": totals}


def far_geometry(nC, nG):
    """Each gamma row's solid angle per C bin (farfield.js:33-41): dC (cos lo - cos hi), the end rows half as wide."""
    dG = 180.0 / (nG - 1)
    j = np.arange(nG, dtype=np.float64)
    lo = np.radians(np.maximum(0.0, (j - 0.5) * dG))
    hi = np.radians(np.minimum(180.0, (j + 0.5) * dG))
    return (2 * math.pi / nC) * (np.cos(lo) - np.cos(hi))


def intensity(far, nC, nG, scale=1.0):
    """Luminous intensity per bin (farfield.js:63-85, symmetry 'none'): flux over the bin's solid angle, the caps at
    the poles pooled over every C. `far` is (nG, nC) in ray weight; `scale` the flux a unit of weight carries (lm)."""
    far = np.asarray(far, np.float64).reshape(nG, nC) * scale
    om = far_geometry(nC, nG)
    I = far / om[:, None]
    for j in (0, nG - 1):
        I[j, :] = far[j].sum() / (om[j] * nC)
    return I


def lux(tally, cells, half, scale=1.0):
    """The lux map: the flux that crossed each cell of the plane over the cell's area (lm / m^2 = lx)."""
    cell = 2.0 * half / cells
    return np.asarray(tally, np.float64).reshape(cells, cells) * scale / (cell * cell)


def virtual_plane(I, nC, nG, h=1.0, half=1.0, cells=64):
    """The far field on a plane square to the axis, h metres off, the luminaire a point (illum.js:206-248
    virtualPlane): E = I(gamma, C) cos^3(gamma) / h^2, I bilinear on the grid (C wraps)."""
    dC, dG = 360.0 / nC, 180.0 / (nG - 1)
    cell = 2 * half / cells
    c = -half + (np.arange(cells) + 0.5) * cell
    a, b = np.meshgrid(c, c)
    rho = np.hypot(a, b)
    cg = h / np.hypot(h, rho)
    gamma = np.degrees(np.arctan2(rho, h))
    Cd = np.degrees(np.arctan2(b, a)) % 360
    g = np.clip(gamma, 0, 180) / dG
    j0 = np.minimum(nG - 1, np.floor(g).astype(int))
    j1 = np.minimum(nG - 1, j0 + 1)
    tg = g - np.floor(g)
    x = Cd / dC
    i0 = np.floor(x).astype(int) % nC
    i1 = (i0 + 1) % nC
    tc = x - np.floor(x)
    v = lambda j: I[j, i0] * (1 - tc) + I[j, i1] * tc
    Ig = v(j0) * (1 - tg) + v(j1) * tg
    return Ig * cg ** 3 / (h * h)
