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

    def set_rays(self, rays):
        """The ray table the ray-set sources (shape 3) read: N x 8 floats -- position (m), weight, direction, wavelength
        (nm) -- as ray_set_rays gives them (optics/sources.js RAYSET_VEC4)."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        check(self.L.st_optics_set_rays(self.rt.ctx, r.ctypes.data_as(C.c_void_p), len(r)), self.rt.ctx,
              "st_optics_set_rays")
        self.rays = r

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


# ------------------------------------------------------------------------------------------------------------
# ZEMAX SOURCE FILES (optics/zemax.js): ray sets as LED makers publish them, and the rays a ray-set source draws.
# ------------------------------------------------------------------------------------------------------------
ZEMAX_HEADER_BYTES = 208
ZEMAX_UNITS = {0: ("m", 1.0), 1: ("in", 0.0254), 2: ("cm", 0.01), 3: ("ft", 0.3048), 4: ("mm", 0.001)}


def _rot_xyz(rx, ry, rz):
    """Rotations about x, then y, then z (radians), as one matrix (zemax.js: the builder's own convention)."""
    cx, sx, cy, sy, cz, sz = math.cos(rx), math.sin(rx), math.cos(ry), math.sin(ry), math.cos(rz), math.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def parse_zemax(data):
    """A Zemax OpticStudio source file (zemax.js parseZemax): the 208-byte little-endian header -- identifier, count,
    description, source and ray-set flux, wavelength, the angles, the length unit, the placement, the ray format (0
    flux only: x y z l m n flux; 2 spectral: + wavelength), the flux unit -- then the rays. Returns (header, rays), rays
    N x 8 float32 (x, y, z in metres with the file's own placement applied, flux, l, m, n unit, wavelength in nm or 0).
    Raises ValueError, saying why, for a file it cannot read honestly (a length that disagrees with the header's count
    and format, an unknown unit or format)."""
    import struct
    b = bytes(data)
    if len(b) < ZEMAX_HEADER_BYTES:
        raise ValueError("not a Zemax source file: %d bytes, the header alone is %d" % (len(b), ZEMAX_HEADER_BYTES))
    identifier, count = struct.unpack_from("<iI", b, 0)
    desc = b[8:108].split(b"\0", 1)[0].decode("latin-1")
    source_flux, rayset_flux, wavelength, inc0, inc1, az0, az1 = struct.unpack_from("<7f", b, 108)
    (units,) = struct.unpack_from("<i", b, 136)
    loc = struct.unpack_from("<3f", b, 140)
    rot = struct.unpack_from("<3f", b, 152)
    fmt, flux_type = struct.unpack_from("<ii", b, 192)
    if units not in ZEMAX_UNITS:
        raise ValueError("unknown length unit %d" % units)
    if fmt not in (0, 2):
        raise ValueError("unknown ray format %d (0 flux only, 2 spectral)" % fmt)
    nf = 7 if fmt == 0 else 8
    if len(b) != ZEMAX_HEADER_BYTES + count * nf * 4:
        raise ValueError("%d bytes for %d rays of %d floats: the file and its header disagree" % (len(b), count, nf))
    raw = np.frombuffer(b, "<f4", count * nf, ZEMAX_HEADER_BYTES).reshape(count, nf).astype(np.float64)
    m = ZEMAX_UNITS[units][1]
    R = _rot_xyz(*rot)
    pos = (raw[:, 0:3] @ R.T + np.array(loc)) * m
    d = raw[:, 3:6] @ R.T
    d /= np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-30)
    rays = np.zeros((count, 8), np.float32)
    rays[:, 0:3] = pos
    rays[:, 3] = raw[:, 6]
    rays[:, 4:7] = d
    rays[:, 7] = raw[:, 7] * 1000.0 if fmt == 2 else (wavelength * 1000.0 if wavelength > 0 else 0.0)
    header = {"identifier": identifier, "count": count, "description": desc, "source_flux": source_flux,
              "rayset_flux": rayset_flux, "wavelength_um": wavelength, "units": ZEMAX_UNITS[units][0],
              "loc": loc, "rot": rot, "rotated": any(abs(x) > 0 for x in rot), "format": fmt,
              "flux_type": "lm" if flux_type == 1 else "W"}
    return header, rays


def ray_set_rays(rays, origin=(0.0, 0.0, 0.0), rot=None):
    """A file's rays placed in the scene (sources.js placeRays): turned by `rot` (3 x 3, optional) and moved to
    `origin`, each ray's weight its flux over the set's mean (sources.js RAYSET_VEC4)."""
    r = np.array(rays, np.float64, copy=True)
    if rot is not None:
        R = np.asarray(rot, np.float64)
        r[:, 0:3] = r[:, 0:3] @ R.T
        r[:, 4:7] = r[:, 4:7] @ R.T
    r[:, 0:3] += np.asarray(origin, np.float64)
    mean = r[:, 3].mean() if len(r) else 1.0
    r[:, 3] = r[:, 3] / (mean if mean > 0 else 1.0)
    return r.astype(np.float32)


def ray_set_source(first, count, flux, instance=0, emit_n=1.0):
    """A ray-set source (shape 3) of `flux` lumens over rays [first, first + count) of the ray table."""
    s = T.StOpticsSource()
    s.shape, s.flux, s.instance, s.emit_n = 3, flux, instance, emit_n
    s.axis[2] = 1.0
    s.tangent[0] = 1.0
    s.ray_first, s.ray_count = first, count
    return s
