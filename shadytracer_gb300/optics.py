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
        self.detail = T.StOpticsDetail()
        self.n_instances = 0

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

    def set_spectra(self, spectra):
        """The spectra a source may name (st_optics_source.spectrum, 1-based): rows of ST_SPECTRUM_NODES values at 1 nm
        from 360 nm, any scale."""
        a = np.ascontiguousarray(np.asarray(spectra, np.float32).reshape(-1, 471))
        check(self.L.st_optics_set_spectra(self.rt.ctx, a.ctypes.data_as(C.c_void_p), len(a)), self.rt.ctx,
              "st_optics_set_spectra")
        self.spectra = a

    def run(self, ray_counts, lux_cells=512, lux_half=1.0, lux_height=1.0, maxbounce=32, seed=1, spectral=0):
        n = len(ray_counts)
        rc = (C.c_uint32 * n)(*[int(x) for x in ray_counts])
        b = T.StOpticsBatch()
        b.n_instances = n
        b.ray_count = C.cast(rc, C.POINTER(C.c_uint32))
        b.lux_cells, b.lux_half, b.lux_height = lux_cells, lux_half, lux_height
        b.maxbounce, b.seed, b.spectral = maxbounce, seed, int(spectral)
        nG, nC = self.far.nG, self.far.nC
        far = np.zeros((n, nG, nC), np.float64)
        lux = np.zeros((n, lux_cells, lux_cells), np.float64)
        tot = (T.StOpticsTotals * n)()
        P = C.c_void_p
        check(self.L.st_optics_run(self.rt.ctx, C.byref(b), far.ctypes.data_as(P), lux.ctypes.data_as(P), tot),
              self.rt.ctx, "st_optics_run")
        totals = [{f: getattr(tot[i], f) for f, _ in T.StOpticsTotals._fields_} for i in range(n)]
        self.n_instances = n
        return {"far": far, "lux": lux, "totals": totals}

    def autotune(self, ray_counts, lux_cells=512, lux_half=1.0, lux_height=1.0, maxbounce=32, seed=1):
        """The optics autotuner (st_optics_autotune): the batch run with each queue tile and march chunk, the fastest
        kept for the runs that follow. Returns {claim, chunk, ms, ms_default}."""
        n = len(ray_counts)
        rc = (C.c_uint32 * n)(*[int(x) for x in ray_counts])
        b = T.StOpticsBatch()
        b.n_instances = n
        b.ray_count = C.cast(rc, C.POINTER(C.c_uint32))
        b.lux_cells, b.lux_half, b.lux_height = lux_cells, lux_half, lux_height
        b.maxbounce, b.seed = maxbounce, seed
        t = T.StTune()
        check(self.L.st_optics_autotune(self.rt.ctx, C.byref(b), C.byref(t)), self.rt.ctx, "st_optics_autotune")
        return {f: getattr(t, f) for f, _ in T.StTune._fields_}

    def set_detail(self, det_cap=0, path_rays=0, path_verts=0, esc_len=0.0):
        """What a run keeps beyond its tallies (st_optics_set_detail): up to det_cap detector hits, and the paths of
        each instance's first path_rays rays, path_verts vertices each, an escaped ray's last esc_len metres on."""
        d = T.StOpticsDetail()
        d.det_cap, d.path_rays, d.path_verts, d.esc_len = det_cap, path_rays, path_verts, esc_len
        check(self.L.st_optics_set_detail(self.rt.ctx, C.byref(d)), self.rt.ctx, "st_optics_set_detail")
        self.detail = d

    def tallies(self):
        """The last run's tallies by object and by material (kernels.js O_TAG / O_MAT): tags (256, 3) and mats
        (instances, materials, 3), each row weight incident, weight leaving, interactions. A tag is an item of the
        table, by its first primitive's index."""
        nm = self.rt.scene.desc.n_materials
        tags = np.zeros((256, 3))
        mats = np.zeros((self.n_instances, nm, 3))
        P = C.c_void_p
        check(self.L.st_optics_tallies(self.rt.ctx, tags.ctypes.data_as(P), mats.ctypes.data_as(P)), self.rt.ctx,
              "st_optics_tallies")
        return tags, mats

    def hits(self, max_n=None):
        """The last run's detector hits (optRecordHit): an (n, 12) array -- position, weight, direction, tag, instance,
        CIE X, Z, 0 -- and how many reached a detector in all (past det_cap they were not kept)."""
        n = C.c_uint32()
        check(self.L.st_optics_hits(self.rt.ctx, None, 0, C.byref(n)), self.rt.ctx, "st_optics_hits")
        k = min(n.value, self.detail.det_cap if max_n is None else max_n)
        out = np.zeros((k, 12), np.float32)
        check(self.L.st_optics_hits(self.rt.ctx, out.ctypes.data_as(C.c_void_p), k, C.byref(n)), self.rt.ctx,
              "st_optics_hits")
        return out, n.value

    def paths(self):
        """The last run's kept paths (optVertex): counts (instances, path_rays) and verts (instances, path_rays,
        path_verts, 8): position, weight, optical length, hue rgb."""
        d = self.detail
        counts = np.zeros((self.n_instances, d.path_rays), np.uint32)
        verts = np.zeros((self.n_instances, d.path_rays, d.path_verts, 8), np.float32)
        P = C.c_void_p
        check(self.L.st_optics_paths(self.rt.ctx, verts.ctypes.data_as(P), counts.ctypes.data_as(P)), self.rt.ctx,
              "st_optics_paths")
        return verts, counts


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


# ---------------------------------------------------------------------------------------------------------------
# THE DETECTOR MAP (optics/detmap.js:104-213 mapFrame / detectorMap / smoothMap): the recorded detector hits as an
# illuminance map, in FP64 on the host. The plane is fitted to the hits (the principal axes of their positions; within
# about a degree of a world axis, squared up to the other two); square cells over the hits' extent (`cells` along the
# longer side); each cell the flux that landed in it over its area in square metres. Smoothing: 'none' (the
# histogram), 'gauss' or 'epan' (kernel density estimates whose kernel is normalised over the cells each hit reaches,
# so each hit deposits exactly its flux; bandwidth in cells), 'knn' (the photon-map estimate at each cell centre: the
# k nearest hits' flux over the disc they fill, the reach capped at KNN_MAX_CELLS).
# ---------------------------------------------------------------------------------------------------------------
KNN_MAX_CELLS = 16


def map_frame(pos, cells=64, rng=None):
    """The plane of the hits and their in-plane coordinates: (centre, u, v, normal, ab, a0, a1, b0, b1, size, nx,
    ny, flatness), or None for fewer than 3 hits."""
    pos = np.asarray(pos, np.float64)
    n = len(pos)
    if n < 3:
        return None
    c = pos.mean(0)
    d = pos - c
    cov = d.T @ d / n
    w, V = np.linalg.eigh(cov)                       # ascending: the normal is the direction they spread least along
    order = np.argsort(w)[::-1]
    w, V = w[order], V[:, order]
    u, v, nrm = V[:, 0], V[:, 1], V[:, 2]
    k = int(np.argmax(np.abs(nrm)))
    if abs(nrm[k]) > 0.9998:                         # a floor, a wall: squared up to the world's axes
        i, j = [q for q in range(3) if q != k]
        u, v, nrm = np.eye(3)[i], np.eye(3)[j], np.eye(3)[k]
    ab = np.stack([d @ u, d @ v], 1)
    a0, a1 = ab[:, 0].min(), ab[:, 0].max()
    b0, b1 = ab[:, 1].min(), ab[:, 1].max()
    if rng is not None:
        (a0, a1), (b0, b1) = rng
    span = max(a1 - a0, b1 - b0) or 1e-9
    size = span / max(1, int(cells))
    nx = max(1, int(math.ceil((a1 - a0) / size - 1e-9)))
    ny = max(1, int(math.ceil((b1 - b0) / size - 1e-9)))
    return {"c": c, "u": u, "v": v, "normal": nrm, "ab": ab, "a0": a0, "a1": a1, "b0": b0, "b1": b1, "size": size,
            "nx": nx, "ny": ny, "flatness": math.sqrt(max(w[2], 0.0)) / span}


def detector_map(pos, flux, cells=64, metres_per_unit=1.0, smooth="none", bandwidth=1.5, k=32, rng=None):
    """The illuminance map of hits at `pos` (n x 3) carrying `flux` (n, lm): a dict with E (ny x nx, lx), the hits'
    count per cell, the frame, and the statistics detmap.js reports (total, max, meanLit, minLit, uniformity,
    hitsPerLitCell, relNoise)."""
    F = map_frame(pos, cells, rng)
    if F is None:
        return None
    flux = np.asarray(flux, np.float64)
    ab, a0, a1, b0, b1, size, nx, ny = F["ab"], F["a0"], F["a1"], F["b0"], F["b1"], F["size"], F["nx"], F["ny"]
    inr = (ab[:, 0] >= a0) & (ab[:, 0] <= a1) & (ab[:, 1] >= b0) & (ab[:, 1] <= b1)
    cx = np.minimum(nx - 1, np.floor((ab[:, 0] - a0) / size).astype(int))
    cy = np.minimum(ny - 1, np.floor((ab[:, 1] - b0) / size).astype(int))
    fl = np.zeros((ny, nx))
    cnt = np.zeros((ny, nx), np.int64)
    np.add.at(fl, (cy[inr], cx[inr]), flux[inr])
    np.add.at(cnt, (cy[inr], cx[inr]), 1)
    m2 = metres_per_unit * metres_per_unit
    area = size * size * m2
    h = max(0.1, float(bandwidth))
    if smooth == "none":
        E = fl / area
    elif smooth in ("gauss", "epan"):
        E = np.zeros((ny, nx))
        hs = h * size
        reach = 3 * h if smooth == "gauss" else h
        R = int(math.ceil(reach)) + 1
        for i in np.nonzero(inr)[0]:
            a, b = ab[i]
            x0, y0 = cx[i], cy[i]
            ys = np.arange(max(0, y0 - R), min(ny - 1, y0 + R) + 1)
            xs = np.arange(max(0, x0 - R), min(nx - 1, x0 + R) + 1)
            db = (b0 + (ys + 0.5) * size - b) / hs
            da = (a0 + (xs + 0.5) * size - a) / hs
            r2 = db[:, None] ** 2 + da[None, :] ** 2
            wk = np.where(r2 < 9, np.exp(-0.5 * r2), 0.0) if smooth == "gauss" else np.where(r2 < 1, 1 - r2, 0.0)
            ws = wk.sum()
            f = flux[i] / area
            if not ws > 0:
                E[y0, x0] += f
            else:
                E[np.ix_(ys, xs)] += f * wk / ws
    elif smooth == "knn":
        E = np.zeros((ny, nx))
        kk = max(1, int(k))
        bins = {}
        for i in np.nonzero(inr)[0]:
            bins.setdefault((cy[i], cx[i]), []).append(i)
        for y in range(ny):
            for x in range(nx):
                ca, cb = a0 + (x + 0.5) * size, b0 + (y + 0.5) * size
                r, got = 0, cnt[y, x]
                while got < kk and r < KNN_MAX_CELLS:
                    r += 1
                    ring = 0
                    for yy in range(y - r, y + r + 1):
                        if yy < 0 or yy >= ny:
                            continue
                        for xx in (range(x - r, x + r + 1) if abs(yy - y) == r else (x - r, x + r)):
                            if 0 <= xx < nx:
                                ring += cnt[yy, xx]
                    got += ring
                if got < kk:
                    continue
                Rr = min(int(math.ceil((r + 0.5) * math.sqrt(2))), KNN_MAX_CELLS * 2)
                idx = [i for yy in range(max(0, y - Rr), min(ny - 1, y + Rr) + 1)
                       for xx in range(max(0, x - Rr), min(nx - 1, x + Rr) + 1) for i in bins.get((yy, xx), ())]
                idx = np.array(idx)
                d2 = (ab[idx, 0] - ca) ** 2 + (ab[idx, 1] - cb) ** 2
                order = np.argsort(d2, kind="stable")[:kk]
                rk2 = d2[order[-1]]
                if rk2 > 0:
                    E[y, x] = flux[idx[order]].sum() / (math.pi * rk2 * m2)
    else:
        raise ValueError("smooth: none, gauss, epan or knn")
    lit = cnt > 0
    inside = int(inr.sum())
    hpc = inside / lit.sum() if lit.any() else 0.0
    rel = None
    if hpc:
        rel = 1 / math.sqrt(kk) if smooth == "knn" else 1 / math.sqrt(
            hpc * (4 * math.pi * h * h if smooth == "gauss" else 0.75 * math.pi * h * h if smooth == "epan" else 1))
    meanLit = float(E[lit].mean()) if lit.any() else 0.0
    minLit = float(E[lit].min()) if lit.any() else 0.0
    return {"E": E, "count": cnt, "frame": F, "total": float(flux[inr].sum()), "max": float(E.max()),
            "meanLit": meanLit, "minLit": minLit, "uniformity": minLit / meanLit if meanLit > 0 else None,
            "litCells": int(lit.sum()), "hitsPerLitCell": hpc, "relNoise": rel, "cell_m": size * metres_per_unit}
