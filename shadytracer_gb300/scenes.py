"""The workloads, as scene tables: the scene-as-data form of the reference's scene contract.

A scene here is what the reference's builder generates (builder/codegen.js:974-1060 generate -> an SDF and a
getMaterial2) written as data: a table of primitives folded the way core/scene_api.js:28-80 folds them, and a
material table (core/materials.js:12-60 Material2, the fields the hot path reads). Material 0 is the air.

Each builder returns a `Scene` holding the ctypes arrays (kept alive here) and the st_scene_desc that points
at them, plus the st_params and st_view of its workload.
"""
import ctypes as C
import math

import numpy as np

from .st_types import (StPrim, StMaterial, StSceneDesc, StView, StLight, default_params, ST_ENV_SUNSKY,
                       ST_LIGHT_DISC, ST_LIGHT_RECTANGLE, ST_LIGHT_COSINE, ST_LIGHT_UNIFORM,
                       ST_PRIM_PLANE, ST_PRIM_SPHERE, ST_PRIM_BOX, ST_PRIM_ROUNDBOX, ST_PRIM_TORUS,
                       ST_PRIM_PRISM, ST_PRIM_ASPHERE, ST_PRIM_CYLINDER,
                       ST_OP_ITEM, ST_OP_SMOOTH, ST_OP_UNION, ST_OP_SUB)

IDENTITY = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)


class Scene:
    def __init__(self, prims, materials, env_radius=400.0, tolerance=0.0, haze=None, name="scene", lights=()):
        self.name = name
        self.light_list = list(lights)
        self.prim_list = list(prims)
        self.material_list = list(materials)
        self.prims = (StPrim * len(prims))(*prims)
        self.materials = (StMaterial * len(materials))(*materials)
        d = StSceneDesc()
        d.prims = C.cast(self.prims, C.POINTER(StPrim))
        d.n_prims = len(prims)
        d.materials = C.cast(self.materials, C.POINTER(StMaterial))
        d.n_materials = len(materials)
        d.env_radius = env_radius
        d.tolerance = tolerance
        for i in range(9):
            d.haze_axes[i] = IDENTITY[i]
        if haze:
            for i in range(3):
                d.haze_centre[i] = haze["centre"][i]
                d.haze_half[i] = haze["half"][i]
                d.haze_albedo[i] = haze.get("albedo", (1.0, 1.0, 1.0))[i]
            d.haze_sigma_t = haze["sigma_t"]
            d.haze_g = haze.get("g", 0.0)
            if "axes" in haze:
                for i in range(9):
                    d.haze_axes[i] = haze["axes"][i]
        if self.light_list:
            self.lights = (StLight * len(self.light_list))(*self.light_list)
            d.lights = C.cast(self.lights, C.POINTER(StLight))
            d.n_lights = len(self.light_list)
        self.desc = d
        self.params = None
        self.view = None
        self.info = {}


def flux_factor(dist=ST_LIGHT_COSINE, n=1.0, half_deg=90.0):
    """builder/lights.js fluxFactor: a face's flux per unit luminance straight out and unit area -- the integral of
    its beam's shape times cos over the cone: 2 pi (1 - c^(n+1)) / (n + 1) for cos^n, 2 pi (1 - c) for even
    intensity (c the cosine of the half angle)."""
    c = math.cos(math.radians(min(90.0, max(0.0, half_deg))))
    if dist == ST_LIGHT_UNIFORM:
        return 2 * math.pi * (1 - c)
    n = max(0.0, n)
    return 2 * math.pi * (1 - max(c, 0.0) ** (n + 1)) / (n + 1)


def light_face(centre, u, v, half_w, half_h=None, flux=None, le=None, colour=(1.0, 1.0, 1.0), material=1,
               dist=ST_LIGHT_COSINE, n=1.0, half_deg=90.0, shape=ST_LIGHT_RECTANGLE):
    """A light's face (the builder's light object): a rectangle (half_w x half_h about centre along the unit axes u,
    v) or a disc (radius half_w), emitting along u x v in a cos^n or even-intensity beam of half angle half_deg.
    Its luminance straight out is `le` (cd/m^2), or what puts `flux` lumens through the face: flux / (A k), k the
    beam's flux factor, coloured by `colour` at that luminance (lights.js, codegen's emissive / luminance)."""
    L = StLight()
    area = 4 * half_w * (half_h if half_h is not None else half_w) if shape == ST_LIGHT_RECTANGLE else math.pi * half_w ** 2
    if le is None:
        lum = flux / (area * flux_factor(dist, n, half_deg))
        y = 0.2126 * colour[0] + 0.7152 * colour[1] + 0.0722 * colour[2]
        le = [c / max(y, 1e-6) * lum for c in colour]
    for i in range(3):
        L.centre[i], L.u[i], L.v[i], L.le[i] = centre[i], u[i], v[i], le[i]
    L.shape = shape
    L.half_w = half_w
    L.half_h = half_h if half_h is not None else half_w
    L.material, L.dist, L.n = material, dist, n
    L.beam_cos = math.cos(math.radians(half_deg)) if half_deg < 90.0 else 0.0
    return L


def face_axes(axis):
    """Unit axes u, v of a face that emits along `axis` (u x v = axis)."""
    R = spot_rot([-c for c in axis])                  # its rows: local x, y and z = axis
    return R[0:3], R[3:6]


def prim(type_, pos=(0, 0, 0), params=(), material=1, op=ST_OP_ITEM, k=0.0, rot=IDENTITY, flags=0):
    p = StPrim()
    p.type, p.op, p.material, p.flags = type_, op, material, flags
    for i in range(3):
        p.pos[i] = pos[i]
    p.k = k
    for i in range(9):
        p.rot[i] = rot[i]
    for i, v in enumerate(params):
        p.p[i] = v
    return p


def material(base=(0.8, 0.8, 0.8), metallic=0.0, roughness=0.5, specular=0.5, specular_tint=0.0,
             transmission=0.0, ior=1.0, abbe=0.0, attenuation=0.0, detector=0.0, emissive=(0, 0, 0),
             scatter_distance=0.0, scatter_g=0.0):
    """makeDefaultMaterial's defaults (core/materials.js:170-191), then the fields given."""
    m = StMaterial()
    for i in range(3):
        m.base[i] = base[i]
        m.emissive[i] = emissive[i]
    m.metallic, m.roughness, m.specular, m.specular_tint = metallic, roughness, specular, specular_tint
    m.transmission, m.ior, m.abbe, m.attenuation, m.detector = transmission, ior, abbe, attenuation, detector
    m.coat_edge, m.coat_width, m.coat_index = 550.0, 0.0, 1.8          # read only where coat != 0
    m.scatter_distance, m.scatter_g = scatter_distance, scatter_g
    return m


COAT_NONE, COAT_AR_BACK, COAT_BARE_BACK, COAT_EVERY_FACE = 0, 1, 2, 3


def coated(m, where=COAT_AR_BACK, lo=0.0, hi=0.0, edge=600.0, width=20.0, index=1.8):
    """coatMaterial (core/materials.js:150-161): a coating put on material m -- R(lambda) from lo below `edge` (nm) to
    hi above it, a logistic of 10-90 % width `width` (nm), its edge moving with the angle through the stack's effective
    index; `where` the faces it is on (COAT_*). lo = hi is a beam splitter (no edge), 0 on every face a perfect AR."""
    m.coat = min(int(where), 3)
    m.coat_lo, m.coat_hi = min(max(lo, 0.0), 1.0), min(max(hi, 0.0), 1.0)
    m.coat_edge, m.coat_width, m.coat_index = edge, max(width, 0.0), max(index, 1.0)
    return m


def air():
    return material(base=(1, 1, 1), specular=0.0, ior=1.0)


def diffuse(c, roughness=1.0):
    """makeDiffuse (core/materials.js:197-207): a Lambertian of albedo c exactly, no coat."""
    return material(base=c, metallic=0.0, roughness=roughness, specular=0.0, transmission=0.0, ior=1.5)


def plastic(c, roughness, specular=0.5):
    """makePlastic (core/materials.js:220-229)."""
    return material(base=c, metallic=0.0, roughness=roughness, specular=specular, transmission=0.0, ior=1.5)


def metal(c, roughness):
    """makeMetal (core/materials.js:231-239)."""
    return material(base=c, metallic=1.0, roughness=roughness, specular=1.0, transmission=0.0)


def glass(c=(1, 1, 1), ior=1.5, roughness=0.0, abbe=0.0):
    """makeGlassSmooth / makeGlassRough (core/materials.js:241-256)."""
    return material(base=c, metallic=0.0, roughness=roughness, specular=0.5, transmission=1.0, ior=max(ior, 1.0),
                    abbe=abbe)


def look_at(eye, target, vfov_deg, aspect, up=(0.0, 0.0, 1.0)):
    """The camera as genrays reads it (core/genrays.js:65-92): right, up and fwd (target -> camera) from the
    view, fx = tan(fov/2) * aspect, fy = tan(fov/2)."""
    d = [target[i] - eye[i] for i in range(3)]
    ln = math.sqrt(sum(x * x for x in d))
    d = [x / ln for x in d]
    r = [d[1] * up[2] - d[2] * up[1], d[2] * up[0] - d[0] * up[2], d[0] * up[1] - d[1] * up[0]]
    ln = math.sqrt(sum(x * x for x in r))
    r = [x / ln for x in r]
    u = [r[1] * d[2] - r[2] * d[1], r[2] * d[0] - r[0] * d[2], r[0] * d[1] - r[1] * d[0]]
    v = StView()
    for i in range(3):
        v.cam_pos[i] = eye[i]
        v.right[i] = r[i]
        v.up[i] = u[i]
        v.fwd[i] = -d[i]
    fy = math.tan(math.radians(vfov_deg) / 2)
    v.fy = fy
    v.fx = fy * aspect
    v.camtype = 0
    return v


def rot_from_quat(q):
    """World -> local rotation (row major) of the unit quaternion q = (w, x, y, z): the transpose of its matrix."""
    w, x, y, z = q
    m = [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]
    return (m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8])


class Pcg32:
    """PCG32 (O'Neill 2014, XSH RR 64/32), the seeded generator the room's primitives are drawn from."""

    def __init__(self, seed, seq=54):
        self.state = 0
        self.inc = ((seq << 1) | 1) & 0xFFFFFFFFFFFFFFFF
        self.next_u32()
        self.state = (self.state + seed) & 0xFFFFFFFFFFFFFFFF
        self.next_u32()

    def next_u32(self):
        old = self.state
        self.state = (old * 6364136223846793005 + self.inc) & 0xFFFFFFFFFFFFFFFF
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * (self.next_u32() / 4294967296.0)


# ---------------------------------------------------------------------------------------------------------------
# The photometry row (lib/pathtracer/tests.js:447-509): a white floor under a uniform environment.
# ---------------------------------------------------------------------------------------------------------------
def floor_furnace(width=256, height=256, spp=16, albedo=0.8, sky=1000.0, maxbounce=4, seed=1):
    """An infinite Lambertian floor (reflectance `albedo`, the plane z = 0) under a uniform environment of `sky`
    cd/m^2, a pinhole camera 1 m above it looking 30 degrees down (vertical field 70 degrees). Closed form: every
    floor pixel is albedo * sky, every sky pixel sky."""
    s = Scene([prim(ST_PRIM_PLANE, material=1)], [air(), diffuse((albedo, albedo, albedo))], name="floor")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, env_uniform=sky, sun_hint=0,
                              seed=seed)
    pitch = math.radians(30.0)
    eye = (0.0, 0.0, 1.0)
    target = (0.0, math.cos(pitch), 1.0 - math.sin(pitch))
    s.view = look_at(eye, target, 70.0, width / height)
    s.info = {"spp": spp, "closed_form_floor": albedo * sky, "closed_form_sky": sky, "workload": "floor-256"}
    return s


def floor_sky(width=64, height=64, env_mode=1, albedo=0.8, sun_elevation=45.0, sun_outside=128000.0, turbidity=0.7,
              studio_illuminance=10000.0, studio_top=0.5, maxbounce=4, seed=1):
    """The floor of floor_furnace under one of the environment's presets (environment.js): env_mode 1 the sun and sky
    physically (sunlight of `sun_outside` lux above the air, `turbidity`), 2 the studio (`studio_illuminance` lux on a
    level surface, brighter above by `studio_top`). The floor's closed form is albedo / pi times the illuminance the
    environment puts on it: the studio's by its construction; the sun and sky's integrated from its radiance."""
    s = floor_furnace(width=width, height=height, albedo=albedo, maxbounce=maxbounce, seed=seed)
    s.params.env_uniform = 0.0
    s.params.sun_hint = 1
    s.params.env_mode = env_mode
    s.params.sun_elevation = sun_elevation
    s.params.sun_azimuth = 0.0
    s.params.sun_outside = sun_outside
    s.params.sky_turbidity = turbidity
    s.params.studio_illuminance = studio_illuminance
    s.params.studio_top = studio_top
    for i in range(3):
        s.params.studio_color[i] = 1.0
    s.info = {"albedo": albedo, "workload": "floor-sky"}
    return s


def sky_illuminance(radiance, sun_elevation, sun_azimuth=0.0, sun_diameter=0.53, nz=400, nphi=800):
    """What an environment puts on a level surface facing up, lux: its sun's disc at normal incidence times
    sin(elevation), plus its sky over the upper hemisphere (midpoint rule in z and azimuth), the disc left out of that.
    `radiance(dirs)` gives rgb at n x 3 unit directions. Returns (sun at normal incidence, sun on the level, sky)."""
    luma = np.array([0.2126, 0.7152, 0.0722])
    e, a = math.radians(sun_elevation), math.radians(sun_azimuth)
    sun = np.array([math.cos(e) * math.sin(a), math.cos(e) * math.cos(a), math.sin(e)])
    half = math.radians(sun_diameter / 2)
    omega = 2 * math.pi * (1 - math.cos(half))
    e_sun = float(radiance(sun[None])[0] @ luma) * omega
    z = (np.arange(nz) + 0.5) / nz
    ph = (np.arange(nphi) + 0.5) / nphi * 2 * math.pi
    Z, PH = np.meshgrid(z, ph, indexing="ij")
    R = np.sqrt(1 - Z * Z)
    d = np.stack([R * np.cos(PH), R * np.sin(PH), Z], -1).reshape(-1, 3)
    L = radiance(d) @ luma
    L[(d @ sun) > math.cos(half)] = 0.0
    e_sky = float((L * d[:, 2]).sum() / nz * (2 * math.pi / nphi))
    return e_sun, e_sun * max(math.sin(e), 0.0), e_sky


def emitter(le, beam_deg=0.0):
    """makeEmissive (core/materials.js:263-268): emitted luminance `le` (cd/m^2, rgb), air beyond; beam_deg > 0
    limits the emission to a cone of that half angle about the surface's outward normal (a cosine light's beam,
    builder/lights.js beamShape)."""
    m = material(base=(0, 0, 0), specular=0.0, ior=1.0, emissive=le)
    m.beam_cos = math.cos(math.radians(beam_deg)) if beam_deg > 0 else 0.0
    return m


def spot_luminance(flux_lm, area_m2, half_deg):
    """A face's luminance straight out for `flux_lm` lumens into a cone of `half_deg` (builder/lights.js fluxFactor, a
    cosine light, n = 1: flux = L A pi sin^2(half))."""
    return flux_lm / (area_m2 * math.pi * math.sin(math.radians(half_deg)) ** 2)


def spot_rot(axis):
    """The world -> local rotation (row major) of a thin lamp whose lower face (local -z) looks along `axis`: its rows
    are the local axes in world coordinates, z = -axis."""
    n = math.sqrt(sum(x * x for x in axis))
    z = [-x / n for x in axis]
    h = (0.0, 1.0, 0.0) if abs(z[1]) < 0.9 else (1.0, 0.0, 0.0)
    x = [h[1] * z[2] - h[2] * z[1], h[2] * z[0] - h[0] * z[2], h[0] * z[1] - h[1] * z[0]]
    n = math.sqrt(sum(c * c for c in x))
    x = [c / n for c in x]
    y = [z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]]
    return tuple(x) + tuple(y) + tuple(z)


def spot_floor(width=128, height=128, spp=64, flux=1000.0, half_deg=10.0, side=0.2, albedo=0.8, seed=1,
               light="emitter"):
    """A 10-degree spot of `flux` lumens -- a thin square lamp `side` x `side` m whose lower face emits into a cone of
    `half_deg` about its normal -- at (-1, 0, 1) aimed at the origin, over an infinite Lambertian floor in a black
    environment, seen straight down by an orthographic camera over 2 x 2 m about the origin. All the beam's flux lands
    on the floor, so pi / albedo times the floor's luminance summed over its area is the flux (the lamp's other faces
    light no floor in view). A lamp of 20 cm keeps the emitter list's first boxes -- bounds of the few points the
    camera found on it -- from leaving most of it to the BSDF's rare hits.
    light="face": the lamp is a light's face instead (one-sided, its flux set through fluxFactor), which light
    sampling aims at from the start."""
    le = spot_luminance(flux, side * side, half_deg)
    axis = (1.0, 0.0, -1.0)
    if light == "face":
        u, v = face_axes(axis)
        s = Scene([prim(ST_PRIM_PLANE, material=1)], [air(), diffuse((albedo, albedo, albedo)), diffuse((0, 0, 0))],
                  env_radius=20.0, name="spot-face-floor",
                  lights=[light_face((-1.0, 0.0, 1.0), u, v, side / 2, side / 2, flux=flux, material=2,
                                     half_deg=half_deg)])
    else:
        lamp = prim(ST_PRIM_BOX, pos=(-1.0, 0.0, 1.0), params=(side / 2, side / 2, 0.0005), material=2,
                    rot=spot_rot(axis))
        s = Scene([prim(ST_PRIM_PLANE, material=1), lamp],
                  [air(), diffuse((albedo, albedo, albedo)), emitter((le, le, le), beam_deg=half_deg)],
                  env_radius=20.0, name="spot-floor")
    s.params = default_params(width=width, height=height, maxbounce=2, sun_hint=0, sun_illuminance=0.0,
                              sky_luminance=0.0, ground_luminance=0.0, seed=seed, eps=1e-4)
    v = StView()
    for i, c in enumerate((0.0, 0.0, 3.0)):
        v.cam_pos[i] = c
    for i in range(3):
        v.right[i] = (1.0, 0.0, 0.0)[i]
        v.up[i] = (0.0, 1.0, 0.0)[i]
        v.fwd[i] = (0.0, 0.0, 1.0)[i]
    v.fx, v.fy, v.camtype = 1.0, 1.0, 1
    s.view = v
    s.info = {"spp": spp, "workload": "spot-floor", "flux": flux, "albedo": albedo, "pixel_area": 4.0 / (width * height)}
    return s


def haze_beam(width=1280, height=720, spp=256, sigma_s=0.2, g=0.7, flux=1000.0, half_deg=10.0, maxbounce=32, seed=1,
              light="face"):
    """The haze-box beam: a 2 x 2 x 4 m box of homogeneous haze (scattering sigma_s, absorbing nothing, HG g), crossed
    along its length by a 10-degree spot of 1000 lm -- a 5 cm square lamp 0.5 m below the box aiming up its axis -- in a
    black environment, seen from the side. The lamp is a light's face (light="face"): one-sided, aimed at by light
    sampling from the air. light="emitter": a thin box of one beam material instead, found by discovery, whose other
    faces emit too, each into its own cone."""
    side = 0.05
    le = spot_luminance(flux, side * side, half_deg)
    haze = {"centre": (0.0, 0.0, 2.0), "half": (1.0, 1.0, 2.0), "sigma_t": sigma_s, "g": g, "albedo": (1.0, 1.0, 1.0)}
    if light == "face":
        # a far floor below keeps the table of primitives from being empty; nothing of it is in view or lit
        s = Scene([prim(ST_PRIM_PLANE, pos=(0.0, 0.0, -100.0), material=2)], [air(), diffuse((0, 0, 0)),
                  diffuse((0, 0, 0))], env_radius=40.0, haze=haze, name="haze-beam",
                  lights=[light_face((0.0, 0.0, -0.5), (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), side / 2, side / 2, flux=flux,
                                     material=1, half_deg=half_deg)])
    else:
        lamp = prim(ST_PRIM_BOX, pos=(0.0, 0.0, -0.5), params=(side / 2, side / 2, 0.0005), material=1,
                    rot=spot_rot((0.0, 0.0, 1.0)))
        s = Scene([lamp], [air(), emitter((le, le, le), beam_deg=half_deg)], env_radius=40.0, haze=haze,
                  name="haze-beam")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_hint=0, sun_illuminance=0.0,
                              sky_luminance=0.0, ground_luminance=0.0, seed=seed, eps=1e-4)
    s.view = look_at((0.0, -7.0, 1.8), (0.0, 0.0, 1.8), 45.0, width / height)
    s.info = {"spp": spp, "workload": "haze-beam", "paths": width * height * spp}
    return s


def lamp_floor(width=96, height=64, spp=64, radius=0.1, lamp_height=1.0, le=1000.0, albedo=0.8, maxbounce=2,
               seed=1, haze_sigma_t=0.0, haze_g=0.0):
    """An emissive sphere of `radius` and luminance `le` (cd/m^2) at `lamp_height` over an infinite Lambertian floor
    (reflectance `albedo`) in a black environment. A sphere of uniform luminance lights a point it is wholly above as a
    point source of intensity pi a^2 Le at its centre, so a floor pixel's closed form is albedo Le a^2 h / D^3, D the
    distance to the centre (h = lamp_height); the floor cannot see itself, so any bounce cap of 1 or more keeps it.
    haze_sigma_t > 0 fills a 3 x 3 x 2 m box about the lamp with albedo-1 haze (no closed form then)."""
    s = Scene([prim(ST_PRIM_PLANE, material=1), prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, lamp_height), params=(radius,),
                                                      material=2)],
              [air(), diffuse((albedo, albedo, albedo)), emitter((le, le, le))], env_radius=20.0, name="lamp-floor",
              haze=None if haze_sigma_t <= 0 else {"centre": (0.0, 0.0, 1.0), "half": (1.5, 1.5, 1.0),
                                                   "sigma_t": haze_sigma_t, "g": haze_g, "albedo": (1.0, 1.0, 1.0)})
    # a march tolerance of 1e-4 m: a ray meets the lamp within the tolerance of its surface, so the lamp lights the
    # floor as a sphere that much larger (the scene's default, from its 20 m radius, would add 4 %)
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_hint=0, sun_illuminance=0.0,
                              sky_luminance=0.0, ground_luminance=0.0, seed=seed, eps=1e-4)
    eye = (0.0, -2.5, 2.0)
    target = (0.0, 0.6, 0.0)
    s.view = look_at(eye, target, 55.0, width / height)
    s.info = {"spp": spp, "workload": "lamp-floor", "lamp": (0.0, 0.0, lamp_height, radius, le), "albedo": albedo}
    return s


def lamp_floor_closed_form(scene, points):
    """The floor's luminance at floor points (n x 3, z = 0): albedo Le a^2 h / D^3."""
    import numpy as np
    cx, cy, cz, a, le = scene.info["lamp"]
    d = np.asarray(points, np.float64) - np.array([cx, cy, cz])
    D = np.linalg.norm(d, axis=-1)
    return scene.info["albedo"] * le * a * a * cz / D ** 3


def lamp_floor_pixels(scene):
    """Each pixel's closed form at its centre ray's floor point, and which pixels it holds for: the ray meets the
    floor within 8 m (a ray leaves the 20 m scene before it meets the floor farther out) and passes clear of the lamp."""
    import numpy as np
    W, H = scene.params.width, scene.params.height
    v = scene.view
    fwd, right, up, eye = [np.array(list(x), np.float64) for x in (v.fwd, v.right, v.up, v.cam_pos)]
    X, Y = np.meshgrid((np.arange(W) + 0.5) / W * 2 - 1, (np.arange(H) + 0.5) / H * 2 - 1)
    d = -fwd + right * (X[..., None] * v.fx) + up * (Y[..., None] * v.fy)
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    t = -eye[2] / d[..., 2]
    pts = eye + d * t[..., None]
    cx, cy, cz, a, le = scene.info["lamp"]
    oc = eye - np.array([cx, cy, cz])
    b = np.sum(d * oc, -1)
    clear = (b * b - (oc @ oc - (1.5 * a) ** 2)) <= 0
    near = np.linalg.norm(pts[..., :2], axis=-1) < 8.0
    return lamp_floor_closed_form(scene, pts), (t > 0) & clear & near


# ---------------------------------------------------------------------------------------------------------------
# The path-traced SDF room.
# ---------------------------------------------------------------------------------------------------------------
ROOM_HALF = (3.0, 2.0, 1.5)          # a 6 x 4 x 3 m room, floor at z = 0
ROOM_WALL = 0.1


def sdf_room(width=1920, height=1080, spp=64, maxbounce=8, seed=1, n_prims=24, prim_seed=2, finish="mixed",
             sky_illuminance=10000.0, ground_luminance=1000.0, sky="uniform"):
    """A 6 x 4 x 3 m room (its walls a hollow box 0.1 m thick, a 2 x 1.5 m window in the +y wall) holding
    `n_prims` primitives drawn from PCG32(prim_seed): types uniform over {box, sphere, torus, rounded prism}, sizes
    0.15-0.4 m, placed uniformly in the room, randomly turned, smooth-unioned in order with radii U(0.02, 0.1) m.
    Materials: roughness U(0.05, 1), albedo U(0.2, 0.9) per channel, 20 % metallic (the rest plastic). Lit by a
    100 klx sun (0.53 degrees, 35 degrees up) and a uniform sky of 10 klx on the level (3183 cd/m^2) through the
    window. March tolerance 1e-4 m. finish="diffuse": every object Lambertian of its drawn albedo (the same draws, the
    same geometry), so most of the room is lit by the light the sunlit floor and walls send on -- the learned
    proposal's workload; sky_illuminance and ground_luminance near 0 leave the sun's patch on the floor the room's only
    light after the sun itself. sky="physical": the environment's physical sun and sky preset instead (environment.js
    SUNSKY_FN, turbidity 0.7), its light above the air set so that the sun gives 100 klx at normal incidence."""
    rng = Pcg32(prim_seed)
    mats = [air(), diffuse((0.75, 0.73, 0.70))]
    hx, hy, hz = ROOM_HALF
    t = ROOM_WALL
    prims = [
        prim(ST_PRIM_BOX, pos=(0, 0, hz), params=(hx + t, hy + t, hz + t), material=1, op=ST_OP_ITEM),
        prim(ST_PRIM_BOX, pos=(0, 0, hz), params=(hx, hy, hz), material=1, op=ST_OP_SUB),
        prim(ST_PRIM_BOX, pos=(0.0, hy + t / 2, 1.65), params=(1.0, t, 0.75), material=1, op=ST_OP_SUB),
    ]
    kinds = [ST_PRIM_BOX, ST_PRIM_SPHERE, ST_PRIM_TORUS, ST_PRIM_PRISM]
    for i in range(n_prims):
        kind = kinds[min(3, int(rng.uniform() * 4))]
        size = rng.uniform(0.15, 0.4)
        pos = (rng.uniform(-hx + 0.5, hx - 0.5), rng.uniform(-hy + 0.5, hy - 0.5), rng.uniform(0.3, 2 * hz - 0.5))
        # a uniformly random rotation (Shoemake's quaternion from three uniforms)
        u1, u2, u3 = rng.uniform(), rng.uniform(), rng.uniform()
        q = (math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
             math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3))
        k = rng.uniform(0.02, 0.1)
        rough = rng.uniform(0.05, 1.0)
        albedo = (rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9))
        is_metal = rng.uniform() < 0.2
        if finish == "diffuse":
            mats.append(diffuse(albedo))
        else:
            mats.append(metal(albedo, rough) if is_metal else plastic(albedo, rough))
        if kind == ST_PRIM_BOX:
            params = (size, size * rng.uniform(0.5, 1.0), size * rng.uniform(0.5, 1.0))
        elif kind == ST_PRIM_SPHERE:
            params = (size,)
        elif kind == ST_PRIM_TORUS:
            params = (size, size * rng.uniform(0.2, 0.45))
        else:
            params = (float(3 + int(rng.uniform() * 4)), size, size * rng.uniform(0.8, 2.0), 0.02)
        prims.append(prim(kind, pos=pos, params=params, material=len(mats) - 1,
                          op=ST_OP_ITEM if i == 0 else ST_OP_SMOOTH, k=k, rot=rot_from_quat(q)))
    s = Scene(prims, mats, env_radius=20.0, name="room24" if finish == "mixed" else "room24-diffuse")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_elevation=35.0, sun_azimuth=20.0,
                              sun_illuminance=100000.0, sky_luminance=sky_illuminance / math.pi,
                              ground_luminance=ground_luminance,
                              eps=1e-4, seed=seed)
    eye = (-2.6, -1.6, 1.7)
    target = (0.8, 0.9, 1.1)
    s.view = look_at(eye, target, 60.0, width / height)
    s.info = {"spp": spp, "workload": "room24-1080p", "paths": width * height * spp}
    if sky == "physical":
        s.params.env_mode = ST_ENV_SUNSKY
        s.params.sky_turbidity = 0.7
        s.params.sun_outside = 100000.0 / sun_sky_transmittance(35.0, 0.7)
        s.info["sky"] = "physical sun and sky, 100 klx sun, turbidity 0.7"
    return s


def sun_sky_transmittance(elevation, turbidity):
    """The share of the light above the air that reaches the ground as the sun's disc in the physical sun and sky
    (environment.js SUNSKY_FN): sum over its 16 bands of each band's luminance share times exp(-tau m), m the
    Kasten-Young air mass at the sun's elevation, tau the band's Rayleigh, aerosol (0.05 + 0.1 turbidity at 550 nm,
    Angstrom 1.3) and ozone (300 DU) depths -- the bands as the library builds them (csrc/st_sky.h)."""
    sigma = (6.2648e-24, 3.1169e-23, 1.0195e-22, 2.4886e-22, 5.4883e-22, 1.1517e-21, 2.0211e-21, 3.0497e-21, 4.2480e-21,
             4.5252e-21, 4.7153e-21, 3.4726e-21, 2.3885e-21, 1.5936e-21, 9.8370e-22, 6.3061e-22)

    def lobe(l, mu, lo, hi):
        t = (l - mu) / (lo if l < mu else hi)
        return math.exp(-0.5 * t * t)
    c = math.sin(math.radians(elevation))
    m = 1.0 / (c + 0.15 * max(93.885 - (90.0 - elevation), 0.1) ** -1.253)
    aerosol = 0.05 + 0.1 * max(turbidity, 0.0)
    step, lum, trans = 350.0 / 16, [], []
    for k in range(16):
        X = Y = Z = wl = ws = 0.0
        l = 380.0 + k * step
        while l < 380.0 + (k + 1) * step:
            li, mm = round(l), l * 1e-9
            w = 1.0 / (mm ** 5 * (math.exp(1.438776877e-2 / (mm * 5778.0)) - 1.0))
            x = 1.056 * lobe(li, 599.8, 37.9, 31.0) + 0.362 * lobe(li, 442.0, 16.0, 26.7) - 0.065 * lobe(li, 501.1, 20.4, 26.2)
            y = 0.821 * lobe(li, 568.8, 46.9, 40.5) + 0.286 * lobe(li, 530.9, 16.3, 31.1)
            z = 1.217 * lobe(li, 437.0, 11.8, 36.0) + 0.681 * lobe(li, 459.0, 26.0, 13.8)
            X, Y, Z, wl, ws = X + w * x, Y + w * y, Z + w * z, wl + w * (x + y + z) * l, ws + w * (x + y + z)
            l += 1.0
        nm = wl / ws
        um = nm / 1000.0
        tau = (0.008569 * um ** -4 * (1 + 0.0113 * um ** -2 + 0.00013 * um ** -4) + aerosol * (nm / 550.0) ** -1.3 +
               sigma[k] * 300.0 * 2.6867e16)
        r = 3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z
        g = -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z
        b = 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z
        lum.append(0.2126 * r + 0.7152 * g + 0.0722 * b)
        trans.append(math.exp(-tau * m))
    return sum(a * t for a, t in zip(lum, trans)) / sum(lum)


# ---------------------------------------------------------------------------------------------------------------
# Dispersion (spectral.js cauchyN, lightspectra.js specDraw): the glass of the photon map's caustic.
# ---------------------------------------------------------------------------------------------------------------
def dispersive_furnace(width=64, height=64, ior=1.5168, abbe=40.0, sky=1000.0, maxbounce=16, seed=1, floor=False):
    """A clear glass sphere (r 0.3 m) of index `ior` at the d line and Abbe number `abbe` in a uniform environment of
    `sky` cd/m^2 (with `floor`, on a white Lambertian floor, albedo 0.7). Without the floor every pixel must read `sky`
    on average: the glass absorbs nothing, and the wavelength a refraction draws weighs each channel by 1 on average
    (spectral.js / lightspectra.js: the draw's colour over its chance)."""
    mats = [air(), glass((1.0, 1.0, 1.0), ior=ior, abbe=abbe), diffuse((0.7, 0.7, 0.7))]
    prims = [prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, 0.3 if floor else 1.0), params=(0.3,), material=1)]
    if floor:
        prims.append(prim(ST_PRIM_PLANE, material=2))
    s = Scene(prims, mats, env_radius=40.0, name="dispersive-furnace")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, env_uniform=sky, sun_hint=0, seed=seed)
    s.view = look_at((0.0, -1.6, 1.2 if floor else 1.0), (0.0, 0.0, 0.3 if floor else 1.0), 40.0, width / height)
    s.info = {"closed_form": None if floor else sky}
    return s


# ---------------------------------------------------------------------------------------------------------------
# The photon map (core/sppm.js) -- a caustic under glass, and its closed form through a pane.
# ---------------------------------------------------------------------------------------------------------------
def cauchy_glass(a=1.50, b_um2=0.0042):
    """n(lambda) = a + b / lambda^2 (lambda in um) as the reference's materials take it: n_d and the Abbe number V_d
    (spectral.js cauchyN goes through both)."""
    ld, lf, lc = 0.58756, 0.48613, 0.65627
    nd = a + b_um2 / ld ** 2
    vd = (nd - 1.0) / (b_um2 * (1 / lf ** 2 - 1 / lc ** 2))
    return nd, vd


def sppm_caustic(width=1024, height=1024, photons=4_000_000, r1=0.005, alpha=0.7, maxbounce=8, seed=1,
                 sun_elevation=50.0, sun_illuminance=100000.0, sky=3000.0, dispersion=True):
    """The caustic: a glass sphere (r 0.3 m, n(lambda) = 1.50 + 0.0042 / lambda^2 um) on a diffuse floor (albedo 0.7) under
    the sun and a sky; the photon map on: `photons` sun photons a sample over a 0.5 m square, first radius r1, alpha."""
    nd, vd = cauchy_glass()
    mats = [air(), glass((1.0, 1.0, 1.0), ior=nd, abbe=vd if dispersion else 0.0), diffuse((0.7, 0.7, 0.7))]
    prims = [prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, 0.3), params=(0.3,), material=1), prim(ST_PRIM_PLANE, material=2)]
    s = Scene(prims, mats, env_radius=20.0, name="sppm-caustic")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, seed=seed, sun_elevation=sun_elevation,
                              sun_azimuth=200.0, sun_illuminance=sun_illuminance, sky_luminance=sky,
                              ground_luminance=0.0, sppm=1, sppm_photons=photons, sppm_r1=r1, sppm_alpha=alpha,
                              sppm_half=0.5)
    s.view = look_at((1.2, -1.4, 1.3), (0.15, 0.3, 0.1), 45.0, width / height)
    s.info = {"workload": "sppm-caustic-%dx%d" % (width, height), "photons": photons}
    return s


def caustic_mask(scene, centre=(0.0, 0.0, 0.3), radius=0.3, grow=1.25):
    """The caustic's pixels: those whose centre's camera ray meets the floor (z = 0) before the sphere, at a point
    whose line to the sun passes within grow x radius of the sphere's centre -- the sphere's shadow on the floor,
    widened, where the glass focuses the sun. A boolean array of the picture's shape (row 0 the bottom)."""
    import numpy as np
    p, v = scene.params, scene.view
    W, H = p.width, p.height
    ux = (np.arange(W) + 0.5) / W
    uy = (np.arange(H) + 0.5) / H
    xx, yy = np.meshgrid(ux * 2 - 1, uy * 2 - 1)
    R, U, F = (np.array(list(v.right)), np.array(list(v.up)), np.array(list(v.fwd)))
    d = xx[..., None] * v.fx * R + yy[..., None] * v.fy * U - F
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    o = np.array(list(v.cam_pos))
    c = np.array(centre)
    t_floor = np.where(d[..., 2] < 0, -o[2] / np.minimum(d[..., 2], -1e-12), np.inf)
    oc = o - c                                          # the sphere first?
    b = (d * oc).sum(-1)
    disc = b * b - (oc @ oc - radius * radius)
    t_sph = np.where(disc > 0, -b - np.sqrt(np.maximum(disc, 0)), np.inf)
    seen = np.isfinite(t_floor) & ((t_sph <= 0) | (t_floor < t_sph))
    q = o + d * np.where(np.isfinite(t_floor), t_floor, 0)[..., None]
    e, az = math.radians(p.sun_elevation), math.radians(p.sun_azimuth)
    sun = np.array([math.cos(e) * math.sin(az), math.cos(e) * math.cos(az), math.sin(e)])
    w = q - c                                           # the line q + t sun's nearest approach to the centre
    dist2 = (w * w).sum(-1) - ((w * sun).sum(-1)) ** 2
    return seen & (dist2 <= (grow * radius) ** 2)


def sppm_pane(width=48, height=48, photons=400_000, r1=0.02, alpha=0.7, sun_elevation=60.0, ior=1.5, seed=1,
              pane_half=1.0, photon_half=1.6, vfov=12.0):
    """The photon map's closed form: a clear pane (2 x 2 m, 2 cm thick, index `ior`) 0.5 m over a white-ish floor
    (albedo 0.7) under the sun alone, seen from straight above through the pane's middle. The floor is a slab cut to
    the pane's shadow (the sun at 60 degrees from +y puts it at y in [-1.29, 0.71]), so it is lit only through the
    glass -- the map's light:
        L = T(view) rho / pi * E_sun sin(elevation) T(sun),  T = (1 - F) / (1 + F) for a slab (every inner
    reflection summed), F the dielectric Fresnel reflectance at the face's angle. (The light a floor inter-reflection
    through the pane's underside brings is neither side's: the map stores a photon at its first D only, and light
    sampling from the floor is blocked by the glass -- as in the reference.)"""
    mats = [air(), glass((1.0, 1.0, 1.0), ior=ior), diffuse((0.7, 0.7, 0.7))]
    h = pane_half
    off = 0.5 / math.tan(math.radians(sun_elevation))        # the shadow's shift away from the sun (+y)
    prims = [prim(ST_PRIM_BOX, pos=(0.0, 0.0, 0.5), params=(h, h, 0.01), material=1),
             prim(ST_PRIM_BOX, pos=(0.0, -off, -0.05), params=(h, h, 0.05), material=2)]
    s = Scene(prims, mats, env_radius=20.0, name="sppm-pane")
    # depth 5: the pane's two faces, the floor, the pane again -- no second floor vertex, so the floor-pane-floor
    # inter-reflection (light nobody's closed form counts, and a path tracer's rare hit of the sun) is cut
    s.params = default_params(width=width, height=height, maxbounce=5, seed=seed, sun_elevation=sun_elevation,
                              sun_azimuth=0.0, sun_illuminance=100000.0, sky_luminance=0.0, ground_luminance=0.0,
                              sppm=1, sppm_photons=photons, sppm_r1=r1, sppm_alpha=alpha, sppm_half=photon_half)
    s.view = look_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), vfov, width / height, up=(0.0, 1.0, 0.0))
    s.info = {"ior": ior, "albedo": 0.7, "sun_elevation": sun_elevation, "E_sun": 100000.0}
    return s


def sppm_pane_closed_form(scene, fresnel):
    """The pane's radiance, T(view) rho / pi E_sun sin(elevation) T(sun); `fresnel(cos_i, eta)` the dielectric
    Fresnel reflectance (the caller's: the oracle's, in the tests)."""
    i = scene.info
    ior, el = i["ior"], i["sun_elevation"]
    Fv = fresnel(1.0, 1.0 / ior)
    Fs = fresnel(math.cos(math.radians(90.0 - el)), 1.0 / ior)
    return (1 - Fv) / (1 + Fv) * i["albedo"] / math.pi * i["E_sun"] * math.sin(math.radians(el)) * (1 - Fs) / (1 + Fs)


def lt_pane(width=64, height=48, photons=400_000, sun_elevation=60.0, ior=1.5, seed=1, pane_z=1.0, photon_half=1.6,
            lens_radius=0.0, sppm=0, vfov=40.0):
    """Light tracing's closed form: the pane of sppm_pane (2 x 2 m, 2 cm thick), `pane_z` over a floor (albedo 0.7)
    cut to its shadow under the sun alone, now seen DIRECTLY from the side, from under the pane: the class
    light -> delta+ -> D -> eye, which light tracing owns. With the depth cap at 3 (the pane's two faces, the floor)
    the photons that reach the floor have crossed each face once, so
        L = rho / pi * E_sun sin(elevation) (1 - F)^2,  F the dielectric Fresnel reflectance at the sun's angle
    (the camera's paths keep only the sky, which is black). `lens_radius` puts a thin lens focused on the floor's
    middle in front of the camera."""
    mats = [air(), glass((1.0, 1.0, 1.0), ior=ior), diffuse((0.7, 0.7, 0.7))]
    off = pane_z / math.tan(math.radians(sun_elevation))      # the shadow's shift away from the sun (+y)
    prims = [prim(ST_PRIM_BOX, pos=(0.0, 0.0, pane_z), params=(1.0, 1.0, 0.01), material=1),
             prim(ST_PRIM_BOX, pos=(0.0, -off, -0.05), params=(1.0, 1.0, 0.05), material=2)]
    s = Scene(prims, mats, env_radius=20.0, name="lt-pane")
    s.params = default_params(width=width, height=height, maxbounce=3, seed=seed, sun_elevation=sun_elevation,
                              sun_azimuth=0.0, sun_illuminance=100000.0, sky_luminance=0.0, ground_luminance=0.0,
                              lt=1, lt_photons=photons, sppm=sppm, sppm_photons=photons, sppm_half=photon_half)
    eye, target = (-2.0, -off, 0.8 * pane_z), (0.3, -off, 0.0)
    s.view = look_at(eye, target, vfov, width / height)
    if lens_radius > 0:
        s.view.lens_radius = lens_radius
        s.view.focus_distance = math.dist(eye, target)
    s.info = {"ior": ior, "albedo": 0.7, "sun_elevation": sun_elevation, "E_sun": 100000.0, "eye": eye,
              "floor": (-1.0, 1.0, -1.0 - off, 1.0 - off)}
    return s


def lt_lamp(width=64, height=48, photons=400_000, le=20000.0, radius=0.1, lamp_height=1.2, pane_z=0.8, ior=1.5,
            albedo=0.7, seed=1):
    """Light tracing's emitter photons: a glowing sphere (`radius`, luminance `le`) above a clear pane (3 x 3 m, 2 mm
    thick, `pane_z` up) over a floor (albedo) in the dark, the floor seen from the side from under the pane. The
    floor under the pane is lit only through the glass: the lamp's light sampling is blocked by it, and a camera path
    that meets the lamp through it is in light tracing's class -- the emitter photons' (the probes' from the third
    sample on, once the lamp is listed). A sphere of uniform luminance lights a point wholly below it as a point of
    intensity pi a^2 Le at its centre, and a thin slab turns no ray, so within a depth cap of 3 (the faces, the floor)
        L = albedo Le a^2 h / D^3 (1 - F)^2,  F at the line's angle to the pane."""
    mats = [air(), glass((1.0, 1.0, 1.0), ior=ior), diffuse((albedo, albedo, albedo)), emitter((le, le, le))]
    prims = [prim(ST_PRIM_PLANE, material=2),
             prim(ST_PRIM_BOX, pos=(0.0, 0.0, pane_z), params=(1.5, 1.5, 0.001), material=1),
             prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, lamp_height), params=(radius,), material=3)]
    s = Scene(prims, mats, env_radius=20.0, name="lt-lamp")
    s.params = default_params(width=width, height=height, maxbounce=3, seed=seed, sun_hint=0, sun_illuminance=0.0,
                              sky_luminance=0.0, ground_luminance=0.0, lt=1, lt_photons=photons, eps=1e-4)
    s.view = look_at((-1.4, -0.2, 0.6), (0.2, 0.1, 0.0), 50.0, width / height)
    s.info = {"ior": ior, "albedo": albedo, "le": le, "radius": radius, "lamp_height": lamp_height}
    return s


def lt_lamp_closed_form(scene, fresnel):
    """lt_lamp's floor, per pixel (its centre's ray; 0 where it misses the floor under the pane, 1 m in)."""
    v, p, i = scene.view, scene.params, scene.info
    W, H = p.width, p.height
    xx, yy = np.meshgrid((np.arange(W) + 0.5) / W * 2 - 1, (np.arange(H) + 0.5) / H * 2 - 1)
    right, up, fwd = (np.array([getattr(v, k)[j] for j in range(3)]) for k in ("right", "up", "fwd"))
    cam = np.array([v.cam_pos[j] for j in range(3)])
    d = right * (xx[..., None] * v.fx) + up * (yy[..., None] * v.fy) - fwd
    t = np.where(d[..., 2] < 0, -cam[2] / np.minimum(d[..., 2], -1e-12), np.inf)
    x = cam + d * np.where(np.isfinite(t), t, 0.0)[..., None]
    lamp = np.array([0.0, 0.0, i["lamp_height"]])
    D = np.linalg.norm(lamp - x, axis=-1)
    cos = i["lamp_height"] / D
    F = np.vectorize(lambda c: fresnel(c, 1.0 / i["ior"]))(cos)
    L = i["albedo"] * i["le"] * i["radius"] ** 2 * i["lamp_height"] / D ** 3 * (1 - F) ** 2
    under = np.isfinite(t) & (np.abs(x[..., 0]) < 1.0) & (np.abs(x[..., 1]) < 1.0)
    return np.where(under, L, 0.0)


def lt_pane_closed_form(scene, fresnel):
    """The floor's radiance in lt_pane, rho / pi E_sun sin(elevation) (1 - F)^2; `fresnel(cos_i, eta)` the
    caller's dielectric Fresnel reflectance."""
    i = scene.info
    el = i["sun_elevation"]
    F = fresnel(math.cos(math.radians(90.0 - el)), 1.0 / i["ior"])
    return i["albedo"] / math.pi * i["E_sun"] * math.sin(math.radians(el)) * (1 - F) ** 2


def lt_haze(width=48, height=36, photons=400_000, pane=True, sun_elevation=60.0, ior=1.5, sigma_t=0.3, g=0.5, seed=1,
            photon_half=2.0):
    """Light tracing in the haze (haze.js:404-460 ltConnectMedium): a box of haze (1 x 1 x 0.6 m, albedo 1, HG g)
    under a clear pane (3 x 3 m, 2 cm thick, 1 m up) that the sun lights it through, seen from the side from under the
    pane. A parallel slab turns no ray, so the haze is lit as without the pane times (1 - F)^2 (each face crossed once,
    within a depth cap of 3: the faces, one collision): the single scattering light tracing's connections carry
    (pane=True) is (1 - F)^2 that of the camera's light samples with the pane gone and a cap of 1 (pane=False). A
    black sky, no floor: a far dark plane keeps the table from being empty."""
    mats = [air(), glass((1.0, 1.0, 1.0), ior=ior), diffuse((0.0, 0.0, 0.0))]
    off = 1.0 / math.tan(math.radians(sun_elevation))
    prims = [prim(ST_PRIM_PLANE, pos=(0.0, 0.0, -50.0), material=2)]
    if pane:
        prims.append(prim(ST_PRIM_BOX, pos=(0.0, 0.0, 1.0), params=(1.5, 1.5, 0.01), material=1))
    haze = {"centre": (0.0, -off * 0.6, 0.4), "half": (0.5, 0.5, 0.3), "sigma_t": sigma_t, "g": g,
            "albedo": (1.0, 1.0, 1.0)}
    s = Scene(prims, mats, env_radius=20.0, haze=haze, name="lt-haze")
    s.params = default_params(width=width, height=height, maxbounce=3 if pane else 1, seed=seed,
                              sun_elevation=sun_elevation, sun_azimuth=0.0, sun_illuminance=100000.0,
                              sky_luminance=0.0, ground_luminance=0.0, lt=1 if pane else 0, lt_photons=photons,
                              sppm_half=photon_half, eps=1e-4)
    s.view = look_at((-2.5, -off * 0.6, 0.4), (0.0, -off * 0.6, 0.4), 30.0, width / height)
    s.info = {"ior": ior, "sun_elevation": sun_elevation}
    return s


def lt_haze_single_scatter(scene, fresnel, n_t=4000):
    """lt_haze's closed form, by quadrature along each pixel's centre ray: the sun's single-scattered light in the box,
    sum over t of sigma_t p_HG(s . d) E_sun (1 - F)^2 exp(-sigma_t (t - t0)) exp(-sigma_t l_sun) dt (albedo 1), l_sun
    the way out of the box toward the sun; (H, W), 0 where the ray misses the box."""
    d, p, v = scene.desc, scene.params, scene.view
    c = np.array([d.haze_centre[i] for i in range(3)])
    h = np.array([d.haze_half[i] for i in range(3)])
    sig, g = d.haze_sigma_t, d.haze_g
    el, az = math.radians(p.sun_elevation), math.radians(p.sun_azimuth)
    sun = np.array([math.sin(az) * math.cos(el), math.cos(az) * math.cos(el), math.sin(el)])
    F = fresnel(math.cos(math.radians(90.0) - el), 1.0 / scene.info["ior"])
    W, H = p.width, p.height
    xx, yy = np.meshgrid((np.arange(W) + 0.5) / W * 2 - 1, (np.arange(H) + 0.5) / H * 2 - 1)
    right, up, fwd = (np.array([getattr(v, k)[i] for i in range(3)]) for k in ("right", "up", "fwd"))
    cam = np.array([v.cam_pos[i] for i in range(3)])
    rd = right * (xx[..., None] * v.fx) + up * (yy[..., None] * v.fy) - fwd
    rd /= np.linalg.norm(rd, axis=-1, keepdims=True)

    def chord(o, dd):                                                 # the slab intersection [t0, t1] of o + dd t
        with np.errstate(divide="ignore", invalid="ignore"):
            a = (c - h - o) / dd
            b = (c + h - o) / dd
        t0 = np.nanmax(np.minimum(a, b), axis=-1)
        t1 = np.nanmin(np.maximum(a, b), axis=-1)
        return np.maximum(t0, 0.0), t1

    t0, t1 = chord(cam, rd)
    out = np.zeros((H, W))
    hit = t1 > t0
    cos = rd @ sun
    ph = (1 - g * g) / (4 * math.pi * (1 + g * g - 2 * g * cos) ** 1.5)
    for iy, ix in zip(*np.nonzero(hit)):
        ts = np.linspace(t0[iy, ix], t1[iy, ix], n_t + 1)
        tm = 0.5 * (ts[1:] + ts[:-1])
        x = cam + rd[iy, ix] * tm[:, None]
        _, ls = chord(x, np.broadcast_to(sun, x.shape))               # the way out toward the sun, from inside
        integrand = sig * np.exp(-sig * (tm - t0[iy, ix])) * np.exp(-sig * ls)
        out[iy, ix] = ph[iy, ix] * float(np.sum(integrand) * (ts[1] - ts[0]))
    return out * p.sun_illuminance * (1 - F) ** 2


def floor_mask(scene, margin=0.1):
    """The pixels whose centre's ray meets the floor's top (z = 0) inside its rectangle, `margin` metres in."""
    v, p = scene.view, scene.params
    W, H = p.width, p.height
    x0, x1, y0, y1 = scene.info["floor"]
    cam = [v.cam_pos[i] for i in range(3)]
    mask = [[False] * W for _ in range(H)]
    for py in range(H):
        for px in range(W):
            xx, yy = (px + 0.5) / W * 2 - 1, (py + 0.5) / H * 2 - 1
            d = [v.right[i] * xx * v.fx + v.up[i] * yy * v.fy - v.fwd[i] for i in range(3)]
            if d[2] >= -1e-6:
                continue
            t = -cam[2] / d[2]
            x, y = cam[0] + t * d[0], cam[1] + t * d[1]
            mask[py][px] = x0 + margin < x < x1 - margin and y0 + margin < y < y1 - margin
    return mask


# ---------------------------------------------------------------------------------------------------------------
# The haze box (lib/pathtracer/tests.js:1818-1866 'haze' row; core/haze.js).
# ---------------------------------------------------------------------------------------------------------------
def haze_furnace(width=64, height=64, sigma_t=0.2, g=0.0, albedo=1.0, sky=1000.0, maxbounce=32, seed=1):
    """The haze row's furnace: an albedo-1 haze box (2 x 2 x 4 m) in a uniform environment with nothing else in
    it but a far-away dark plane the camera never sees -- every pixel must read `sky` exactly, whatever sigma_t and
    g (energy conservation: what the dust scatters out of a camera ray it scatters back in)."""
    s = Scene([prim(ST_PRIM_PLANE, pos=(0, 0, -50.0), material=1)], [air(), diffuse((1.0, 1.0, 1.0))],
              env_radius=40.0,
              haze={"centre": (0.0, 0.0, 2.0), "half": (1.0, 1.0, 2.0), "sigma_t": sigma_t, "g": g,
                    "albedo": (albedo, albedo, albedo)}, name="haze-furnace")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, env_uniform=sky, sun_hint=0, seed=seed)
    s.view = look_at((0.0, -6.0, 2.0), (0.0, 0.0, 2.0), 50.0, width / height)
    s.info = {"closed_form": sky}
    return s


# ---------------------------------------------------------------------------------------------------------------
# The batched optics bench (optics/index.js; the reference's aspheric condenser, scenes/aspheric-condenser.json)
# ---------------------------------------------------------------------------------------------------------------
MM = 1e-3


def led_lens_instance(inst, k1, a4_mm, a6_mm, mats_ids=(1, 2), ior=1.49):
    """One emitter + lens: a 1 x 1 x 0.2 mm die (its top face at z = 0) under a plano-convex aspheric lens (6 mm
    across, 2.5 mm thick, front radius 3.2 mm, conic k1, 4th/6th coefficients a4, a6 given in mm^-3, mm^-5), its flat
    back 0.5 mm above the die. Primitives flagged with the instance (flags >> 8)."""
    die = prim(ST_PRIM_BOX, pos=(0, 0, -0.1 * MM), params=(0.5 * MM, 0.5 * MM, 0.1 * MM), material=mats_ids[0],
               flags=inst << 8)
    t, D, R1 = 2.5 * MM, 6.0 * MM, 3.2 * MM
    lens = prim(ST_PRIM_ASPHERE, pos=(0, 0, 0.5 * MM + t / 2),
                params=(D, t, R1, k1, a4_mm * 1e9, a6_mm * 1e15, 0.0, 0.0, 0.0, 0.0), material=mats_ids[1],
                flags=inst << 8)
    return [die, lens]


def led_source(inst, flux=1.0):
    """The die's top face as a Lambertian source (cos^1 over the hemisphere), 1 x 1 mm, stepped off its sheet."""
    s = __import__("shadytracer_gb300.st_types", fromlist=["StOpticsSource"]).StOpticsSource()
    for i, v in enumerate((0.0, 0.0, 0.0)):
        s.centre[i] = v
    s.flux = flux
    for i, v in enumerate((0.0, 0.0, 1.0)):
        s.axis[i] = v
    for i, v in enumerate((1.0, 0.0, 0.0)):
        s.tangent[i] = v
    s.shape = 2
    s.size_x = s.size_y = 0.5 * MM
    s.dist = 2
    s.cos_half = 0.0
    s.n_exp = 1.0
    s.emit_n = 1.0
    s.two_sided = 0
    s.on_surface = 1
    s.instance = inst
    return s


def optics_bench(n_instances=64, seed=5, ray_min=1e5, ray_max=1e7, ray_scale=1.0):
    """The batched optics bench: n instances of led_lens_instance with k1 ~ U(-1.5, 0), a4, a6 ~ U(-1e-3, 1e-3)
    (mm units) and IOR 1.49, each with its die's source and a ray count log-uniform in [ray_min, ray_max] (times
    ray_scale), all drawn from PCG32(seed). Far field 1 x 1 degree (360 x 181 bins), lux 512 x 512 at 1 m."""
    rng = Pcg32(seed)
    mats = [air(), diffuse((0.5, 0.5, 0.5)), glass((1, 1, 1), ior=1.49)]
    prims, srcs, rays, lenses = [], [], [], []
    for i in range(n_instances):
        k1 = rng.uniform(-1.5, 0.0)
        a4 = rng.uniform(-1e-3, 1e-3)
        a6 = rng.uniform(-1e-3, 1e-3)
        n = math.exp(rng.uniform(math.log(ray_min), math.log(ray_max)))
        prims += led_lens_instance(i, k1, a4, a6)
        srcs.append(led_source(i))
        rays.append(max(1, int(n * ray_scale)))
        lenses.append({"k1": k1, "a4_mm": a4, "a6_mm": a6})
    s = Scene(prims, mats, env_radius=0.02, tolerance=1e-6, name="optics-bench")
    s.params = default_params(width=16, height=16, maxbounce=32)
    s.view = look_at((0, -0.05, 0.01), (0, 0, 0.002), 30.0, 1.0)
    s.info = {"sources": srcs, "rays": rays, "lenses": lenses, "nC": 360, "nG": 181, "lux_cells": 512,
              "lux_half": 1.0, "lux_height": 1.0, "workload": "optics-bench-%d" % n_instances}
    return s


def optics_detector_bench(n_instances=2, seed=5, height=0.02, radius=0.015, rays=200_000):
    """The optics bench's emitter + lens instances, each with a detector above it (optics/kernels.js optIsDetector): a
    thin disc of radius `radius` at `height` over the die, of a detector material, so the trace records the hits that
    reach it (optRecordHit) and tallies them by object and by material."""
    rng = Pcg32(seed)
    det = material(base=(1, 1, 1), detector=1.0)
    mats = [air(), diffuse((0.5, 0.5, 0.5)), glass((1, 1, 1), ior=1.49), det]
    prims, srcs = [], []
    for i in range(n_instances):
        k1 = rng.uniform(-1.5, 0.0)
        a4 = rng.uniform(-1e-3, 1e-3)
        a6 = rng.uniform(-1e-3, 1e-3)
        prims += led_lens_instance(i, k1, a4, a6)
        prims.append(prim(ST_PRIM_CYLINDER, pos=(0, 0, height), params=(0.0005, radius), material=3, flags=i << 8))
        srcs.append(led_source(i))
    s = Scene(prims, mats, env_radius=0.1, tolerance=1e-6, name="optics-detector")
    s.params = default_params(width=16, height=16, maxbounce=32)
    s.view = look_at((0, -0.05, 0.01), (0, 0, 0.002), 30.0, 1.0)
    s.info = {"sources": srcs, "rays": [rays] * n_instances, "workload": "optics-detector-%d" % n_instances}
    return s


# ------------------------------------------------------------------------------------------------------------
# An environment image (core/envimage.js) and the map light sampling draws from it (core/envmap.js).
# ------------------------------------------------------------------------------------------------------------
def env_image_lookup(img, dirs, luminance=179.0, turn=0.0):
    """envImageAt (envimage.js:56-70) for many directions: the equirectangular image `img` (H x W x 3, top row first)
    looked up bilinearly in each unit direction, wrapping across the seam, clamped at the poles, times `luminance`."""
    import numpy as np
    img = np.asarray(img, np.float64)
    h, w = img.shape[:2]
    d = np.asarray(dirs, np.float64)
    d = d / np.linalg.norm(d, axis=-1, keepdims=True)
    a = 0.5 - np.arctan2(d[..., 1], d[..., 0]) / (2 * np.pi) + turn / 360.0
    a = a - np.floor(a)
    u = a * w - 0.5
    v = np.arccos(np.clip(d[..., 2], -1, 1)) / np.pi * h - 0.5
    x0, y0 = np.floor(u), np.floor(v)
    fx, fy = (u - x0)[..., None], (v - y0)[..., None]
    xa = (x0.astype(np.int64) % w + w) % w
    xb = (xa + 1) % w
    ya = np.clip(y0.astype(np.int64), 0, h - 1)
    yb = np.clip(y0.astype(np.int64) + 1, 0, h - 1)
    top = img[ya, xa] * (1 - fx) + img[ya, xb] * fx
    bot = img[yb, xa] * (1 - fx) + img[yb, xb] * fx
    return np.maximum(top * (1 - fy) + bot * fy, 0.0) * luminance


def env_patch_image(w=256, h=128, background=1.0, patch=2000.0, row=40, col=100, size=6):
    """A dim uniform panorama with one bright square patch `size` pixels across, its top-left pixel at (row, col)."""
    import numpy as np
    img = np.full((h, w, 3), background, np.float32)
    img[row:row + size, col:col + size] = patch
    return img


def env_level_illuminance(img, luminance=179.0, turn=0.0, n=2048):
    """What the image puts on a level surface facing up: the integral of L cos over the upper hemisphere, by an
    equal-area midpoint grid of n x n/2 cells over the sphere (rows of equal steps in z)."""
    import numpy as np
    W, H = n, n // 2
    z = 1 - 2 * (np.arange(H) + 0.5) / H
    phi = 2 * np.pi * (np.arange(W) + 0.5) / W
    Z, PH = np.meshgrid(z[z > 0], phi, indexing="ij")
    S = np.sqrt(1 - Z * Z)
    d = np.stack([S * np.cos(PH), S * np.sin(PH), Z], -1)
    L = env_image_lookup(img, d, luminance, turn) @ np.array([0.2126, 0.7152, 0.0722])
    return float((L * Z).sum() * 4 * np.pi / (W * H))


def env_floor(width=32, height=32, albedo=0.8, maxbounce=2, seed=1):
    """A Lambertian floor (albedo 0.8) under whatever environment is set, seen straight down by an orthographic camera
    over 2 x 2 m: every pixel reads albedo / pi times the illuminance the environment's upper half puts on it."""
    s = Scene([prim(ST_PRIM_PLANE, material=1)], [air(), diffuse((albedo, albedo, albedo))], env_radius=20.0,
              name="env-floor")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_hint=0, sun_illuminance=0.0,
                              sky_luminance=0.0, ground_luminance=0.0, seed=seed)
    v = StView()
    for i, c in enumerate((0.0, 0.0, 3.0)):
        v.cam_pos[i] = c
    for i in range(3):
        v.right[i] = (1.0, 0.0, 0.0)[i]
        v.up[i] = (0.0, 1.0, 0.0)[i]
        v.fwd[i] = (0.0, 0.0, 1.0)[i]
    v.fx, v.fy, v.camtype = 1.0, 1.0, 1
    s.view = v
    s.info = {"workload": "env-floor", "albedo": albedo}
    return s


def translucent_furnace(kind="opal", width=48, height=48, sky=1000.0, maxbounce=32, seed=1):
    """The side beyond (materials_pbr.js THE SIDE BEYOND; transmission.js): a sphere in the uniform furnace, seen whole --
    "opal" a white body that diffuses all it passes (transmission 1, haze 1), "hazy" clear glass with a veil
    (transmission 1, haze 0.3), "rough" rough glass (roughness 0.5), "frosted" a white base passing half (transmission
    0.5, haze 1, roughness 0.3). Light samples aim through its faces from inside wherever the medium beyond is air."""
    mats = {"opal": material(base=(1, 1, 1), roughness=0.2, specular=0.5, transmission=1.0, ior=1.5),
            "hazy": material(base=(1, 1, 1), roughness=0.0, specular=0.5, transmission=1.0, ior=1.5),
            "rough": material(base=(1, 1, 1), roughness=0.5, specular=0.5, transmission=1.0, ior=1.5),
            "frosted": material(base=(1, 1, 1), roughness=0.3, specular=0.5, transmission=0.5, ior=1.5)}
    m = mats[kind]
    m.haze = {"opal": 1.0, "hazy": 0.3, "rough": 0.0, "frosted": 1.0}[kind]
    s = Scene([prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, 0.0), params=(0.5,), material=1)], [air(), m], env_radius=20.0,
              name="translucent-" + kind)
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, env_uniform=sky, sun_hint=0, seed=seed)
    s.view = look_at((0.0, -3.0, 0.0), (0.0, 0.0, 0.0), 25.0, 1.0)
    s.info = {"sky": sky}
    return s


def translucent_sun(kind="opal", width=64, height=48, maxbounce=12, seed=1):
    """A translucent sphere (translucent_furnace's materials) half sunk in a grey floor under the sun and sky: what
    light reaches the camera through it comes from light samples aimed through its faces from inside."""
    f = translucent_furnace(kind)
    m = f.material_list[1]
    s = Scene([prim(ST_PRIM_PLANE, material=1), prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, 0.2), params=(0.5,), material=2)],
              [air(), diffuse((0.5, 0.5, 0.5)), m], env_radius=20.0, name="translucent-sun-" + kind)
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_elevation=40.0, sun_azimuth=30.0,
                              sun_illuminance=100000.0, sky_luminance=3000.0, ground_luminance=0.0, seed=seed)
    s.view = look_at((0.0, -3.0, 1.2), (0.0, 0.0, 0.3), 35.0, width / height)
    return s


def aniso_spheres(anisotropy=0.8, width=64, height=48, maxbounce=8, seed=1, furnace=False):
    """Anisotropic gloss (microfacet.js mfAnisoAlpha; materials_pbr.js:185-194): a rough gold-ish metal sphere and a
    glossy plastic one whose lobes are stretched along their first tangent, on a grey floor under the sun and sky (or
    in the white furnace)."""
    m1 = metal((0.95, 0.8, 0.5), 0.5)
    m2 = plastic((0.2, 0.4, 0.8), 0.4)
    m1.anisotropy = anisotropy
    m2.anisotropy = anisotropy
    s = Scene([prim(ST_PRIM_PLANE, material=1), prim(ST_PRIM_SPHERE, pos=(-0.6, 0.0, 0.5), params=(0.5,), material=2),
               prim(ST_PRIM_SPHERE, pos=(0.6, 0.0, 0.5), params=(0.5,), material=3)],
              [air(), diffuse((0.5, 0.5, 0.5)), m1, m2], env_radius=20.0, name="aniso")
    if furnace:
        s.params = default_params(width=width, height=height, maxbounce=maxbounce, env_uniform=1000.0, sun_hint=0,
                                  seed=seed)
    else:
        s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_elevation=35.0,
                                  sun_azimuth=200.0, sun_illuminance=100000.0, sky_luminance=3000.0,
                                  ground_luminance=0.0, seed=seed)
    s.view = look_at((0.0, -3.5, 1.4), (0.0, 0.0, 0.45), 35.0, width / height)
    return s


def absorbing_box(width=32, height=32, base=(0.5, 0.25, 0.8), attenuation=1.0, sky=1000.0, seed=1):
    """Absorption inside (tracebasics.js absorbAlong; materials.js mediumMu): a 1 m cube of a clear material of index 1
    (no reflection, no bending) that takes its colour `base` off light over `attenuation` metres, seen straight through
    by an orthographic camera against the white furnace: every ray through it reads sky x base^(1 / attenuation)."""
    m = material(base=base, roughness=0.0, specular=0.0, transmission=1.0, ior=1.0, attenuation=attenuation)
    s = Scene([prim(ST_PRIM_BOX, pos=(0.0, 0.0, 0.0), params=(0.5, 0.5, 0.5), material=1)], [air(), m],
              env_radius=20.0, name="absorbing-box")
    # a fine march tolerance: the path inside is the cube's width less up to a tolerance at each face
    s.params = default_params(width=width, height=height, maxbounce=8, env_uniform=sky, sun_hint=0, seed=seed, eps=1e-5)
    v = StView()
    for i, c in enumerate((0.0, -3.0, 0.0)):
        v.cam_pos[i] = c
    for i in range(3):
        v.right[i] = (1.0, 0.0, 0.0)[i]
        v.up[i] = (0.0, 0.0, 1.0)[i]
        v.fwd[i] = (0.0, -1.0, 0.0)[i]
    v.fx, v.fy, v.camtype = 0.4, 0.4, 1
    s.view = v
    s.info = {"expected": [sky * b ** (1.0 / attenuation) for b in base]}
    return s


# ------------------------------------------------------------------------------------------------------------
# A coating on a slab (core/materials.js coat; optics/fresnel.js coatedSlabT): the optics trace's collimated beam
# through a clear coated slab onto a detector floor.
# ------------------------------------------------------------------------------------------------------------
def coated_slab(where=COAT_AR_BACK, lo=0.5, hi=0.5, edge=600.0, width=20.0, index=1.8, deg=0.0, ior=1.5,
                rays=100_000):
    """A clear smooth slab (n `ior`, white, 0.1 m thick, its middle at z 0.5, 8 m across) coated as `coated` says, over a
    black detector floor at z 0; a collimated disc of radius 0.3 m at z 1 shining down, tilted `deg` degrees about y.
    What reaches the floor is what the slab let through: the incoherent series (1 - R)(1 - Ri) / (1 - Ri^2), Ri what
    each face reflects from within -- 0 with an AR back, the glass's Fresnel bare, R coated (coated_slab_t)."""
    from .st_types import StOpticsSource
    glass_m = coated(material(base=(1, 1, 1), roughness=0.0, specular=0.5, transmission=1.0, ior=ior), where, lo, hi,
                     edge, width, index)
    det = material(base=(0, 0, 0), specular=0.0, detector=1.0)
    mats = [air(), glass_m, det]
    prims = [prim(ST_PRIM_BOX, pos=(0, 0, 0.5), params=(4.0, 4.0, 0.05), material=1),
             prim(ST_PRIM_BOX, pos=(0, 0, -0.05), params=(8.0, 8.0, 0.05), material=2)]
    s = Scene(prims, mats, env_radius=20.0, tolerance=1e-5, name="coated-slab")
    s.params = default_params(width=16, height=16, maxbounce=32)
    s.view = look_at((0, -3, 2), (0, 0, 0.5), 40.0, 1.0)
    a = math.radians(deg)
    src = StOpticsSource()
    for i, v in enumerate((0.0, 0.0, 1.0)):
        src.centre[i] = v
    for i, v in enumerate((math.sin(a), 0.0, -math.cos(a))):
        src.axis[i] = v
    for i, v in enumerate((0.0, 1.0, 0.0)):
        src.tangent[i] = v
    src.flux, src.shape, src.size_x, src.size_y = 1000.0, 1, 0.3, 0.3
    src.dist, src.cos_half, src.n_exp, src.emit_n = 0, 1.0, 1.0, 1.0
    s.info = {"sources": [src], "rays": [rays], "workload": "coated-slab"}
    return s


def coated_slab_t(deg, ior, R, where):
    """optics/fresnel.js coatedSlabT: the slab's transmission for a coating of reflectance R on the faces light enters
    by, the leaving faces as `where` says (Ri 0 with an AR back, the glass's unpolarised Fresnel bare, R coated)."""
    if where == COAT_AR_BACK:
        Ri = 0.0
    elif where == COAT_BARE_BACK:
        c = math.cos(math.radians(deg))
        s2 = (1.0 / ior) ** 2 * (1.0 - c * c)                          # from outside: the Fresnel of the entry angle
        ct = math.sqrt(1.0 - s2)
        rs = ((c - ior * ct) / (c + ior * ct)) ** 2
        rp = ((ct - ior * c) / (ct + ior * c)) ** 2
        Ri = 0.5 * (rs + rp)
    else:
        Ri = R
    return (1.0 - R) * (1.0 - Ri) / (1.0 - Ri * Ri)


def coat_edge_rgb(lo, hi, edge, width):
    """spectral.js edgeRGB, restated in numpy: a coating's reflectance per channel -- R(lambda) averaged against each
    channel's 10 nm bin weights (the clipped Rec.709 colour-matching functions of the Wyman-Sloan-Shirley fit), each
    bin's mean of the logistic exact (a softplus difference)."""
    import numpy as np
    l = 380.0 + (np.arange(4000) + 0.5) * 0.1
    g = lambda x, mu, s1, s2: np.exp(-0.5 * ((x - mu) / np.where(x < mu, s1, s2)) ** 2)
    X = 1.056 * g(l, 599.8, 37.9, 31.0) + 0.362 * g(l, 442.0, 16.0, 26.7) - 0.065 * g(l, 501.1, 20.4, 26.2)
    Y = 0.821 * g(l, 568.8, 46.9, 40.5) + 0.286 * g(l, 530.9, 16.3, 31.1)
    Z = 1.217 * g(l, 437.0, 11.8, 36.0) + 0.681 * g(l, 459.0, 26.0, 13.8)
    M = np.array([[3.2404542, -1.5371385, -0.4985314], [-0.9692660, 1.8760108, 0.0415560],
                  [0.0556434, -0.2040259, 1.0572252]])
    rgb = np.maximum(M @ np.stack([X, Y, Z]), 0.0)                    # 3 x 4000
    W = rgb.reshape(3, 40, 100).mean(axis=2)
    W /= W.sum(axis=1, keepdims=True)
    s = max(width, 0.01) / (2 * math.log(9))
    sp = lambda x: np.maximum(x, 0) + np.log1p(np.exp(-np.abs(x)))
    b = 380.0 + 10.0 * np.arange(41)
    F = sp((b - edge) / s)
    mean = s * np.diff(F) / 10.0
    return lo + (hi - lo) * (W @ mean)


def coat_edge_at(edge0, n_sin, n_eff):
    """spectral.js edgeAt: the edge for light of invariant n0 sin(theta0) through a stack of effective index n_eff."""
    return edge0 * math.sqrt(max(0.0, 1.0 - (n_sin / max(n_eff, 1e-6)) ** 2))


def coated_spheres(width=64, height=48, maxbounce=12, seed=1, furnace=False, where=COAT_EVERY_FACE, abbe=30.0):
    """Coatings in a render: a dichroic clear glass sphere (R 0 to 1 above 600 nm, 20 nm wide, coated as `where`
    says), a rough gold-ish metal under a 30 % beam-splitter coating, and a dispersive glass sphere (Abbe `abbe`)
    with the dichroic on every face -- its rays meet the inner faces with a wavelength of their own -- on a grey floor
    under the sun and sky. `furnace`: the dichroic glass alone in a uniform environment, where a lossless coating
    (R + T = 1 in every channel) must read the environment in every channel."""
    dichroic = coated(glass((1, 1, 1), ior=1.5), where, 0.0, 1.0, 600.0, 20.0, 1.8)
    if furnace:
        s = Scene([prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, 1.0), params=(0.3,), material=1)], [air(), dichroic],
                  env_radius=40.0, name="coated-furnace")
        s.params = default_params(width=width, height=height, maxbounce=maxbounce, env_uniform=1000.0, sun_hint=0,
                                  seed=seed)
        s.view = look_at((0.0, -1.6, 1.0), (0.0, 0.0, 1.0), 40.0, width / height)
        s.info = {"closed_form": 1000.0}
        return s
    gold = coated(metal((0.95, 0.8, 0.5), 0.3), COAT_AR_BACK, 0.3, 0.3, 600.0, 20.0, 1.8)
    disp = coated(glass((1, 1, 1), ior=1.6, abbe=abbe), COAT_EVERY_FACE, 0.0, 1.0, 560.0, 30.0, 1.8)
    s = Scene([prim(ST_PRIM_PLANE, material=1), prim(ST_PRIM_SPHERE, pos=(-0.7, 0.0, 0.35), params=(0.35,), material=2),
               prim(ST_PRIM_SPHERE, pos=(0.0, 0.3, 0.35), params=(0.35,), material=3),
               prim(ST_PRIM_SPHERE, pos=(0.7, 0.0, 0.35), params=(0.35,), material=4)],
              [air(), diffuse((0.6, 0.6, 0.6)), dichroic, gold, disp], env_radius=20.0, name="coated-spheres")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_elevation=40.0, sun_azimuth=30.0,
                              sun_illuminance=100000.0, sky_luminance=3000.0, ground_luminance=0.0, seed=seed)
    s.view = look_at((0.0, -3.0, 1.4), (0.0, 0.0, 0.3), 40.0, width / height)
    return s


# ------------------------------------------------------------------------------------------------------------
# Scattering inside a material (materials.js scatterDistance; haze.js THE MEDIUM'S WALK).
# ------------------------------------------------------------------------------------------------------------
def volume_slab(tau=1.0, g=0.0, width=32, height=32, thickness=0.1, le=1000.0, maxiter=20000, seed=1):
    """An index-matched slab (ior 1: its faces do nothing) 0.1 m thick and 10 m wide, its mean free path thickness / tau
    and Henyey-Greenstein asymmetry g, seen head-on (a 6 degree view from 1 m) in front of a glowing plane of `le`
    cd/m^2, in a black world: each pixel reads le x what the slab passes of a beam at normal incidence -- the walk's
    transmission T(tau, g), which radiative transfer pins (exp(-tau) of it never collides; T + R = 1; deep in the slab
    T (tau + 2 q) stops depending on tau, q = 0.7104 for isotropic scattering)."""
    slab = material(base=(1, 1, 1), roughness=0.0, specular=0.0, transmission=1.0, ior=1.0,
                    scatter_distance=thickness / tau, scatter_g=g)
    glow = material(base=(0, 0, 0), specular=0.0, emissive=(le, le, le))
    mats = [air(), slab, glow]
    prims = [prim(ST_PRIM_BOX, pos=(0, 0, 0), params=(5.0, 5.0, thickness / 2), material=1),
             prim(ST_PRIM_BOX, pos=(0, 0, -0.5), params=(49.99, 49.99, 0.001), material=2)]
    s = Scene(prims, mats, env_radius=80.0, name="volume-slab")
    s.params = default_params(width=width, height=height, maxbounce=16, env_uniform=1e-6, sun_hint=0, seed=seed)
    s.params.maxiter = maxiter
    s.params.emit_off = 1
    s.view = look_at((0.0, 0.0, 1.0), (0.0, 0.0, 0.0), 6.0, width / height, up=(0.0, 1.0, 0.0))
    s.info = {"closed_form": None, "le": le, "tau": tau, "g": g}
    return s


def milky_spheres(width=64, height=48, maxbounce=12, seed=1, furnace=False, maxiter=4000):
    """Milky glass: a clear glass sphere (n 1.5) whose volume scatters (mean free path 5 cm, g 0.6) and a diffusing
    opal-coloured one (mean free path 2 cm, g 0, a colour depth of 20 cm at (0.9, 0.7, 0.5)), on a grey floor under
    the sun and sky; `furnace`: the first alone in a uniform environment, where it absorbs nothing and must vanish."""
    milky = material(base=(1, 1, 1), roughness=0.0, specular=0.5, transmission=1.0, ior=1.5, scatter_distance=0.05,
                     scatter_g=0.6)
    if furnace:
        s = Scene([prim(ST_PRIM_SPHERE, pos=(0.0, 0.0, 1.0), params=(0.3,), material=1)], [air(), milky],
                  env_radius=40.0, name="milky-furnace")
        # (inside glass most of a walk's arrivals at the wall are past the critical angle: bounces enough for them)
        s.params = default_params(width=width, height=height, maxbounce=64, env_uniform=1000.0, sun_hint=0, seed=seed)
        s.params.maxiter = maxiter
        s.view = look_at((0.0, -1.6, 1.0), (0.0, 0.0, 1.0), 40.0, width / height)
        s.info = {"closed_form": 1000.0}
        return s
    opal = material(base=(0.9, 0.7, 0.5), roughness=0.0, specular=0.5, transmission=1.0, ior=1.45, attenuation=0.2,
                    scatter_distance=0.02, scatter_g=0.0)
    s = Scene([prim(ST_PRIM_PLANE, material=1), prim(ST_PRIM_SPHERE, pos=(-0.45, 0.0, 0.35), params=(0.35,), material=2),
               prim(ST_PRIM_SPHERE, pos=(0.45, 0.1, 0.3), params=(0.3,), material=3)],
              [air(), diffuse((0.6, 0.6, 0.6)), milky, opal], env_radius=20.0, name="milky-spheres")
    s.params = default_params(width=width, height=height, maxbounce=maxbounce, sun_elevation=40.0, sun_azimuth=30.0,
                              sun_illuminance=100000.0, sky_luminance=3000.0, ground_luminance=0.0, seed=seed)
    s.params.maxiter = maxiter
    s.view = look_at((0.0, -2.6, 1.2), (0.0, 0.0, 0.3), 40.0, width / height)
    return s


def milky_slab(width=64, height=48, photons=200_000, r1=0.01, r1v=0.02, sun_diameter=5.0, seed=1, sppm=True,
               maxiter=4000):
    """The photon map in the volume: a slab of milky glass (n 1.5, 0.6 x 0.6 x 0.1 m, mean free path 3 cm, g 0.5) 0.25 m
    over a grey floor, lit by the sun alone (50 degrees up; its disc `sun_diameter` wide so the camera's own paths find
    it through the walk often enough to check the map against), seen from the side and above. With the map on, the sun's
    photons walk the slab and store where they collide; a camera ray that came in through the slab's face gathers them
    at its first collision; the floor under it gathers what the slab let through."""
    milky = material(base=(1, 1, 1), roughness=0.0, specular=0.5, transmission=1.0, ior=1.5, scatter_distance=0.03,
                     scatter_g=0.5)
    s = Scene([prim(ST_PRIM_PLANE, material=1), prim(ST_PRIM_BOX, pos=(0.0, 0.0, 0.3), params=(0.3, 0.3, 0.05),
                                                     material=2)],
              [air(), diffuse((0.6, 0.6, 0.6)), milky], env_radius=10.0, name="milky-slab")
    s.params = default_params(width=width, height=height, maxbounce=16, sun_elevation=50.0, sun_azimuth=30.0,
                              sun_illuminance=100000.0, sun_diameter=sun_diameter, sky_luminance=0.0,
                              ground_luminance=0.0, seed=seed)
    s.params.maxiter = maxiter
    if sppm:
        s.params.sppm = 1
        s.params.sppm_photons = photons
        s.params.sppm_r1 = r1
        s.params.sppm_r1_volume = r1v
        s.params.sppm_alpha = 0.7
        s.params.sppm_half = 0.6
    s.view = look_at((0.0, -1.4, 0.75), (0.0, 0.0, 0.2), 45.0, width / height)
    return s


def dispersive_wedge(abbe=28.0, ior=1.75, wedge_deg=30.0, rays=100_000):
    """optics-dispersion's bench (lib/pathtracer/tests.js testScene 'wedge'): a collimated white beam (a disc of 0.1 m
    at z 1) straight down through a glass wedge -- a block whose top face is tilted `wedge_deg` about y (outward normal
    (sin a, 0, cos a)) and whose bottom is level -- of index `ior` at the d line and Abbe number `abbe`, onto a black
    detector floor. Each ray refracted into the glass takes a wavelength and refracts at n(l): the beam fans out."""
    from .st_types import StOpticsSource
    a = math.radians(wedge_deg)
    glass_m = material(base=(1, 1, 1), roughness=0.0, specular=0.5, transmission=1.0, ior=ior, abbe=abbe)
    det = material(base=(0, 0, 0), specular=0.0, detector=1.0)
    # the tilted top: a half-space subtracted from the block, its local z (into the wedge) -(sin a, 0, cos a)
    rot = (-math.cos(a), 0.0, math.sin(a), 0.0, 1.0, 0.0, -math.sin(a), 0.0, -math.cos(a))
    prims = [prim(ST_PRIM_BOX, pos=(0, 0, 0.5), params=(0.5, 0.5, 0.2), material=1),
             prim(ST_PRIM_PLANE, pos=(0, 0, 0.55), material=1, op=ST_OP_SUB, rot=rot),
             prim(ST_PRIM_BOX, pos=(0, 0, -0.05), params=(8.0, 8.0, 0.05), material=2)]
    # (the surface tolerance the normal's differences are taken at: at 1e-5 m a tilted face's f32 differences turn the
    # normal by about 0.03 degree, at 1e-3 m a hundred times less)
    s = Scene(prims, [air(), glass_m, det], env_radius=20.0, tolerance=1e-3, name="dispersive-wedge")
    s.params = default_params(width=16, height=16, maxbounce=32)
    s.view = look_at((0, -3, 2), (0, 0, 0.5), 40.0, 1.0)
    src = StOpticsSource()
    for i, v in enumerate((0.0, 0.0, 1.0)):
        src.centre[i] = v
    for i, v in enumerate((0.0, 0.0, -1.0)):
        src.axis[i] = v
    for i, v in enumerate((0.0, 1.0, 0.0)):
        src.tangent[i] = v
    src.flux, src.shape, src.size_x, src.size_y = 1000.0, 1, 0.1, 0.1
    src.dist, src.cos_half, src.n_exp, src.emit_n = 0, 1.0, 1.0, 1.0
    s.info = {"sources": [src], "rays": [rays], "workload": "dispersive-wedge"}
    return s


def wedge_exit_deg(wedge_deg, n):
    """optics/fresnel.js wedgeExitDeg: the beam straight down refracted into the wedge's tilted top (into index n) and
    out of its level bottom; the leaving ray's angle from straight down, degrees, signed as atan2(x, -z)."""
    def refract(d, nrm, eta):
        c = -(d[0] * nrm[0] + d[1] * nrm[1] + d[2] * nrm[2])
        k = 1 - eta * eta * (1 - c * c)
        if k < 0:
            return None
        t = eta * c - math.sqrt(k)
        return [eta * d[i] + t * nrm[i] for i in range(3)]
    a = math.radians(wedge_deg)
    inside = refract([0.0, 0.0, -1.0], [math.sin(a), 0.0, math.cos(a)], 1.0 / n)
    out = inside and refract(inside, [0.0, 0.0, 1.0], n)
    return math.degrees(math.atan2(out[0], -out[2])) if out else None
