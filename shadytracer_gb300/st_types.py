"""ctypes mirrors of the C ABI's structs (include/shadytracer.h), field for field.

The host side (renderer.py, optics.py) fills these and passes pointers across the boundary; nothing here
computes. A struct whose size drifts from the header's is caught by tests/test_capi.py, which compares
ctypes.sizeof against the sizes the library itself reports.
"""
import ctypes as C

ST_OK = 0
ST_ERR_ARG = -1
ST_ERR_OOM = -2
ST_ERR_CUDA = -3
ST_ERR_TIMEOUT = -4
ST_ERR_BUSY = -5
ST_ERR_COMPILE = -6
ST_ERR_STATE = -7

ST_PRIM_PLANE, ST_PRIM_SPHERE, ST_PRIM_BOX, ST_PRIM_ROUNDBOX, ST_PRIM_TORUS, ST_PRIM_PRISM, \
    ST_PRIM_ASPHERE, ST_PRIM_CYLINDER = range(8)
ST_OP_ITEM, ST_OP_SMOOTH, ST_OP_UNION, ST_OP_SUB = range(4)
ST_ENV_ANALYTIC, ST_ENV_SUNSKY, ST_ENV_STUDIO = range(3)
ST_MAX_PRIMS = 256
ST_MAX_MATERIALS = 256


class StPrim(C.Structure):
    _fields_ = [("type", C.c_uint32), ("op", C.c_uint32), ("material", C.c_uint32), ("flags", C.c_uint32),
                ("pos", C.c_float * 3), ("k", C.c_float),
                ("rot", C.c_float * 9), ("pad0", C.c_float * 3),
                ("p", C.c_float * 12)]


class StMaterial(C.Structure):
    _fields_ = [("base", C.c_float * 3), ("metallic", C.c_float),
                ("roughness", C.c_float), ("specular", C.c_float), ("specular_tint", C.c_float),
                ("transmission", C.c_float), ("ior", C.c_float), ("abbe", C.c_float),
                ("attenuation", C.c_float), ("detector", C.c_float),
                ("emissive", C.c_float * 3), ("beam_cos", C.c_float), ("haze", C.c_float), ("anisotropy", C.c_float),
                ("coat", C.c_uint32), ("coat_lo", C.c_float), ("coat_hi", C.c_float), ("coat_edge", C.c_float),
                ("coat_width", C.c_float), ("coat_index", C.c_float),
                ("scatter_distance", C.c_float), ("scatter_g", C.c_float), ("pad", C.c_float * 2)]


ST_LIGHT_DISC, ST_LIGHT_RECTANGLE = 1, 2
ST_LIGHT_COSINE, ST_LIGHT_UNIFORM = 0, 1
ST_MAX_LIGHTS = 64


class StLight(C.Structure):
    _fields_ = [("centre", C.c_float * 3), ("shape", C.c_uint32), ("u", C.c_float * 3), ("half_w", C.c_float),
                ("v", C.c_float * 3), ("half_h", C.c_float), ("le", C.c_float * 3), ("material", C.c_uint32),
                ("dist", C.c_uint32), ("n", C.c_float), ("beam_cos", C.c_float), ("pad", C.c_uint32)]


class StSceneDesc(C.Structure):
    _fields_ = [("prims", C.POINTER(StPrim)), ("n_prims", C.c_uint32),
                ("materials", C.POINTER(StMaterial)), ("n_materials", C.c_uint32),
                ("env_radius", C.c_float), ("tolerance", C.c_float),
                ("haze_centre", C.c_float * 3), ("haze_sigma_t", C.c_float),
                ("haze_axes", C.c_float * 9), ("haze_half", C.c_float * 3),
                ("haze_albedo", C.c_float * 3), ("haze_g", C.c_float),
                ("lights", C.POINTER(StLight)), ("n_lights", C.c_uint32)]


class StParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32),
                ("maxbounce", C.c_uint32), ("maxiter", C.c_uint32), ("stepscale", C.c_float),
                ("nee", C.c_uint32), ("rr", C.c_uint32), ("nee_sun_pick", C.c_float),
                ("sun_elevation", C.c_float), ("sun_azimuth", C.c_float), ("sun_diameter", C.c_float),
                ("sun_illuminance", C.c_float), ("sky_luminance", C.c_float), ("ground_luminance", C.c_float),
                ("env_uniform", C.c_float), ("env_sun_gain", C.c_float), ("env_sky_gain", C.c_float),
                ("sun_hint", C.c_uint32), ("seed", C.c_uint32), ("maxaverages", C.c_uint32),
                ("eps", C.c_float), ("budget", C.c_uint32), ("samples_per_wave", C.c_uint32),
                ("sppm", C.c_uint32), ("sppm_photons", C.c_uint32), ("sppm_r1", C.c_float),
                ("sppm_alpha", C.c_float), ("sppm_half", C.c_float), ("sppm_learn", C.c_uint32),
                ("guide", C.c_uint32), ("guide_alpha", C.c_float), ("guide_lr", C.c_float),
                ("guide_train", C.c_uint32), ("guide_seed", C.c_uint32),
                ("emit_share", C.c_float), ("emit_radius", C.c_float), ("emit_off", C.c_uint32),
                ("env_map_off", C.c_uint32), ("step_cache", C.c_uint32), ("step_cache_cells", C.c_float),
                ("lt", C.c_uint32), ("lt_photons", C.c_uint32),
                ("env_mode", C.c_uint32), ("sun_outside", C.c_float), ("sky_turbidity", C.c_float),
                ("studio_illuminance", C.c_float), ("studio_top", C.c_float), ("studio_color", C.c_float * 3),
                ("lt_emit_share", C.c_float), ("env_cache", C.c_uint32), ("env_cache_size", C.c_uint32),
                ("sppm_r1_volume", C.c_float)]


class StView(C.Structure):
    _fields_ = [("cam_pos", C.c_float * 3), ("right", C.c_float * 3), ("up", C.c_float * 3),
                ("fwd", C.c_float * 3), ("fx", C.c_float), ("fy", C.c_float), ("camtype", C.c_uint32),
                ("lens_radius", C.c_float), ("focus_distance", C.c_float)]


class StCounters(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("segments", C.c_uint64), ("march_steps", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("shadow_steps", C.c_uint64),
                ("nonfinite", C.c_uint32), ("flushed", C.c_uint32), ("shadowcut", C.c_uint32),
                ("samples", C.c_uint32), ("launches", C.c_uint64), ("prim_evals", C.c_uint64 * 8),
                ("prim_warp_evals", C.c_uint64 * 8), ("bound_tests", C.c_uint64), ("bound_warp_tests", C.c_uint64),
                ("op_evals", C.c_uint64 * 4)]


class StImageStats(C.Structure):
    _fields_ = [("mean_luma", C.c_double), ("median_luma", C.c_double), ("trimmed_mean_luma", C.c_double),
                ("mean_rel_se", C.c_double), ("sampled", C.c_uint32), ("samples", C.c_uint32)]


class StKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 24), ("launches", C.c_uint32), ("ms", C.c_double)]


class StSppmStats(C.Structure):
    _fields_ = [("stored", C.c_uint32), ("gathers", C.c_uint32), ("cut", C.c_uint32),
                ("visits_max", C.c_uint32), ("visits", C.c_uint64)]


class StMlpStats(C.Structure):
    _fields_ = [("steps", C.c_uint32), ("samples", C.c_uint32), ("loss", C.c_float), ("mean_weight", C.c_float),
                ("box_lo", C.c_float * 3), ("box_inv_ext", C.c_float), ("inferred", C.c_uint32)]


MLP_PARAMS = 13824 + 131072         # ST_MLP_PARAMS: W1 W2 W3 W4 then the hash grid's features


class StOpticsSource(C.Structure):
    _fields_ = [("centre", C.c_float * 3), ("flux", C.c_float),
                ("axis", C.c_float * 3), ("shape", C.c_uint32),
                ("tangent", C.c_float * 3), ("size_x", C.c_float),
                ("size_y", C.c_float), ("dist", C.c_uint32), ("cos_half", C.c_float), ("n_exp", C.c_float),
                ("emit_n", C.c_float), ("two_sided", C.c_uint32), ("on_surface", C.c_uint32),
                ("instance", C.c_uint32), ("ray_first", C.c_uint32), ("ray_count", C.c_uint32),
                ("colour", C.c_float * 3), ("cct", C.c_float), ("spectrum", C.c_uint32), ("pad", C.c_uint32 * 5)]


class StOpticsFar(C.Structure):
    _fields_ = [("nC", C.c_uint32), ("nG", C.c_uint32), ("axis", C.c_float * 3), ("c0", C.c_float * 3)]


class StOpticsBatch(C.Structure):
    _fields_ = [("n_instances", C.c_uint32), ("ray_count", C.POINTER(C.c_uint32)),
                ("lux_cells", C.c_uint32), ("lux_half", C.c_float), ("lux_height", C.c_float),
                ("maxbounce", C.c_uint32), ("seed", C.c_uint32), ("spectral", C.c_uint32)]


class StOpticsTotals(C.Structure):
    _fields_ = [("emitted", C.c_double), ("escaped", C.c_double), ("lost", C.c_double),
                ("detected", C.c_double), ("absorbed", C.c_double),
                ("interactions", C.c_uint64), ("rays", C.c_uint64),
                ("n_escaped", C.c_uint64), ("n_lost", C.c_uint64), ("n_detected", C.c_uint64),
                ("n_absorbed", C.c_uint64)]


class StTune(C.Structure):
    _fields_ = [("claim", C.c_uint32), ("chunk", C.c_uint32), ("ms", C.c_float), ("ms_default", C.c_float)]


class StOpticsDetail(C.Structure):
    _fields_ = [("det_cap", C.c_uint32), ("path_rays", C.c_uint32), ("path_verts", C.c_uint32),
                ("esc_len", C.c_float)]


def default_params(**kw):
    """The reference's defaults for the settings the hot path reads (core/uniforms.schema.js UniformSpec)."""
    p = StParams()
    p.width, p.height = 256, 256
    p.maxbounce = 10
    p.maxiter = 400
    p.stepscale = 0.9
    p.nee = 1
    p.rr = 0
    p.nee_sun_pick = 0.5
    p.sun_elevation = 45.0
    p.sun_azimuth = 0.0
    p.sun_diameter = 0.53
    p.sun_illuminance = 100000.0
    p.sky_luminance = 0.0
    p.ground_luminance = 0.0
    p.env_uniform = 0.0
    p.env_sun_gain = 1.0
    p.env_sky_gain = 1.0
    p.sun_hint = 1
    p.seed = 1
    p.maxaverages = 0
    p.eps = 0.0
    p.budget = 0
    p.samples_per_wave = 0
    p.sppm = 0
    p.sppm_photons = 0
    p.sppm_r1 = 0.0
    p.sppm_alpha = 0.0
    p.sppm_half = 0.0
    p.sppm_learn = 0
    p.guide = 0
    p.guide_alpha = 0.0
    p.guide_lr = 0.0
    p.guide_train = 1
    p.guide_seed = 0
    p.emit_share = 0.0
    p.emit_radius = 0.0
    p.emit_off = 0
    p.env_cache = 1                   # the environment's presets from a texture (UniformSpec envCache: on)
    p.env_cache_size = 2048
    p.sppm_r1_volume = 0.0
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p
