"""Loading libshadytracer.so and declaring its C ABI for ctypes (include/shadytracer.h).

There is no fallback: if the library is not built, or no GPU answers, the call that needs it raises.
"""
import ctypes as C
import os

from . import st_types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libshadytracer.so")

_lib = None

# every entry point include/shadytracer.h declares, with its argument and result types
P = C.c_void_p
SIGNATURES = {
    "st_abi_version": ([], C.c_int),
    "st_create": ([C.c_int, C.POINTER(P)], C.c_int),
    "st_destroy": ([P], C.c_int),
    "st_last_error": ([P], C.c_char_p),
    "st_set_scene": ([P, C.c_char_p, C.POINTER(T.StSceneDesc), C.c_char_p, C.c_size_t], C.c_int),
    "st_set_params": ([P, C.POINTER(T.StParams), C.POINTER(C.c_uint64)], C.c_int),
    "st_set_view": ([P, C.POINTER(T.StView)], C.c_int),
    "st_scene_code_info": ([P, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_uint64)], C.c_int),
    "st_compile_scene": ([C.c_char_p, C.c_char_p, C.c_size_t, C.POINTER(C.c_double)], C.c_int),
    "st_set_env_image": ([P, P, C.c_uint32, C.c_uint32, C.c_float, C.c_float], C.c_int),
    "st_optics_set_rays": ([P, P, C.c_uint32], C.c_int),
    "st_optics_set_spectra": ([P, P, C.c_uint32], C.c_int),
    "st_checkpoint_size": ([P, C.POINTER(C.c_size_t)], C.c_int),
    "st_checkpoint_save": ([P, P, C.c_size_t], C.c_int),
    "st_checkpoint_load": ([P, P, C.c_size_t], C.c_int),
    "st_env_map_tables": ([P, P], C.c_int),
    "st_invalidate": ([P], C.c_int),
    "st_step": ([P, C.c_int], C.c_int),
    "st_step_async": ([P, C.c_int], C.c_int),
    "st_sync": ([P, C.c_int], C.c_int),
    "st_set_wait_limit": ([P, C.c_uint32, C.c_int], C.c_int),
    "st_autotune": ([P, C.c_int, C.POINTER(T.StTune)], C.c_int),
    "st_set_tune": ([P, C.POINTER(T.StTune)], C.c_int),
    "st_read_accum": ([P, P, P, P, P], C.c_int),
    "st_image_stats": ([P, C.POINTER(T.StImageStats)], C.c_int),
    "st_read_counters": ([P, C.POINTER(T.StCounters)], C.c_int),
    "st_enable_kernel_times": ([P, C.c_int], C.c_int),
    "st_kernel_times": ([P, C.POINTER(T.StKernelTime), C.c_int, C.POINTER(C.c_int)], C.c_int),
    "st_reset_kernel_times": ([P], C.c_int),
    "st_mf_tables": ([P, P, P, P], C.c_int),
    "st_sppm_build": ([P, P, P, P, P, P, C.c_uint32, C.c_float], C.c_int),
    "st_sppm_read_grid": ([P, P, P, P, P], C.c_int),
    "st_sppm_gather": ([P, P, P, P, P, C.c_uint32, C.c_float, C.c_uint32, C.c_uint32, C.c_uint32, P], C.c_int),
    "st_sppm_stats_read": ([P, C.POINTER(T.StSppmStats)], C.c_int),
    "st_sppm_emission_map": ([P, P, P, P], C.c_int),
    "st_lt_counts": ([P, P], C.c_int),
    "st_set_views": ([P, P, C.c_uint32], C.c_int),
    "st_read_accum_view": ([P, C.c_uint32, P, P, P, P], C.c_int),
    "st_optics_set_sources": ([P, C.POINTER(T.StOpticsSource), C.c_uint32], C.c_int),
    "st_optics_set_far": ([P, C.POINTER(T.StOpticsFar)], C.c_int),
    "st_optics_run": ([P, C.POINTER(T.StOpticsBatch), P, P, C.POINTER(T.StOpticsTotals)], C.c_int),
    "st_optics_set_detail": ([P, C.POINTER(T.StOpticsDetail)], C.c_int),
    "st_optics_autotune": ([P, C.POINTER(T.StOpticsBatch), C.POINTER(T.StTune)], C.c_int),
    "st_optics_tallies": ([P, P, P], C.c_int),
    "st_optics_hits": ([P, P, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int),
    "st_optics_paths": ([P, P, P], C.c_int),
    "st_render_noalloc": ([C.c_int, C.POINTER(T.StSceneDesc), C.POINTER(T.StParams), C.POINTER(T.StView), C.c_int,
                           P, P, P, P], C.c_int),
    "st_eval_sdf": ([P, P, C.c_uint32, P], C.c_int),
    "st_mlp_get_weights": ([P, P, C.c_size_t], C.c_int),
    "st_mlp_set_weights": ([P, P, C.c_size_t], C.c_int),
    "st_mlp_eval": ([P, P, P, C.c_uint32, P, P], C.c_int),
    "st_mlp_grad": ([P, P, P, P, P, C.c_uint32, P, P], C.c_int),
    "st_mlp_train": ([P, P, P, P, P, C.c_uint32, C.c_uint32, C.c_float], C.c_int),
    "st_mlp_stats_read": ([P, C.POINTER(T.StMlpStats)], C.c_int),
    "st_mlp_read_batch": ([P, P, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int),
    "st_emit_list": ([P, P, C.c_uint32, C.POINTER(C.c_uint32)], C.c_int),
    "st_struct_sizes": ([P, C.c_int], C.c_int),
    "st_stream": ([P], C.c_void_p),
}

STRUCT_ORDER = [T.StPrim, T.StMaterial, T.StSceneDesc, T.StParams, T.StView, T.StCounters, T.StImageStats,
                T.StKernelTime, T.StSppmStats, T.StOpticsSource, T.StOpticsFar, T.StOpticsBatch, T.StOpticsTotals,
                T.StMlpStats, T.StLight, T.StOpticsDetail, T.StTune]


def load(path=None):
    """The library, loaded once. Raises if it has not been built (shadytracer_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libshadytracer.so is not built (%s): run `python -m shadytracer_gb300.build` or "
                           "__graft_entry__.build(); there is no CPU fallback" % path)
    L = C.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
    _lib = L
    return L


class StError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


def check(rc, ctx=None, what="call"):
    if rc != 0:
        msg = what
        if ctx:
            m = load().st_last_error(ctx)
            if m:
                msg = "%s: %s" % (what, m.decode(errors="replace"))
        raise StError(rc, msg)
    return rc
