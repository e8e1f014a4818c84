"""The renderer facade: the reference's createPathTracer / RT (lib/pathtracer/index.js:90, contract in
lib/pathtracer/README.md:38-124), over the C ABI of libshadytracer.so.

    rt = create_path_tracer(scene)     # createPathTracer({scene, ...}); RT.init()
    rt.set(maxbounce=8)                # RT.set(values) -> the keys it did not recognise
    rt.step(16)                        # RT.step(n): returns when the GPU has finished
    rt.image_stats()                   # RT.imageStats()
    rt.measure(x, y)                   # RT.measure: the pixel's luminance and its standard error
    rt.set_scene(other)                # RT.setScene(s): on a failed build the old scene is kept
    rt.invalidate()                    # RT.invalidate()

Errors are exceptions (StError), as the reference's are (core/raytrace_main.js:1580-1581). Everything runs on the
GPU through the library; a missing library or GPU raises.
"""
import ctypes as C

import numpy as np

from . import st_types as T
from ._lib import load, check, StError  # noqa: F401

PARAM_KEYS = [f for f, _ in T.StParams._fields_]


class PathTracer:
    def __init__(self, scene=None, device=0, code=None):
        self.L = load()
        self.ctx = C.c_void_p()
        check(self.L.st_create(device, C.byref(self.ctx)), None, "st_create (no GPU, or no device %d)" % device)
        self.params = None
        self.view = None
        self.scene = None
        if scene is not None:
            self.set_scene(scene, code=code)
            self.set_params(scene.params)
            self.set_view(scene.view)

    # ---- life cycle ----
    def close(self):
        if self.ctx:
            self.L.st_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- the scene, the settings, the camera ----
    def set_scene(self, scene, code=None):
        """RT.setScene(s). code: None, the scene's primitive table (the scene as data); True, the table written as
        code by codegen.generate and compiled for sm_103a; a string, that CUDA source (st_set_scene's contract).
        Returns NVRTC's milliseconds for it (0 for a table or a source compiled before). On failure the old scene is
        kept and StError says why."""
        if code is True:
            from .codegen import generate
            code = generate(scene)
        err = C.create_string_buffer(1 << 16)
        src = code.encode() if isinstance(code, str) else None
        rc = self.L.st_set_scene(self.ctx, src, C.byref(scene.desc), err, 1 << 16)
        if rc != 0:
            raise StError(rc, "setScene: " + err.value.decode(errors="replace"))
        self.scene = scene
        self.code = code
        return self.scene_code_info()["compile_ms"]

    def autotune(self, samples=2):
        """The autotuner (st_autotune): the queue tile and march chunk timed on this scene and view, the fastest kept.
        Returns {claim, chunk, ms, ms_default}."""
        t = T.StTune()
        check(self.L.st_autotune(self.ctx, int(samples), C.byref(t)), self.ctx, "st_autotune")
        return {f: getattr(t, f) for f, _ in T.StTune._fields_}

    def set_tune(self, claim=0, chunk=0):
        """The queue tile and march chunk set by hand (st_set_tune; 0 the defaults)."""
        t = T.StTune(claim=int(claim), chunk=int(chunk))
        check(self.L.st_set_tune(self.ctx, C.byref(t)), self.ctx, "st_set_tune")

    def scene_code_info(self):
        is_code, ms, nbytes = C.c_int(), C.c_double(), C.c_uint64()
        check(self.L.st_scene_code_info(self.ctx, C.byref(is_code), C.byref(ms), C.byref(nbytes)), self.ctx,
              "st_scene_code_info")
        return {"code": bool(is_code.value), "compile_ms": ms.value, "cubin_bytes": nbytes.value}

    def set_params(self, p):
        check(self.L.st_set_params(self.ctx, C.byref(p), None), self.ctx, "st_set_params")
        self.params = T.StParams.from_buffer_copy(p)

    def set_view(self, v):
        check(self.L.st_set_view(self.ctx, C.byref(v)), self.ctx, "st_set_view")
        self.view = v

    def set_views(self, views):
        """Many cameras of the scene rendered together (st_set_views): every step a sample of each, a picture each
        (read_accum(view=i))."""
        arr = (T.StView * len(views))(*views)
        check(self.L.st_set_views(self.ctx, arr, len(views)), self.ctx, "st_set_views")
        self.view = views[0]

    def set_env_image(self, rgb=None, luminance=0.0, turn=0.0):
        """The environment as an equirectangular image (envimage.js): `rgb` H x W x 3 linear floats, top row first,
        `luminance` cd/m^2 a unit (0: 179), turned `turn` degrees about z; None goes back to the sun and sky."""
        if rgb is None:
            check(self.L.st_set_env_image(self.ctx, None, 0, 0, 0.0, 0.0), self.ctx, "st_set_env_image")
            self.env_image = None
            return
        img = np.ascontiguousarray(rgb, dtype=np.float32)
        if img.ndim != 3 or img.shape[2] != 3:
            raise ValueError("the environment image is H x W x 3")
        h, w = img.shape[:2]
        check(self.L.st_set_env_image(self.ctx, img.ctypes.data_as(C.c_void_p), w, h, luminance, turn), self.ctx,
              "st_set_env_image")
        self.env_image = (img, luminance, turn)

    def set(self, reset=True, **values):
        """RT.set(values): applies the settings it knows, returns the names it does not (README.md:56)."""
        p = T.StParams.from_buffer_copy(self.params) if self.params else T.default_params()
        unknown = []
        for k, v in values.items():
            if k in PARAM_KEYS:
                setattr(p, k, v)
            else:
                unknown.append(k)
        self.set_params(p)
        return unknown

    def get(self):
        return {k: getattr(self.params, k) for k in PARAM_KEYS} if self.params else {}

    def invalidate(self):
        check(self.L.st_invalidate(self.ctx), self.ctx, "st_invalidate")

    # ---- tracing ----
    def step(self, n=1):
        check(self.L.st_step(self.ctx, int(n)), self.ctx, "st_step")

    def step_async(self, n=1):
        check(self.L.st_step_async(self.ctx, int(n)), self.ctx, "st_step_async")

    def sync(self, timeout_ms=-1):
        check(self.L.st_sync(self.ctx, int(timeout_ms)), self.ctx, "st_sync")

    # ---- readings ----
    def lt_counts(self):
        """Light tracing's connections that reached each pixel since the last invalidate (st_lt_counts), HxW."""
        W, H = self.params.width, self.params.height
        out = np.zeros((H, W), np.uint32)
        check(self.L.st_lt_counts(self.ctx, out.ctypes.data_as(C.c_void_p)), self.ctx, "st_lt_counts")
        return out

    def read_accum(self, view=0):
        """(rgb HxWx3, V HxW, S HxW, count HxW): the FP64 mean, the error bar's moments, the samples per pixel (of
        the view'th camera, with many)."""
        W, H = self.params.width, self.params.height
        rgb = np.zeros((H, W, 3), np.float64)
        V = np.zeros((H, W), np.float64)
        S = np.zeros((H, W), np.float64)
        cnt = np.zeros((H, W), np.uint32)
        P = C.c_void_p
        check(self.L.st_read_accum_view(self.ctx, int(view), rgb.ctypes.data_as(P), V.ctypes.data_as(P),
                                        S.ctypes.data_as(P), cnt.ctypes.data_as(P)), self.ctx, "st_read_accum_view")
        return rgb, V, S, cnt

    def checkpoint(self):
        """The render's state between samples (st_checkpoint_save): bytes a later resume() continues from."""
        n = C.c_size_t()
        check(self.L.st_checkpoint_size(self.ctx, C.byref(n)), self.ctx, "st_checkpoint_size")
        buf = C.create_string_buffer(n.value)
        check(self.L.st_checkpoint_save(self.ctx, buf, n.value), self.ctx, "st_checkpoint_save")
        return buf.raw

    def resume(self, blob):
        """Go on from a checkpoint of the same scene, settings and picture (st_checkpoint_load)."""
        buf = C.create_string_buffer(bytes(blob), len(blob))
        check(self.L.st_checkpoint_load(self.ctx, buf, len(blob)), self.ctx, "st_checkpoint_load")

    def image_stats(self):
        s = T.StImageStats()
        check(self.L.st_image_stats(self.ctx, C.byref(s)), self.ctx, "st_image_stats")
        return {f: getattr(s, f) for f, _ in T.StImageStats._fields_}

    def counters(self):
        c = T.StCounters()
        check(self.L.st_read_counters(self.ctx, C.byref(c)), self.ctx, "st_read_counters")
        out = {}
        for f, _ in T.StCounters._fields_:
            v = getattr(c, f)
            out[f] = list(v) if hasattr(v, "__len__") else v
        return out

    def measure(self, x, y):
        """The reading at pixel (x, y), row 0 the bottom (core/measure.js:56-66 reading): L, se, nEff, count."""
        rgb, V, S, cnt = self.read_accum()
        c = int(cnt[y, x])
        if not c:
            return None
        L = float(rgb[y, x] @ np.array([0.2126, 0.7152, 0.0722]))
        s, v = float(S[y, x]), float(V[y, x])
        se = float(np.sqrt(s * v / (1 - s))) if 0 < s < 1 and v >= 0 else None
        return {"L": L, "se": se, "nEff": 1.0 / s if s > 0 else None, "count": c, "rgb": rgb[y, x].tolist()}

    def mf_tables(self):
        ec = np.zeros(16 * 32 * 32, np.float32)
        ecavg = np.zeros(16 * 32, np.float32)
        e1 = np.zeros(32 * 32, np.float32)
        P = C.c_void_p
        check(self.L.st_mf_tables(self.ctx, ec.ctypes.data_as(P), ecavg.ctypes.data_as(P), e1.ctypes.data_as(P)),
              self.ctx, "st_mf_tables")
        return ec, ecavg, e1

    # ---- kernel times (core/kerneltime.js) ----
    def enable_kernel_times(self, on=True, count_work=False):
        mode = (2 if count_work else 1) if on else 0
        check(self.L.st_enable_kernel_times(self.ctx, mode), self.ctx, "st_enable_kernel_times")

    def kernel_times(self):
        buf = (T.StKernelTime * 32)()
        n = C.c_int()
        check(self.L.st_kernel_times(self.ctx, buf, 32, C.byref(n)), self.ctx, "st_kernel_times")
        return {buf[i].name.decode(): (buf[i].launches, buf[i].ms) for i in range(min(n.value, 32))}

    def reset_kernel_times(self):
        check(self.L.st_reset_kernel_times(self.ctx), self.ctx, "st_reset_kernel_times")

    def stream(self):
        return self.L.st_stream(self.ctx)

    # ---- emissive surfaces ----
    def emit_list(self):
        """The emitter list light sampling aims at: n x [centre xyz, radius, probability, running sum]."""
        out = np.zeros((64, 6), np.float32)
        n = C.c_uint32()
        check(self.L.st_emit_list(self.ctx, out.ctypes.data_as(C.c_void_p), 64, C.byref(n)), self.ctx, "st_emit_list")
        return out[:n.value]

    # ---- the learned proposal (st_params.guide; include/shadytracer.h st_mlp_*) ----
    def mlp_weights(self):
        """Every parameter, FP32: W1 (64x48), W2, W3 (64x64), W4 (40x64), then the hash grid's features."""
        w = np.zeros(T.MLP_PARAMS, np.float32)
        check(self.L.st_mlp_get_weights(self.ctx, w.ctypes.data_as(C.c_void_p), w.size), self.ctx, "st_mlp_get_weights")
        return w

    def set_mlp_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        check(self.L.st_mlp_set_weights(self.ctx, w.ctypes.data_as(C.c_void_p), w.size), self.ctx, "st_mlp_set_weights")

    def mlp_eval(self, pos, nrm):
        """The network at n points: (raw outputs n x 40, mixture n x 8 x [mean xyz, kappa, weight] as sampled)."""
        pos = np.ascontiguousarray(pos, np.float32)
        nrm = np.ascontiguousarray(nrm, np.float32)
        n = len(pos)
        raw = np.zeros((n, 40), np.float32)
        mix = np.zeros((n, 8, 5), np.float32)
        P = C.c_void_p
        check(self.L.st_mlp_eval(self.ctx, pos.ctypes.data_as(P), nrm.ctypes.data_as(P), n, raw.ctypes.data_as(P),
                                 mix.ctypes.data_as(P)), self.ctx, "st_mlp_eval")
        return raw, mix

    def mlp_grad(self, pos, nrm, dirs, weight):
        """The gradient of the training loss at a batch (no step): (gradient of every parameter, summed loss)."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in (pos, nrm, dirs, weight)]
        g = np.zeros(T.MLP_PARAMS, np.float32)
        loss = C.c_float()
        P = C.c_void_p
        check(self.L.st_mlp_grad(self.ctx, *[a.ctypes.data_as(P) for a in arrs], len(arrs[0]), g.ctypes.data_as(P),
                                 C.byref(loss)), self.ctx, "st_mlp_grad")
        return g, loss.value

    def mlp_train(self, pos, nrm, dirs, weight, steps, lr=0.0):
        """`steps` Adam steps on a given batch (what a wave's end does with its paths' records)."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in (pos, nrm, dirs, weight)]
        P = C.c_void_p
        check(self.L.st_mlp_train(self.ctx, *[a.ctypes.data_as(P) for a in arrs], len(arrs[0]), int(steps), float(lr)),
              self.ctx, "st_mlp_train")

    def mlp_batch(self):
        """The last wave's training batch: (n x 3 positions, normals, directions; n weights)."""
        out = np.zeros((131072, 10), np.float32)
        n = C.c_uint32()
        check(self.L.st_mlp_read_batch(self.ctx, out.ctypes.data_as(C.c_void_p), 131072, C.byref(n)), self.ctx,
              "st_mlp_read_batch")
        b = out[:n.value]
        return b[:, 0:3], b[:, 3:6], b[:, 6:9], b[:, 9]

    def mlp_stats(self):
        s = T.StMlpStats()
        check(self.L.st_mlp_stats_read(self.ctx, C.byref(s)), self.ctx, "st_mlp_stats_read")
        return {"steps": s.steps, "samples": s.samples, "loss": s.loss, "mean_weight": s.mean_weight,
                "box_lo": list(s.box_lo), "box_inv_ext": s.box_inv_ext, "inferred": s.inferred}


def create_path_tracer(scene=None, device=0, code=None):
    """createPathTracer (lib/pathtracer/index.js:90) + RT.init: a context on `device` with `scene` loaded (as code
    compiled for sm_103a when `code` is True or a source; PathTracer.set_scene)."""
    return PathTracer(scene, device, code=code)
