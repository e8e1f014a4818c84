"""bench.py -- the headline benchmark: Mpaths/s of the path-traced SDF room on one GB300.

Workload (the second of the reference's benchmark configurations): a 6 x 4 x 3 m room of 24 seeded SDF primitives
(boxes, spheres, tori, rounded prisms, smooth-unioned), GGX metal and plastic, a 100 klx sun and a sky through one
window; 1920 x 1080, 64 samples per pixel, max depth 8, march tolerance 1e-4 m, FP64 pixel tallies. One STEP is
the whole render -- 64 samples of every pixel, 132.7 M camera paths -- folded into the FP64 accumulation.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--small] [--spp S]
                    [--leg sppm|rmse|optics|mlp|emit|haze|env|sc]   # one leg alone, its JSON printed

value: paths / s with the scene resident on the GPU (graph replays; the timed region brackets K renders with a
       synchronize), the reference's step cache on (one look, 16 M cells; `step_cache` below has it off too). e2e: the same through the C ABI as a host calls it -- scene, settings and camera uploaded from
       host memory, the render, and the FP64 picture and its error bar read back to host memory, every step.
roofline: the march kernel (the dominant one), FP32 arithmetic: the fold's work counted on the device in a counting
       pass (evaluations by primitive type and fold operation, bounding-sphere tests, steps; one more render of the
       same seeds through an instrumented march), weighed by FP32 operations (shadytracer_gb300/flops.py), per
       launch, over the plain kernel's average CUDA-event time on the library's stream (a second pass over the same
       K renders with per-kernel events on).
cpu_baseline: the oracle (oracle/, the CPU restatement of the reference's path) in f32 on every host core, over a
       bounded band of the same picture's paths.
--impl reference: the reference's own implementation cannot run here (JavaScript + WGSL through WebGPU); its CPU
       restatement, the oracle, is timed instead on the host's cores, on the same workload and metric.
sppm: the photon map's caustic (1024^2, 4 M sun photons a pass, 64 passes): photons/s over the photon
       pass's kernels, and the render's paths/s with the map on.
time_to_rmse: seconds to 1 % relative RMSE against a closed form, the photon map guided by the learned emission map
       vs plain.
optics: the batched optics bench (64 emitter + aspheric-lens instances, 120.2 M rays, FP64 far-field and lux
       tallies) in rays/s, with the tallies on the device (`value`) and read back every run (`e2e`).
mlp: the learned proposal (a BF16 network guiding BSDF sampling): relative RMSE and GPU time, plain against guided,
       on the diffuse room lit by the sun's patch; the network's inference and training flops a second.
emit: emissive surfaces: a sphere lamp over a floor (its closed form): Mpaths/s with the discovered lamp light-sampled,
       and the relative RMSE with and without that light sample at equal samples.
haze_beam: the haze-box beam (a 10-degree 1000 lm spot, a light face, through 2 x 2 x 4 m of albedo-1 haze;
       1280 x 720, 256 samples, 32 bounces) at each of its nine (sigma_s, g) cells: Mpaths/s per cell and overall.
env: the environment image's map: a floor under a panorama with one small bright patch (its closed form), the relative
       RMSE with the map's light samples and with the cosine lobe's alone at equal samples.
step_cache: the headline room with the reference's step cache off, on one cell and on three: Mpaths/s and the scene
       distance evaluations a path.
Multi-GPU (torchrun): replicas -- each rank renders the whole workload on its own GPU; value sums the ranks' paths
       over the slowest rank's time (weak scaling). There is no data exchange in the path tracer.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="a 480 x 270, 4-spp render (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-optics", action="store_true", help="skip the optics bench's rays/s leg")
    ap.add_argument("--no-sppm", action="store_true", help="skip the photon map's photons/s leg")
    ap.add_argument("--spp", type=int, default=0, help="samples per pixel a step (profiling runs; default: 64)")
    ap.add_argument("--no-mlp", action="store_true", help="skip the learned proposal's leg")
    ap.add_argument("--no-emit", action="store_true", help="skip the emissive surfaces' leg")
    ap.add_argument("--no-haze", action="store_true", help="skip the haze-box beam's leg")
    ap.add_argument("--no-env", action="store_true", help="skip the environment image's leg")
    ap.add_argument("--no-sc", action="store_true", help="skip the step cache's leg")
    ap.add_argument("--tune", default="", help="CLAIM,CHUNK: set by hand, no autotuner (profiling runs)")
    ap.add_argument("--leg", default="all", choices=["all", "sppm", "rmse", "caustic_rmse", "optics", "mlp", "emit",
                                                     "haze", "env", "sc", "views"],
                    help="run one leg alone and print its JSON (profiling runs of the photon map or the optics bench)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(x, dist=None, device="cpu"):
    """The largest of every rank's x -- the slowest rank's time -- over the process group (x itself with none)."""
    if not dist:
        return float(x)
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, paths_per_step, ms):
    """Replicas (weak scaling): every rank renders the whole workload, so the job's paths a second are the ranks'
    paths over the slowest rank's time, in millions."""
    return world * paths_per_step / (ms / 1e3) / 1e6


def workload(small, spp=0):
    """The room as the reference renders it by default: its scene as code (the builder's generated SDF, here
    codegen.py's CUDA compiled by NVRTC for sm_103a at st_set_scene), the step cache off (the reference's developer
    setting; the scene_forms leg measures it on), lit by the physical sun and sky (the reference's default
    environment, environment.js; a 100 klx sun 35 degrees up)."""
    from shadytracer_gb300 import scenes
    if small:
        s = scenes.sdf_room(width=480, height=270, spp=spp or 4, maxbounce=8, sky="physical")
    else:
        s = scenes.sdf_room(width=1920, height=1080, spp=spp or 64, maxbounce=8, sky="physical")
    s.params.step_cache = 0
    return s


def scene_code(s):
    from shadytracer_gb300 import codegen
    return codegen.generate(s)


def config_of(s):
    p = s.params
    return {"workload": "room24 SDF room %dx%d, %d spp, max depth %d, eps 1e-4 m" % (p.width, p.height,
                                                                                     s.info["spp"], p.maxbounce),
            "width": p.width, "height": p.height, "spp": s.info["spp"], "maxbounce": p.maxbounce,
            "paths_per_step": p.width * p.height * s.info["spp"], "primitives": 24,
            "environment": s.info.get("sky", "a 100 klx sun disc and a uniform sky of 10 klx on the level"),
            "scene": "code: codegen.py's CUDA for the room, compiled by NVRTC for sm_103a at st_set_scene",
            "step_cache": ("%d look%s, %g M cells" % (1 if p.step_cache == 1 else 3, "" if p.step_cache == 1 else "s",
                                                    p.step_cache_cells or 4.0)) if p.step_cache else "off",
            "l2": "working set above L2: path state + queues of 2.07 M paths are 300 MB a wave (> 129 MB L2)"}


# ---------------------------------------------------------------------------------------------------------------
# clocks during the timed region (nvidia-smi sampled every 200 ms)
# ---------------------------------------------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]) if f[3] not in ("[N/A]", "N/A") else 0.0, f[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [r for r in rows if r[2] > 200] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in load])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


# ---------------------------------------------------------------------------------------------------------------
# the CPU baseline: the oracle in f32 over a band of the picture's paths, all host threads
# ---------------------------------------------------------------------------------------------------------------
def cpu_baseline(s, budget_s=15.0):
    """The oracle in f32 with the reference's bounding-box culling at the root (the work the reference's generated
    code does a step, builder/codegen.js:2141-2193), every host thread, bands of the picture's paths."""
    from oracle import oracle
    threads = os.cpu_count() or 1
    p = s.params
    P = p.width * p.height
    acc = oracle.Accum(p.width, p.height)
    # bands of consecutive paths from the middle of the picture outwards, one sample each, until the budget is spent
    band = min(P, 16384)
    oracle.render(s, 1, acc, fp64=False, threads=threads, sample0=0, path_first=P // 2, path_count=band,
                  cull=True)  # warm
    first0 = P // 2
    n, k = 0, 0
    t = time.perf_counter()
    while True:
        first = (first0 + k * band) % max(P - band, 1)
        oracle.render(s, 1, acc, fp64=False, threads=threads, sample0=1, path_first=first, path_count=band, cull=True)
        n += band
        k += 1
        dt = time.perf_counter() - t
        if dt >= budget_s or k * band >= P:
            break
    return {"value": n / dt / 1e6, "unit": "Mpaths/s", "cores": threads, "kind": "port",
            "sample": "%d paths of sample 1 (%d bands of %d consecutive paths from row %d on, %dx%d), %.1f s; f32, the "
                      "reference's root bounding-box cull" % (n, k, band, first0 // p.width, p.width, p.height, dt)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    s = workload(args.small, args.spp)
    metric = "Mpaths/s"
    for _ in range(max(args.warmup, 0)):
        cpu_baseline(s, budget_s=3.0)
    vals, samples = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cb = cpu_baseline(s, budget_s=10.0)
        vals.append(cb["value"])
        samples.append(cb["sample"])
    dt = time.perf_counter() - t0
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": metric, "value": v, "unit": "Mpaths/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(config_of(s), scene="the reference's fold: every top-level group culled by its box "
                                              "where it is farther than ten tolerances (its generated code's work)"),
            "cpu_baseline": {"value": v, "unit": "Mpaths/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "each step: " + samples[-1]},
            "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference is JavaScript + WGSL run by WebGPU (no JS runtime or graphics stack here); its "
                    "path is timed through the oracle, its CPU restatement, on every host core"}
    print(json.dumps(line), flush=True)
    return 0


def optics_leg(args, dev, with_cpu):
    """The batched optics bench (64 emitter + aspheric-lens instances, log-uniform ray counts from PCG32(5): 120.2 M
    rays; far field 1 x 1 degree, lux 512 x 512 at 1 m, FP64 tallies) in rays/s: `value` with the tallies left on
    the device, `e2e` with every instance's far field and lux map read back to host memory each run."""
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.optics import Optics
    from shadytracer_gb300.renderer import create_path_tracer
    # --small: the same 64 instances at a tenth of the rays (12 M), a profiling case still larger than L2
    b = scenes.optics_bench(n_instances=64, seed=5, ray_scale=0.1 if args.small else 1.0)
    rays = b.info["rays"]
    total = int(sum(rays))
    rt = create_path_tracer(b, device=dev)
    O = Optics(rt)
    O.set_sources(b.info["sources"])
    O.set_far(nC=360, nG=181)
    L = rt.L
    n = len(rays)
    rc = (C.c_uint32 * n)(*rays)
    from shadytracer_gb300 import st_types as T
    batch = T.StOpticsBatch()
    batch.n_instances, batch.ray_count = n, C.cast(rc, C.POINTER(C.c_uint32))
    batch.lux_cells, batch.lux_half, batch.lux_height, batch.maxbounce, batch.seed = 512, 1.0, 1.0, 32, 1
    tot = (T.StOpticsTotals * n)()
    far = np.zeros((n, 181, 360))
    lux = np.zeros((n, 512, 512))

    def run(out):
        f = far.ctypes.data_as(C.c_void_p) if out else None
        x = lux.ctypes.data_as(C.c_void_p) if out else None
        r = L.st_optics_run(rt.ctx, C.byref(batch), f, x, tot)
        if r != 0:
            raise RuntimeError(L.st_last_error(rt.ctx))

    tune = O.autotune(rays, lux_cells=512, lux_half=1.0, lux_height=1.0, maxbounce=32, seed=1)
    for _ in range(max(args.warmup, 3)):
        run(False)
    K = max(args.steps, 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        run(False)
    torch.cuda.synchronize()
    dev_s = (time.perf_counter() - t0) / K
    t0 = time.perf_counter()
    for _ in range(K):
        run(True)
    e2e_s = (time.perf_counter() - t0) / K
    emitted = sum(tot[i].emitted for i in range(n))
    escaped = sum(tot[i].escaped for i in range(n))
    out = {"workload": "optics bench: %d LED die + aspheric lens instances, %d rays (log-uniform per instance), far "
                       "field 360 x 181, lux 512 x 512 at 1 m, FP64 tallies" % (n, total),
           "metric": "rays/s", "value": total / dev_s, "unit": "rays/s", "ms_per_run": 1e3 * dev_s,
           "e2e": {"value": total / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": 4 * n + C.sizeof(batch),
                   "d2h_bytes_per_step": int(far.nbytes + lux.nbytes + C.sizeof(tot))},
           "autotune": {"claim": tune["claim"], "chunk": tune["chunk"],
                        "speedup_over_defaults": tune["ms_default"] / tune["ms"] if tune["ms"] else None},
           "graph": "the batch's whole chain replayed as one CUDA graph",
           "interactions_per_ray": sum(tot[i].interactions for i in range(n)) / max(total, 1),
           "escaped_share": escaped / max(emitted, 1)}
    rt.close()
    if with_cpu:
        from oracle import oracle
        import os as _os
        sub = [2000000] * 4
        o_t = time.perf_counter()
        oracle.optics_run(b, sub, nC=360, nG=181, cells=0, maxbounce=32, seed=1, threads=_os.cpu_count() or 1)
        dt = time.perf_counter() - o_t
        out["cpu_baseline"] = {"value": sum(sub) / dt, "unit": "rays/s", "cores": _os.cpu_count(), "kind": "port",
                               "sample": "instances 0-3 of the same batch, 2 M rays each, far field only, %.1f s" % dt}
    return out


def sppm_leg(args, dev, with_cpu):
    """The photon map's caustic: a dispersive glass sphere on a floor under the sun, 1024 x 1024, 4 M sun photons a
    pass, r1 5 mm, alpha 0.7, 64 passes a render. `value`: photons/s over the photon pass's kernels (their CUDA-event
    time: generation, sort, march, surface, store); `render`: the whole render's camera paths/s with the map on."""
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    small = args.small
    W = 256 if small else 1024
    N = 250_000 if small else 4_000_000
    passes = 8 if small else 64
    s = scenes.sppm_caustic(width=W, height=W, photons=N, r1=0.005, alpha=0.7)
    rt = create_path_tracer(s, device=dev, code=True)
    stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
    for _ in range(max(args.warmup, 3)):
        rt.invalidate()
        rt.step_async(2)
        rt.sync()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    rt.invalidate()
    e0.record(stream)
    rt.step_async(passes)
    e1.record(stream)
    rt.sync()
    render_ms = e0.elapsed_time(e1)
    Lmean = float((rt.read_accum()[0] @ np.array([0.2126, 0.7152, 0.0722])).mean())
    # the photon pass's own kernels, from per-kernel events over a few passes
    rt.enable_kernel_times(True)
    rt.reset_kernel_times()
    rt.invalidate()
    kp = 4
    rt.step(kp)
    kt = rt.kernel_times()
    rt.enable_kernel_times(False)
    ph_keys = ("photons", "photon_sort", "photon_march", "photon_surface", "photon_shade")
    ph_ms = sum(kt.get(k, (0, 0.0))[1] for k in ph_keys)
    tot_ms = sum(v[1] for v in kt.values()) or 1.0
    import ctypes as _C
    from shadytracer_gb300.st_types import StSppmStats
    stt = StSppmStats()
    rt.L.st_sppm_stats_read(rt.ctx, _C.byref(stt))
    rt.close()
    out = {"workload": "sppm caustic: glass sphere r 0.3 m (Cauchy 1.50 + 0.0042/um^2) on a floor (albedo 0.7) under "
                       "the sun, %dx%d, %d sun photons a pass, r1 5 mm, alpha 0.7, %d passes" % (W, W, N, passes),
           "metric": "photons/s", "value": N * kp / (ph_ms / 1e3) if ph_ms > 0 else None, "unit": "photons/s",
           "photon_pass_share": ph_ms / tot_ms,
           "render": {"metric": "Mpaths/s (with the photon pass)", "value": W * W * passes / (render_ms / 1e3) / 1e6,
                      "ms_per_render": render_ms, "passes": passes, "photons_per_s_whole": N * passes / (render_ms / 1e3)},
           "stored_per_pass": stt.stored, "dropped": stt.cut, "mean_luma": Lmean,
           "kernel_share": {k: round(v[1] / tot_ms, 4) for k, v in kt.items()}}
    if with_cpu:
        # the oracle on every host thread over whole passes -- the sun's photons traced and stored, the grid built,
        # the camera's paths traced and gathered -- against the GPU's whole-render photons a second
        from oracle import oracle
        import os as _os
        Wc = 256
        Nc = N * Wc * Wc // (W * W)              # the same photons a camera path as the GPU's render
        sc = scenes.sppm_caustic(width=Wc, height=Wc, photons=Nc, r1=0.005, alpha=0.7)
        threads = _os.cpu_count() or 1
        oracle.render(sc, 1, threads=threads)                       # warm
        t0 = time.perf_counter()
        k = 0
        while True:
            oracle.render(scenes.sppm_caustic(width=Wc, height=Wc, photons=Nc, r1=0.005, alpha=0.7), 1,
                          threads=threads, sample0=k)
            k += 1
            if time.perf_counter() - t0 > 10.0 or k >= 8:
                break
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": Nc * k / dt, "unit": "photons/s (whole passes)", "cores": threads,
                               "kind": "port", "compare_to": "render.photons_per_s_whole",
                               "sample": "%d whole passes of the caustic at %dx%d with %d sun photons a pass (trace, "
                                         "store, grid, camera paths, gather), every host thread, %.1f s"
                                         % (k, Wc, Wc, Nc, dt)}
    return out


MLP_FWD_FLOPS = 2 * (48 * 64 + 64 * 64 + 64 * 64 + 40 * 64)     # 27 648 a vertex: 13 824 BF16 multiply-adds
MLP_TRAIN_FLOPS = 3 * MLP_FWD_FLOPS                               # forward, backward to the inputs, weight GEMM


def mlp_leg(args, dev):
    """The learned proposal, plain and guided (trained online from the first wave), 160 x 90, relative RMSE and GPU time
    at 1024 samples against a plain render of 8192 on seeds of its own, on two rooms: the diffuse room lit by the sun's
    patch alone (sky almost black: the light every vertex sees is indirect) and the headline's room as configured (the
    physical sun and sky through the window, the mixed finish: the sky's light through the window is what light
    sampling's cosine draw finds worst); the network's inference and training on the first."""
    W, H = (96, 54) if args.small else (160, 90)
    ref_spp, spp = (1024, 256) if args.small else (8192, 1024)
    out = {"metric": "relative RMSE at equal samples", "workloads": {}}
    for name, kw in (("diffuse_sun_patch", dict(finish="diffuse", sky_illuminance=10.0, ground_luminance=1.0)),
                     ("configured", dict(sky="physical"))):
        out["workloads"][name] = mlp_workload(args, dev, W, H, spp, ref_spp, kw, stats=name == "diffuse_sun_patch")
    d = out["workloads"]["diffuse_sun_patch"]
    for k in ("legs", "rmse_ratio_guided_over_plain", "time_ratio_guided_over_plain", "speedup_to_equal_rmse", "workload"):
        out[k] = d[k]
    out["speedup_to_equal_rmse_configured"] = out["workloads"]["configured"]["speedup_to_equal_rmse"]
    return out


def mlp_workload(args, dev, W, H, spp, ref_spp, kw, stats):
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    luma = np.array([0.2126, 0.7152, 0.0722])

    def scene(guide):
        s = scenes.sdf_room(width=W, height=H, spp=spp, **kw)
        s.params.guide = guide
        return s
    # the reference on seeds of its own: a plain run on the same seeds would share its first samples with it and read
    # an error too small by the shared part (at 1024 of 8192 samples, a variance 0.875 of its true one against 1.125
    # for any run on other numbers)
    ref = scene(0)
    ref.params.seed = 7919
    rt = create_path_tracer(ref, device=dev, code=True)
    left = ref_spp
    while left > 0:
        rt.step(min(512, left))
        left -= 512
    rgb, V, S, cnt = rt.read_accum()
    Lref = rgb @ luma
    ok = (S > 0) & (S < 1)
    se2 = np.zeros_like(V)
    se2[ok] = S[ok] * V[ok] / (1 - S[ok])
    ref_noise = float(np.mean(se2))                 # the reference's own variance, taken out of each run's error
    rt.close()
    out = {"workload": "room24 %s, %dx%d, %d samples against a %d-sample plain render on seeds of its own (its own "
                       "noise taken out)" % (", ".join("%s=%s" % kv for kv in kw.items()), W, H, spp, ref_spp),
           "legs": {}}
    for guide in (0, 1):
        rt = create_path_tracer(scene(guide), device=dev, code=True)
        stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rt.invalidate()
        e0.record(stream)
        rt.step_async(spp)
        e1.record(stream)
        rt.sync()
        L = rt.read_accum()[0] @ luma
        leg = {"rmse": float(np.sqrt(max(np.mean((L - Lref) ** 2) - ref_noise, 0.0)) / Lref.mean()),
               "ms": e0.elapsed_time(e1)}
        if guide and stats:
            st = rt.mlp_stats()
            rt.enable_kernel_times(True)
            rt.reset_kernel_times()
            rt.step(64)
            kt = rt.kernel_times()
            st2 = rt.mlp_stats()
            rt.enable_kernel_times(False)
            n_i, ms_i = kt.get("guide", (0, 0.0))
            n_t, ms_t = kt.get("guide_train", (0, 0.0))
            waves = max(kt.get("resolve", (1, 0.0))[0], 1)
            inferred = st2["inferred"] * waves              # the last wave's count, each wave alike
            pk = peaks()
            peak = pk.get("bf16_tflops") if pk else None
            tf_i = MLP_FWD_FLOPS * inferred / (ms_i / 1e3) / 1e12 if ms_i > 0 else None
            tf_t = MLP_TRAIN_FLOPS * st2["samples"] * waves / (ms_t / 1e3) / 1e12 if ms_t > 0 else None
            leg.update({"train_steps": st["steps"], "loss": st["loss"],
                        "infer": {"launches": n_i, "ms": ms_i, "vertices": inferred, "tflops": tf_i,
                                  "frac_of_bf16_peak": tf_i / peak if (tf_i and peak) else None},
                        "train": {"waves": waves, "ms": ms_t, "samples_per_wave": st2["samples"], "tflops": tf_t},
                        "share_of_render": (ms_i + ms_t + kt.get("guide_collect", (0, 0.0))[1]) /
                                           max(sum(v[1] for v in kt.values()), 1e-9)})
        out["legs"]["guided" if guide else "plain"] = leg
        rt.close()
    out["rmse_ratio_guided_over_plain"] = out["legs"]["guided"]["rmse"] / out["legs"]["plain"]["rmse"]
    out["time_ratio_guided_over_plain"] = out["legs"]["guided"]["ms"] / out["legs"]["plain"]["ms"]
    # at equal time the guided render's RMSE would scale by sqrt(time ratio): the speed-up to equal error
    out["speedup_to_equal_rmse"] = 1.0 / (out["rmse_ratio_guided_over_plain"] ** 2 * out["time_ratio_guided_over_plain"])
    return out


def emit_leg(args, dev):
    """Emissive surfaces: a sphere lamp over a floor in the dark (its closed form, albedo Le a^2 h / D^3), 480 x 320,
    256 samples: camera paths a second with the discovered lamp light-sampled, and the relative RMSE against the closed
    form with the light sample and with the BSDF's hits alone, at equal samples and their GPU times."""
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    W, H = (192, 128) if args.small else (480, 320)
    spp = 64 if args.small else 256
    out = {"workload": "lamp-floor: a 0.1 m sphere of 1000 cd/m^2 at 1 m over a 0.8 floor, black environment, %dx%d, "
                       "%d samples" % (W, H, spp), "metric": "Mpaths/s", "legs": {}}
    luma = np.array([0.2126, 0.7152, 0.0722])
    for off in (0, 1):
        s = scenes.lamp_floor(width=W, height=H, spp=spp)
        s.params.emit_off = off
        cf, ok = scenes.lamp_floor_pixels(s)
        rt = create_path_tracer(s, device=dev, code=True)
        stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
        for _ in range(max(args.warmup, 3)):
            rt.invalidate()
            rt.step(spp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rt.invalidate()
        e0.record(stream)
        rt.step_async(spp)
        e1.record(stream)
        rt.sync()
        ms = e0.elapsed_time(e1)
        L = rt.read_accum()[0] @ luma
        out["legs"]["bsdf_only" if off else "light_sampled"] = {
            "ms": ms, "Mpaths_per_s": W * H * spp / (ms / 1e3) / 1e6,
            "rmse": float(np.sqrt(np.mean((L[ok] - cf[ok]) ** 2)) / cf[ok].mean()),
            "mean_over_closed_form": float(L[ok].sum() / cf[ok].sum()), "listed": int(len(rt.emit_list()))}
        rt.close()
    a, b = out["legs"]["light_sampled"], out["legs"]["bsdf_only"]
    out["value"] = a["Mpaths_per_s"]
    out["speedup_to_equal_rmse"] = (b["rmse"] / a["rmse"]) ** 2 * (b["ms"] / a["ms"])
    return out


def haze_leg(args, dev):
    """The haze-box beam: a 2 x 2 x 4 m box of albedo-1 haze crossed by a 10-degree, 1000 lm spot (a 5 cm light face
    below it), 1280 x 720, 256 samples, 32 bounces, at each of the nine cells sigma_s in {0.05, 0.2, 1.0} per metre x
    g in {0, 0.7, 0.9}: camera paths a second per cell (CUDA events around one render), and over the nine."""
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    W, H = (320, 180) if args.small else (1280, 720)
    spp = 16 if args.small else 256
    out = {"workload": "haze-beam: 2x2x4 m albedo-1 haze, 10 deg 1000 lm spot (5 cm face), %dx%d, %d samples, "
                       "32 bounces" % (W, H, spp), "metric": "Mpaths/s", "cells": {}}
    tot_paths, tot_ms = 0, 0.0
    for sig in (0.05, 0.2, 1.0):
        for g in (0.0, 0.7, 0.9):
            s = scenes.haze_beam(width=W, height=H, sigma_s=sig, g=g)
            rt = create_path_tracer(s, device=dev, code=True)
            stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
            rt.step(4)                                # the wave's buffers and graphs
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            rt.invalidate()
            e0.record(stream)
            rt.step_async(spp)
            e1.record(stream)
            rt.sync()
            ms = e0.elapsed_time(e1)
            c = rt.counters()
            L = rt.read_accum()[0] @ np.array([0.2126, 0.7152, 0.0722])
            out["cells"]["sigma%g_g%g" % (sig, g)] = {
                "ms": ms, "Mpaths_per_s": W * H * spp / (ms / 1e3) / 1e6, "mean_luminance": float(L.mean()),
                "segments_per_path": c["segments"] / max(c["paths"], 1), "nonfinite": c["nonfinite"]}
            tot_paths += W * H * spp
            tot_ms += ms
            rt.close()
    out["value"] = tot_paths / (tot_ms / 1e3) / 1e6
    return out


def env_leg(args, dev):
    """The environment image's map: a Lambertian floor under a panorama that is dim but for one small bright patch
    (its closed form, albedo / pi times the upper half's illuminance), 256 x 256, 128 samples: camera paths a second
    and the relative RMSE against the closed form with the map's light samples and with the cosine lobe's alone, at
    equal samples, and the speed-up to equal error."""
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    W = 128 if args.small else 256
    spp = 32 if args.small else 128
    img = scenes.env_patch_image(patch=20000.0, size=3)
    cf = 0.8 / np.pi * scenes.env_level_illuminance(img)
    out = {"workload": "env-floor: 0.8 floor under a 256x128 panorama of 179 cd/m^2 with a 3x3-pixel patch of "
                       "3.58 Mcd/m^2, %dx%d, %d samples" % (W, W, spp), "metric": "Mpaths/s", "legs": {}}
    for off in (0, 1):
        s = scenes.env_floor(width=W, height=W)
        s.params.env_map_off = off
        rt = create_path_tracer(s, device=dev, code=True)
        rt.set_env_image(img)
        stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
        for _ in range(max(args.warmup, 3)):
            rt.invalidate()
            rt.step(spp)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rt.invalidate()
        e0.record(stream)
        rt.step_async(spp)
        e1.record(stream)
        rt.sync()
        ms = e0.elapsed_time(e1)
        L = rt.read_accum()[0] @ np.array([0.2126, 0.7152, 0.0722])
        out["legs"]["lobe_only" if off else "map"] = {
            "ms": ms, "Mpaths_per_s": W * W * spp / (ms / 1e3) / 1e6,
            "rmse": float(np.sqrt(np.mean((L - cf) ** 2)) / cf), "mean_over_closed_form": float(L.mean() / cf)}
        rt.close()
    a, b = out["legs"]["map"], out["legs"]["lobe_only"]
    out["value"] = a["Mpaths_per_s"]
    out["speedup_to_equal_rmse"] = (b["rmse"] / a["rmse"]) ** 2 * (b["ms"] / a["ms"])
    return out


def sc_leg(args, dev):
    """The scene's two forms and the step cache (the reference's developer setting, wavefront.js:67-150): the headline
    room at its full size and samples as a primitive table (the scene as data, a loop over the table in shared memory)
    and as code (codegen.py's CUDA, NVRTC), each with the cache off and on (one look, 16 M cells) -- paths a second
    (CUDA events around one render after a warm-up render) and the scene-distance evaluations a path."""
    import torch
    from shadytracer_gb300.renderer import create_path_tracer
    s = workload(args.small, args.spp)
    spp = s.info["spp"]
    P = s.params.width * s.params.height
    out = {"workload": "the headline room as a table and as code, the step cache off and on",
           "metric": "Mpaths/s", "modes": {}}
    for form in ("table", "code"):
        for mode, cells in ((0, 4.0), (1, 16.0)):
            s.params.step_cache = mode
            s.params.step_cache_cells = cells
            rt = create_path_tracer(s, device=dev, code=True if form == "code" else None)
            stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
            rt.step(spp)
            c0 = rt.counters()["march_steps"]
            rt.invalidate()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rt.step_async(spp)
            e1.record(stream)
            rt.sync()
            ms = e0.elapsed_time(e1)
            evals = rt.counters()["march_steps"] - c0
            out["modes"]["%s_%s" % (form, "cache_off" if mode == 0 else "cache_1look_16M")] = {
                "ms": ms, "Mpaths_per_s": P * spp / (ms / 1e3) / 1e6, "evals_per_path": evals / (P * spp)}
            rt.close()
    s.params.step_cache = 0
    s.params.step_cache_cells = 0.0
    m = out["modes"]
    out["code_over_table"] = m["code_cache_off"]["Mpaths_per_s"] / m["table_cache_off"]["Mpaths_per_s"]
    out["value"] = max(v["Mpaths_per_s"] for v in m.values())
    return out


def views_leg(args, dev):
    """Many views in one wavefront (st_set_views): four cameras of the headline room at 960 x 540, 16 samples each,
    rendered together in the same waves, against the four rendered one after another -- paths a second (CUDA events
    around the renders after a warm-up), the pictures the same."""
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    W, H, spp = (240, 135, 8) if args.small else (960, 540, 16)
    s = scenes.sdf_room(width=W, height=H, spp=spp, maxbounce=8, sky="physical")
    s.params.step_cache = 0
    views = [scenes.look_at(e, t, 60.0, W / H) for e, t in (((-2.6, -1.6, 1.7), (0.8, 0.9, 1.1)),
                                                              ((2.5, -1.7, 1.5), (-0.5, 0.8, 0.8)),
                                                              ((0.0, 1.6, 2.6), (0.0, -0.5, 0.3)),
                                                              ((-2.5, 1.5, 1.2), (1.0, -0.5, 1.0)))]
    paths = len(views) * W * H * spp
    rt = create_path_tracer(s, device=dev, code=True)
    stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))

    def timed(run):
        run()
        rt.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        rt.sync()
        return e0.elapsed_time(e1)

    def together():
        rt.set_views(views)
        rt.step_async(spp)

    def apart():
        for v in views:
            rt.set_views([v])
            rt.step(spp)                  # (a view's settings change only between traces)
    ms_t = timed(together)
    ms_a = timed(apart)
    rt.close()
    return {"workload": "the headline room from 4 cameras, %dx%d, %d samples each" % (W, H, spp), "metric": "Mpaths/s",
            "together": {"ms": ms_t, "Mpaths_per_s": paths / ms_t / 1e3},
            "one_after_another": {"ms": ms_a, "Mpaths_per_s": paths / ms_a / 1e3},
            "speedup": ms_a / ms_t, "value": paths / ms_t / 1e3}


def rmse_leg(args, dev):
    """Time to 1 % relative RMSE against the closed form, guided vs plain: the photon map's pane (a 0.5 m glass pane
    over a floor lit only through it, the sun's photons drawn over a 4 m square), plain -- the photons uniform over the
    square -- against guided -- drawn from the learned emission map (rebuilt every 4 passes from each cell's stores per
    photon). RMSE over the picture's pixels of (L - closed form) / closed form; GPU time of the passes (CUDA events),
    checked every 8 passes (every 64 past 512), up to 12288 passes."""
    import torch
    from oracle import oracle as _o        # the closed form's Fresnel term only (the checker's), not the path
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    W = 64 if args.small else 128
    N = 1_000_000 if args.small else 4_000_000
    out = {"metric": "seconds to 1% relative RMSE vs the closed form", "unit": "s", "higher_is_better": False,
           "workload": "sppm pane: 0.5 m pane 0.5 m over a floor lit only through it, sun at 75 deg, %dx%d, %d sun "
                       "photons a pass over a 4 m square, r1 5 mm, alpha 0.7" % (W, W, N)}
    for name, learn in (("plain", 0), ("guided", 1)):
        s = scenes.sppm_pane(width=W, height=W, photons=N, r1=0.005, alpha=0.7, sun_elevation=75.0, pane_half=0.25,
                             photon_half=2.0, vfov=3.5)
        s.params.sppm_learn = learn
        cf = scenes.sppm_pane_closed_form(s, _o.fresnel_dielectric)
        rt = create_path_tracer(s, device=dev, code=True)
        stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
        rt.step(1)                                    # the graph captured
        rt.invalidate()
        ms, passes, rm, hit = 0.0, 0, None, None
        curve = []
        while passes < 12288:
            k = 8 if passes < 512 else 64
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rt.step_async(k)
            e1.record(stream)
            rt.sync()
            ms += e0.elapsed_time(e1)
            passes += k
            L = rt.read_accum()[0] @ np.array([0.2126, 0.7152, 0.0722])
            rm = float(np.sqrt(np.mean((L - cf) ** 2)) / cf)
            if passes in (8, 32, 128, 512, 2048, 8192) or rm <= 0.01:
                curve.append([passes, round(ms / 1e3, 3), round(rm, 4)])
            if rm <= 0.01:
                hit = ms / 1e3
                break
        rt.close()
        out[name] = {"seconds": hit, "passes": passes, "rmse": rm, "curve": curve}
    if out["plain"]["seconds"] and out["guided"]["seconds"]:
        out["speedup"] = out["plain"]["seconds"] / out["guided"]["seconds"]
    return out


# the march's DRAM traffic per scene evaluation: ncu's dram__bytes_read.sum + dram__bytes_write.sum over the 26 march
# launches of one render of the room at 1920 x 1080, 2 samples (claim 32, chunk 24), over that render's evaluations
# as the counting pass finds them (15.54 GB / 1.127 G); scaled by each launch's evaluations: the path state a ray's
# refill and hand-off move, spread over its steps (the scene itself is code)
MARCH_DRAM_BYTES_PER_EVAL = 13.8
MARCH_DRAM_PROFILE = "profiles/launches-room24-code-1920x1080-2spp.md"


def caustic_rmse_leg(args, dev):
    """Time to 1 % relative RMSE on the caustic as configured (1024^2, 4 M sun photons a pass, r1 5 mm, alpha 0.7),
    four ways: the photon map alone with the sun's photons uniform over their square ("plain") or drawn from the
    learned 128^2 emission map ("guided"), and the reference's own split -- light tracing to the camera for the caustic
    seen directly, the map past glass from the eye -- uniform ("lt") or guided ("lt_guided", the map then taught by
    the connections, as the reference's is).

    Against an FP64-accumulated render of 16 x the runs' passes of the split, on seeds of its own (no pass of it is a
    pass of a run). The RMSE over the pixels of the luminance's difference, less the reference's own variance (its
    pixels' squared standard errors), over the reference's mean; over the pixels the reference has converged on (its
    standard error within 10 % of its value, and below its 99.9th percentile: a camera path that reaches the sun's disc
    through glass along a line the photons' square does not cover is a single sample of ~1e9 cd/m^2 in a pixel, in any
    of the four), the largest 0.1 % of each run's squared differences left out (the same rare paths of its own). The
    passes are timed with CUDA events; past the first checks the error is the noise's, falling as passes^-1/2, so the
    time to 1 % is the last check's time x (RMSE / 1 %)^2 -- and the ratio of two arms' is their efficiency's."""
    import torch
    from shadytracer_gb300 import scenes
    from shadytracer_gb300.renderer import create_path_tracer
    W = 256 if args.small else 1024
    N = 250_000 if args.small else 4_000_000
    run_passes = 64 if args.small else 256
    ref_passes = 16 * run_passes
    luma = np.array([0.2126, 0.7152, 0.0722])
    mk = lambda: scenes.sppm_caustic(width=W, height=W, photons=N, r1=0.005, alpha=0.7)
    ref = mk()
    ref.params.lt = 1
    ref.params.seed = 7919                   # the reference's own streams: no pass of it is a pass of the runs
    rt = create_path_tracer(ref, device=dev, code=True)
    left = ref_passes
    while left > 0:
        rt.step(min(64, left))
        left -= 64
    rgb, V, S, cnt = rt.read_accum()
    rt.close()
    Lref = rgb @ luma
    ok = (S > 0) & (S < 1)
    se2 = np.zeros_like(V)
    se2[ok] = S[ok] * V[ok] / (1 - S[ok])
    keep = (Lref <= np.quantile(Lref, 0.999)) & (np.sqrt(se2) <= 0.1 * np.maximum(Lref, 1.0))
    cm = scenes.caustic_mask(mk()) & keep           # the sphere's shadow on the floor, seen directly
    regions = {"picture": (keep, float(np.mean(se2[keep])), float(Lref[keep].mean())),
               "caustic": (cm, float(np.mean(se2[cm])), float(Lref[cm].mean()))}

    def rmse(L, region):
        mask, noise, mean = regions[region]
        d2 = np.sort((L[mask] - Lref[mask]) ** 2)
        d2 = d2[:max(1, int(len(d2) * 0.999))]
        return float(np.sqrt(max(d2.mean() - noise, 0.0)) / mean)

    out = {"metric": "seconds to 1% relative RMSE vs an FP64 render at 16x the passes", "unit": "s",
           "higher_is_better": False,
           "workload": "sppm caustic %dx%d, %d sun photons a pass, r1 5 mm, alpha 0.7; %d passes a run, the reference "
                       "%d passes of light tracing + the map on seeds of its own (its own relative noise %.4f, taken "
                       "out); %.1f %% of the pixels converged in it" % (W, W, N, run_passes, ref_passes,
                                                                      np.sqrt(regions["picture"][1]) / regions["picture"][2],
                                                                      100 * keep.mean()),
           "caustic_pixels": int(cm.sum())}
    for name, learn, lt in (("plain", 0, 0), ("guided", 1, 0), ("lt", 0, 1), ("lt_guided", 1, 1)):
        s = mk()
        s.params.sppm_learn = learn
        s.params.lt = lt
        rt = create_path_tracer(s, device=dev, code=True)
        stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))
        rt.step(1)
        rt.invalidate()
        ms, passes, curve = 0.0, 0, []
        while passes < run_passes:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rt.step_async(run_passes // 4)
            e1.record(stream)
            rt.sync()
            ms += e0.elapsed_time(e1)
            passes += run_passes // 4
            L = rt.read_accum()[0] @ luma
            curve.append([passes, round(ms / 1e3, 3), round(rmse(L, "picture"), 5), round(rmse(L, "caustic"), 5)])
        rt.close()
        _, t, rp, rc = curve[-1]
        out[name] = {"seconds": t * (rp / 0.01) ** 2, "seconds_caustic": t * (rc / 0.01) ** 2, "passes": passes,
                     "rmse": rp, "rmse_caustic": rc, "ms_per_pass": ms / passes,
                     "curve (passes, s, rmse, rmse over the caustic)": curve}

    def ratio(a, b, key):
        return out[a][key] / out[b][key] if out[a][key] and out[b][key] else None
    out["speedup"] = ratio("plain", "guided", "seconds")                 # guided emission, the map alone
    out["speedup_caustic"] = ratio("plain", "guided", "seconds_caustic")
    out["speedup_lt_over_plain"] = ratio("plain", "lt", "seconds")       # the reference's split over the map alone
    out["speedup_lt_over_plain_caustic"] = ratio("plain", "lt", "seconds_caustic")
    out["speedup_lt_guided_over_lt"] = ratio("lt", "lt_guided", "seconds")   # guided emission within the split
    out["speedup_lt_guided_over_lt_caustic"] = ratio("lt", "lt_guided", "seconds_caustic")
    return out


def run_ours(args):
    rank, world, local = dist_env()
    import torch
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    if args.leg != "all":
        with_cpu = rank == 0 and world == 1 and not args.no_cpu
        out = {"sppm": lambda: sppm_leg(args, dev, with_cpu), "rmse": lambda: rmse_leg(args, dev),
               "caustic_rmse": lambda: caustic_rmse_leg(args, dev),
               "optics": lambda: optics_leg(args, dev, with_cpu), "mlp": lambda: mlp_leg(args, dev),
               "emit": lambda: emit_leg(args, dev), "haze": lambda: haze_leg(args, dev),
               "env": lambda: env_leg(args, dev), "sc": lambda: sc_leg(args, dev),
               "views": lambda: views_leg(args, dev)}[args.leg]()
        if rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))
    from shadytracer_gb300 import flops
    from shadytracer_gb300.renderer import create_path_tracer
    s = workload(args.small, args.spp)
    spp = s.info["spp"]
    p = s.params
    P = p.width * p.height
    paths_per_step = P * spp
    src = scene_code(s)                     # the builder's step: the scene written as code, once
    rt = create_path_tracer(s, device=dev, code=src)
    compile_ms = rt.scene_code_info()["compile_ms"]
    # the autotuner picks the queue tile and the march chunk on this workload (2 samples each candidate, untimed)
    if args.tune:
        claim, chunk = (int(x) for x in args.tune.split(","))
        rt.set_tune(claim, chunk)
        tune = {"claim": claim, "chunk": chunk, "ms": 0.0, "ms_default": 0.0}
    else:
        tune = rt.autotune(2)
    stream = torch.cuda.ExternalStream(rt.stream(), device=torch.device("cuda", dev))

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def one_step():
        rt.invalidate()
        rt.step_async(spp)

    # ---- warm-up ----
    for _ in range(max(args.warmup, 3)):
        one_step()
        rt.sync()
    # ---- timed: value (device-resident scene; graph replays) ----
    launches0 = rt.counters()["launches"]
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            one_step()
        e1.record(stream)
        rt.sync()
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    clocks = clk.summary()
    c = rt.counters()
    launches = c["launches"] - launches0          # the library's kernels (graph nodes) in the timed region
    ms = reduce_max(ms, dist, "cuda")
    value = replica_value(world, paths_per_step, ms)

    # ---- e2e: through the C ABI from host memory, the picture read back every step ----
    rgb = np.zeros((p.height, p.width, 3), np.float64)
    V = np.zeros((p.height, p.width), np.float64)
    S = np.zeros((p.height, p.width), np.float64)
    cnt = np.zeros((p.height, p.width), np.uint32)
    Pv = C.c_void_p
    L = rt.L
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rt.set_scene(s, code=src)           # the scene's code (its compiled library, from the process's cache) and
                                            # its materials and table, host -> device
        rt.set_params(p)                    # the settings (resets the accumulation)
        rt.set_view(s.view)
        rt.step(spp)
        L.st_read_accum(rt.ctx, rgb.ctypes.data_as(Pv), V.ctypes.data_as(Pv), S.ctypes.data_as(Pv),
                        cnt.ctypes.data_as(Pv))
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = reduce_max(e2e_s, dist, "cuda")
    h2d = (C.sizeof(type(s.prims)) + C.sizeof(type(s.materials)) + C.sizeof(p) + C.sizeof(s.view) +
           len(src.encode()))
    d2h = P * (32 + 16)
    Lmean = float((rgb @ np.array([0.2126, 0.7152, 0.0722])).mean())

    # ---- per-kernel times (CUDA events on the library's stream) over the same K renders ----
    rt.enable_kernel_times(True)
    rt.reset_kernel_times()
    c0 = rt.counters()
    for _ in range(args.steps):
        one_step()
        rt.sync()
    kt = rt.kernel_times()
    c1 = rt.counters()
    rt.enable_kernel_times(False)
    evals = c1["march_steps"] - c0["march_steps"]
    m_launches, m_ms = kt.get("march", (0, 0.0))
    tot_ms = sum(v[1] for v in kt.values()) or 1.0

    # ---- a counting pass: one render with an instrumented march, its fold's work counted on the device ----
    rt.enable_kernel_times(True, count_work=True)
    w0 = rt.counters()
    one_step()
    rt.sync()
    w1 = rt.counters()
    rt.enable_kernel_times(False)
    dw = {k: [b - a for a, b in zip(w0[k], w1[k])] for k in ("prim_evals", "prim_warp_evals", "op_evals")}
    for k in ("bound_tests", "bound_warp_tests", "march_steps"):
        dw[k] = w1[k] - w0[k]
    f_render, sfu_render = flops.counted_flops(dw, dw["march_steps"])
    f_table, _ = flops.march_step_flops(s)                   # the whole table, every step: the uncull'd worst case
    per_launch_flops = f_render / max(m_launches / max(args.steps, 1), 1)
    avg_launch_s = m_ms / max(m_launches, 1) / 1e3
    achieved = per_launch_flops / avg_launch_s / 1e12 if avg_launch_s > 0 else 0.0   # TFLOP/s per march launch
    simd = sum(dw["prim_evals"]) / max(32 * sum(dw["prim_warp_evals"]), 1)
    pk = peaks()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    if pk and pk.get("sm_max_mhz"):
        peak = sms * 128 * 2 * pk["sm_max_mhz"] * 1e6 / 1e12
        peak_src = "FP32 FMA peak from MEASURED_PEAKS.json's sm_max_mhz: %d SMs x 128 lanes x 2 x %.0f MHz" % (
            sms, pk["sm_max_mhz"])
    else:
        peak = sms * 128 * 2 * 2070e6 / 1e12
        peak_src = "FP32 FMA peak at the nominal 2070 MHz (fallback)"
    line = {"metric": "Mpaths/s", "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 pixel tallies)", "data": "synthetic (seeded scene)",
            "config": dict(config_of(s), parallelism="replicas" if world > 1 else "1 GPU"),
            "e2e": {"value": world * paths_per_step / e2e_s / 1e6, "unit": "Mpaths/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "scene_compile_ms": compile_ms,
            "autotune": {"claim": tune["claim"], "chunk": tune["chunk"],
                         "speedup_over_defaults": tune["ms_default"] / tune["ms"] if tune["ms"] else None},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None,
                         "traffic": MARCH_DRAM_BYTES_PER_EVAL * evals / max(m_launches, 1),
                         "traffic_unit": "bytes of DRAM read + written per launch: ncu's dram__bytes per scene "
                                         "evaluation over one render's march launches at 1920x1080, 2 samples (%s), "
                                         "times this launch's evaluations" % MARCH_DRAM_PROFILE,
                         "kernel": "k_march", "flops_per_launch": per_launch_flops,
                         "flops_per_eval": f_render / max(dw["march_steps"], 1),
                         "flops_per_eval_whole_table": f_table,
                         "sfu_per_eval": sfu_render / max(dw["march_steps"], 1),
                         "evals_per_launch": evals / max(m_launches, 1),
                         "evals_per_render": evals / max(args.steps, 1),
                         "prims_evaluated_per_eval": sum(dw["prim_evals"]) / max(dw["march_steps"], 1),
                         "fold_simd_efficiency": simd,
                         "evals_by_type": {flops.TYPE_NAMES.get(t, str(t)): {
                             "per_step": n / max(dw["march_steps"], 1),
                             "simd_efficiency": n / max(32 * w, 1)}
                             for t, (n, w) in enumerate(zip(dw["prim_evals"], dw["prim_warp_evals"])) if n},
                         "bound_tests_per_step": dw["bound_tests"] / max(dw["march_steps"], 1),
                         "avg_launch_ms": m_ms / max(m_launches, 1), "peak_source": peak_src,
                         "work": "counted on the device in a counting pass (an instrumented march over one more "
                                 "render of the same seeds): evaluations by primitive type and fold operation, "
                                 "bounding-sphere tests, steps, each weighed by its FP32 operations "
                                 "(shadytracer_gb300/flops.py)"},
            "kernel_share": {k: round(v[1] / tot_ms, 4) for k, v in kt.items()},
            "clocks": clocks,
            "stats": {"mean_luma": Lmean, "segments_per_path": c["segments"] / max(c["paths"], 1),
                      "steps_per_segment": c["march_steps"] / max(c["segments"], 1),
                      "shadow_steps_per_ray": c["shadow_steps"] / max(c["shadow_rays"], 1),
                      "flushed": c["flushed"], "nonfinite": c["nonfinite"]}}
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(s)
    elif rank == 0:
        line["cpu_baseline"] = None
    if not args.no_sppm:
        line["sppm"] = sppm_leg(args, dev, rank == 0 and world == 1 and not args.no_cpu)
        line["time_to_rmse"] = {"caustic": caustic_rmse_leg(args, dev), "pane": rmse_leg(args, dev)}
    if not args.no_mlp:
        line["mlp"] = mlp_leg(args, dev)
    if not args.no_emit:
        line["emit"] = emit_leg(args, dev)
    if not args.no_haze:
        line["haze_beam"] = haze_leg(args, dev)
    if not args.no_env:
        line["env"] = env_leg(args, dev)
    if not args.no_sc:
        line["step_cache"] = sc_leg(args, dev)
        line["views"] = views_leg(args, dev)
    if not args.no_optics:
        line["optics"] = optics_leg(args, dev, rank == 0 and world == 1 and not args.no_cpu)
        if world > 1:
            line["optics"]["note"] = "per rank (each rank runs the whole batch)"
    if rank == 0:
        print(json.dumps(line), flush=True)
    rt.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
