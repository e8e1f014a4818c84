"""Build libshadytracer.so in-tree: every csrc/*.cu compiled for sm_103a in parallel, then linked (cudart static).

    python -m shadytracer_gb300.build          # or __graft_entry__.build()

The library lands beside this file (shadytracer_gb300/libshadytracer.so, git-ignored) and is rebuilt only when a
source or header is newer. No torch, no cmake: nvcc and the C ABI of include/shadytracer.h.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libshadytracer.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# f32 division and square root by the hardware's fast sequences (within 2 ulp), denormals flushed: the SDF fold,
# the march and the shading are bound by instruction issue, and these cut their instruction counts by about a
# quarter. Where a result must be the reference's to the bit (the photon grid's cells, its gather's radius and
# normal tests) the kernels call the IEEE-rounded intrinsics (__fdiv_rn, __fmul_rn, __fsqrt_rn) explicitly.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-prec-div=false", "-prec-sqrt=false", "-ftz=true",
         "-Xcompiler", "-fPIC", "-diag-suppress", "1444",
         "-I", os.path.join(ROOT, "include")]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def cuda_lib_dir():
    """The toolkit's library directory, beside the nvcc in use (lib64, or lib on some layouts)."""
    import shutil
    n = nvcc()
    path = n if os.path.isabs(n) else (shutil.which(n) or "/usr/local/cuda/bin/nvcc")
    root = os.path.dirname(os.path.dirname(os.path.realpath(path)))
    for d in ("lib64", "lib"):
        if os.path.exists(os.path.join(root, d, "libnvrtc.so")):
            return os.path.join(root, d)
    return os.path.join(root, "lib64")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "shadytracer.h"), os.path.abspath(__file__)]   # the flags live here
    objs, jobs = [], []
    for s in sources:
        o = os.path.join(OBJ, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc()] + ARCH + FLAGS + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        # NVRTC (a scene given as code is compiled at st_set_scene): the toolkit's shared library, found at run time
        # where it was at link time
        lib = cuda_lib_dir()
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + \
            ["-L" + lib, "-lnvrtc", "-Xlinker", "-rpath=" + lib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
