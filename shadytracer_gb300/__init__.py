"""shadytracer_gb300 -- a GB300-native (sm_103a) rebuild of lampmaker/ShadyTracer's rendering hot path.

The compute path is libshadytracer.so (shadytracer_gb300/csrc, CUDA C++ for sm_103a) behind the C ABI of
include/shadytracer.h. This package is the host side above it: ctypes mirrors of the ABI's structs (st_types),
the workloads as scene tables (scenes), and the reference's renderer and optics APIs (renderer, optics), which
raise if the CUDA library is missing -- there is no CPU fallback.
"""
from . import st_types, scenes  # noqa: F401

__all__ = ["st_types", "scenes"]
