"""The C ABI boundary, on the CPU: the library builds, loads without a GPU, exports every function
include/shadytracer.h declares, and agrees with the ctypes mirrors on every struct's size. Nothing here launches a
kernel; the one runtime call (st_create) must fail cleanly when there is no GPU.
"""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "shadytracer.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    src = re.sub(r"#[^\n]*", " ", src)
    names = set(re.findall(r"\b(st_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from shadytracer_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_the_api():
    names = declared_functions()
    for n in ("st_create", "st_destroy", "st_set_scene", "st_step", "st_read_accum", "st_sppm_build",
              "st_optics_run", "st_render_noalloc", "st_struct_sizes"):
        assert n in names
    assert len(names) >= 28


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_every_declared_symbol_has_a_ctypes_signature():
    from shadytracer_gb300._lib import SIGNATURES
    missing = [n for n in declared_functions() if n not in SIGNATURES]
    assert not missing, missing


def test_struct_sizes_match_the_mirrors(lib):
    from shadytracer_gb300._lib import STRUCT_ORDER
    out = (C.c_uint32 * 32)()
    n = lib.st_struct_sizes(C.cast(out, C.c_void_p), 32)
    assert n == len(STRUCT_ORDER)
    for i, T in enumerate(STRUCT_ORDER):
        assert out[i] == C.sizeof(T), (T.__name__, out[i], C.sizeof(T))


def test_fixed_record_sizes():
    from shadytracer_gb300 import st_types as T
    assert C.sizeof(T.StPrim) == 128
    assert C.sizeof(T.StMaterial) == 112


def test_abi_version(lib):
    assert lib.st_abi_version() >= 1


def test_create_fails_loudly_without_a_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = C.c_void_p()
    rc = lib.st_create(0, C.byref(ctx))
    assert rc != 0
    assert not ctx.value
    from shadytracer_gb300.renderer import PathTracer
    from shadytracer_gb300._lib import StError
    with pytest.raises(StError):
        PathTracer(None, device=0)


def test_null_arguments_are_rejected(lib):
    assert lib.st_create(0, None) != 0
    assert lib.st_step(None, 1) != 0
    assert lib.st_sppm_build(None, None, None, None, None, None, 0, C.c_float(1.0)) != 0
    assert lib.st_optics_run(None, None, None, None, None) != 0
