"""The scene as code, on the CPU: the emitter (shadytracer_gb300/codegen.py, the twin of builder/codegen.js:974-1060)
writes the scene-as-code contract for the workloads, NVRTC compiles it for sm_103a with the library's kernels (no GPU
is needed to compile: st_compile_scene), and a source that does not compile is refused with the scene's line and the
node it belongs to (builder/codegen.js:20-41 maps WGSL errors to nodes the same way).
"""
import ctypes as C

import pytest

from shadytracer_gb300 import codegen, scenes, st_types as T


@pytest.fixture(scope="module")
def lib():
    from shadytracer_gb300 import build, _lib
    build.build()
    return _lib.load()


def compile_src(lib, src):
    err = C.create_string_buffer(1 << 16)
    ms = C.c_double()
    rc = lib.st_compile_scene(src.encode(), err, 1 << 16, C.byref(ms))
    return rc, err.value.decode(), ms.value


@pytest.mark.parametrize("make", [
    lambda: scenes.sdf_room(width=64, height=36),
    lambda: scenes.floor_furnace(width=16, height=16),
    lambda: scenes.sppm_caustic(width=16, height=16),
    lambda: scenes.spot_floor(width=16, height=16, light="face"),
    lambda: scenes.optics_bench(n_instances=2),
])
def test_the_workloads_compile(lib, make):
    s = make()
    src = codegen.generate(s)
    assert "st_scene_dist" in src and "st_scene_full" in src and "st_scene_dist_count" in src
    rc, err, ms = compile_src(lib, src)
    assert rc == 0, err
    # a second compile of the same text comes from the cache
    rc, err, ms2 = compile_src(lib, src)
    assert rc == 0 and ms2 == 0.0


def test_every_primitive_is_tagged_and_no_table_is_read():
    s = scenes.sdf_room(width=64, height=36)
    src = codegen.generate(s)
    for i in range(len(s.prim_list)):
        assert "// node %d:" % i in src
    assert "DPrim" not in src and "switch" not in src       # no table, no type switch: constants in the code
    # the prisms' sectors from their edge normals, no arctangent or sine-cosine per evaluation
    assert "atan2" not in src and "sincos" not in src


def test_a_bad_scene_is_refused_with_its_line_and_node(lib):
    s = scenes.floor_furnace(width=16, height=16)
    src = codegen.generate(s)
    lines = src.splitlines()
    # break the floor plane's distance: an undefined name on the node's line
    k = next(i for i, l in enumerate(lines) if "out = q.z;" in l)
    lines[k] = lines[k].replace("out = q.z;", "out = q.z + not_a_name;")
    rc, err, _ = compile_src(lib, "\n".join(lines))
    assert rc == T.ST_ERR_COMPILE
    assert "not_a_name" in err
    assert "at scene line %d:" % (k + 1) in err, err
    # the line reported is the node's own code; the node is named by the block it sits in
    block = "\n".join(lines[max(0, k - 4):k + 1])
    assert "node 0: plane" in block


def test_a_source_without_the_contract_is_refused(lib):
    rc, err, _ = compile_src(lib, "__device__ float f(st::f3 p) { return 0.f; }")
    assert rc == T.ST_ERR_COMPILE and "st_scene_dist" in err


def test_a_node_tree_lowers_to_the_table():
    tree = {"kind": "scene", "children": [
        {"kind": "object", "shape": "plane", "material": 2},
        {"kind": "group", "csg": "smooth", "k": 0.05, "children": [
            {"kind": "object", "shape": "sphere", "params": [0.3], "position": [0, 0, 0.3], "material": 1},
            {"kind": "object", "shape": "box", "params": [0.2, 0.2, 0.2], "position": [0.3, 0, 0.2], "material": 1},
            {"kind": "object", "shape": "torus", "params": [0.3, 0.05], "position": [0, 0, 0.6], "material": 1,
             "enabled": False},
        ]},
    ]}
    P = codegen.lower(tree)
    assert [p.type for p in P] == [T.ST_PRIM_PLANE, T.ST_PRIM_SPHERE, T.ST_PRIM_BOX]
    assert [p.op for p in P] == [T.ST_OP_ITEM, T.ST_OP_ITEM, T.ST_OP_SMOOTH]
    assert abs(P[2].k - 0.05) < 1e-7 and P[1].material == 1 and P[0].material == 2
    src = codegen.generate(tree)
    assert "node 2: box" in src and "smooth_union" in src


def test_literals_round_trip_to_the_table_floats():
    import numpy as np
    for x in (0.1, 1.0 / 3.0, 1e-30, 3.4e38, -2.5e-7, 0.0, 1234567.8):
        s = codegen.lit(x)
        assert np.float32(float(s[:-1])) == np.float32(x), (x, s)
