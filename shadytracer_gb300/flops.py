"""The algorithmic work of one scene-SDF evaluation, counted from the scene table.

The march and the occlusion pass are bound by FP32 arithmetic on the SDF: a step is one evaluation of the whole
table plus the step's own bookkeeping. This module counts the FP32 operations of one evaluation statically, the
way the kernels (csrc/st_device.cuh prim_sdf / scene_dist, csrc/st_render.cu k_march) write them: an add, a
multiply, a min/max/abs, a compare are 1; a fused multiply-add is 2; sqrt, reciprocal, divide and the
transcendentals run on the special-function unit and are counted apart (`sfu`). The achieved FLOP/s a roofline
reports is (evaluations counted on the device) x (this count) / (the kernel's time).

The fold skips primitives by their bounding spheres, so a step evaluates fewer than the whole table: `counted_flops`
weighs the work a counting pass of the march counted on the device (evaluations by primitive type and by fold
operation, bounding-sphere tests, steps) -- the work the kernel did, not the table's worst case.
"""
from .st_types import (ST_PRIM_PLANE, ST_PRIM_SPHERE, ST_PRIM_BOX, ST_PRIM_ROUNDBOX, ST_PRIM_TORUS, ST_PRIM_PRISM,
                       ST_PRIM_ASPHERE, ST_PRIM_CYLINDER, ST_OP_ITEM, ST_OP_SMOOTH, ST_OP_UNION, ST_OP_SUB)

# the world -> local transform: 3 subtracts, 3 x (3 multiplies, 2 adds) as 3 x (1 multiply + 2 FMAs)
TRANSFORM = (3 + 3 * (1 + 2 * 2), 0)
# per type: (flops, sfu ops) after the transform
PRIM = {
    ST_PRIM_PLANE: (0, 0),
    ST_PRIM_SPHERE: (2 + 2 * 2 + 1, 1),          # dot (mul + 2 fma), sqrt, subtract
    ST_PRIM_BOX: (3 + 3 + 3 + 1 + 2 * 2 + 2 + 1 + 1, 1),   # abs, sub, max 0, dot(mul + 2 fma), sqrt, max x2, min, add
    ST_PRIM_ROUNDBOX: (3 + 3 + 3 + 1 + 2 * 2 + 2 + 1 + 1 + 1, 1),
    ST_PRIM_TORUS: (1 + 2 + 1 + 1 + 2 + 1, 2),   # lxy (mul + fma), sqrt, sub, (mul + fma), sqrt, sub
    ST_PRIM_PRISM: (34, 6),                      # polygon: rint, atan2, 2 sincos, 2 dots, clamps; extrude; round
    ST_PRIM_ASPHERE: (2 * 40 + 6, 8),            # two faces (sag, slope bound), the rim
    ST_PRIM_CYLINDER: (2 + 1 + 1 + 1 + 2 + 2 + 1 + 2 + 1, 2),
}
TYPE_NAMES = {ST_PRIM_PLANE: "plane", ST_PRIM_SPHERE: "sphere", ST_PRIM_BOX: "box", ST_PRIM_ROUNDBOX: "roundbox",
              ST_PRIM_TORUS: "torus", ST_PRIM_PRISM: "prism", ST_PRIM_ASPHERE: "asphere", ST_PRIM_CYLINDER: "cylinder"}
OP = {ST_OP_SMOOTH: (9, 1), ST_OP_UNION: (1, 0), ST_OP_SUB: (2, 0), ST_OP_ITEM: (0, 0)}
FOLD = (3, 0)                                      # |d| compare and select per item
STEP = (30, 1)                                     # marchTol, the escape and hit tests, the step and its length


def sdf_flops(scene):
    """(flops, sfu) of one evaluation of the scene's SDF (distance only)."""
    f = s = 0
    for p in scene.prim_list:
        a, b = PRIM.get(p.type, (0, 0))
        f += TRANSFORM[0] + a
        s += TRANSFORM[1] + b
        o = OP.get(p.op, (0, 0))
        f += o[0]
        s += o[1]
        if p.op == ST_OP_ITEM:
            f += FOLD[0]
    return f, s


def march_step_flops(scene):
    """(flops, sfu) of one march step: the SDF and the step."""
    f, s = sdf_flops(scene)
    return f + STEP[0], s + STEP[1]


BOUND_TEST = (10, 0)        # |p - c|^2 against (t + R)^2: 3 subtracts, a multiply and 2 FMAs, an add, a multiply, 2 compares


def counted_flops(c, n_steps):
    """(flops, sfu) of the march's fold as a counting pass counted it: `c` the counters' differences (prim_evals by
    type, op_evals by fold operation, bound_tests), `n_steps` the evaluations (march steps)."""
    f = s = 0
    for t, n in enumerate(c["prim_evals"]):
        a, b = PRIM.get(t, (0, 0))
        f += n * (TRANSFORM[0] + a)
        s += n * (TRANSFORM[1] + b)
    for op, n in enumerate(c["op_evals"]):
        o = OP.get(op, (0, 0))
        f += n * (o[0] + (FOLD[0] if op == ST_OP_ITEM else 0))
        s += n * o[1]
    f += c["bound_tests"] * BOUND_TEST[0]
    f += n_steps * STEP[0]
    s += n_steps * STEP[1]
    return f, s
