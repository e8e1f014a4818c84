"""The scene as code: a CUDA C++ emitter for the scene's SDF, the twin of the reference builder's code generator
(builder/codegen.js:974-1060 generate -> the scene's SDF and material functions as WGSL; scene_api.js:28-93 the fold
they implement and its bounding-box culling, :288-305).

    src = codegen.generate(scene)            # a Scene (scenes.py) or a node tree (below) -> CUDA source
    rt.set_scene(scene, code=src)            # st_set_scene(ctx, src, desc): NVRTC for sm_103a at scene load

The source defines what st_set_scene's contract asks (include/shadytracer.h):

    __device__ float        st_scene_dist(st::f3 p);                    FOLD_DIST
    __device__ st::SceneHit st_scene_full(st::f3 p);                    FOLD_FULL (distance, material, medium)
    __device__ float        st_scene_dist_count(st::f3 p, uint32_t* wc) FOLD_DIST tallying its work (ST_SCENE_COUNTS)

It folds the scene exactly as the table path does (st_device.cuh scene_dist / scene_full): items by the nearest
surface, each item a CSG chain (smooth union, union, subtraction into the item), a chain member evaluated only where
its bounding sphere says it could change the running value -- the same test, so the same value bit for bit where the
arithmetic is the same. What the code gains over the table's loop is what a compiler does with constants: no type
switch, no table in shared memory, every parameter an immediate, the rotation skipped where it cannot matter (a
sphere; an axis-aligned primitive), only the rows a shape reads (a plane's one), and a regular prism's sector found
from its few edge normals (the polygon folded about its mirror axis) instead of an arctangent and a sine-cosine.

Every primitive's line ends with a tag naming its item and its node, so an NVRTC error on it (the library reports the
scene's line and its text) names the part of the scene that failed (builder/codegen.js:20-41 maps a WGSL error to
its node the same way).

A NODE TREE (the builder's tree, reduced to what the table can hold): {"kind": "scene", "children": [...]} of
objects {"kind": "object", "shape": "box"|"sphere"|"roundbox"|"torus"|"prism"|"asphere"|"cylinder"|"plane",
"params": [...], "position": [x, y, z], "rotation": [9 floats, world -> local rows], "material": m} and CSG groups
{"kind": "group", "csg": "smooth"|"union"|"subtract", "k": radius, "children": [objects]} -- a group is one item, its
first child the head and the rest folded into it by the group's operation. `lower(tree)` gives the table.
"""
import math

import numpy as np

from .st_types import (StPrim, ST_PRIM_PLANE, ST_PRIM_SPHERE, ST_PRIM_BOX, ST_PRIM_ROUNDBOX, ST_PRIM_TORUS,
                       ST_PRIM_PRISM, ST_PRIM_ASPHERE, ST_PRIM_CYLINDER, ST_OP_ITEM, ST_OP_SMOOTH, ST_OP_UNION,
                       ST_OP_SUB, ST_LIGHT_DISC)

SHAPES = {"plane": ST_PRIM_PLANE, "sphere": ST_PRIM_SPHERE, "box": ST_PRIM_BOX, "roundbox": ST_PRIM_ROUNDBOX,
          "torus": ST_PRIM_TORUS, "prism": ST_PRIM_PRISM, "asphere": ST_PRIM_ASPHERE, "cylinder": ST_PRIM_CYLINDER}
TYPE_NAMES = {v: k for k, v in SHAPES.items()}
OPS = {"smooth": ST_OP_SMOOTH, "union": ST_OP_UNION, "subtract": ST_OP_SUB}
IDENTITY = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)
CULL_REL = "1.001f"
CULL_ABS = "1e-6f"


def lit(x):
    """A float32 literal that parses back to exactly x's float32."""
    v = np.float32(x)
    if np.isnan(v):
        return "__int_as_float(0x7fc00000)"
    if np.isinf(v):
        return "__int_as_float(0x7f800000)" if v > 0 else "__int_as_float(0xff800000)"
    s = np.format_float_scientific(v, unique=True, trim="0")
    return s + "f"


def f32(x):
    return float(np.float32(x))


# ---------------------------------------------------------------------------------------------------------------
# what the table path works out once a primitive, in double, then rounds (st_capi.cu pack_prim): the bound's radius
# (inflated, +inf where none is exact) and a prism's edge constants
# ---------------------------------------------------------------------------------------------------------------
def bound_radius(t, q):
    if t == ST_PRIM_SPHERE:
        R = abs(q[0])
    elif t == ST_PRIM_BOX:
        R = math.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2])
    elif t == ST_PRIM_ROUNDBOX:
        R = math.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]) + abs(q[3])
    elif t == ST_PRIM_TORUS:
        R = abs(q[0]) + abs(q[1])
    elif t == ST_PRIM_PRISM:
        R = math.sqrt(q[1] * q[1] + 0.25 * q[2] * q[2]) + abs(q[3])
    elif t == ST_PRIM_CYLINDER:
        R = math.sqrt(q[0] * q[0] + q[1] * q[1])
    else:
        return math.inf
    return f32(R * 1.001 + 1e-5)


def light_sheets(scene):
    """The lights' faces as the table path draws them (st_capi.cu light_faces): each a sheet of its material after the
    scene's primitives, a rectangle a box of no thickness, a disc a cylinder of none, its frame made orthonormal in
    double."""
    out = []
    for L in getattr(scene, "light_list", []):
        u = [float(c) for c in L.u]
        v = [float(c) for c in L.v]
        lu = math.sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2])
        u = [c / lu for c in u]
        uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2]
        v = [v[k] - uv * u[k] for k in range(3)]
        lv = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
        v = [c / lv for c in v]
        n = [u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]]
        p = StPrim()
        p.type = ST_PRIM_CYLINDER if L.shape == ST_LIGHT_DISC else ST_PRIM_BOX
        p.op = ST_OP_ITEM
        p.material = L.material
        for k in range(3):
            p.pos[k] = L.centre[k]
            p.rot[k], p.rot[3 + k], p.rot[6 + k] = u[k], v[k], n[k]
        if L.shape == ST_LIGHT_DISC:
            p.p[0], p.p[1] = 0.0, L.half_w
        else:
            p.p[0], p.p[1], p.p[2] = L.half_w, L.half_h, 0.0
        out.append(p)
    return out


# ---------------------------------------------------------------------------------------------------------------
# one primitive's distance, as statements that leave it in `out`
# ---------------------------------------------------------------------------------------------------------------
class Prim:
    def __init__(self, p, index):
        self.i = index
        self.type = int(p.type)
        self.op = int(p.op)
        self.material = int(p.material)
        self.c = [f32(p.pos[k]) for k in range(3)]
        self.k = f32(p.k)
        self.rot = [f32(p.rot[k]) for k in range(9)]
        self.q = [f32(p.p[k]) for k in range(12)]
        self.R = bound_radius(self.type, self.q)

    @property
    def tag(self):
        return "node %d: %s" % (self.i, TYPE_NAMES.get(self.type, "?"))

    def local(self, rows=(0, 1, 2)):
        """The statements putting p in the primitive's frame: d = p - c, then q = rot d (the rows asked for)."""
        c = self.c
        s = ["const f3 d = mk(p.x - %s, p.y - %s, p.z - %s);" % (lit(c[0]), lit(c[1]), lit(c[2]))]
        if tuple(self.rot) == IDENTITY:
            s.append("const f3 q = d;")
            return s
        comp = []
        for r in range(3):
            if r not in rows:
                comp.append("0.f")
                continue
            a, b, e = self.rot[3 * r: 3 * r + 3]
            terms = []
            for coef, v in ((a, "d.x"), (b, "d.y"), (e, "d.z")):
                if coef == 0.0:
                    continue
                terms.append(v if coef == 1.0 else ("-" + v if coef == -1.0 else "%s * %s" % (lit(coef), v)))
            comp.append(" + ".join(terms) if terms else "0.f")
        s.append("const f3 q = mk(%s, %s, %s);" % tuple(comp))
        return s

    def body(self):
        t, q = self.type, self.q
        if t == ST_PRIM_PLANE:
            return self.local(rows=(2,)) + ["out = q.z;"]
        if t == ST_PRIM_SPHERE:
            # rotation-invariant: the distance from the centre
            c = self.c
            return ["const f3 d = mk(p.x - %s, p.y - %s, p.z - %s);" % (lit(c[0]), lit(c[1]), lit(c[2])),
                    "out = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z) - %s;" % lit(q[0])]
        if t == ST_PRIM_BOX:
            return self.local() + ["out = sd_box(q, mk(%s, %s, %s));" % (lit(q[0]), lit(q[1]), lit(q[2]))]
        if t == ST_PRIM_ROUNDBOX:
            return self.local() + ["out = sd_box(q, mk(%s, %s, %s)) - %s;" % (lit(q[0]), lit(q[1]), lit(q[2]),
                                                                                lit(q[3]))]
        if t == ST_PRIM_TORUS:
            return self.local() + ["const float t = sqrtf(q.x * q.x + q.y * q.y) - %s;" % lit(q[0]),
                                   "out = sqrtf(t * t + q.z * q.z) - %s;" % lit(q[1])]
        if t == ST_PRIM_CYLINDER:
            return self.local() + [
                "const float lx = sqrtf(q.x * q.x + q.y * q.y) - %s, lz = fabsf(q.z) - %s;" % (lit(q[1]), lit(q[0])),
                "const float ox = fmaxf(lx, 0.f), oz = fmaxf(lz, 0.f);",
                "out = fminf(fmaxf(lx, lz), 0.f) + sqrtf(ox * ox + oz * oz);"]
        if t == ST_PRIM_PRISM:
            return self.local() + self.prism()
        if t == ST_PRIM_ASPHERE:
            rho = max(0.5 * q[0], 1e-6)
            return self.local() + [
                "const float l = sqrtf(q.x * q.x + q.y * q.y);",
                "float dd = l - %s;" % lit(rho),
                "const float top = asph_face(q, l, %s, %s, %s, %s, %s, %s, 1.f);" % (
                    lit(rho), lit(0.5 * q[1]), lit(q[2]), lit(q[3]), lit(q[4]), lit(q[5])),
                "if (top > dd) dd = top;",
                "const float bot = asph_face(q, l, %s, %s, %s, %s, %s, %s, -1.f);" % (
                    lit(rho), lit(0.5 * q[1]), lit(q[6]), lit(q[7]), lit(q[8]), lit(q[9])),
                "if (bot > dd) dd = bot;",
                "out = dd;"]
        return ["out = 1e7f;"]

    def prism(self):
        """g2RegularPolygon (shapes.js:266-283) extruded: the edge nearest in angle is the one whose outward normal
        has the largest dot product with the point; the polygon is its own mirror image across x = 0 (its first edge
        normal is -y), so |x| leaves only the normals with x >= 0 to try. Then the edge's distance, extruded."""
        q = self.q
        n = min(max(float(np.rint(q[0])), 3.0), 64.0)
        an = math.pi / n
        Rp = max(q[1], 0.0)
        ap, he = f32(Rp * math.cos(an)), f32(Rp * math.sin(an))
        s = ["const float ax = fabsf(q.x);",
             "float pu = -q.y, pv = ax;"]                   # k = 0: normal (0, -1)
        for k in range(1, int(n) // 2 + 1):
            sk, ck = math.sin(2 * math.pi * k / n), math.cos(2 * math.pi * k / n)
            if sk < -1e-12:
                continue
            # u = ax sk - y ck (the normal (sk, -ck)); v = ax ck + y sk
            s.append("{ const float uk = %s * ax - %s * q.y; if (uk > pu) { pu = uk; pv = %s * ax + %s * q.y; } }" % (
                lit(sk), lit(ck), lit(ck), lit(sk)))
        s += ["float gz;",
              "if (pu <= %s) gz = pu - %s;" % (lit(ap), lit(ap)),
              "else { const float ex = pu - %s, ey = pv - clampf(pv, %s, %s); gz = sqrtf(ex * ex + ey * ey); }" % (
                  lit(ap), lit(-he), lit(he)),
              "out = g2_extrude(q.z, gz, %s) - %s;" % (lit(max(0.5 * q[2], 0.0)), lit(q[3]))]
        return s

    def value(self, var, indent):
        """`var` = the primitive's distance, in a block of its own, tagged."""
        pad = " " * indent
        lines = [pad + "{   // %s" % self.tag]
        lines += [pad + "    float out;"]
        lines += [pad + "    " + b for b in self.body()]
        lines += [pad + "    %s = out;" % var, pad + "}"]
        return lines

    def culled(self, t_expr):
        """The bounding-sphere test's condition that the distance here is at least t (st_device.cuh beyond): None
        where the primitive has no exact bound (it is always evaluated)."""
        if not math.isfinite(self.R):
            return None
        c = self.c
        return ("beyond_at(p, %s, %s, %s, %s, %s)" % (lit(c[0]), lit(c[1]), lit(c[2]), lit(self.R), t_expr))


PRELUDE = r"""// generated by shadytracer_gb300/codegen.py: the scene's SDF as code (st_set_scene's contract)
#define ST_SCENE_COUNTS 1
using st::f3;
using st::mk;
using st::SceneHit;
namespace stscene {
using namespace st;
// st_device.cuh beyond, with the primitive's centre and bound radius as immediates
__device__ __forceinline__ bool beyond_at(f3 p, float cx, float cy, float cz, float R, float t) {
    const float s = t + R;
    if (!(s < 3.0e38f)) return false;
    if (s < 0.f) return true;
    const float dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
    return dx * dx + dy * dy + dz * dz >= s * s;
}
"""


def items_of(prims):
    items = []
    for p in prims:
        if p.op == ST_OP_ITEM or not items:
            items.append([p])
        else:
            items[-1].append(p)
    return items


def emit_dist(items, count):
    name = "dist_count" if count else "dist"
    sig = "__device__ __forceinline__ float %s(f3 p%s)" % (name, ", uint32_t* wc" if count else "")
    L = [sig + " {", "    float best = 1e7f;"]
    for ii, it in enumerate(items):
        head = it[0]
        L.append("    {   // item %d" % ii)
        L.append("        float di;")
        if count:
            L.append("        wc_prim(wc, %du, 0u);" % head.type)
        L += head.value("di", 8)
        for m in it[1:]:
            if count:
                L.append("        wc_test(wc);")
            if m.op == ST_OP_SMOOTH:
                t = "di + %s * %s + %s" % (lit(max(m.k, 0.0)), CULL_REL, CULL_ABS)
                fold = "di = smooth_union(di, dj, %s);" % lit(m.k)
            elif m.op == ST_OP_UNION:
                t = "di + %s" % CULL_ABS
                fold = "di = fminf(di, dj);"
            else:
                t = "-di + %s" % CULL_ABS
                fold = "di = fmaxf(di, -dj);"
            cond = m.culled(t)
            L.append("        if (%s) {" % ("!" + cond if cond else "true"))
            if count:
                L.append("            wc_prim(wc, %du, %du);" % (m.type, m.op))
            L.append("            float dj;")
            L += m.value("dj", 12)
            L.append("            " + fold)
            L.append("        }")
        L.append("        if (fabsf(di) < fabsf(best)) best = di;")
        L.append("    }")
    L += ["    return best;", "}"]
    return L


def emit_full(items):
    L = ["__device__ __forceinline__ SceneHit full(f3 p) {",
         "    SceneHit H;", "    H.d = 1e7f; H.m = 0u; H.a = 0u;", "    float insideW = -1e7f;"]
    for ii, it in enumerate(items):
        head = it[0]
        L.append("    {   // item %d" % ii)
        L.append("        float di;")
        L += head.value("di", 8)
        L.append("        uint32_t mat = %du;" % head.material)
        L.append("        float nearv = fabsf(di);")
        for m in it[1:]:
            if m.op == ST_OP_SMOOTH:
                t = "fmaxf(di + %s * %s, nearv) + %s" % (lit(max(m.k, 0.0)), CULL_REL, CULL_ABS)
                fold = ["di = smooth_union(di, dj, %s);" % lit(m.k),
                        "if (fabsf(dj) < nearv) { nearv = fabsf(dj); mat = %du; }" % m.material]
            elif m.op == ST_OP_UNION:
                t = "fmaxf(di, nearv) + %s" % CULL_ABS
                fold = ["di = fminf(di, dj);",
                        "if (fabsf(dj) < nearv) { nearv = fabsf(dj); mat = %du; }" % m.material]
            else:
                t = "-di + %s" % CULL_ABS
                fold = ["di = fmaxf(di, -dj);"]
            cond = m.culled(t)
            L.append("        if (%s) {" % ("!" + cond if cond else "true"))
            L.append("            float dj;")
            L += m.value("dj", 12)
            L += ["            " + f for f in fold]
            L.append("        }")
        L.append("        if (di < 0.f && di > insideW) { insideW = di; H.a = mat; }")
        L.append("        if (fabsf(di) < fabsf(H.d)) { H.d = di; H.m = mat; }")
        L.append("    }")
    L += ["    return H;", "}"]
    return L


def generate(scene_or_tree):
    """CUDA source for st_set_scene from a Scene (its primitives, then its lights' sheets) or a node tree."""
    if isinstance(scene_or_tree, dict):
        prims = lower(scene_or_tree)
        sheets = []
    else:
        prims = list(scene_or_tree.prim_list)
        sheets = light_sheets(scene_or_tree)
    P = [Prim(p, i) for i, p in enumerate(list(prims) + sheets)]
    items = items_of(P)
    L = [PRELUDE]
    L += emit_dist(items, False)
    L += emit_dist(items, True)
    L += emit_full(items)
    L += ["}  // namespace stscene",
          "__device__ float st_scene_dist(st::f3 p) { return stscene::dist(p); }",
          "__device__ float st_scene_dist_count(st::f3 p, uint32_t* wc) { return stscene::dist_count(p, wc); }",
          "__device__ st::SceneHit st_scene_full(st::f3 p) { return stscene::full(p); }", ""]
    return "\n".join(L)


def lower(tree):
    """A node tree (module docstring) as the primitive table: a CSG group one item, its children folded into its
    first by its operation; an object an item of its own."""
    out = []

    def obj(node, op, k):
        p = StPrim()
        p.type = SHAPES[node["shape"]]
        p.op = op
        p.material = int(node.get("material", 1))
        pos = node.get("position", (0.0, 0.0, 0.0))
        rot = node.get("rotation", IDENTITY)
        for i in range(3):
            p.pos[i] = pos[i]
        for i in range(9):
            p.rot[i] = rot[i]
        p.k = k
        for i, v in enumerate(node.get("params", ())):
            p.p[i] = v
        return p

    for child in tree.get("children", ()):
        if child.get("kind") == "group":
            op = OPS[child.get("csg", "union")]
            k = float(child.get("k", 0.0))
            kids = [c for c in child.get("children", ()) if c.get("enabled", True)]
            for j, c in enumerate(kids):
                if c.get("kind") != "object":
                    raise ValueError("a CSG group holds objects (nested groups do not fit the table)")
                out.append(obj(c, ST_OP_ITEM if j == 0 else op, k))
        elif child.get("kind") == "object":
            if child.get("enabled", True):
                out.append(obj(child, ST_OP_ITEM, 0.0))
        else:
            raise ValueError("unknown node kind %r" % child.get("kind"))
    return out
