// st_optics.cu -- the optics bench (optics/kernels.js, optics/index.js) for sm_103a: many emitter + lens instances
// traced in one launch chain, with FP64 tallies.
//
// THE REFERENCE traces one luminaire at a time: prog_opt_gen (kernels.js:429) draws rays from the sources, the
// renderer's march moves them, prog_opt_shade (kernels.js:571-699) walks each through every event -- a photon that is
// never ended by a scatter (TAG_OPTIC) -- and tallies, per interaction, what escaped, was lost, was absorbed or reached
// a detector, and the far field by direction, in u64 fixed point. The host turns the far field into candela
// (farfield.js) and a lux plane (illum.js).
//
// HERE a BATCH of instances -- each its own table range of primitives and its own sources, with its own ray count --
// runs as one wave chain: k_opt_gen fills the wave with the rays of every instance (each instance's rays split evenly
// over the waves, photons.js planBatches), the renderer's persistent march (k_march<INST>) moves each ray through its
// own instance's primitives only, and k_opt_shade shades and tallies. The tallies are FP64: per instance the totals
// (shared-memory atomics per CTA, one global add each at the end), the far field on a (C, gamma) grid and the lux map
// on a plane at a set height along the axis (global FP64 atomics, spread over their bins).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "st_ext.h"
#include "st_kernels.cuh"
#include "st_spectral.h"

using namespace st;

#define OPT_MAX_INST 256u
// per instance, in fixed point (OPT_FX a unit of weight) or counts: the weight emitted (a ray set's), escaped, lost,
// detected, absorbed; the interactions; the rays escaped, lost, detected and absorbed
#define OPT_TOT 16u
#define T_EMIT 0u
#define T_ESC 1u
#define T_LOST 2u
#define T_DET 3u
#define T_ABS 4u
#define T_INTER 5u
#define T_NESC 6u
#define T_NLOST 7u
#define T_NDET 8u
#define T_NABS 9u
#define OPT_WAVE (4u << 20)
// THE TALLIES IN FIXED POINT (the reference's optAdd, kernels.js:174-179, keeps u64 in lo/hi words at 2^20 a unit):
// signed 64-bit integers at 2^24 a unit of weight, so every sum is exact and the same whatever order the atomics ran
// in; FP64 only where the sums are read out (k_opt_flush)
#define OPT_FX 16777216.0
#define OPT_TAG_MAX 256u    // the tags: an item of the table, by its first primitive's index
#define DET_F4 3u           // a detector hit: position | weight, direction | tag, colour X | Z | 0 | 0
#define VERT_F4 2u          // a path vertex: position | weight, optical length | hue rgb

namespace {

struct OptArgs {
    WaveArgs w;
    const st_optics_source* src;    // sorted by instance
    const float* cdf;               // each source's cumulative share within its instance
    const uint2* src_range;         // per instance [first, count) of src
    const float4* rays;             // the ray table (two float4s a ray), and its rays
    uint32_t n_rays;
    uint32_t has_sets;              // a ray set among the sources: the weights emitted are summed (tot[7])
    const float4* origin;           // per instance: where its axis starts (its first source's centre)
    const uint32_t* wave_first;     // per instance: the first ray id of this wave
    const uint32_t* wave_prefix;    // per instance: the wave's slots before it (n_inst + 1 entries)
    uint32_t n_inst;
    uint32_t seed;
    f3 axis, c0, c90;
    uint32_t nC, nG, cells;
    float half, height;
    unsigned long long* far;        // n_inst * nG * nC, fixed point
    unsigned long long* lux;        // n_inst * cells * cells, fixed point
    unsigned long long* tot;        // n_inst * OPT_TOT
    unsigned long long* tag;        // OPT_TAG_MAX * 3: incident, leaving (fixed point), interactions
    unsigned long long* mat;        // n_inst * n_mats * 3: the same by material
    // the detector hits recorded (optRecordHit, kernels.js:237-251) and the paths kept (optVertex, :193-206)
    float4* det;                    // det_cap * DET_F4
    uint32_t* det_n;                // hits reached (may pass det_cap: the rest were not kept)
    uint32_t det_cap;
    float4* verts;                  // n_inst * path_rays * path_verts * VERT_F4
    uint32_t* vcount;               // n_inst * path_rays
    uint32_t path_rays, path_verts;
    float esc_len;                  // an escaped ray's last vertex, this far past its last interaction
    // THE TRACE BY WAVELENGTH (optics/spectral.js): on, and its tables -- the draw's CDF, the colour-matching
    // functions, the basis an RGB colour becomes a spectrum by (SPO_NODES values each), then each source's spectrum
    // (in src's order) at luminance 1
    uint32_t spectral;
    const float* spo;
};

// ---- the trace by wavelength's device half (optics/spectral.js SPECTRAL_CORE_WGSL, specOfRGB) ----
#define SPO_NODES 471u
#define SPO_LO 360.f
// a table at l, linear between its 1 nm nodes
__device__ __forceinline__ float spo_node(const float* __restrict__ t, uint32_t off, float l) {
    const float x = l - SPO_LO;
    const uint32_t i = (uint32_t)fminf(fmaxf(floorf(x), 0.f), (float)(SPO_NODES - 2u));
    const float f = fminf(fmaxf(x - (float)i, 0.f), 1.f);
    const float a = __ldg(&t[off + i]), b = __ldg(&t[off + i + 1u]);
    return a + f * (b - a);
}
// the draw: u to (l, its density per nm) through the CDF of x-bar + y-bar + z-bar
__device__ __forceinline__ float2 spo_lambda(const float* __restrict__ t, float u) {
    uint32_t lo = 0u, hi = SPO_NODES - 1u;
    while (hi - lo > 1u) {
        const uint32_t m = (lo + hi) >> 1;
        if (__ldg(&t[m]) <= u) lo = m;
        else hi = m;
    }
    const float c0 = __ldg(&t[lo]), mass = __ldg(&t[hi]) - c0;
    const float f = mass > 0.f ? fminf(fmaxf((u - c0) / mass, 0.f), 1.f) : 0.5f;
    return make_float2(SPO_LO + (float)lo + f, mass);
}
// a ray's three wavelengths, u, u + 1/3, u + 2/3 (mod 1) through the draw
__device__ __forceinline__ f3 spo_lams(const float* t, float u) {
    float u1 = u + 1.f / 3.f, u2 = u + 2.f / 3.f;
    if (u1 >= 1.f) u1 -= 1.f;
    if (u2 >= 1.f) u2 -= 1.f;
    return mk(spo_lambda(t, u).x, spo_lambda(t, u1).x, spo_lambda(t, u2).x);
}
__device__ __forceinline__ f3 spo_cmf(const float* t, float l) {
    return mk(spo_node(t, SPO_NODES, l), spo_node(t, 2u * SPO_NODES, l), spo_node(t, 3u * SPO_NODES, l));
}
__device__ __forceinline__ f3 spo_basis(const float* t, float l) {
    return mk(spo_node(t, 4u * SPO_NODES, l), spo_node(t, 5u * SPO_NODES, l), spo_node(t, 6u * SPO_NODES, l));
}
// what a ray carries as XYZ: each wavelength's weight times the colour-matching functions there (specXYZ)
__device__ __forceinline__ f3 spo_xyz(const float* t, f3 c, f3 l) {
    return spo_cmf(t, l.x) * c.x + spo_cmf(t, l.y) * c.y + spo_cmf(t, l.z) * c.z;
}
// a ray's wavelength word (PathBuf.lam): its u, or u + 2 once a dispersive glass collapsed it to its first wavelength
__device__ __forceinline__ float spo_u(float w) { return w >= 2.f ? w - 2.f : w; }
// THE LOBES AT THE RAY'S WAVELENGTHS (optics/spectral.js specOfRGB): the material's colour a reflectance at each, the
// coating taken at each -- out of line, so the trace in colour keeps its registers
__device__ __noinline__ void spectral_lobes(const float* spo, f3 l3, f3 nrm, f3 v, const st_material& m, float eta,
                                            const MfTab& tab, float trans, float spec, float hz, float n0, bool inside,
                                            Lobes& out) {
    st_material mw = m;
    const f3 rgb = mk(m.base[0], m.base[1], m.base[2]);
    mw.base[0] = dot(rgb, spo_basis(spo, l3.x));
    mw.base[1] = dot(rgb, spo_basis(spo, l3.y));
    mw.base[2] = dot(rgb, spo_basis(spo, l3.z));
    out = make_lobes(nrm, v, mw, eta, tab, trans, spec, hz, n0, inside, 0.f, &l3);
}
// optWeight: what a ray carries, as luminance -- its colour's, or by wavelength its Y
__device__ __forceinline__ float opt_weight(const OptArgs& o, f3 beta, float lamw) {
    return o.spectral ? spo_xyz(o.spo, beta, spo_lams(o.spo, spo_u(lamw))).y : luma(beta);
}

__device__ __forceinline__ long long fx(float w) { return __double2ll_rn((double)w * OPT_FX); }

// THE WARP'S TALLY: for every key the warp's lanes hold, the sums of their NV values over the lanes holding it, added
// to base[key * stride + j] by one lane -- a few shuffles and one atomic a key instead of one a lane. Every lane of
// the warp calls it; a lane with nothing to add passes has = false.
template <int NV>
__device__ __forceinline__ void warp_tally(bool has, uint32_t key, const long long (&v)[NV], unsigned long long* base,
                                           uint32_t stride) {
    uint32_t pending = __ballot_sync(FULL_MASK, has);
    const uint32_t lane = threadIdx.x & 31u;
    while (pending) {
        const uint32_t leader = __ffs(pending) - 1;
        const uint32_t k = __shfl_sync(FULL_MASK, key, leader);
        const bool mine = has && key == k;
#pragma unroll
        for (int j = 0; j < NV; j++) {
            long long x = mine ? v[j] : 0ll;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL_MASK, x, o);
            if (lane == leader && x != 0ll) atomicAdd(&base[(size_t)k * stride + j], (unsigned long long)x);
        }
        pending &= ~__ballot_sync(FULL_MASK, mine);
    }
}

// scene_full with the item it answered from: the first primitive of the item whose surface is nearest (the tag the
// reference's capture pass finds, scene_api.js tagCaptureBegin/End)
__device__ __forceinline__ SceneHit scene_full_item(const DPrim* __restrict__ pr, uint32_t n, f3 p, uint32_t& item) {
    SceneHit H{1e7f, 0u, 0u};
    float insideW = -1e7f;
    item = 0;
    uint32_t i = 0;
    while (i < n) {
        float di = prim_sdf(pr[i], p);
        uint32_t mat = pr[i].h.z;
        float nearv = fabsf(di);
        uint32_t j = i + 1;
        while (j < n) {
            const uint32_t op = pr[j].h.y;
            if (op == ST_OP_ITEM) break;
            if (op == ST_OP_SMOOTH) {
                float k = pr[j].r0.w;
                if (!beyond(pr[j], p, fmaxf(di + fmaxf(k, 0.f) * CULL_REL, nearv) + CULL_ABS)) {
                    float dj = prim_sdf(pr[j], p);
                    di = smooth_union(di, dj, k);
                    if (fabsf(dj) < nearv) { nearv = fabsf(dj); mat = pr[j].h.z; }
                }
            } else if (op == ST_OP_UNION) {
                if (!beyond(pr[j], p, fmaxf(di, nearv) + CULL_ABS)) {
                    float dj = prim_sdf(pr[j], p);
                    di = fminf(di, dj);
                    if (fabsf(dj) < nearv) { nearv = fabsf(dj); mat = pr[j].h.z; }
                }
            } else {
                if (!beyond(pr[j], p, -di + CULL_ABS)) di = fmaxf(di, -prim_sdf(pr[j], p));
            }
            j++;
        }
        if (di < 0.f && di > insideW) { insideW = di; H.a = mat; }
        if (fabsf(di) < fabsf(H.d)) { H.d = di; H.m = mat; item = i; }
        i = j;
    }
    return H;
}

// a kept path's next vertex (the reference's optVertex): one thread holds a ray at a time, so no atomics
__device__ __forceinline__ void opt_vertex(const OptArgs& o, uint32_t inst, uint32_t id, f3 p, float w, float opl, f3 c) {
    if (id >= o.path_rays) return;
    const size_t r = (size_t)inst * o.path_rays + id;
    const uint32_t k = o.vcount[r];
    if (k >= o.path_verts) return;
    const float y = luma(c);
    const f3 hue = y > 0.f ? c / y : mk(1.f);
    float4* v = o.verts + (r * o.path_verts + k) * VERT_F4;
    v[0] = f4(p, w);
    v[1] = make_float4(opl, hue.x, hue.y, hue.z);
    o.vcount[r] = k + 1u;
}

// the far field's bin (kernels.js:251-272 optFarAdd), in f32 as the kernel bins it
__device__ __forceinline__ uint32_t far_bin(const OptArgs& o, f3 d) {
    f3 dn = normalize(d);
    float g = acosf(clampf(dot(dn, o.axis), -1.f, 1.f));
    float c = atan2f(dot(dn, o.c90), dot(dn, o.c0));
    if (c < 0.f) c += 6.28318530718f;
    uint32_t ig = min((uint32_t)(g / 3.14159265359f * (float)(o.nG - 1) + 0.5f), o.nG - 1);
    uint32_t ic = (uint32_t)(c / 6.28318530718f * (float)o.nC + 0.5f) % o.nC;
    return ig * o.nC + ic;
}

// A SOURCE'S RAY (kernels.js:299-408 optSourceRay): the source by flux, a point on it, the side, the direction from
// its distribution, two march tolerances off the sheet when it is geometry
__device__ __forceinline__ void source_ray(const OptArgs& o, uint32_t inst, Rng& rng, f3& org, f3& dir, float& en,
                                           float& w, uint32_t& ks) {
    const uint2 rg = o.src_range[inst];
    float4 pick = rng.next();
    uint32_t k = rg.x;
    for (uint32_t i = 0; i < rg.y; i++) { k = rg.x + i; if (pick.x <= o.cdf[rg.x + i]) break; }
    ks = k;
    const st_optics_source& s = o.src[k];
    w = 1.f;
    if (s.shape == 3u) {                                              // A RAY SET: one of its rays, as it is, weighted
        const uint32_t cnt = max(s.ray_count, 1u);
        const float4 u = rng.next();
        const uint32_t j = min(s.ray_first + min((uint32_t)(u.x * (float)cnt), cnt - 1u), o.n_rays - 1u);
        const float4 a = o.rays[2u * j], d = o.rays[2u * j + 1u];
        org = mk(a.x, a.y, a.z);
        dir = normalize(mk(d.x, d.y, d.z));
        w = a.w;
        en = fmaxf(1.f, s.emit_n);
        return;
    }
    f3 front = normalize(mk(s.axis[0], s.axis[1], s.axis[2]));
    f3 t0 = mk(s.tangent[0], s.tangent[1], s.tangent[2]);
    f3 tu = normalize(t0 - front * dot(t0, front));
    f3 tv = cross(front, tu);
    float4 u = rng.next();
    f3 p = mk(s.centre[0], s.centre[1], s.centre[2]);
    if (s.shape == 1u) {
        float r = s.size_x * sqrtf(u.x);
        float sp, cp;
        sincosf(6.28318530718f * u.y, &sp, &cp);
        p = p + (tu * cp + tv * sp) * r;
    } else if (s.shape == 2u) {
        p = p + tu * ((2.f * u.x - 1.f) * s.size_x) + tv * ((2.f * u.y - 1.f) * s.size_y);
    }
    f3 ax = front;
    if (s.two_sided && pick.y < 0.5f) ax = -front;
    float4 u2 = rng.next();
    float c = 1.f;
    if (s.dist == 1u) c = 1.f - u2.x * (1.f - s.cos_half);
    else if (s.dist == 2u) {
        float e = s.n_exp + 1.f;
        float lo = powf(fmaxf(s.cos_half, 0.f), e);
        c = powf(1.f - u2.x * (1.f - lo), 1.f / e);
    }
    float sn = sqrtf(fmaxf(0.f, 1.f - c * c));
    float sp2, cp2;
    sincosf(6.28318530718f * u2.y, &sp2, &cp2);
    dir = normalize(tu * (sn * cp2) + tv * (sn * sp2) + ax * c);
    float off = s.on_surface ? 2.f * march_tol(p, o.w.u.tol) : 0.f;
    org = p + ax * off;
    en = fmaxf(1.f, s.emit_n);
}

__global__ void __launch_bounds__(256) k_opt_gen(OptArgs o) {
    __shared__ uint32_t pre[OPT_MAX_INST + 1];
    for (uint32_t i = threadIdx.x; i <= o.n_inst; i += blockDim.x) pre[i] = o.wave_prefix[i];
    __syncthreads();
    const WaveArgs& a = o.w;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.slots; i += gridDim.x * blockDim.x) {
        // the instance whose slots hold i: the first j in [1, n] with pre[j] > i, less one
        uint32_t lo = 1, hi = o.n_inst;
        while (lo < hi) { uint32_t mid = (lo + hi) >> 1; if (pre[mid] > i) hi = mid; else lo = mid + 1; }
        const uint32_t inst = lo - 1;
        uint32_t id = o.wave_first[inst] + (i - pre[inst]);
        Rng rng;
        rng.h = sample_seed(o.seed, inst);
        rng.seed(id);
        rng.seed(0x9E3779B9u);
        f3 org, dir;
        float en, w;
        uint32_t ks = 0;
        source_ray(o, inst, rng, org, dir, en, w, ks);
        a.pb.pos[i] = make_float4(org.x, org.y, org.z, 0.f);
        a.pb.dir[i] = make_float4(dir.x, dir.y, dir.z, en);
        // a ray set's ray carries its weight; a light its colour at that luminance -- or, by wavelength, three
        // wavelengths of its spectrum, each weighing S(l) / (3 p(l)) (optics/spectral.js: sum_k w_k y-bar(l_k) is w
        // on average)
        const st_optics_source& s = o.src[ks];
        f3 c = mk(w);
        if (o.spectral) {
            const float4 ur = rng.next();
            const float* sp = o.spo + 7u * SPO_NODES + (size_t)ks * SPO_NODES;
            float uk = ur.x;
            float b[3];
            for (int k = 0; k < 3; k++) {
                const float2 lp = spo_lambda(o.spo, uk);
                b[k] = lp.y > 0.f ? w * spo_node(sp, 0u, lp.x) / (3.f * lp.y) : 0.f;
                uk += 1.f / 3.f;
                if (uk >= 1.f) uk -= 1.f;
            }
            c = mk(b[0], b[1], b[2]);
            a.pb.lam[i] = ur.x;
        } else {
            a.pb.lam[i] = 0.f;                                          // no wavelength yet
            if (s.colour[0] != 0.f || s.colour[1] != 0.f || s.colour[2] != 0.f) {
                const f3 col = mk(s.colour[0], s.colour[1], s.colour[2]);
                const float y = luma(col);
                if (y > 0.f) c = col * (w / y);
            }
        }
        // w: what it carries as luminance (optWeight), carried with it so that every interaction's weight in is exactly
        // the last one's weight out, and the tallies' sums telescope to what was emitted bit for bit (a weight worked
        // out again from the stored colour could round to another integer of the fixed point)
        const float wt = o.spectral ? spo_xyz(o.spo, c, spo_lams(o.spo, a.pb.lam[i])).y
                                    : ((c.x == c.y && c.y == c.z) ? c.x : luma(c));
        a.pb.beta[i] = make_float4(c.x, c.y, c.z, wt);
        if (o.has_sets) atomicAdd(&o.tot[(size_t)inst * OPT_TOT + T_EMIT], (unsigned long long)fx(w));
        if (id < o.path_rays) {                                         // a kept path starts where the ray leaves
            o.vcount[(size_t)inst * o.path_rays + id] = 0u;
            opt_vertex(o, inst, id, org, w, 0.f, c);
        }
        a.pb.rad[i] = make_float4(1.f, 1.f, 1.f, 0.f);          // a photon's radiance field is its flux: weight 1
        a.pb.meta[i] = make_uint4(id, meta_y(0, 0, RAY_ACTIVE), 0u, inst);
        a.q.ray[0][i] = i;
    }
}

// THE SHADE (kernels.js:571-699): escaped, lost, a detector's, or an interaction -- pathBegin..pathEnd with a
// photon's rules: no light sampling, no end at a scatter, the bounce cap. Each lane works out what its ray adds to the
// tallies; then the warp adds them, the instance's totals into the CTA's shared sums (flushed once at its end), the
// object's and the material's incident / leaving / interactions into global sums, one atomic a key a warp.
__global__ void __launch_bounds__(256) k_opt_shade(OptArgs o, int nxt, int last) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ __align__(8) uint64_t mbar2;
    const WaveArgs& a = o.w;
    const Uni& u = a.u;
    DPrim* sp = reinterpret_cast<DPrim*>(smem);
    st_material* sm = reinterpret_cast<st_material*>(smem + u.n_prims * sizeof(DPrim));
    unsigned long long* stot =
        reinterpret_cast<unsigned long long*>(smem + u.n_prims * sizeof(DPrim) + u.n_mats * sizeof(st_material));
    for (uint32_t i = threadIdx.x; i < o.n_inst * OPT_TOT; i += blockDim.x) stot[i] = 0ull;
    if (!stage_table(sp, a.prims, u.n_prims * (uint32_t)sizeof(DPrim), &mbar, a.ctr)) return;
    if (!stage_table(sm, a.mats, u.n_mats * (uint32_t)sizeof(st_material), &mbar2, a.ctr)) return;
    const uint32_t count = a.ctr->hitCount;
    uint32_t* __restrict__ outq = nxt ? a.q.ray[1] : a.q.ray[0];
    uint32_t* outc = nxt ? &a.ctr->rayCount[1] : &a.ctr->rayCount[0];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t nrounds = (count + stride - 1) / stride;
    for (uint32_t r = 0; r < nrounds; r++) {
        uint32_t q = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool cont = false;
        float wcar = 0.f;                                            // the weight a ray going on carries
        uint32_t slot = 0, inst = 0, tag = 0, mati = 0;
        f3 pos, dir, beta;
        float ltot = 0.f, n = 1.f;
        uint4 m4 = make_uint4(0, 0, 0, 0);
        // this ray's part of the tallies
        long long tv[OPT_TOT - 6] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};   // T_EMIT .. T_NABS
        long long iv[3] = {0, 0, 0};                                 // incident, leaving, interactions (its object, material)
        bool interacted = false;
        if (q < count) {
            slot = a.q.hit[q];
            const float dh = a.q.hitd[q];
            float4 p4 = a.pb.pos[slot], d4 = a.pb.dir[slot], b4 = a.pb.beta[slot];
            m4 = a.pb.meta[slot];
            pos = xyz(p4); ltot = p4.w; dir = xyz(d4); n = d4.w; beta = xyz(b4);
            inst = m4.w;
            const uint32_t id = m4.x;
            uint32_t bounces = m4.y & 0xffu, state = (m4.y >> 16) & 0xffu;
            // by wavelength its u (and whether it collapsed); in colour the wavelength a dispersive glass gave it (0 none)
            const float lamw = a.pb.lam[slot];
            const float wIn = b4.w;                                   // optWeight: beta x radiance (1), as luminance
            wcar = wIn;
            if (state == RAY_ESCAPED) {                               // kernels.js:609-625
                tv[T_ESC] = fx(wIn);
                tv[T_NESC] = 1;
                atomicAdd(&o.far[(size_t)inst * o.nG * o.nC + far_bin(o, dir)], (unsigned long long)fx(wIn));
                if (id < o.path_rays) {                               // drawn esc_len past its last vertex
                    const size_t pr = (size_t)inst * o.path_rays + id;
                    const uint32_t k = o.vcount[pr];
                    if (k > 0u && k <= o.path_verts) {
                        const float4* lv = o.verts + (pr * o.path_verts + (k - 1u)) * VERT_F4;
                        opt_vertex(o, inst, id, xyz(lv[0]) + dir * o.esc_len, wIn, lv[1].x + o.esc_len * n, beta);
                    }
                }
                // the lux plane: the escaping ray's line at `height` along the axis (nothing lies beyond the scene)
                float dn = dot(dir, o.axis);
                if (o.cells && dn > 0.f) {
                    float4 og = o.origin[inst];
                    f3 rel = pos - xyz(og);
                    float t = (o.height - dot(rel, o.axis)) / dn;
                    f3 hp = rel + dir * t;
                    float ha = dot(hp, o.c0), hb = dot(hp, o.c90);
                    float cell = 2.f * o.half / (float)o.cells;
                    if (t >= 0.f && fabsf(ha) < o.half && fabsf(hb) < o.half) {
                        uint32_t ix = min((uint32_t)((ha + o.half) / cell), o.cells - 1);
                        uint32_t iy = min((uint32_t)((hb + o.half) / cell), o.cells - 1);
                        atomicAdd(&o.lux[(size_t)inst * o.cells * o.cells + (size_t)iy * o.cells + ix],
                                  (unsigned long long)fx(wIn));
                    }
                }
            } else if (state != RAY_ACTIVE) {                          // out of steps or length: lost
                tv[T_LOST] = fx(wIn);
                tv[T_NLOST] = 1;
                opt_vertex(o, inst, id, pos, wIn, ltot, beta);
            } else {
                const uint2 rg = o.w.inst_range[inst];
                const DPrim* ip = sp + rg.x;
                const uint32_t np = rg.y;
                float eps = march_tol(pos, u.tol);
                float gx = scene_dist(ip, np, mk(pos.x + eps, pos.y, pos.z)) - dh;
                float gy = scene_dist(ip, np, mk(pos.x, pos.y + eps, pos.z)) - dh;
                float gz = scene_dist(ip, np, mk(pos.x, pos.y, pos.z + eps)) - dh;
                f3 nn = normalize(mk(gx, gy, gz));
                bool inside = dh < 0.f;
                f3 nrm = inside ? -nn : nn;
                float otol = 10.f * eps;
                uint32_t item = 0;
                SceneHit h = scene_full_item(ip, np, pos, item);
                tag = min(rg.x + item, OPT_TAG_MAX - 1u);
                mati = min(h.m, u.n_mats - 1);
                const st_material& m = sm[mati];
                if (m.detector > 0.5f && dot(-dir, nrm) >= 0.f) {     // kernels.js:660-672: a detector stops it
                    tv[T_DET] = fx(wIn);
                    tv[T_NDET] = 1;
                    tv[T_INTER] = 1;
                    iv[0] = fx(wIn);
                    iv[2] = 1;
                    interacted = true;
                    opt_vertex(o, inst, id, pos, wIn, ltot, beta);
                    const uint32_t k = atomicAdd(o.det_n, 1u);        // optRecordHit
                    if (k < o.det_cap) {
                        float4* d = o.det + (size_t)k * DET_F4;
                        d[0] = f4(pos, wIn);
                        d[1] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(tag | (inst << 16)));
                        // the colour as CIE X and Z of its linear Rec.709 rgb, or by wavelength its XYZ (Y is the weight)
                        if (o.spectral) {
                            const f3 X = spo_xyz(o.spo, beta, spo_lams(o.spo, spo_u(lamw)));
                            d[2] = make_float4(X.x, X.z, 0.f, 0.f);
                        } else {
                            d[2] = make_float4(0.4124f * beta.x + 0.3576f * beta.y + 0.1805f * beta.z,
                                               0.0193f * beta.x + 0.1192f * beta.y + 0.9505f * beta.z, 0.f, 0.f);
                        }
                    }
                } else if (dot(-dir, nrm) < 0.f) {                    // seen from behind: moved on, no interaction
                    f3 off = dir * otol;
                    pos = pos + off; ltot += length(off) * n;
                    if (last) { tv[T_LOST] = fx(wIn); tv[T_NLOST] = 1; opt_vertex(o, inst, id, pos, wIn, ltot, beta); }
                    else cont = true;
                } else {
                    Rng rng;
                    rng.h = sample_seed(o.seed, inst);
                    rng.seed(id);
                    rng.seed(bounces);
                    bounces += 1;
                    const f3 hit_pos = pos, beta_in = beta;
                    const float hit_ltot = ltot;
                    float n0 = n, n1 = fmaxf(m.ior, n0), v1 = 0.f;
                    if (m.transmission > 0.f && m.metallic < 1.f) {
                        SceneHit mb = scene_full(ip, np, pos + (-nrm) * (otol * 2.f));
                        n1 = sm[min(mb.a, u.n_mats - 1)].ior;
                        v1 = sm[min(mb.a, u.n_mats - 1)].abbe;
                    }
                    // BY WAVELENGTH (optics/spectral.js WHAT A MATERIAL IS AT A WAVELENGTH): the colour a reflectance at
                    // each of the ray's wavelengths, the coating taken at each; a dispersive glass beyond refracts the
                    // first wavelength (at its n, the pick the d line's) and drops the other two
                    f3 l3 = mk(0.f);
                    float nT = n1;
                    bool collapse = false;
                    SpecDraw sd;
                    bool draw = false;
                    if (o.spectral) {
                        l3 = spo_lams(o.spo, spo_u(lamw));
                        if (v1 > 0.f) { nT = cauchy_n(n1, v1, l3.x); collapse = lamw < 2.f; }
                    } else if (v1 > 0.f) {
                        // IN COLOUR (materials_pbr.js:1116-1139, as the renderer's): a ray with a wavelength meets the
                        // dispersive glass at n(its wavelength); one without draws one from the camera's table, used
                        // if it refracts, its channels weighed by what that wavelength is to them; the pick the d line's
                        if (lamw > 0.f) nT = cauchy_n(n1, v1, lamw);
                        else {
                            const float4 rl = rng.next();
                            sd = spec_draw(a.spec, rl.x);
                            sd.lam = lambda_coded(sd.lam);
                            nT = cauchy_n(n1, v1, sd.lam);
                            draw = true;
                        }
                    }
                    float pG = refract_share_of(m.transmission, m.haze), trans = m.transmission, specv = m.specular;
                    float hz = m.haze;
                    bool diffFace = pG <= 0.f && m.transmission > 0.f;
                    if (inside && pG > 0.f && pG < 1.f) {
                        float k = mixf(2.f * m.specular, 1.f, pG);
                        float4 r4 = rng.next();
                        if (r4.x < pG) { trans = 1.f; hz = 0.f; }
                        else {
                            trans = sat(sat(m.transmission) * sat(m.haze) / fmaxf(1.f - pG, 1e-6f));
                            hz = 1.f; specv = 0.5f * k; diffFace = true;
                        }
                    }
                    float etaFace = diffFace ? fminf(n0, n1) / fmaxf(n0, n1) : n0 / n1;
                    Lobes lb;
                    if (o.spectral) spectral_lobes(o.spo, l3, nrm, -dir, m, etaFace, a.tab, trans, specv, hz, n0, inside, lb);
                    else lb = make_lobes(nrm, -dir, m, etaFace, a.tab, trans, specv, hz, n0, inside, 0.f);
                    lb.etaT = n0 / nT;
                    coat_pick(lb, beta);
                    LobeSample smp = lobes_sample(lb, a.tab, rng.next());
                    dir = smp.dir;
                    beta = beta * smp.w;
                    float lamo = lamw;
                    if (smp.transmitted) {
                        n = nT;
                        if (collapse) { beta = mk(3.f * beta.x, 0.f, 0.f); lamo = lamw + 2.f; }
                        if (draw) { beta = beta * sd.w; lamo = sd.lam; }
                    }
                    uint32_t st = RAY_ACTIVE;
                    if (max3(smp.w) <= 0.f) st = RAY_ABSORBED;
                    f3 off = dir * otol;
                    pos = pos + off; ltot += length(off) * n;
                    if (bounces > u.maxbounce) st = RAY_TERMINATED;
                    bool goesOn = st == RAY_ACTIVE || st == RAY_TERMINATED;
                    float wOut = goesOn ? opt_weight(o, beta, lamo) : 0.f;
                    wcar = wOut;
                    if (lamo != lamw) a.pb.lam[slot] = lamo;
                    tv[T_INTER] = 1;
                    tv[T_ABS] = fx(wIn) - fx(wOut);
                    if (!goesOn) tv[T_NABS] = 1;
                    iv[0] = fx(wIn);
                    iv[1] = fx(wOut);
                    iv[2] = 1;
                    interacted = true;
                    opt_vertex(o, inst, id, hit_pos, wIn, hit_ltot, beta_in);
                    if (st == RAY_TERMINATED || (st == RAY_ACTIVE && last)) { tv[T_LOST] = fx(wOut); tv[T_NLOST] = 1; }
                    else if (st == RAY_ACTIVE) cont = true;
                    m4.y = meta_y(bounces, (m4.y >> 8) & 0xffu, RAY_ACTIVE);
                }
            }
        }
        // the warp's tallies: the instances' totals into shared memory, the objects' and materials' into global
        warp_tally<OPT_TOT - 6>(q < count, inst, tv, stot, OPT_TOT);
        warp_tally<3>(interacted, tag, iv, o.tag, 3u);
        warp_tally<3>(interacted, inst * u.n_mats + mati, iv, o.mat, 3u);
        uint32_t rq = warp_append(outc, cont);
        if (cont) {
            a.pb.pos[slot] = f4(pos, ltot);
            a.pb.dir[slot] = f4(dir, n);
            a.pb.beta[slot] = f4(beta, wcar);
            m4.y = (m4.y & 0xffffu) | (RAY_ACTIVE << 16);
            a.pb.meta[slot] = m4;
            outq[rq] = slot;
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < o.n_inst * OPT_TOT; i += blockDim.x)
        if (stot[i] != 0ull) atomicAdd(&o.tot[i], stot[i]);
}

// THE FLUSH: the fixed-point sums as FP64 weight (counts stay counts), where they are read out
__global__ void k_opt_flush(const unsigned long long* __restrict__ in, double* __restrict__ out, size_t n, int counts) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = counts ? (double)in[i] : (double)(long long)in[i] / OPT_FX;
}

uint32_t __float_as_uint_host(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

f3 normalize_host(f3 a) {
    float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return mk(a.x / l, a.y / l, a.z / l);
}

template <class X>
cudaError_t grow(X*& p, size_t& have, size_t want) {
    if (have >= want && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    have = 0;
    cudaError_t e = cudaMalloc(&p, want * sizeof(X));
    if (e == cudaSuccess) have = want;
    return e;
}

// the optics run's device buffers, kept in the context between runs
struct OptBuf {
    float4 *pos = nullptr, *dir = nullptr, *beta = nullptr, *rad = nullptr;
    uint4* meta = nullptr;
    uint32_t *ray0 = nullptr, *ray1 = nullptr, *hit = nullptr;
    float* hitd = nullptr;
    size_t cap = 0, c1 = 0, c2 = 0, c3 = 0, c4 = 0, c5 = 0, c6 = 0, c7 = 0, c8 = 0, c9 = 0;
    unsigned long long *far = nullptr, *lux = nullptr, *tot = nullptr, *tag = nullptr, *mat = nullptr;
    size_t nfar = 0, nlux = 0, ntot = 0, ntag = 0, nmat = 0;
    st_optics_source* src = nullptr; size_t nsrc = 0;
    float* cdf = nullptr; size_t ncdf = 0;
    uint2 *range = nullptr, *srange = nullptr; size_t nrange = 0, nsrange = 0;
    float4* origin = nullptr; size_t norigin = 0;
    uint32_t *wfirst = nullptr, *wpre = nullptr; size_t nwfirst = 0, nwpre = 0;
    DevCtr* ctr = nullptr; size_t nctr = 0;
    float4 *det = nullptr, *verts = nullptr; size_t ndet = 0, nverts = 0;
    uint32_t *det_n = nullptr, *vcount = nullptr; size_t ndetn = 0, nvcount = 0;
    float* lam = nullptr; size_t nlam = 0;      // the trace by wavelength: each ray's u (and whether it collapsed)
    float* spo = nullptr; size_t nspo = 0;      // ...its tables and the sources' spectra
    uint64_t spo_gen = 0;                       // the spectra's change the tables were made with
    // the last run, kept for the readings after it (st_optics_tallies / _hits / _paths)
    uint32_t last_ni = 0, last_mats = 0, last_det_cap = 0, last_path_rays = 0, last_path_verts = 0;
    // THE BATCH AS ONE CUDA GRAPH: its whole chain captured at its first run and replayed while nothing it was
    // captured with changes (the key: the scene, the batch, the far field, the sources, the detail, the buffers)
    cudaGraphExec_t graph = nullptr;
    std::vector<uint64_t> graph_key;
    uint32_t graph_launches = 0;
};

}  // namespace

void optics_free(OpticsState& os) {
    if (os.rays) { cudaFree(os.rays); os.rays = nullptr; os.n_rays = 0; }
    if (!os.scratch) return;
    OptBuf* B = static_cast<OptBuf*>(os.scratch);
    void* ps[] = {B->pos, B->dir, B->beta, B->rad, B->meta, B->ray0, B->ray1, B->hit, B->hitd, B->far, B->lux, B->tot,
                  B->tag, B->mat, B->src, B->cdf, B->range, B->srange, B->origin, B->wfirst, B->wpre, B->ctr, B->det,
                  B->verts, B->det_n, B->vcount, B->lam, B->spo};
    for (void* p : ps)
        if (p) cudaFree(p);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    delete B;
    os.scratch = nullptr;
}

extern "C" {

int st_optics_set_sources(st_ctx* ctx, const st_optics_source* src, uint32_t n) {
    if (!ctx || (n && !src)) return ST_ERR_ARG;
    for (uint32_t i = 0; i < n; i++)
        if (src[i].shape > 3 || src[i].dist > 2 || !(src[i].flux >= 0) || src[i].instance >= OPT_MAX_INST) {
            ctx_set_error(ctx, "source " + std::to_string(i) + ": shape, distribution, flux or instance out of range");
            return ST_ERR_ARG;
        }
    ctx_ext(ctx).optics.sources.assign(src, src + n);
    ctx_ext(ctx).optics.sources_gen++;
    return ST_OK;
}

int st_optics_set_spectra(st_ctx* ctx, const float* values, uint32_t n) {
    if (!ctx || (n && !values)) return ST_ERR_ARG;
    OpticsState& os = ctx_ext(ctx).optics;
    os.spectra.assign(values, values + (size_t)n * ST_SPECTRUM_NODES);
    os.sources_gen++;
    return ST_OK;
}

int st_optics_set_rays(st_ctx* ctx, const float* rays, uint32_t n) {
    if (!ctx || (n && !rays)) return ST_ERR_ARG;
    OpticsState& os = ctx_ext(ctx).optics;
    if (os.rays) { cudaFree(os.rays); os.rays = nullptr; os.n_rays = 0; }
    if (!n) return ST_OK;
    std::vector<float4> h((size_t)n * 2);
    for (uint32_t i = 0; i < n; i++) {
        const float* r = rays + (size_t)i * 8;
        h[2 * i] = make_float4(r[0], r[1], r[2], r[3]);
        h[2 * i + 1] = make_float4(r[4], r[5], r[6], r[7]);
    }
    cudaError_t e = cudaMalloc(&os.rays, h.size() * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemcpy(os.rays, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (os.rays) cudaFree(os.rays);
        os.rays = nullptr;
        ctx_set_error(ctx, std::string("ray table: ") + cudaGetErrorString(e));
        return ST_ERR_CUDA;
    }
    os.n_rays = n;
    os.sources_gen++;
    return ST_OK;
}

int st_optics_set_far(st_ctx* ctx, const st_optics_far* far) {
    if (!ctx || !far) return ST_ERR_ARG;
    if (far->nC == 0 || far->nG < 2 || (uint64_t)far->nC * far->nG > (1u << 24)) {
        ctx_set_error(ctx, "far field grid out of range");
        return ST_ERR_ARG;
    }
    ctx_ext(ctx).optics.far = *far;
    ctx_ext(ctx).optics.has_far = true;
    return ST_OK;
}

int st_optics_run(st_ctx* ctx, const st_optics_batch* b, double* far_out, double* lux_out, st_optics_totals* totals) {
    if (!ctx || !b || !b->ray_count || b->n_instances == 0 || b->n_instances > OPT_MAX_INST) return ST_ERR_ARG;
    OpticsState& os = ctx_ext(ctx).optics;
    if (!ctx_has_scene(ctx)) { ctx_set_error(ctx, "set a scene first"); return ST_ERR_STATE; }
    if (!os.has_far) { ctx_set_error(ctx, "set the far field first (st_optics_set_far)"); return ST_ERR_STATE; }
    for (const st_optics_source& q : os.sources)
        if (q.shape == 3u && (q.ray_count == 0 || (uint64_t)q.ray_first + q.ray_count > os.n_rays)) {
            ctx_set_error(ctx, "a ray set's rays are past the ray table (st_optics_set_rays)");
            return ST_ERR_ARG;
        }
    if (b->lux_cells > 4096) { ctx_set_error(ctx, "lux map over 4096 cells a side"); return ST_ERR_ARG; }
    if (b->maxbounce > 250) { ctx_set_error(ctx, "maxbounce over 250 (a ray's bounces are counted in 8 bits)"); return ST_ERR_ARG; }
    const uint32_t NI = b->n_instances;
    if ((uint64_t)NI * b->lux_cells * b->lux_cells > (1ull << 28) ||
        (uint64_t)NI * os.far.nC * os.far.nG > (1ull << 28)) {
        ctx_set_error(ctx, "the batch's far fields or lux maps hold over 2^28 bins");
        return ST_ERR_ARG;
    }
    cudaSetDevice(ctx_device(ctx));
    cudaStream_t st = ctx_stream(ctx);
    if (!os.scratch) os.scratch = new OptBuf();
    OptBuf& B = *static_cast<OptBuf*>(os.scratch);
    auto fail = [&](cudaError_t e, const char* what) {
        ctx_set_error(ctx, std::string(what) + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? ST_ERR_OOM : ST_ERR_CUDA;
    };

    // each instance's table range: the primitives whose flags >> 8 name it, contiguous (st_optics_batch)
    const uint32_t np = ctx_n_prims(ctx);
    std::vector<st_prim> prims(np);
    {
        std::vector<DPrim> dp(np);
        cudaMemcpy(dp.data(), ctx_d_prims(ctx), np * sizeof(DPrim), cudaMemcpyDeviceToHost);
        for (uint32_t i = 0; i < np; i++) prims[i].flags = dp[i].h.w;
    }
    std::vector<uint2> range(NI, make_uint2(0, 0));
    for (uint32_t i = 0; i < np; i++) {
        uint32_t inst = prims[i].flags >> 8;
        if (inst >= NI) { ctx_set_error(ctx, "primitive " + std::to_string(i) + " names an instance past the batch"); return ST_ERR_ARG; }
        if (range[inst].y == 0) range[inst] = make_uint2(i, 1);
        else if (range[inst].x + range[inst].y == i) range[inst].y++;
        else { ctx_set_error(ctx, "instance " + std::to_string(inst) + "'s primitives are not contiguous"); return ST_ERR_ARG; }
    }
    // sources by instance, their cumulative shares, each instance's axis origin
    std::vector<st_optics_source> src;
    std::vector<float> cdf;
    std::vector<uint2> srange(NI, make_uint2(0, 0));
    std::vector<float4> origin(NI, make_float4(0, 0, 0, 0));
    for (uint32_t inst = 0; inst < NI; inst++) {
        srange[inst].x = (uint32_t)src.size();
        double tot = 0;
        for (auto& s : os.sources) if (s.instance == inst) { src.push_back(s); tot += s.flux; }
        srange[inst].y = (uint32_t)src.size() - srange[inst].x;
        if (b->ray_count[inst] && (!srange[inst].y || range[inst].y == 0)) {
            ctx_set_error(ctx, "instance " + std::to_string(inst) + " has rays but no source or no geometry");
            return ST_ERR_ARG;
        }
        double acc = 0;
        for (uint32_t k = 0; k < srange[inst].y; k++) {
            acc += src[srange[inst].x + k].flux;
            cdf.push_back(tot > 0 ? (float)(acc / tot) : (float)(k + 1) / srange[inst].y);
        }
        if (srange[inst].y) {
            cdf.back() = 1.f;
            const st_optics_source& s0 = src[srange[inst].x];
            origin[inst] = make_float4(s0.centre[0], s0.centre[1], s0.centre[2], 0.f);
        }
    }
    const st_optics_far& F = os.far;
    const st_optics_detail& D = os.detail;
    const size_t nfar = (size_t)NI * F.nG * F.nC, nlux = (size_t)NI * b->lux_cells * b->lux_cells;
    const uint32_t NM = ctx_n_mats(ctx);
    uint64_t total = 0;
    for (uint32_t i = 0; i < NI; i++) total += b->ray_count[i];
    const uint32_t K = (uint32_t)std::max<uint64_t>(1, (total + OPT_WAVE - 1) / OPT_WAVE);   // planBatches
    const size_t W = (size_t)std::min<uint64_t>(OPT_WAVE + NI, total + NI);
    const size_t nverts = (size_t)NI * D.path_rays * D.path_verts * VERT_F4;
    cudaError_t e;
    if ((e = grow(B.pos, B.cap, W)) || (e = grow(B.dir, B.c1, W)) || (e = grow(B.beta, B.c2, W)) || (e = grow(B.rad, B.c3, W)) ||
        (e = grow(B.meta, B.c4, W)) || (e = grow(B.ray0, B.c5, W)) || (e = grow(B.ray1, B.c6, W)) || (e = grow(B.hit, B.c7, W)) ||
        (e = grow(B.hitd, B.c8, W)) || (e = grow(B.far, B.nfar, std::max<size_t>(nfar, 1))) ||
        (e = grow(B.lux, B.nlux, std::max<size_t>(nlux, 1))) || (e = grow(B.tot, B.ntot, (size_t)NI * OPT_TOT)) ||
        (e = grow(B.tag, B.ntag, (size_t)OPT_TAG_MAX * 3)) || (e = grow(B.mat, B.nmat, (size_t)NI * NM * 3)) ||
        (e = grow(B.src, B.nsrc, std::max<size_t>(src.size(), 1))) || (e = grow(B.cdf, B.ncdf, std::max<size_t>(cdf.size(), 1))) ||
        (e = grow(B.range, B.nrange, (size_t)NI)) || (e = grow(B.srange, B.nsrange, (size_t)NI)) ||
        (e = grow(B.origin, B.norigin, (size_t)NI)) || (e = grow(B.wfirst, B.nwfirst, (size_t)NI * K)) ||
        (e = grow(B.wpre, B.nwpre, (size_t)(NI + 1) * K)) || (e = grow(B.ctr, B.nctr, (size_t)1)) ||
        (e = grow(B.det, B.ndet, std::max<size_t>((size_t)D.det_cap * DET_F4, 1))) ||
        (e = grow(B.det_n, B.ndetn, (size_t)1)) || (e = grow(B.verts, B.nverts, std::max<size_t>(nverts, 1))) ||
        (e = grow(B.vcount, B.nvcount, std::max<size_t>((size_t)NI * D.path_rays, 1))) ||
        (e = grow(B.lam, B.nlam, W)) ||
        (b->spectral && (e = grow(B.spo, B.nspo, (size_t)(7 + src.size()) * SPO_N))))
        return fail(e, "cudaMalloc optics buffers");
    // THE TRACE BY WAVELENGTH's tables and each source's spectrum at luminance 1 (optics/spectral.js spectralBuffer)
    if (b->spectral) {
        for (const st_optics_source& q : src)
            if (q.spectrum && (size_t)q.spectrum * ST_SPECTRUM_NODES > os.spectra.size()) {
                ctx_set_error(ctx, "a source names spectrum " + std::to_string(q.spectrum) + " past the table");
                return ST_ERR_ARG;
            }
        const std::vector<double> tab = spo_tables();
        std::vector<float> h((size_t)(7 + src.size()) * SPO_N);
        for (size_t i = 0; i < tab.size(); i++) h[i] = (float)tab[i];
        for (size_t k = 0; k < src.size(); k++) {
            const st_optics_source& q = src[k];
            const float* row = q.spectrum ? os.spectra.data() + (size_t)(q.spectrum - 1) * ST_SPECTRUM_NODES : nullptr;
            const std::vector<double> sv = spo_source(tab, row, q.cct, q.colour);
            for (int i = 0; i < SPO_N; i++) h[(7 + k) * SPO_N + i] = (float)sv[i];
        }
        if ((e = cudaMemcpyAsync(B.spo, h.data(), h.size() * 4, cudaMemcpyHostToDevice, st)))
            return fail(e, "optics spectra upload");
    }
    // the waves: each instance's rays split evenly over K of them (photons.js:31-62 splitPart), all K tables at once
    std::vector<uint32_t> wf((size_t)NI * K), wp((size_t)(NI + 1) * K, 0);
    std::vector<uint32_t> wslots(K);
    for (uint32_t k = 0; k < K; k++) {
        uint32_t* pre = wp.data() + (size_t)k * (NI + 1);
        for (uint32_t i = 0; i < NI; i++) {
            uint64_t n = b->ray_count[i];
            uint64_t f0 = n * k / K, f1 = n * (k + 1) / K;
            wf[(size_t)k * NI + i] = (uint32_t)f0;
            pre[i + 1] = pre[i] + (uint32_t)(f1 - f0);
        }
        wslots[k] = pre[NI];
    }
    if ((e = cudaMemcpyAsync(B.src, src.data(), src.size() * sizeof(st_optics_source), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(B.cdf, cdf.data(), cdf.size() * 4, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(B.range, range.data(), NI * sizeof(uint2), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(B.srange, srange.data(), NI * sizeof(uint2), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(B.origin, origin.data(), NI * sizeof(float4), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(B.wfirst, wf.data(), wf.size() * 4, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(B.wpre, wp.data(), wp.size() * 4, cudaMemcpyHostToDevice, st)) ||
        (e = cudaStreamSynchronize(st)))
        return fail(e, "optics upload");

    // the uniforms the march and the shade read: the scene's tolerance and radius, the settings' march controls
    const st_scene_desc& sd = ctx_desc(ctx);
    OptArgs o;
    Uni& u = o.w.u;
    u = Uni{};
    u.maxbounce = b->maxbounce ? b->maxbounce : 32;
    u.maxiter = 400;
    u.nee = 0; u.rr = 0;
    u.stepscale = 0.9f;
    u.claim = os.tune_claim;
    u.chunk = os.tune_chunk;
    const uint32_t chunk = u.chunk ? u.chunk : MARCH_CHUNK;
    u.budget = u.maxbounce + 1 + (u.maxiter + chunk - 1) / chunk + 4;
    double tol = sd.tolerance > 0 ? sd.tolerance : 1e-3;
    double R = sd.env_radius > 0 ? sd.env_radius : 400.0;
    u.tol = (float)tol; u.envR = (float)R; u.envR2 = (float)(R * R);
    u.n_prims = np; u.n_mats = NM;
    u.P = 1;
    o.w.prims = ctx_d_prims(ctx);
    o.w.mats = ctx_d_mats(ctx);
    o.w.tab = ctx_tab(ctx);
    o.w.pb = PathBuf{B.pos, B.dir, B.beta, B.rad, B.meta};
    o.w.pb.lam = B.lam;                 // by wavelength its u; in colour the wavelength a dispersive glass gave it
    o.w.spec = ctx_spec(ctx);
    o.spectral = b->spectral ? 1u : 0u;
    o.spo = b->spectral ? B.spo : nullptr;
    o.w.q = Queues{};
    o.w.q.ray[0] = B.ray0; o.w.q.ray[1] = B.ray1; o.w.q.hit = B.hit; o.w.q.hitd = B.hitd;
    o.w.q.cap = (uint32_t)W;
    o.w.ctr = B.ctr;
    o.w.frame = nullptr; o.w.acc = nullptr; o.w.mom = nullptr;
    o.w.spw = 1;
    o.w.inst_range = B.range;
    o.src = B.src; o.cdf = B.cdf; o.src_range = B.srange; o.origin = B.origin;
    o.rays = os.rays; o.n_rays = os.n_rays;
    o.has_sets = 0;
    for (const st_optics_source& q : os.sources) if (q.shape == 3u) o.has_sets = 1;
    o.n_inst = NI;
    o.seed = b->seed;
    f3 ax = normalize_host(mk(F.axis[0], F.axis[1], F.axis[2]));
    f3 c0 = normalize_host(mk(F.c0[0], F.c0[1], F.c0[2]));
    o.axis = ax; o.c0 = c0;
    o.c90 = mk(ax.y * c0.z - ax.z * c0.y, ax.z * c0.x - ax.x * c0.z, ax.x * c0.y - ax.y * c0.x);
    o.nC = F.nC; o.nG = F.nG; o.cells = b->lux_cells;
    o.half = b->lux_half; o.height = b->lux_height;
    o.far = B.far; o.lux = B.lux; o.tot = B.tot; o.tag = B.tag; o.mat = B.mat;
    o.det = B.det; o.det_n = B.det_n; o.det_cap = D.det_cap;
    o.verts = B.verts; o.vcount = B.vcount; o.path_rays = D.path_rays; o.path_verts = D.path_verts;
    o.esc_len = D.esc_len > 0.f ? D.esc_len : 0.1f;
    const int sms = ctx_sms(ctx);
    const size_t shade_smem = np * sizeof(DPrim) + u.n_mats * sizeof(st_material) + (size_t)NI * OPT_TOT * 8;
    cudaFuncSetAttribute(k_opt_shade, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shade_smem);
    int shade_blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&shade_blocks, k_opt_shade, 256, shade_smem);
    shade_blocks = std::max(1, shade_blocks) * sms;

    // THE CHAIN, every wave: the tallies cleared, then per wave its rays generated and traced to their ends
    auto chain = [&](uint32_t& launches) -> cudaError_t {
        cudaError_t r;
        launches = 0;
        if ((r = cudaMemsetAsync(B.far, 0, std::max<size_t>(nfar, 1) * 8, st)) ||
            (r = cudaMemsetAsync(B.lux, 0, std::max<size_t>(nlux, 1) * 8, st)) ||
            (r = cudaMemsetAsync(B.tot, 0, (size_t)NI * OPT_TOT * 8, st)) ||
            (r = cudaMemsetAsync(B.tag, 0, (size_t)OPT_TAG_MAX * 3 * 8, st)) ||
            (r = cudaMemsetAsync(B.mat, 0, (size_t)NI * NM * 3 * 8, st)) ||
            (r = cudaMemsetAsync(B.det_n, 0, 4, st)) ||
            (r = cudaMemsetAsync(B.ctr, 0, sizeof(DevCtr), st)))
            return r;
        for (uint32_t k = 0; k < K; k++) {
            const uint32_t slots = wslots[k];
            if (!slots) continue;
            OptArgs ok = o;
            ok.wave_first = B.wfirst + (size_t)k * NI;
            ok.wave_prefix = B.wpre + (size_t)k * (NI + 1);
            ok.w.slots = slots;
            if ((r = launch_iter_begin(ok.w, 0, 1, 1, st))) return r;
            k_opt_gen<<<std::min((slots + 255) / 256, (uint32_t)sms * 8u), 256, 0, st>>>(ok);
            launches += 2;
            int cur = 0;
            for (uint32_t it = 0; it < u.budget; it++) {
                int nxt = cur ^ 1, last = it + 1 == u.budget;
                if (it > 0 && (r = launch_iter_begin(ok.w, (int)it, nxt, 0, st))) return r;
                if ((r = launch_march(ok.w, cur, nxt, last, sms, st))) return r;
                k_opt_shade<<<shade_blocks, 256, shade_smem, st>>>(ok, nxt, last);
                launches += 3;
                cur = nxt;
            }
            if ((r = cudaGetLastError())) return r;
        }
        return cudaSuccess;
    };
    // the graph's key: everything the chain was recorded with
    std::vector<uint64_t> key = {ctx_scene_gen(ctx), NI, K, b->seed, b->lux_cells, b->maxbounce,
                                 (uint64_t)(uintptr_t)B.pos, (uint64_t)(uintptr_t)B.far, (uint64_t)(uintptr_t)B.lux,
                                 (uint64_t)(uintptr_t)B.det, (uint64_t)(uintptr_t)B.verts, (uint64_t)(uintptr_t)B.mat,
                                 (uint64_t)(uintptr_t)B.wfirst, (uint64_t)(uintptr_t)B.src, os.sources_gen,
                                 (uint64_t)(uintptr_t)os.rays, D.det_cap, D.path_rays, D.path_verts,
                                 (uint64_t)__float_as_uint_host(o.esc_len), F.nC, F.nG,
                                 (uint64_t)__float_as_uint_host(b->lux_half), (uint64_t)__float_as_uint_host(b->lux_height),
                                 u.claim, u.chunk, b->spectral, (uint64_t)(uintptr_t)B.lam, (uint64_t)(uintptr_t)B.spo};
    for (int k = 0; k < 3; k++) {
        key.push_back(__float_as_uint_host(F.axis[k]));
        key.push_back(__float_as_uint_host(F.c0[k]));
    }
    for (uint32_t i = 0; i < NI; i++) key.push_back(b->ray_count[i]);
    if (!B.graph || key != B.graph_key) {
        if (B.graph) { cudaGraphExecDestroy(B.graph); B.graph = nullptr; }
        cudaGraph_t g;
        uint32_t launches = 0;
        if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal))) return fail(e, "optics capture");
        cudaError_t e1 = chain(launches);
        cudaError_t e2 = cudaStreamEndCapture(st, &g);
        if (e1 || e2) { cudaGetLastError(); return fail(e1 ? e1 : e2, "optics capture"); }
        e = cudaGraphInstantiate(&B.graph, g, 0);
        cudaGraphDestroy(g);
        if (e) { B.graph = nullptr; return fail(e, "optics graph"); }
        B.graph_key = key;
        B.graph_launches = launches;
    }
    if ((e = cudaGraphLaunch(B.graph, st))) return fail(e, "optics graph launch");
    os.launches += B.graph_launches;
    // the readings: the totals as they are, the far field and the lux map flushed to FP64 in place, then read out
    std::vector<unsigned long long> tot((size_t)NI * OPT_TOT);
    if ((e = cudaMemcpyAsync(tot.data(), B.tot, tot.size() * 8, cudaMemcpyDeviceToHost, st))) return fail(e, "optics readback");
    if (far_out && nfar) {
        k_opt_flush<<<std::min<size_t>((nfar + 255) / 256, (size_t)sms * 16), 256, 0, st>>>(
            B.far, reinterpret_cast<double*>(B.far), nfar, 0);
        if ((e = cudaMemcpyAsync(far_out, B.far, nfar * 8, cudaMemcpyDeviceToHost, st))) return fail(e, "optics readback");
    }
    if (lux_out && nlux) {
        k_opt_flush<<<std::min<size_t>((nlux + 255) / 256, (size_t)sms * 16), 256, 0, st>>>(
            B.lux, reinterpret_cast<double*>(B.lux), nlux, 0);
        if ((e = cudaMemcpyAsync(lux_out, B.lux, nlux * 8, cudaMemcpyDeviceToHost, st))) return fail(e, "optics readback");
    }
    if ((e = cudaStreamSynchronize(st))) return fail(e, "optics readback");
    DevCtr c;
    cudaMemcpy(&c, B.ctr, sizeof(DevCtr), cudaMemcpyDeviceToHost);
    B.last_ni = NI; B.last_mats = NM; B.last_det_cap = D.det_cap;
    B.last_path_rays = D.path_rays; B.last_path_verts = D.path_verts;
    if (c.errflag) { ctx_set_error(ctx, "a kernel's wait for its scene table ran out of iterations"); return ST_ERR_TIMEOUT; }
    auto w = [&](uint32_t i, uint32_t j) { return (double)(long long)tot[(size_t)i * OPT_TOT + j] / OPT_FX; };
    auto n = [&](uint32_t i, uint32_t j) { return (uint64_t)tot[(size_t)i * OPT_TOT + j]; };
    if (totals)
        for (uint32_t i = 0; i < NI; i++) {
            totals[i].emitted = o.has_sets ? w(i, T_EMIT) : (double)b->ray_count[i];   // a ray set's: its rays' weights
            totals[i].escaped = w(i, T_ESC); totals[i].lost = w(i, T_LOST); totals[i].detected = w(i, T_DET);
            totals[i].absorbed = w(i, T_ABS);
            totals[i].interactions = n(i, T_INTER);
            totals[i].rays = b->ray_count[i];
            totals[i].n_escaped = n(i, T_NESC); totals[i].n_lost = n(i, T_NLOST);
            totals[i].n_detected = n(i, T_NDET); totals[i].n_absorbed = n(i, T_NABS);
        }
    return ST_OK;
}

// THE OPTICS AUTOTUNER: the batch run with each (queue tile, march chunk) pair of the candidates (its graph recorded by
// one untimed run, then one timed: CUDA events on the context's stream), the fastest kept for the runs that follow
int st_optics_autotune(st_ctx* ctx, const st_optics_batch* b, st_tune* out) {
    if (!ctx || !b) return ST_ERR_ARG;
    OpticsState& os = ctx_ext(ctx).optics;
    static const uint32_t claims[] = {32u, 64u, 128u};
    static const uint32_t chunks[] = {24u, 32u, 48u, 64u, 96u, 160u};
    cudaSetDevice(ctx_device(ctx));
    cudaStream_t st = ctx_stream(ctx);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return ST_ERR_CUDA;
    float best = 1e30f, base = 0.f;
    uint32_t bc = CLAIM, bk = MARCH_CHUNK;
    int rc = ST_OK;
    for (uint32_t cl : claims) {
        for (uint32_t ch : chunks) {
            os.tune_claim = cl;
            os.tune_chunk = ch;
            if ((rc = st_optics_run(ctx, b, nullptr, nullptr, nullptr))) break;     // records the graph
            cudaEventRecord(e0, st);
            if ((rc = st_optics_run(ctx, b, nullptr, nullptr, nullptr))) break;
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (cl == CLAIM && ch == MARCH_CHUNK) base = ms;
            if (ms < best) { best = ms; bc = cl; bk = ch; }
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    os.tune_claim = rc ? 0u : bc;
    os.tune_chunk = rc ? 0u : bk;
    if (rc) return rc;
    if (out) { out->claim = bc; out->chunk = bk; out->ms = best; out->ms_default = base; }
    return ST_OK;
}

int st_optics_set_detail(st_ctx* ctx, const st_optics_detail* d) {
    if (!ctx || !d) return ST_ERR_ARG;
    if (d->det_cap > (1u << 24) || d->path_rays > 4096 || d->path_verts > 256 || !(d->esc_len >= 0.f)) {
        ctx_set_error(ctx, "optics detail out of range (det_cap <= 2^24, path_rays <= 4096, path_verts <= 256)");
        return ST_ERR_ARG;
    }
    ctx_ext(ctx).optics.detail = *d;
    return ST_OK;
}

static OptBuf* last_run(st_ctx* ctx) {
    OpticsState& os = ctx_ext(ctx).optics;
    OptBuf* B = static_cast<OptBuf*>(os.scratch);
    if (!B || !B->last_ni) { ctx_set_error(ctx, "no optics run yet"); return nullptr; }
    return B;
}

int st_optics_tallies(st_ctx* ctx, double* tags, double* mats) {
    if (!ctx) return ST_ERR_ARG;
    OptBuf* B = last_run(ctx);
    if (!B) return ST_ERR_STATE;
    cudaSetDevice(ctx_device(ctx));
    auto out = [&](const unsigned long long* d, size_t n, double* h) -> bool {
        std::vector<unsigned long long> v(n);
        if (cudaMemcpy(v.data(), d, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
        for (size_t i = 0; i < n; i++) h[i] = i % 3 == 2 ? (double)v[i] : (double)(long long)v[i] / OPT_FX;
        return true;
    };
    if (tags && !out(B->tag, (size_t)OPT_TAG_MAX * 3, tags)) return ST_ERR_CUDA;
    if (mats && !out(B->mat, (size_t)B->last_ni * B->last_mats * 3, mats)) return ST_ERR_CUDA;
    return ST_OK;
}

int st_optics_hits(st_ctx* ctx, float* hits, uint32_t max_n, uint32_t* n_out) {
    if (!ctx || (max_n && !hits)) return ST_ERR_ARG;
    OptBuf* B = last_run(ctx);
    if (!B) return ST_ERR_STATE;
    cudaSetDevice(ctx_device(ctx));
    uint32_t n = 0;
    if (cudaMemcpy(&n, B->det_n, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return ST_ERR_CUDA;
    if (n_out) *n_out = n;
    const uint32_t k = std::min(std::min(n, B->last_det_cap), max_n);
    if (!k) return ST_OK;
    std::vector<float4> v((size_t)k * DET_F4);
    if (cudaMemcpy(v.data(), B->det, v.size() * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess) return ST_ERR_CUDA;
    for (uint32_t i = 0; i < k; i++) {
        const float4* d = &v[(size_t)i * DET_F4];
        float* h = hits + (size_t)i * 12;
        uint32_t t;
        std::memcpy(&t, &d[1].w, 4);
        h[0] = d[0].x; h[1] = d[0].y; h[2] = d[0].z; h[3] = d[0].w;          // position, weight
        h[4] = d[1].x; h[5] = d[1].y; h[6] = d[1].z;                          // direction
        h[7] = (float)(t & 0xffffu); h[8] = (float)(t >> 16);                  // tag, instance
        h[9] = d[2].x; h[10] = d[2].y; h[11] = 0.f;                           // CIE X, Z
    }
    return ST_OK;
}

int st_optics_paths(st_ctx* ctx, float* verts, uint32_t* counts) {
    if (!ctx) return ST_ERR_ARG;
    OptBuf* B = last_run(ctx);
    if (!B) return ST_ERR_STATE;
    cudaSetDevice(ctx_device(ctx));
    const size_t nr = (size_t)B->last_ni * B->last_path_rays;
    if (counts && nr && cudaMemcpy(counts, B->vcount, nr * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return ST_ERR_CUDA;
    const size_t nv = nr * B->last_path_verts * VERT_F4;
    if (verts && nv && cudaMemcpy(verts, B->verts, nv * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess)
        return ST_ERR_CUDA;
    return ST_OK;
}

}  // extern "C"
