// st_device.cuh -- device-side arithmetic of the rendering hot path for sm_103a: vectors, the PCG4D generator, the
// surface tolerance, the scene table's SDF fold, the environment, the GGX lobes and their albedo tables.
//
// Each function restates the reference (lampmaker/ShadyTracer v0.88.0) at the file:line given; the kernels that
// use them are in st_render.cu. Everything is f32 with f32 accumulation, as the reference's WGSL computes.
#pragma once
#ifndef __CUDACC_RTC__                 // NVRTC (st_scene_rtc.cu) compiles this header too; it has the types built in
#include <cstdint>
#include <cuda_runtime.h>
#endif
#include "../../include/shadytracer.h"

#define ST_PI 3.14159265358979f

namespace st {

// ------------------------------------------------------------------------------------------------------------
// vectors
// ------------------------------------------------------------------------------------------------------------
struct f3 { float x, y, z; };
__host__ __device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__host__ __device__ __forceinline__ f3 mk(float a) { return f3{a, a, a}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator/(f3 a, f3 b) { return f3{a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return f3{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 operator-(f3 a) { return f3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) { return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ float length(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ f3 normalize(f3 a) { return a / length(a); }
__device__ __forceinline__ float max3(f3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ f3 vmin(f3 a, float s) { return f3{fminf(a.x, s), fminf(a.y, s), fminf(a.z, s)}; }
__device__ __forceinline__ f3 vmax(f3 a, float s) { return f3{fmaxf(a.x, s), fmaxf(a.y, s), fmaxf(a.z, s)}; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float sat(float x) { return clampf(x, 0.f, 1.f); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.f - t) + b * t; }
__device__ __forceinline__ float luma(f3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }
__device__ __forceinline__ f3 reflectv(f3 I, f3 N) { return I - N * (2.f * dot(N, I)); }
__device__ __forceinline__ f3 refractv(f3 I, f3 N, float eta) {
    float d = dot(N, I);
    float k = 1.f - eta * eta * (1.f - d * d);
    if (k < 0.f) return mk(0.f);
    return I * eta - N * (eta * d + sqrtf(k));
}
__device__ __forceinline__ f3 xyz(float4 v) { return f3{v.x, v.y, v.z}; }
__device__ __forceinline__ float4 f4(f3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// ------------------------------------------------------------------------------------------------------------
// PCG4D (core/tracebasics.js:330-380): SEED_u32, pcg4d, PRNG -- the top 24 bits of each lane
// ------------------------------------------------------------------------------------------------------------
struct Rng {
    uint4 h;
    __device__ __forceinline__ static uint4 pcg4d(uint4 v) {
        v.x = v.x * 1664525u + 1013904223u; v.y = v.y * 1664525u + 1013904223u;
        v.z = v.z * 1664525u + 1013904223u; v.w = v.w * 1664525u + 1013904223u;
        v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
        v.x ^= v.x >> 16; v.y ^= v.y >> 16; v.z ^= v.z >> 16; v.w ^= v.w >> 16;
        v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
        return v;
    }
    __device__ __forceinline__ void seed(uint32_t v) {
        uint4 o = h;
        h.x = (o.y ^ v) * 2313257647u; h.y = (o.z ^ v) * 2700274807u;
        h.z = (o.w ^ v) * 3152041561u; h.w = (o.x ^ v) * 3679390633u;
    }
    __device__ __forceinline__ float4 next() {
        h = pcg4d(h);
        const float s = 1.0f / 16777216.0f;
        return make_float4(float(h.x >> 8) * s, float(h.y >> 8) * s, float(h.z >> 8) * s, float(h.w >> 8) * s);
    }
};
// the sample's seed from the base seed, and a path's generator at an event (0 the camera ray, 1 + i the shade of its
// i-th segment): seeded by the path, as the reference's optics shade seeds by the ray (optics/kernels.js:598-606)
#define PHOTON_SEED_SALT 0x50484F54u       // the photons' sample seed: the picture's seed xor this
__host__ __device__ __forceinline__ uint4 sample_seed(uint32_t base, uint32_t sample) {
    uint4 v = make_uint4(base, sample, 0xA53B3F17u, 0xC0FFEE42u);
    for (int r = 0; r < 2; r++) {
        v.x = v.x * 1664525u + 1013904223u; v.y = v.y * 1664525u + 1013904223u;
        v.z = v.z * 1664525u + 1013904223u; v.w = v.w * 1664525u + 1013904223u;
        v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
        v.x ^= v.x >> 16; v.y ^= v.y >> 16; v.z ^= v.z >> 16; v.w ^= v.w >> 16;
        v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    }
    return v;
}
// the photons' sample seed (their own streams: the photon's id, then its shade count)
__host__ __device__ __forceinline__ uint4 photon_seed_of(uint32_t base, uint32_t sample) {
    return sample_seed(base ^ PHOTON_SEED_SALT, sample);
}
__device__ __forceinline__ Rng path_rng(uint4 sseed, uint32_t path, uint32_t event) {
    Rng r; r.h = sseed; r.seed(path); r.seed(event); return r;
}
#define ST_SALT_HAZE 0x48410000u
#define ST_SALT_WALK 0x57410000u          // a scattering material's walk: a leg's first flight (+ the path's steps)
#define ST_SALT_WALK_HIT 0x57480000u      // ...a collision's turn and next flight (+ the path's steps)

// ------------------------------------------------------------------------------------------------------------
// The uniforms a launch reads: the settings and their host-derived values (core/photometry.js:182-237, in double
// on the host, rounded once to f32 here), passed by value in the kernel's parameter bank.
// ------------------------------------------------------------------------------------------------------------
struct Uni {
    uint32_t W, H, P;            // picture, paths per sample (P = W * H)
    uint32_t tilesX, tilesY;
    float invTX, invTY;
    uint32_t maxbounce, maxiter, nee, rr, budget;
    float stepscale, tol, envR2, envR;
    // camera (genrays.js:65-92)
    f3 cam, right, up, fwd; float fx, fy; uint32_t camtype;
    float lens_r, lens_f;        // the thin lens (lens.js): aperture radius and focus distance; 0 a pinhole
    // environment (sdf.js:70-160)
    f3 sun_dir; float sun_sin2, sun_omc, sun_omega, pick; int sun_on;
    f3 disc; float sky, ground, uniform, sun_gain, sky_gain;
    // the environment image (envimage.js) and the map light sampling draws from (envmap.js); null, none
    const float4* env_img; uint32_t env_w, env_h; float env_lum, env_turn;
    const float4* env_map; float env_mshare;
    // the presets (environment.js): the mode, the sun and sky's light above the air, its aerosol depth at 550 nm and
    // its 16 bands (st_sky.h: per band Rayleigh depth, aerosol factor, ozone depth, then its colour); the studio's L0,
    // its top and its colour
    uint32_t env_mode; float sun_outside, aerosol; const float4* sky_tab;
    const float4* env_tex; uint32_t env_tw, env_th;   // the preset in a texture (envmap.js envCacheAt); null, none
    float studio_l0, studio_top; f3 studio_tint;
    // the step cache (wavefront.js:67-118): the cells' distances, the grid's low corner and cell size, its cells, looks
    const float* sc; f3 sc_lo; float sc_cs; uint32_t sc_dx, sc_dy, sc_dz, sc_looks;
    // haze box (haze.js:64-80)
    int haze_on; f3 hc, hu, hv, hw, halb; float hhu, hhv, hhw, hsig, hg;
    uint32_t scatter_on;         // a material that scatters inside (st_material.scatter_distance): the march walks it
    // the sample sequence
    uint32_t seed, maxaverages, n_prims, n_mats;
    uint32_t count_work;         // a counting pass: the march counts its fold's work (WC_*)
    // the autotuner's picks (st_autotune): queue entries a warp claims at a time in the march and the occlusion pass,
    // and the evaluations a ray takes a launch before it waits for the next iteration; 0, the defaults
    uint32_t claim, chunk;
    // the march queue's space order (st_render.cu k_sort_*): a SORT_G^3 grid over the primitives' bounds
    uint32_t sort_on; f3 glo, ginv;
    // the photon map (st_photons.cu): photons a sample, the sun photons' square, the radius schedule, the budget
    uint32_t sppm_on, sppm_n, sppm_budget, sppm_learn; float sppm_half, sppm_r1, sppm_alpha;
    float sppm_r1v;              // the volume's first radius (st_params.sppm_r1_volume)
    // light tracing to the camera (st_photons.cu lt_connect): the photons above connect where they land
    uint32_t lt_on;
    uint32_t photon_pass;        // the wave's photon pass: its rays are photons, seeded by the photon's own stream
    uint32_t lt_emit_n;          // of the sample's sppm_n photons, the first this many are emitter probes (0: none)
    // many views in one wave (st_set_views): nv pictures of P pixels; a wave's frame k (slot / P) is sample k / nv of
    // view k % nv; each view's camera in the table (VIEW_F4 float4s a view), null with one
    uint32_t nv; const float4* views;
};
#define VIEW_F4 5
// a slot's sample within its wave (what seeds its paths) and its view
__device__ __forceinline__ uint32_t slot_sample(const Uni& u, uint32_t slot) { return (slot / u.P) / max(u.nv, 1u); }
__device__ __forceinline__ uint32_t slot_view(const Uni& u, uint32_t slot) { return (slot / u.P) % max(u.nv, 1u); }

// ------------------------------------------------------------------------------------------------------------
// DISPERSION (spectral.js:121-128 cauchyN, :136-137 lambdaCode; lightspectra.js specDraw): Cauchy's index through a
// glass's n_d and Abbe number, the wavelength as the reference's 15-bit code keeps it, and the camera's draw of a
// wavelength from the 1 nm table (csrc/st_spectral.h builds it on the host: per cell the CDF and its colour).
// ------------------------------------------------------------------------------------------------------------
#define SPEC_NCELLS 400
__device__ __forceinline__ float cauchy_n(float nd, float vd, float lam) {
    if (!(vd > 0.f)) return nd;
    const float FC = (float)(1.0 / (486.13 * 486.13) - 1.0 / (656.27 * 656.27));   // 1/lambda_F^2 - 1/lambda_C^2
    const float LD2 = (float)(587.56 * 587.56);
    const float B = (nd - 1.f) / (vd * FC);
    return nd + B * (1.f / (lam * lam) - 1.f / LD2);
}
__device__ __forceinline__ float lambda_coded(float lam) {
    const float c = 1.f + rintf(fminf(fmaxf((lam - 380.f) / 400.f, 0.f), 1.f) * 32766.f);
    return 380.f + (c - 1.f) * (400.f / 32766.f);
}
struct SpecDraw { float lam; f3 w; };
__device__ __forceinline__ SpecDraw spec_draw(const float4* __restrict__ tab, float u) {
    uint32_t lo = 0, hi = SPEC_NCELLS - 1;
    while (lo < hi) {                                                  // the first cell whose CDF passes u
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&tab[mid].x) > u) hi = mid;
        else lo = mid + 1;
    }
    const float c0 = lo ? __ldg(&tab[lo - 1].x) : 0.f;
    const float4 t = __ldg(&tab[lo]);
    const float q = t.x - c0;
    const float f = q > 0.f ? fminf(fmaxf((u - c0) / q, 0.f), 1.f) : 0.5f;
    SpecDraw d;
    d.lam = 380.f + (float)lo + f;
    d.w = mk(t.y, t.z, t.w);
    return d;
}

// ------------------------------------------------------------------------------------------------------------
// THE TOLERANCE (core/tolerances.js:27-37 marchTol); offsetTol = 10 marchTol (tracebasics.js:165)
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ float march_tol(f3 p, float setting) {
    float f = 128.0f * 1.1920928955078125e-7f * fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z)));
    return fmaxf(fmaxf(setting, 1e-9f), f);
}

// THE STEP CACHE (wavefront.js:95-118 scStep): the step a ball allows from pos along dir -- the farthest exit of
// the balls of the ray's own cell and, with two looks more, of the cells one and two cells ahead, the ray inside
// them -- or -1 where none holds it as far as a cell
__device__ __forceinline__ float sc_step(const Uni& u, f3 pos, f3 dir) {
    const float cs = u.sc_cs;
    float best = 0.f;
    for (uint32_t k = 0; k < u.sc_looks; k++) {
        const f3 g = (pos + dir * ((float)k * cs) - u.sc_lo) * (1.f / cs);
        if (g.x < 0.f || g.y < 0.f || g.z < 0.f || g.x >= (float)u.sc_dx || g.y >= (float)u.sc_dy || g.z >= (float)u.sc_dz)
            continue;
        const uint32_t cx = min((uint32_t)g.x, u.sc_dx - 1u), cy = min((uint32_t)g.y, u.sc_dy - 1u),
                       cz = min((uint32_t)g.z, u.sc_dz - 1u);
        const float r = __ldg(&u.sc[cx + u.sc_dx * (cy + u.sc_dy * cz)]);
        const f3 oc = pos - (u.sc_lo + mk((float)cx + 0.5f, (float)cy + 0.5f, (float)cz + 0.5f) * cs);
        const float c2 = dot(oc, oc) - r * r;
        if (c2 >= 0.f) continue;                                      // not inside this ball (an empty cell's is none)
        const float b = dot(oc, dir);
        best = fmaxf(best, -b + sqrtf(b * b - c2));                   // where the ray leaves it
    }
    return best >= cs ? best : -1.f;
}

// ------------------------------------------------------------------------------------------------------------
// THE SCENE TABLE'S SDF (core/scene_api.js:28-80 fold; sdf.js:214-256, :602; shapes.js:266-287, :621-726)
// The table sits in shared memory (st_render.cu stages it with a bulk copy); every thread of a warp reads the
// same record at the same time, a broadcast.
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ float sd_box(f3 p, f3 b) {
    f3 q = mk(fabsf(p.x) - b.x, fabsf(p.y) - b.y, fabsf(p.z) - b.z);
    return length(vmax(q, 0.f)) + fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.f);
}
__device__ __forceinline__ float g2_extrude(float pz, float gz, float h) {
    float wz = fabsf(pz) - h;
    if (gz > 0.f && wz > 0.f) return sqrtf(gz * gz + wz * wz);
    if (gz > wz) return gz;
    return wz;
}
__device__ __forceinline__ void asph_sag(float r, float c, float k, float a4, float a6, float& sag, float& slope) {
    float r2 = r * r;
    float w = 1.f - (1.f + k) * c * c * r2;
    float u = sqrtf(fmaxf(w, 1e-4f));
    float poly = r2 * r2 * (a4 + r2 * a6);
    float dpoly = r * r2 * (4.f * a4 + r2 * (6.f * a6));
    sag = c * r2 / (1.f + u) + poly;
    slope = (w >= 1e-4f ? c * r / u : 2.f * c * r / (1.f + u)) + dpoly;
}
__device__ __forceinline__ float asph_face(f3 p, float l, float rho, float ht, float R, float k, float a4, float a6, float s) {
    float c = fabsf(R) > 1e-9f ? 1.f / R : 0.f;
    float sag, slope;
    asph_sag(fminf(l, rho), c, k, a4, a6, sag, slope);
    float r2 = rho * rho;
    float u = sqrtf(fmaxf(1.f - (1.f + k) * c * c * r2, 1e-4f));
    float poly = rho * r2 * (4.f * fabsf(a4) + r2 * (6.f * fabsf(a6)));
    float m = fabsf(c) * rho / u + poly;
    return (s * p.z - ht + sag) / sqrtf(1.f + m * m);
}

// THE TABLE AS THE KERNELS READ IT: each st_prim repacked on the host (st_capi.cu pack_prims) into eight 16-byte
// words, so a record is read with 128-bit shared-memory loads and carries what the host could work out once: the
// radius of a sphere about its centre that holds it (its BOUND, +inf where none is valid) and a prism's edge
// constants. 128 bytes, as st_prim.
struct __align__(16) DPrim {
    float4 a;    // centre xyz, bound radius (inflated; +inf: never culled)
    float4 r0;   // rotation row 0, smooth-union radius k
    float4 r1;   // rotation row 1, p0
    float4 r2;   // rotation row 2, p1
    float4 e;    // p2..p5
    float4 f;    // p6..p9
    float4 g;    // prism: distance to an edge's middle, half an edge, 2 pi / sides, sides
    uint4 h;     // type, op, material, flags
};

__device__ __forceinline__ float prim_sdf(const DPrim& pr, f3 pw) {
    const float4 A = pr.a, R0 = pr.r0, R1 = pr.r1, R2 = pr.r2;
    f3 d = pw - mk(A.x, A.y, A.z);
    f3 q = mk(R0.x * d.x + R0.y * d.y + R0.z * d.z,
              R1.x * d.x + R1.y * d.y + R1.z * d.z,
              R2.x * d.x + R2.y * d.y + R2.z * d.z);
    const float p0 = R1.w, p1 = R2.w;
    switch (pr.h.x) {
        case ST_PRIM_PLANE: return q.z;
        case ST_PRIM_SPHERE: return length(q) - p0;
        case ST_PRIM_BOX: return sd_box(q, mk(p0, p1, pr.e.x));
        case ST_PRIM_ROUNDBOX: { float4 E = pr.e; return sd_box(q, mk(p0, p1, E.x)) - E.y; }
        case ST_PRIM_TORUS: {
            float lxy = sqrtf(q.x * q.x + q.y * q.y);
            float t = lxy - p0;
            return sqrtf(t * t + q.z * q.z) - p1;
        }
        case ST_PRIM_PRISM: {
            // g2RegularPolygon (shapes.js:266-283) with its per-shape constants from the host; the edge normal's
            // angle -pi/2 + 2 pi k / n as sin / cos of pi (2k / n), which need no argument reduction
            const float4 G = pr.g, E = pr.e;
            float k = rintf((atan2f(q.y, q.x) + 0.5f * ST_PI) / G.z);
            float sp, cp;
            sincospif(2.f * k / G.w, &sp, &cp);
            float nkx = sp, nky = -cp;
            float u = q.x * nkx + q.y * nky, v = -q.x * nky + q.y * nkx;
            float gz;
            if (u <= G.x) gz = u - G.x;
            else { float ex = u - G.x, ey = v - clampf(v, -G.y, G.y); gz = sqrtf(ex * ex + ey * ey); }
            return g2_extrude(q.z, gz, fmaxf(0.5f * E.x, 0.f)) - E.y;
        }
        case ST_PRIM_ASPHERE: {
            const float4 E = pr.e, F = pr.f;
            float rho = fmaxf(0.5f * p0, 1e-6f);
            float l = sqrtf(q.x * q.x + q.y * q.y);
            float dd = l - rho;
            float top = asph_face(q, l, rho, 0.5f * p1, E.x, E.y, E.z, E.w, 1.f);
            if (top > dd) dd = top;
            float bot = asph_face(q, l, rho, 0.5f * p1, F.x, F.y, F.z, F.w, -1.f);
            if (bot > dd) dd = bot;
            return dd;
        }
        case ST_PRIM_CYLINDER: {
            float lx = sqrtf(q.x * q.x + q.y * q.y) - p1;
            float lz = fabsf(q.z) - p0;
            float ox = fmaxf(lx, 0.f), oz = fmaxf(lz, 0.f);
            return fminf(fmaxf(lx, lz), 0.f) + sqrtf(ox * ox + oz * oz);
        }
    }
    return 1e7f;
}
__device__ __forceinline__ float smooth_union(float d1, float d2, float k) {          // sdf.js:252-256
    if (!(k > 0.f)) return fminf(d1, d2);
    float h = clampf(0.5f + 0.5f * (d2 - d1) / k, 0.f, 1.f);
    return mixf(d2, d1, h) - k * h * (1.f - h);
}
// THE CULL: whether the primitive's distance at p is at least t, from its bounding sphere alone (|p - c| - R <= d,
// true of every exact distance the table holds; the host gives +inf R where it is not). Exact by construction: a
// culled primitive is one whose fold or union would have left the running value as it was.
__device__ __forceinline__ bool beyond(const DPrim& pr, f3 p, float t) {
    const float4 A = pr.a;
    float s = t + A.w;
    if (!(s < 3.0e38f)) return false;                                 // no bound (+inf)
    if (s < 0.f) return true;
    f3 d = p - mk(A.x, A.y, A.z);
    return dot(d, d) >= s * s;
}
#define CULL_REL 1.001f
#define CULL_ABS 1e-6f

// WORK COUNTS, for a counting pass only (the COUNT instantiations): shared-memory counters a block flushes at its
// end -- per primitive type the evaluations made (threads) and the warp issues that made them, and the same for the
// bounding-sphere tests. Their ratio is the SIMD efficiency of the fold; their sum, weighted by each type's
// operations, the algorithmic work a launch did.
#define WC_EVAL 0u      // [0, 8): evaluations by primitive type
#define WC_WEVAL 8u     // [8, 16): warp issues of those evaluations
#define WC_TEST 16u     // bounding-sphere tests
#define WC_WTEST 17u    // ...their warp issues
#define WC_OP 18u       // [18, 22): evaluations by how they fold in (ST_OP_ITEM: a chain's head, SMOOTH, UNION, SUB)
#define WC_N 22u
// one more of counter k (threads) and of its warp-issue counter wk, from the warp's lowest active lane
template <bool COUNT>
__device__ __forceinline__ void wc_add(uint32_t* c, uint32_t k, uint32_t wk) {
    if (COUNT) {
        const uint32_t m = __activemask();
        if ((threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) {
            atomicAdd(&c[k], (uint32_t)__popc(m));
            atomicAdd(&c[wk], 1u);
        }
    }
}
template <bool COUNT>
__device__ __forceinline__ void wc_eval(uint32_t* c, const DPrim& pr, uint32_t op) {
    if (COUNT) {
        wc_add<COUNT>(c, WC_EVAL + (pr.h.x & 7u), WC_WEVAL + (pr.h.x & 7u));
        const uint32_t m = __activemask();
        if ((threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(&c[WC_OP + (op & 3u)], (uint32_t)__popc(m));
    }
}

// ...and the same tallies from a scene's generated code (st_scene_rtc.cu's st_scene_dist_count): one evaluation of a
// primitive of type t folded in by op, one bounding-sphere test
__device__ __forceinline__ void wc_prim(uint32_t* c, uint32_t t, uint32_t op) {
    wc_add<true>(c, WC_EVAL + (t & 7u), WC_WEVAL + (t & 7u));
    const uint32_t m = __activemask();
    if ((threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(&c[WC_OP + (op & 3u)], (uint32_t)__popc(m));
}
__device__ __forceinline__ void wc_test(uint32_t* c) { wc_add<true>(c, WC_TEST, WC_WTEST); }

struct SceneHit { float d; uint32_t m, a; };
// distance only (scene_api.js FOLD_DIST): the march's and the shadow rays' question. Within an item's CSG chain a
// primitive is evaluated only where it could change the running value: a smooth union of radius k leaves acc alone
// where d_j >= acc + k (sdf.js opSmoothUnion's h is then 1), a union where d_j >= acc, a subtraction where
// d_j >= -acc -- the same number, bit for bit, as evaluating it.
template <bool COUNT = false>
__device__ __forceinline__ float scene_dist(const DPrim* __restrict__ pr, uint32_t n, f3 p, uint32_t* wc = nullptr) {
    float best = 1e7f;
    uint32_t i = 0;
    while (i < n) {
        wc_eval<COUNT>(wc, pr[i], ST_OP_ITEM);
        float di = prim_sdf(pr[i], p);
        uint32_t j = i + 1;
        while (j < n) {
            const uint32_t op = pr[j].h.y;
            if (op == ST_OP_ITEM) break;
            wc_add<COUNT>(wc, WC_TEST, WC_WTEST);
            if (op == ST_OP_SMOOTH) {
                float k = pr[j].r0.w;
                if (!beyond(pr[j], p, di + fmaxf(k, 0.f) * CULL_REL + CULL_ABS)) {
                    wc_eval<COUNT>(wc, pr[j], op);
                    di = smooth_union(di, prim_sdf(pr[j], p), k);
                }
            } else if (op == ST_OP_UNION) {
                if (!beyond(pr[j], p, di + CULL_ABS)) {
                    wc_eval<COUNT>(wc, pr[j], op);
                    di = fminf(di, prim_sdf(pr[j], p));
                }
            } else {
                if (!beyond(pr[j], p, -di + CULL_ABS)) {
                    wc_eval<COUNT>(wc, pr[j], op);
                    di = fmaxf(di, -prim_sdf(pr[j], p));
                }
            }
            j++;
        }
        if (fabsf(di) < fabsf(best)) best = di;
        i = j;
    }
    return best;
}
// the whole answer (FOLD_FULL): the surface's material (the chain's primitive of least |d|) and the medium (the
// least-deep item the point is in). A primitive is culled only where it could change neither the running value
// nor the nearest primitive.
__device__ __forceinline__ SceneHit scene_full(const DPrim* __restrict__ pr, uint32_t n, f3 p) {
    SceneHit H{1e7f, 0u, 0u};
    float insideW = -1e7f;
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
        if (fabsf(di) < fabsf(H.d)) { H.d = di; H.m = mat; }
        i = j;
    }
    return H;
}

// ------------------------------------------------------------------------------------------------------------
// THE ENVIRONMENT (sdf.js:70-182; tracebasics.js:655-699)
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ bool in_sun_disc(const Uni& u, f3 dir) {
    f3 L = normalize(dir);
    f3 c = cross(L, u.sun_dir);
    return dot(L, u.sun_dir) > 0.f && dot(c, c) <= u.sun_sin2;
}
// THE ENVIRONMENT IMAGE in direction dir (envimage.js:33-52 envImage): equirectangular, its middle column +x running
// right as one turns right, top row straight up, turned env_turn degrees about z; bilinear, wrapping across the seam,
// clamped at the poles; its own numbers times env_lum (cd/m^2 a unit)
__device__ __forceinline__ f3 env_image(const Uni& u, f3 dir) {
    const f3 d = normalize(dir);
    const int w = (int)u.env_w, h = (int)u.env_h;
    float a = 0.5f - atan2f(d.y, d.x) * (0.5f / ST_PI) + u.env_turn * (1.f / 360.f);
    a -= floorf(a);
    const float uu = a * (float)w - 0.5f;
    const float vv = acosf(clampf(d.z, -1.f, 1.f)) * (1.f / ST_PI) * (float)h - 0.5f;
    const float x0 = floorf(uu), y0 = floorf(vv), fx = uu - x0, fy = vv - y0;
    const int xa = (((int)x0 % w) + w) % w, xb = (xa + 1) % w;
    const int ya = min(max((int)y0, 0), h - 1), yb = min(max((int)y0 + 1, 0), h - 1);
    const float4 p00 = __ldg(&u.env_img[(size_t)ya * w + xa]), p01 = __ldg(&u.env_img[(size_t)ya * w + xb]);
    const float4 p10 = __ldg(&u.env_img[(size_t)yb * w + xa]), p11 = __ldg(&u.env_img[(size_t)yb * w + xb]);
    const f3 top = mk(p00.x, p00.y, p00.z) * (1.f - fx) + mk(p01.x, p01.y, p01.z) * fx;
    const f3 bot = mk(p10.x, p10.y, p10.z) * (1.f - fx) + mk(p11.x, p11.y, p11.z) * fx;
    const f3 c = top * (1.f - fy) + bot * fy;
    return mk(fmaxf(c.x, 0.f), fmaxf(c.y, 0.f), fmaxf(c.z, 0.f)) * u.env_lum;
}
// Kasten-Young relative air mass (sdf.js:96-100 airMass): 1 / cos(zenith) near the top, finite at the horizon
__device__ __forceinline__ float air_mass(float cz) {
    const float c = clampf(cz, 0.f, 1.f);
    const float zdeg = acosf(c) * (180.f / ST_PI);
    return 1.f / (c + 0.15f * powf(fmaxf(93.885f - zdeg, 0.1f), -1.253f));
}
// THE SUN AND SKY, PHYSICALLY (environment.js SUNSKY_FN): per band the disc -- the sunlight the air lets through,
// exp(-tau m_s), spread over the disc, none once the sun has set -- or the sky, that light scattered once toward the
// eye over the air's whole depth, E0 (tau_R P_R + 0.9 tau_A P_M) / tau  m_v (exp(-tau m_s) - exp(-tau m_v)) / (m_v - m_s)
// (tau m_v exp(-tau m_v) where the two air masses meet), fading over the sun's last 3 degrees below the horizon; the
// ozone in the extinction, not in what scatters; added up as colour, times the light above the air
__device__ __forceinline__ f3 sun_sky(const Uni& u, f3 d) {
    const f3 s = u.sun_dir;
    const float mv = air_mass(fmaxf(d.z, 0.f)), ms = air_mass(fmaxf(s.z, 0.f));
    const bool disc = in_sun_disc(u, d) && s.z > -sqrtf(u.sun_sin2);
    const float c = dot(d, s), g = 0.7f;
    const float phaseR = 3.f / (16.f * ST_PI) * (1.f + c * c);
    const float phaseM = (1.f - g * g) / (4.f * ST_PI * powf(1.f + g * g - 2.f * g * c, 1.5f));
    const float up = clampf((s.z + 0.05f) / 0.05f, 0.f, 1.f);
    const float dm = mv - ms;
    f3 L = mk(0.f);
#pragma unroll 4
    for (int k = 0; k < 16; k++) {
        const float4 b = __ldg(&u.sky_tab[k]);
        const float4 rgb = __ldg(&u.sky_tab[16 + k]);
        const float tr = b.x, ta = u.aerosol * b.y, tau = tr + ta + b.z;
        float v;
        if (disc) {
            v = expf(-tau * ms) / (ST_PI * u.sun_sin2);
        } else {
            const float k1 = fabsf(dm) < 1e-3f ? tau * mv * expf(-tau * mv) : mv * (expf(-tau * ms) - expf(-tau * mv)) / dm;
            v = (tr * phaseR + 0.9f * ta * phaseM) / tau * k1 * up;
        }
        L = L + mk(rgb.x, rgb.y, rgb.z) * v;
    }
    return mk(fmaxf(L.x, 0.f), fmaxf(L.y, 0.f), fmaxf(L.z, 0.f)) * fmaxf(u.sun_outside, 0.f);
}
// THE STUDIO (environment.js STUDIO_FN): L0 (1 + top z) in its colour, L0 such that a level surface facing up receives
// the set illuminance whatever top is
__device__ __forceinline__ f3 studio_light(const Uni& u, f3 d) {
    return u.studio_tint * (u.studio_l0 * fmaxf(1.f + u.studio_top * d.z, 0.f));
}
// THE ENVIRONMENT FROM ITS TEXTURE (envmap.js:162-182 envCacheAt): equirectangular, columns the azimuth from +x, rows
// even in angle from straight up; bilinear, wrapping across the seam, clamped at the poles
__device__ __forceinline__ f3 env_cache_at(const Uni& u, f3 d) {
    const int w = (int)u.env_tw, h = (int)u.env_th;
    float a = atan2f(d.y, d.x) * (0.5f / ST_PI);
    a -= floorf(a);
    const float uu = a * (float)w - 0.5f;
    const float vv = acosf(clampf(d.z, -1.f, 1.f)) * (1.f / ST_PI) * (float)h - 0.5f;
    const float x0 = floorf(uu), y0 = floorf(vv), fx = uu - x0, fy = vv - y0;
    const int xa = (((int)x0 % w) + w) % w, xb = (xa + 1) % w;
    const int ya = min(max((int)y0, 0), h - 1), yb = min(max((int)y0 + 1, 0), h - 1);
    const float4 p00 = __ldg(&u.env_tex[(size_t)ya * w + xa]), p01 = __ldg(&u.env_tex[(size_t)ya * w + xb]);
    const float4 p10 = __ldg(&u.env_tex[(size_t)yb * w + xa]), p11 = __ldg(&u.env_tex[(size_t)yb * w + xb]);
    const f3 top = mk(p00.x, p00.y, p00.z) * (1.f - fx) + mk(p01.x, p01.y, p01.z) * fx;
    const f3 bot = mk(p10.x, p10.y, p10.z) * (1.f - fx) + mk(p11.x, p11.y, p11.z) * fx;
    return top * (1.f - fy) + bot * fy;
}
__device__ __forceinline__ f3 env_base(const Uni& u, f3 dir) {
    if (u.env_img) return env_image(u, dir);
    if (u.uniform > 0.f) return mk(u.uniform);
    f3 d = normalize(dir);
    // a preset from its texture, outside the sun's cone (sdf.js envBase)
    if (u.env_tex && !(u.sun_on && in_sun_disc(u, d))) return env_cache_at(u, d);
    if (u.env_mode == 1u) return sun_sky(u, d);
    if (u.env_mode == 2u) return studio_light(u, d);
    if (in_sun_disc(u, d)) return u.disc;
    return mk(d.z > 0.f ? u.sky : u.ground);
}
__device__ __forceinline__ f3 env_radiance(const Uni& u, f3 dir) {
    bool cone = u.sun_on && in_sun_disc(u, dir);
    return env_base(u, dir) * (cone ? u.sun_gain : u.sky_gain);
}
// the environment outside the sun's cone (sdf.js skyRadiance): what a path the photons own finds there -- nothing in
// the cone, whose light is theirs
__device__ __forceinline__ f3 env_sky(const Uni& u, f3 dir) {
    if (u.sun_on && in_sun_disc(u, dir)) return mk(0.f);
    return env_base(u, dir) * u.sky_gain;
}
// whether the sun's photons were drawn along this line (sdf.js ltCovers): it crosses the square of half width
// sppm_half across the sun's direction through the origin
__device__ __forceinline__ bool sppm_covers(const Uni& u, f3 p, f3 d) {
    const f3 s = u.sun_dir;
    const float ds = dot(d, s);
    if (!(ds > 0.f)) return false;
    const f3 x = p - d * (dot(p, s) / ds);
    const f3 t = fabsf(s.x) > 0.9f ? mk(0, 1, 0) : mk(1, 0, 0);
    const f3 b1 = normalize(cross(t, s));
    const f3 b2 = cross(s, b1);
    return fabsf(dot(x, b1)) <= u.sppm_half && fabsf(dot(x, b2)) <= u.sppm_half;
}
__device__ __forceinline__ f3 sample_sun_cone(const Uni& u, float u0, float u1) {
    f3 sd = u.sun_dir;
    float omc = u0 * u.sun_omc;
    float cosT = 1.f - omc;
    float sinT = sqrtf(fmaxf(0.f, omc * (2.f - omc)));
    float sp, cp;
    sincosf(2.f * ST_PI * u1, &sp, &cp);
    f3 t = fabsf(sd.x) > 0.9f ? mk(0, 1, 0) : mk(1, 0, 0);
    f3 b1 = normalize(cross(t, sd));
    f3 b2 = cross(sd, b1);
    return normalize(b1 * (cp * sinT) + b2 * (sp * sinT) + sd * cosT);
}
__device__ __forceinline__ f3 sample_cosine_hemi(f3 n, float u0, float u1) {
    float r = sqrtf(u0);
    float sp, cp;
    sincosf(2.f * ST_PI * u1, &sp, &cp);
    f3 t = fabsf(n.x) > 0.9f ? mk(0, 1, 0) : mk(1, 0, 0);
    f3 b1 = normalize(cross(t, n));
    f3 b2 = cross(n, b1);
    return normalize(b1 * (r * cp) + b2 * (r * sp) + n * sqrtf(fmaxf(0.f, 1.f - u0)));
}
// THE MAP OF WHERE THE ENVIRONMENT IS BRIGHT (envmap.js:44-98): ENV_MW x ENV_MH texels of equal solid angle, columns
// azimuth, rows equal steps of z from straight up; each a float4 of (the CDF along its row at its end, its density
// per steradian, the CDF down the rows at its row's end, 0). A row by the CDF down column 0, a column by the row's own,
// a point uniform in (azimuth, z) inside the texel: both numbers pick and then place, no more are drawn.
#define ENV_MW 512
#define ENV_MH 256
__device__ __forceinline__ f3 env_map_sample(const Uni& u, float ux, float uy) {
    const float4* __restrict__ m = u.env_map;
    int lo = 0, hi = ENV_MH - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ux < __ldg(&m[mid * ENV_MW]).z) hi = mid; else lo = mid + 1;
    }
    const int row = lo;
    const float r0 = row > 0 ? __ldg(&m[(row - 1) * ENV_MW]).z : 0.f, r1 = __ldg(&m[row * ENV_MW]).z;
    const float fy = clampf((ux - r0) / fmaxf(r1 - r0, 1e-12f), 0.f, 0.999999f);
    lo = 0; hi = ENV_MW - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (uy < __ldg(&m[row * ENV_MW + mid]).x) hi = mid; else lo = mid + 1;
    }
    const int col = lo;
    const float c0 = col > 0 ? __ldg(&m[row * ENV_MW + col - 1]).x : 0.f, c1 = __ldg(&m[row * ENV_MW + col]).x;
    const float fx = clampf((uy - c0) / fmaxf(c1 - c0, 1e-12f), 0.f, 0.999999f);
    const float z = 1.f - 2.f * ((float)row + fy) / (float)ENV_MH;
    const float phi = 2.f * ST_PI * ((float)col + fx) / (float)ENV_MW;
    const float sz = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return mk(sz * cp, sz * sp, z);
}
__device__ __forceinline__ float env_map_pdf(const Uni& u, f3 L) {
    const f3 d = normalize(L);
    float a = atan2f(d.y, d.x) * (0.5f / ST_PI);
    a -= floorf(a);
    const int col = min(max((int)(a * (float)ENV_MW), 0), ENV_MW - 1);
    const int row = min(max((int)((1.f - d.z) * 0.5f * (float)ENV_MH), 0), ENV_MH - 1);
    return __ldg(&u.env_map[row * ENV_MW + col]).y;
}
// the environment's three strategies (tracebasics.js:686-713): the sun's cone with its pick, of the rest the map with
// its share (0 with no map), else the cosine lobe -- one number picks all three, rescaled within its step
__device__ __forceinline__ f3 env_sample_dir(const Uni& u, f3 n, float pick, float u0, float u1) {
    if (pick < u.pick) return sample_sun_cone(u, u0, u1);
    if (u.env_mshare > 0.f && (pick - u.pick) / fmaxf(1.f - u.pick, 1e-6f) < u.env_mshare) return env_map_sample(u, u0, u1);
    return sample_cosine_hemi(n, u0, u1);
}
__device__ __forceinline__ float env_pdf(const Uni& u, f3 L, f3 n) {
    float pSun = in_sun_disc(u, L) ? 1.f / u.sun_omega : 0.f;
    float pCos = fmaxf(dot(L, n), 0.f) / ST_PI;
    const float m = u.env_mshare;
    const float pm = m > 0.f ? m * env_map_pdf(u, L) : 0.f;
    return u.pick * pSun + (1.f - u.pick) * (pm + (1.f - m) * pCos);
}
// ...and with a share q of the sky's cosine draw from the far hemisphere (materials_pbr.js:1089-1105 envSampleDirQ,
// envPdfQ): at q 0 exactly env_sample_dir and env_pdf
__device__ __forceinline__ f3 env_sample_dir_q(const Uni& u, f3 n, float pick, float u0, float u1, float q) {
    if (q <= 0.f || pick < u.pick) return env_sample_dir(u, n, pick, u0, u1);
    const float rest = (pick - u.pick) / fmaxf(1.f - u.pick, 1e-6f);
    const float m = u.env_mshare;
    if (rest < m) return env_map_sample(u, u0, u1);
    const float pc = (rest - m) / fmaxf(1.f - m, 1e-6f);
    return sample_cosine_hemi(pc < q ? n * -1.f : n, u0, u1);
}
__device__ __forceinline__ float env_pdf_q(const Uni& u, f3 L, f3 n, float q) {
    if (q <= 0.f) return env_pdf(u, L, n);
    const float pSun = in_sun_disc(u, L) ? 1.f / u.sun_omega : 0.f;
    const float c = dot(L, n);
    const float pCos = ((1.f - q) * fmaxf(c, 0.f) + q * fmaxf(-c, 0.f)) / ST_PI;
    const float m = u.env_mshare;
    const float pm = m > 0.f ? m * env_map_pdf(u, L) : 0.f;
    return u.pick * pSun + (1.f - u.pick) * (pm + (1.f - m) * pCos);
}
__device__ __forceinline__ float mis_weight(float a, float b) {
    float a2 = a * a, b2 = b * b;
    return a2 / fmaxf(a2 + b2, 1e-20f);
}
// the environment from a point in the air (haze.js:296-310)
__device__ __forceinline__ f3 env_sample_dir_m(const Uni& u, float pick, float u0, float u1) {
    if (pick < u.pick) return sample_sun_cone(u, u0, u1);
    if (u.env_mshare > 0.f && (pick - u.pick) / fmaxf(1.f - u.pick, 1e-6f) < u.env_mshare) return env_map_sample(u, u0, u1);
    float z = 1.f - 2.f * u0;
    float s = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sp, cp;
    sincosf(2.f * ST_PI * u1, &sp, &cp);
    return mk(s * cp, s * sp, z);
}
__device__ __forceinline__ float env_pdf_m(const Uni& u, f3 L) {
    float pSun = in_sun_disc(u, L) ? 1.f / u.sun_omega : 0.f;
    const float m = u.env_mshare;
    const float pm = m > 0.f ? m * env_map_pdf(u, L) : 0.f;
    return u.pick * pSun + (1.f - u.pick) * (pm + (1.f - m) / (4.f * ST_PI));
}

// ------------------------------------------------------------------------------------------------------------
// HAZE (haze.js:191-288): Henyey-Greenstein, the box's span and transmittance, the leg's collision
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ float hg_eval(float cosT, float g) {
    float d = 1.f + g * g - 2.f * g * cosT;
    return (1.f - g * g) / (4.f * ST_PI * powf(fmaxf(d, 1e-12f), 1.5f));
}
__device__ __forceinline__ f3 hg_sample(f3 d, float g, float u0, float u1) {
    float c = 1.f - 2.f * u0;
    if (fabsf(g) >= 1e-3f) {
        float s = (1.f - g * g) / (1.f - g + 2.f * g * u0);
        c = clampf((1.f + g * g - s * s) / (2.f * g), -1.f, 1.f);
    }
    float sn = sqrtf(fmaxf(0.f, 1.f - c * c));
    float sp, cp;
    sincosf(2.f * ST_PI * u1, &sp, &cp);
    f3 t = fabsf(d.x) > 0.9f ? mk(0, 1, 0) : mk(1, 0, 0);
    f3 b1 = normalize(cross(t, d));
    f3 b2 = cross(d, b1);
    return normalize(b1 * (cp * sn) + b2 * (sp * sn) + d * c);
}
__device__ __forceinline__ void haze_slab(float o, float dd, float h, float& t0, float& t1) {
    if (fabsf(dd) < 1e-12f) { if (fabsf(o) > h) { t0 = 1.f; t1 = 0.f; } return; }
    float a = (-h - o) / dd, b = (h - o) / dd;
    t0 = fmaxf(t0, fminf(a, b));
    t1 = fminf(t1, fmaxf(a, b));
}
__device__ __forceinline__ void haze_span(const Uni& u, f3 A, f3 d, float len, float& t0, float& t1) {
    f3 o = A - u.hc;
    t0 = 0.f; t1 = len;
    haze_slab(dot(o, u.hu), dot(d, u.hu), u.hhu, t0, t1);
    haze_slab(dot(o, u.hv), dot(d, u.hv), u.hhv, t0, t1);
    haze_slab(dot(o, u.hw), dot(d, u.hw), u.hhw, t0, t1);
    float b = dot(A, d);
    float disc = b * b - (dot(A, A) - u.envR * u.envR);
    if (disc <= 0.f) { t0 = 1.f; t1 = 0.f; return; }
    float s = sqrtf(disc);
    t0 = fmaxf(t0, -b - s);
    t1 = fminf(t1, -b + s);
}
__device__ __forceinline__ float haze_tr(const Uni& u, f3 A, f3 d, float len) {
    if (!u.haze_on) return 1.f;
    float t0, t1;
    haze_span(u, A, d, len, t0, t1);
    if (t1 <= t0) return 1.f;
    return expf(-u.hsig * (t1 - t0));
}

// ------------------------------------------------------------------------------------------------------------
// MICROFACET (microfacet.js:72-240): GGX, Smith, the VNDF sampler, Fresnel, the isotropic albedo tables' reads
// ------------------------------------------------------------------------------------------------------------
#define MF_NMU 32
#define MF_NR 32
#define MF_NIOR 16
#define MF_ALPHA_MIN 1e-3f
// the albedo tables, and a coating's 10 nm bins (st_spectral.h coat_bin_table: COAT_BINS rows of r, g, b, 0)
struct MfTab {
    const float* __restrict__ ec; const float* __restrict__ ecavg; const float* __restrict__ e1;
    const float4* __restrict__ coat;
};

// the two alphas along the local x and y (microfacet.js mfAnisoAlpha); an isotropic lobe's are equal, and then every
// number below is the one the isotropic formulas give
__device__ __forceinline__ float mf_lambda(f3 w, float2 a) {
    float z2 = fmaxf(w.z * w.z, 1e-12f);
    float t2 = (a.x * a.x * w.x * w.x + a.y * a.y * w.y * w.y) / z2;
    return 0.5f * (-1.f + sqrtf(1.f + t2));
}
__device__ __forceinline__ float mf_g1(f3 w, float2 a) { return 1.f / (1.f + mf_lambda(w, a)); }
__device__ __forceinline__ float mf_g2(f3 o, f3 i, float2 a) { return 1.f / (1.f + mf_lambda(o, a) + mf_lambda(i, a)); }
__device__ __forceinline__ float mf_d(f3 h, float2 a) {
    if (h.z <= 0.f) return 0.f;
    float t = (h.x * h.x) / (a.x * a.x) + (h.y * h.y) / (a.y * a.y) + h.z * h.z;
    return 1.f / (ST_PI * a.x * a.y * t * t);
}
__device__ __forceinline__ f3 mf_sample_vndf(f3 o, float2 a, float u0, float u1) {
    f3 os = normalize(mk(o.x * a.x, o.y * a.y, o.z));
    float z = (1.f - u1) * (1.f + os.z) - os.z;
    float sinT = sqrtf(clampf(1.f - z * z, 0.f, 1.f));
    float sp, cp;
    sincosf(2.f * ST_PI * u0, &sp, &cp);
    f3 c = mk(sinT * cp, sinT * sp, z);
    f3 hs = c + os;
    return normalize(mk(hs.x * a.x, hs.y * a.y, fmaxf(hs.z, 1e-7f)));
}
__device__ __forceinline__ float mf_pdf_reflect(f3 o, f3 i, float2 a) {
    if (o.z <= 0.f || i.z <= 0.f) return 0.f;
    f3 h = normalize(o + i);
    return mf_g1(o, a) * mf_d(h, a) / (4.f * o.z);
}
__device__ __forceinline__ float fresnel_dielectric(float cosI_in, float eta) {
    float cosI = clampf(cosI_in, 0.f, 1.f);
    float sin2T = eta * eta * (1.f - cosI * cosI);
    if (sin2T >= 1.f) return 1.f;
    float cosT = sqrtf(1.f - sin2T);
    float rs = (eta * cosI - cosT) / (eta * cosI + cosT);
    float rp = (cosI - eta * cosT) / (cosI + eta * cosT);
    return 0.5f * (rs * rs + rp * rp);
}
__device__ __forceinline__ float mf_lambda(f3 w, float a) { return mf_lambda(w, make_float2(a, a)); }
__device__ __forceinline__ float mf_g1(f3 w, float a) { return mf_g1(w, make_float2(a, a)); }
__device__ __forceinline__ float mf_g2(f3 o, f3 i, float a) { return mf_g2(o, i, make_float2(a, a)); }
__device__ __forceinline__ float mf_d(f3 h, float a) { return mf_d(h, make_float2(a, a)); }
__device__ __forceinline__ f3 mf_sample_vndf(f3 o, float a, float u0, float u1) { return mf_sample_vndf(o, make_float2(a, a), u0, u1); }
__device__ __forceinline__ float mf_pdf_reflect(f3 o, f3 i, float a) { return mf_pdf_reflect(o, i, make_float2(a, a)); }
__device__ __forceinline__ f3 fresnel_schlick3(float cosI, f3 f0) {
    float m = 1.f - clampf(cosI, 0.f, 1.f);
    float m5 = m * m * m * m * m;
    return f0 + (mk(1.f) - f0) * m5;
}
__device__ __forceinline__ void mf_axis(float x, int n, float& i0, float& f) {
    float c = clampf(x, 0.f, float(n - 1));
    i0 = fminf(floorf(c), float(n - 2));
    f = c - i0;
}
__device__ __forceinline__ float mf_ec(const MfTab& t, float mu, float r, float n) {
    float m0, mf, r0, rf, n0, nf;
    mf_axis(mu * float(MF_NMU) - 0.5f, MF_NMU, m0, mf);
    mf_axis(r * float(MF_NR - 1), MF_NR, r0, rf);
    mf_axis((n - 1.f) * float(MF_NIOR - 1) / 2.f, MF_NIOR, n0, nf);
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        int di = c & 1, dk = (c >> 1) & 1, dj = (c >> 2) & 1;
        float w = (di ? nf : 1.f - nf) * (dk ? rf : 1.f - rf) * (dj ? mf : 1.f - mf);
        int idx = (((int)n0 + di) * MF_NR + (int)r0 + dk) * MF_NMU + (int)m0 + dj;
        acc += w * __ldg(t.ec + idx);
    }
    return acc;
}
__device__ __forceinline__ float mf_ecavg(const MfTab& t, float r, float n) {
    float r0, rf, n0, nf;
    mf_axis(r * float(MF_NR - 1), MF_NR, r0, rf);
    mf_axis((n - 1.f) * float(MF_NIOR - 1) / 2.f, MF_NIOR, n0, nf);
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        int di = c & 1, dk = (c >> 1) & 1;
        float w = (di ? nf : 1.f - nf) * (dk ? rf : 1.f - rf);
        acc += w * __ldg(t.ecavg + ((int)n0 + di) * MF_NR + (int)r0 + dk);
    }
    return acc;
}
__device__ __forceinline__ float mf_e1(const MfTab& t, float mu, float r) {
    float m0, mf, r0, rf;
    mf_axis(mu * float(MF_NMU) - 0.5f, MF_NMU, m0, mf);
    mf_axis(r * float(MF_NR - 1), MF_NR, r0, rf);
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        int dk = c & 1, dj = (c >> 1) & 1;
        float w = (dk ? rf : 1.f - rf) * (dj ? mf : 1.f - mf);
        acc += w * __ldg(t.e1 + ((int)r0 + dk) * MF_NMU + (int)m0 + dj);
    }
    return acc;
}

// ------------------------------------------------------------------------------------------------------------
// THE LOBES (materials_pbr.js:164-596): isotropic, uncoated, no haze share -- the hot path's materials
// ------------------------------------------------------------------------------------------------------------
#define EV_NONE 0u
#define EV_DELTA 1u
#define EV_EVAL 2u
#define EV_OTHER 3u
// the share of a material's light that refracts (materials.js:123 refractShare): what passes, less what its haze
// diffuses through instead
__host__ __device__ __forceinline__ float refract_share_of(float transmission, float haze) {
    const float t = fminf(fmaxf(transmission, 0.f), 1.f), h = fminf(fmaxf(haze, 0.f), 1.f);
    return t * (1.f - h);
}
// ------------------------------------------------------------------------------------------------------------
// A COATING (materials.js:52-89 Material2.coat, :150-163 coatMaterial; spectral.js:80-117 edgeRGB, edgeAt, edgeAt1):
// R(lambda) = lo + (hi - lo) / (1 + exp(-(lambda - edge) / s)), s the 10-90 % width over 2 ln 9, its edge moved to
// shorter wavelengths by the light's invariant n0 sin(theta0) through the stack's effective index. A channel's
// reflectance is R averaged against that channel's weights in 10 nm bins, each bin's mean of the logistic exact (a
// softplus difference); a ray with a wavelength of its own takes R at it in every channel.
// ------------------------------------------------------------------------------------------------------------
#define COAT_NBINS 40
#define COAT_W1090 4.39444915467244f     // the 10-90 % width of a logistic in units of its scale: 2 ln 9
#define COAT_WIDTH_MIN 0.01f             // nm: a width of 0 asks for a step, and this is one to well under a bin
__device__ __forceinline__ float coat_softplus(float x) { return fmaxf(x, 0.f) + log1pf(expf(-fabsf(x))); }
__device__ __forceinline__ float coat_scale(float width) { return fmaxf(width, COAT_WIDTH_MIN) / COAT_W1090; }
__device__ __forceinline__ f3 coat_edge_rgb(const float4* __restrict__ bins, float lo, float hi, float edge, float width) {
    const float s = coat_scale(width);
    f3 acc = mk(0.f);
    float prev = coat_softplus((380.f - edge) / s);
    for (int k = 0; k < COAT_NBINS; k++) {
        const float next = coat_softplus((380.f + 10.f * (float)(k + 1) - edge) / s);
        const float4 w = __ldg(&bins[k]);
        acc = acc + mk(w.x, w.y, w.z) * (next - prev);
        prev = next;
    }
    return mk(lo) + acc * ((hi - lo) * (s / 10.f));
}
__device__ __forceinline__ float coat_edge_at_lambda(float lo, float hi, float edge, float width, float lam) {
    return lo + (hi - lo) / (1.f + expf(-(lam - edge) / coat_scale(width)));
}
__device__ __forceinline__ float coat_edge_at(float edge0, float nSin, float nEff) {
    const float q = nSin / fmaxf(nEff, 1e-6f);
    return edge0 * sqrtf(fmaxf(0.f, 1.f - q * q));
}
// a coating over a metal (materials_pbr.js:114-136 metalFresnel, coatOverMetal): the stack's R and the metal's F summed
// as intensities, 1 - (1 - R)(1 - F) / (1 - R F), F held to [0, 1] first
__device__ __forceinline__ f3 coat_over_metal(f3 r, f3 f) {
    const f3 fc = mk(sat(f.x), sat(f.y), sat(f.z));
    return mk(1.f) - (mk(1.f) - r) * (mk(1.f) - fc) / vmax(mk(1.f) - r * fc, 1e-6f);
}

struct Lobes {
    f3 tX, tY, nZ, o, base, transTint, coatK, cm, ecO, ecAvg;
    f3 coatR;          // a coating's reflectance per channel at the view's angle (0 on an anti-reflective face)
    f3 pw;             // ...and the channels' weights in a reflect-or-pass pick: the ray's own shares (coat_pick)
    float ax, ay;      // the alphas along tX and tY (tX the rough axis of an anisotropic lobe)
    float aMin, r, metallic, trans, transl, eta, etaT, nrel, ps;
    bool isDelta;
    bool coated;       // a coating is the interface here: coatR, not coatK x the Fresnel (materials_pbr.js:106-112)
    bool through;      // THE SIDE BEYOND lit (materials_pbr.js:1176-1190): the lobes below the surface evaluated
    __device__ __forceinline__ float2 al() const { return make_float2(ax, ay); }
    __device__ __forceinline__ f3 to_local(f3 w) const { return mk(dot(w, tX), dot(w, tY), dot(w, nZ)); }
    __device__ __forceinline__ f3 to_world(f3 w) const { return normalize(tX * w.x + tY * w.y + nZ * w.z); }
    // the interface's reflectance at cosI: a coating's at the view's angle for every facet, total past the critical
    // angle, which no coating changes (materials_pbr.js:109-113 coatFresnel)
    __device__ __forceinline__ f3 coat_fresnel(float cosI) const {
        const float f = fresnel_dielectric(cosI, eta);
        if (coated) return f >= 1.f ? mk(1.f) : coatR;
        return vmin(coatK * f, 1.f);
    }
    __device__ __forceinline__ f3 metal_fresnel(float cosI) const {
        const f3 f = fresnel_schlick3(cosI, base);
        return coated ? coat_over_metal(coatR, f) : f;
    }
    // how likely a pick is to reflect, of a reflectance per channel (materials_pbr.js:137-142 reflectPick): the largest
    // channel uncoated, the channels weighed by what the ray carries under a coating
    __device__ __forceinline__ float reflect_pick(f3 c) const { return coated ? dot(c, pw) : max3(c); }
};
__device__ __forceinline__ f3 coat_albedo(const Lobes& lb, const MfTab& t, f3 w) {
    if (lb.coated) return lb.coatR;                 // the coating's at the view, at every angle (materials_pbr.js:151-153)
    return vmin(lb.coatK * mf_ec(t, w.z, lb.r, lb.nrel), 1.f);
}
// the coat's pick probability at the view (materials_pbr.js:274-279 coatPs)
__device__ __forceinline__ float coat_ps(const Lobes& lb) {
    return fminf(lb.reflect_pick(lb.coat_fresnel(lb.o.z)), fresnel_dielectric(lb.o.z, lb.eta) >= 1.f ? 1.f : 0.999f);
}
// A COATING'S PICK WEIGHED BY THE RAY (materials_pbr.js:280-291 coatPick): the channels' shares of |beta|, or alike for a
// ray carrying nothing; only where a ray scatters, so every density its MIS reads is this lobe's own
__device__ __forceinline__ void coat_pick(Lobes& lb, f3 beta) {
    if (!lb.coated) return;
    const f3 a = mk(fabsf(beta.x), fabsf(beta.y), fabsf(beta.z));
    const float t = a.x + a.y + a.z;
    lb.pw = t > 0.f ? a * (1.f / t) : mk(1.f / 3.f);
    lb.ps = coat_ps(lb);
}
// transm, spec and hz: the material's transmission, specular and haze, or the part of the face drawn from inside
// n0 the index of the medium the view is in, inside whether it is seen from within (the normal turned), lam the
// ray's own wavelength (0 none): a coating reads all three (materials_pbr.js:164 makeLobes)
// (lam3: the trace by wavelength's three wavelengths, one a channel, where the coating is taken at each)
__device__ __forceinline__ Lobes make_lobes(f3 n, f3 v, const st_material& m, float eta, const MfTab& t,
                                            float transm, float spec, float hz, float n0, bool inside, float lam,
                                            const f3* lam3 = nullptr) {
    Lobes lb;
    lb.through = false;
    f3 s = fabsf(n.z) < 0.999f ? normalize(cross(n, mk(0, 0, 1))) : normalize(cross(n, mk(0, 1, 0)));
    lb.tX = s; lb.tY = cross(s, n); lb.nZ = n;
    lb.o = mk(dot(v, lb.tX), dot(v, lb.tY), fmaxf(dot(v, n), 1e-4f));
    lb.r = clampf(m.roughness, 0.f, 1.f);
    float aIso = lb.r * lb.r;
    lb.isDelta = aIso < MF_ALPHA_MIN;
    // ANISOTROPY (microfacet.js mfAnisoAlpha; materials_pbr.js:185-194, without a grain): x the rough axis, the two
    // alphas' geometric mean r^2, their ratio 1 / (1 - 0.9 |anisotropy|) -- at most 10
    const float sa = sqrtf(1.f - 0.9f * fminf(fabsf(m.anisotropy), 1.f));
    const float ax = aIso / sa, ay = aIso * sa;
    lb.aMin = fminf(ax, ay);
    lb.ax = clampf(ax, MF_ALPHA_MIN, 1.f);
    lb.ay = clampf(ay, MF_ALPHA_MIN, 1.f);
    lb.metallic = sat(m.metallic);
    // TRANSMISSION AND HAZE (materials_pbr.js:196-204): T (1 - H) refracts; of the diffuse base, the share transl
    // passes through (T H of the whole)
    lb.trans = refract_share_of(transm, hz);
    lb.transl = 1.f - lb.trans > 1e-6f ? sat(sat(transm) * sat(hz) / fmaxf(1.f - lb.trans, 1e-6f)) : 0.f;
    lb.base = mk(m.base[0], m.base[1], m.base[2]);
    lb.transTint = m.attenuation > 0.f ? mk(1.f) : lb.base;
    float lum = max3(lb.base);
    f3 tint = lum > 0.f ? lb.base / fmaxf(lum, 1e-6f) : mk(1.f);
    float st = m.specular_tint;
    f3 tintMix = mk(1.f) * (1.f - st) + tint * st;
    lb.coatK = tintMix * mixf(2.f * spec, 1.f, lb.trans);
    lb.eta = eta; lb.etaT = eta;
    lb.nrel = clampf(1.f / eta, 1.f, 3.f);
    // A COATING (materials_pbr.js:220-245) is the interface on every face the light enters by; on a face it leaves by,
    // as the material says: anti-reflective (coat 1: nothing reflects but total internal reflection), the bare
    // interface (2), or the coating again (3). Evaluated once, at the view: a smooth coating's angle exactly.
    lb.coated = false;
    lb.coatR = mk(0.f);
    lb.pw = mk(1.f / 3.f);
    const uint32_t coat = min(m.coat, 3u);
    if (coat != 0u) {
        if (!inside || coat == 3u) {
            const float sin0 = sqrtf(fmaxf(0.f, 1.f - lb.o.z * lb.o.z));
            const float lo = sat(m.coat_lo), hi = sat(m.coat_hi), w = fmaxf(m.coat_width, 0.f);
            const float edge = coat_edge_at(m.coat_edge, n0 * sin0, fmaxf(m.coat_index, 1.f));
            if (lam3)
                lb.coatR = mk(coat_edge_at_lambda(lo, hi, edge, w, lam3->x), coat_edge_at_lambda(lo, hi, edge, w, lam3->y),
                              coat_edge_at_lambda(lo, hi, edge, w, lam3->z));
            else
                lb.coatR = lam > 0.f ? mk(coat_edge_at_lambda(lo, hi, edge, w, lam)) : coat_edge_rgb(t.coat, lo, hi, edge, w);
            lb.coated = true;
        } else if (coat == 1u) {
            lb.coated = true;
        }
    }
    lb.ps = coat_ps(lb);
    lb.ecO = coat_albedo(lb, t, lb.o);
    float e1 = lb.metallic > 0.f ? mf_e1(t, lb.o.z, lb.r) : 1.f;
    if (lb.coated) {
        lb.ecAvg = lb.coatR;
    } else {
        float eAvg = mf_ecavg(t, lb.r, lb.nrel);
        lb.ecAvg = vmin(lb.coatK * eAvg, 1.f);
    }
    // Turquin's factor from F0: the metal's colour, or under a coating what the two reflect head-on
    const f3 f0 = lb.coated ? coat_over_metal(lb.coatR, lb.base) : lb.base;
    lb.cm = mk(1.f) + f0 * (1.f / fmaxf(e1, 1e-3f) - 1.f);
    return lb;
}
__device__ __forceinline__ f3 lobes_through_eval(const Lobes& lb, const MfTab& t, f3 i, float minAlpha);
__device__ __forceinline__ f3 lobes_eval(const Lobes& lb, const MfTab& t, f3 l, float minAlpha) {
    f3 i = lb.to_local(l);
    if (lb.through && i.z < 0.f) return lobes_through_eval(lb, t, i, minAlpha);
    if (i.z <= 0.f) return mk(0.f);
    f3 f = mk(0.f);
    if (!lb.isDelta && lb.aMin >= minAlpha) {
        f3 h = normalize(lb.o + i);
        float spec = mf_d(h, lb.al()) * mf_g2(lb.o, i, lb.al()) / (4.f * lb.o.z * i.z);
        float oh = dot(lb.o, h);
        f = f + lb.cm * lb.metal_fresnel(oh) * (lb.metallic * spec);
        f = f + lb.coat_fresnel(oh) * ((1.f - lb.metallic) * spec);
    }
    float wDiff = (1.f - lb.metallic) * (1.f - lb.trans) * (1.f - lb.transl);   // ...less what passes through
    if (wDiff > 0.f) {
        f3 ecI = coat_albedo(lb, t, i);
        f3 den = vmax(mk(1.f) - lb.ecAvg, 1e-4f) * ST_PI;
        f = f + lb.base * (mk(1.f) - lb.ecO) * (mk(1.f) - ecI) / den * wDiff;
    }
    return f;
}
__device__ __forceinline__ float interface_reflect_p(const Lobes& lb, float oh) {
    float fh = lb.reflect_pick(lb.coat_fresnel(oh));
    float den = fh + (1.f - fh) * lb.trans;
    return den > 1e-6f ? fh / den : 1.f;
}
// THE SIDE BEYOND (materials_pbr.js:385-432): the refraction's generalised half vector turned to the view's side (w 0:
// none), the translucent base's value below -- the reflected share's form, mirrored -- and rough refraction's, and the
// sampler's density there
__device__ __forceinline__ float4 through_half(const Lobes& lb, f3 i) {
    f3 h = (lb.o * lb.etaT + i) * -1.f;
    const float hl = length(h);
    if (hl < 1e-12f) return make_float4(0.f, 0.f, 0.f, 0.f);
    h = h * (1.f / hl);
    if (h.z < 0.f) h = h * -1.f;
    if (dot(lb.o, h) <= 0.f || dot(i, h) >= 0.f) return make_float4(0.f, 0.f, 0.f, 0.f);
    return make_float4(h.x, h.y, h.z, 1.f);
}
__device__ __forceinline__ f3 lobes_through_eval(const Lobes& lb, const MfTab& t, f3 i, float minAlpha) {
    const float wd = 1.f - lb.metallic;
    f3 f = mk(0.f);
    const float wT = wd * (1.f - lb.trans) * lb.transl;
    if (wT > 0.f) {
        const f3 ecI = coat_albedo(lb, t, mk(i.x, i.y, -i.z));
        f = lb.base * (mk(1.f) - lb.ecO) * (mk(1.f) - ecI) / (vmax(mk(1.f) - lb.ecAvg, 1e-4f) * ST_PI) * wT;
    }
    if (wd <= 0.f || lb.trans <= 0.f || lb.isDelta || lb.aMin < minAlpha) return f;
    const float4 hh = through_half(lb, i);
    if (hh.w == 0.f) return f;
    const f3 h = mk(hh.x, hh.y, hh.z);
    const float oh = dot(lb.o, h), ih = dot(i, h), den = lb.etaT * oh + ih;
    const f3 fc = lb.coat_fresnel(oh);
    return f + (mk(1.f) - fc) * lb.transTint *
               (wd * lb.trans * mf_d(h, lb.al()) * mf_g2(lb.o, i, lb.al()) * oh * (-ih) /
                (lb.o.z * (-i.z) * fmaxf(den * den, 1e-20f)));
}
__device__ __forceinline__ float lobes_through_pdf(const Lobes& lb, f3 i) {
    const float wd = 1.f - lb.metallic;
    const float pd = (1.f - lb.ps) * (1.f - lb.trans);
    const float p = wd * pd * lb.transl * (-i.z) / ST_PI;            // the translucent base's cosine draw
    if (wd <= 0.f || lb.trans <= 0.f || lb.isDelta) return p;
    const float4 hh = through_half(lb, i);
    if (hh.w == 0.f) return p;
    const f3 h = mk(hh.x, hh.y, hh.z);
    const float oh = dot(lb.o, h), ih = dot(i, h), den = lb.etaT * oh + ih;
    return p + wd * (1.f - pd) * (1.f - interface_reflect_p(lb, oh)) * mf_g1(lb.o, lb.al()) * mf_d(h, lb.al()) * oh / lb.o.z *
                   (-ih) / fmaxf(den * den, 1e-20f);
}
__device__ __forceinline__ float lobes_pdf(const Lobes& lb, f3 l) {
    f3 i = lb.to_local(l);
    if (lb.through && i.z < 0.f) return lobes_through_pdf(lb, i);
    if (i.z <= 0.f) return 0.f;
    float wd = 1.f - lb.metallic;
    float pd = (1.f - lb.ps) * (1.f - lb.trans);
    float p = wd * pd * (1.f - lb.transl) * i.z / ST_PI;
    if (!lb.isDelta) {
        float pr = mf_pdf_reflect(lb.o, i, lb.al());
        p += (lb.metallic + wd * (1.f - pd) * interface_reflect_p(lb, dot(lb.o, normalize(lb.o + i)))) * pr;
    }
    return p;
}
__device__ __forceinline__ bool lobes_none(const st_material& m, float transmission, float hz) {
    float r = clampf(m.roughness, 0.f, 1.f);
    return r * r < MF_ALPHA_MIN && (1.f - sat(m.metallic)) * (1.f - refract_share_of(transmission, hz)) <= 0.f;
}
// a transmission lobe that can be evaluated, from the material (or the part drawn) alone (materials_pbr.js:379-384)
__device__ __forceinline__ bool through_evaluable(const st_material& m, float transmission, float hz) {
    const float r = clampf(m.roughness, 0.f, 1.f), wd = 1.f - sat(m.metallic);
    return (wd * refract_share_of(transmission, hz) > 0.f && r * r >= MF_ALPHA_MIN) || wd * sat(transmission) * sat(hz) > 0.f;
}
struct LobeSample { f3 dir, w; uint32_t ev; bool isDelta, transmitted; };
__device__ __forceinline__ LobeSample lobes_sample(const Lobes& lb, const MfTab& t, float4 rnd) {
    LobeSample s;
    s.w = mk(0.f); s.ev = EV_OTHER; s.isDelta = false; s.transmitted = false;
    f3 i = mk(0, 0, 1);
    uint32_t glossyEv = lb.aMin >= 0.05f ? EV_EVAL : EV_OTHER;
    float wd = 1.f - lb.metallic;
    float pick = rnd.x;
    if (pick < lb.metallic) {
        if (lb.isDelta) {
            i = mk(-lb.o.x, -lb.o.y, lb.o.z);
            s.w = lb.metal_fresnel(lb.o.z) * lb.cm;
            s.ev = EV_DELTA; s.isDelta = true;
        } else {
            f3 h = mf_sample_vndf(lb.o, lb.al(), rnd.y, rnd.z);
            i = reflectv(-lb.o, h);
            if (i.z > 0.f) s.w = lb.cm * lb.metal_fresnel(dot(lb.o, h)) * (mf_g2(lb.o, i, lb.al()) / mf_g1(lb.o, lb.al()));
            s.ev = glossyEv;
        }
    } else {
        pick = (pick - lb.metallic) / fmaxf(wd, 1e-6f);
        float pd = (1.f - lb.ps) * (1.f - lb.trans);
        if (pick < 1.f - pd) {
            float sub = pick / fmaxf(1.f - pd, 1e-6f);
            if (lb.isDelta) {
                if (sub < lb.ps / fmaxf(1.f - pd, 1e-6f)) {
                    i = mk(-lb.o.x, -lb.o.y, lb.o.z);
                    s.w = lb.coat_fresnel(lb.o.z) / lb.ps;
                } else {
                    s.transmitted = true;
                    i = refractv(-lb.o, mk(0, 0, 1), lb.etaT);
                    if (i.z < 0.f) s.w = (mk(1.f) - lb.coat_fresnel(lb.o.z)) * lb.transTint / (1.f - lb.ps);
                }
                s.ev = EV_DELTA; s.isDelta = true;
            } else {
                f3 h = mf_sample_vndf(lb.o, lb.al(), rnd.y, rnd.z);
                float oh = dot(lb.o, h);
                f3 fc = lb.coat_fresnel(oh);
                float r = interface_reflect_p(lb, oh);
                if (sub < r) {
                    i = reflectv(-lb.o, h);
                    if (i.z > 0.f) s.w = fc * (mf_g2(lb.o, i, lb.al()) / mf_g1(lb.o, lb.al()) / ((1.f - pd) * r));
                    s.ev = glossyEv;
                } else {
                    s.transmitted = true;
                    i = refractv(-lb.o, h, lb.etaT);
                    if (i.z < 0.f)
                        s.w = (mk(1.f) - fc) * lb.transTint *
                              (lb.trans * mf_g2(lb.o, i, lb.al()) / mf_g1(lb.o, lb.al()) / ((1.f - pd) * (1.f - r)));
                    s.ev = lb.aMin >= 0.05f ? EV_EVAL : EV_OTHER;
                }
            }
        } else {
            // the diffuse base: of it, transl passes through (materials_pbr.js:525-539), a cosine below weighed as the
            // reflected share's draw is, into the medium beyond as a refraction
            float r = sqrtf(rnd.y);
            float sp, cp;
            sincosf(2.f * ST_PI * rnd.z, &sp, &cp);
            const float z = sqrtf(fmaxf(0.f, 1.f - rnd.y));
            const bool thru = rnd.w < lb.transl;
            i = mk(r * cp, r * sp, z);
            f3 ecI = coat_albedo(lb, t, i);
            s.w = lb.base * (mk(1.f) - lb.ecO) * (mk(1.f) - ecI) / vmax(mk(1.f) - lb.ecAvg, 1e-4f) / (1.f - lb.ps);
            s.ev = EV_EVAL;
            if (thru) { i.z = -z; s.transmitted = true; }
        }
    }
    s.dir = lb.to_world(i);
    return s;
}

}  // namespace st
