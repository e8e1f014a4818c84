// st_photons.cu -- the photon map inside the wavefront (core/sppm.js, core/wavefront.js:519-626 prog_genphotons,
// :1150-1235 prog_sppm) for sm_103a.
//
// THE REFERENCE runs a sample's photons before its camera rays through the same wavefront: sun photons are drawn
// over a square across the sun's direction, marched, and at each hit either STORED -- a photon that has passed
// delta events only (glass, mirrors), at least one, landing on a surface a camera connection can evaluate -- or
// bounced; the sample's camera rays that have seen only delta events since the eye then GATHER the stored photons
// where they land (sum f Phi / (pi r^2), over the evaluable lobes), the radius shrinking from sample to sample, and a
// camera path that reaches the sun through delta events after its D leaves the disc's light to the map.
//
// HERE the same order inside one graph a sample: k_sppm_begin (the sample's radius, the count cleared), per chunk of
// photons k_genphotons then the march / surface / k_photon_shade iterations (a photon that is stored, or scatters
// off anything but a delta lobe, is done: it can never be stored again), the grid built by a counting sort
// (st_sppm.cu sppm_grid_launch), then the camera's iterations with k_gather between the surface kernel and shade.
// The photons' random numbers come from their own sample seed, the photon's id and its shade count; the gather's
// from the path's own stream with a salt of its own, so the shading draws are the same with the map on or off.
#include <algorithm>
#include <cmath>

#include "st_emit.cuh"
#include "st_internal.h"
#include "st_kernels.cuh"
#include "st_sppm_dev.cuh"

namespace st {

#define PHOTON_GEN_SALT 0x5A17u            // their draw at the source (wavefront.js:594 SEED_u32(0x5A17))
#define SPPM_STORE_SALT 0x53505031u        // a store's and a gather's own stream (wavefront.js:1186)
#define LT_LENS_SALT 0x4C54434Eu           // a connection's point of the lens, from the photon's own stream

__device__ __forceinline__ uint4 photon_seed(const Uni& u, uint32_t sample) { return photon_seed_of(u.seed, sample); }
// sppmEvaluable (wavefront.js prog_sppm, sppm.js:441-444): a diffuse base, or gloss rough enough to evaluate
__device__ __forceinline__ bool sppm_evaluable(const st_material& m, bool all) {
    const float r = clampf(m.roughness, 0.f, 1.f);
    return (1.f - m.metallic) * (1.f - sat(m.transmission)) > 0.f || r * r >= (all ? 1e-3f : LT_MIN_ALPHA);
}

// THE SAMPLE'S RADIUS (sppm.js:177-181): r_k^2 = r_1^2 prod_{i<k} (i + alpha) / (i + 1), k the sample's number from
// 1; the grid's cell is 2 r; the count of records cleared
// AND IN THE VOLUME (sppm.js:182-191 sppmRadiusVolume): R_k^3 = R_1^3 times the same product, its records' cell 2 R
__global__ void k_sppm_begin(SppmDev* __restrict__ d, const DevCtr* __restrict__ ctr, float r1, float alpha, uint32_t cap,
                             float r1v) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const uint32_t k = ctr->sample + 1u;
    double s = 1.0;
    for (uint32_t i = 1; i < k; i++) s *= (i + (double)alpha) / (i + 1.0);
    const double r = (double)r1 * sqrt(s);
    d->r = (float)r;
    d->r2 = (float)r * (float)r;
    d->cell = (float)(2.0 * r);
    d->inv_area = (float)(1.0 / (3.14159265358979323846 * r * r));
    const double rv = (double)r1v * cbrt(s);
    d->vr = (float)rv;
    d->vr2 = (float)rv * (float)rv;
    d->vcell = (float)(2.0 * rv);
    d->inv_vol = (float)(3.0 / (4.0 * 3.14159265358979323846 * rv * rv * rv));
    d->vstores = 0u;
    d->vgathers = 0u;
    const float room = 0.5f * (float)cap;
    d->vkeep = (k > 1u && (float)d->vdemand > room) ? room / (float)d->vdemand : 1.f;
    d->vdemand = 0u;
    d->count = 0u;
    d->cap = cap;
    d->dropped = 0u;
    d->gathers = 0u;
    d->visits = 0ull;
}

// THE LEARNED EMISSION MAP (wavefront.js:520-536 ltSearch / ltMass, :628-711 prog_lt_build). A cell's worth is its
// stores per photon it sent (the reference's camera connections per photon; this build has no connections to the
// camera, and a stored photon is what the map's camera rays use); both counts halve at every rebuild, so the map
// forgets; the density is (1 - LT_FLOOR) worth / total + LT_FLOOR uniform, as a row CDF and per-row conditional
// CDFs. One block of LT_GRID threads, a row each; run at a sample's start, every fourth sample from the fourth.
__device__ __forceinline__ uint32_t lt_search(const float* __restrict__ cdf, float u) {
    uint32_t lo = 0, hi = LT_GRID - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (u < cdf[mid]) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}
__device__ __forceinline__ float lt_mass(const float* __restrict__ cdf, uint32_t i) {
    return fmaxf(cdf[i] - (i ? cdf[i - 1] : 0.f), 0.f);
}
__global__ void __launch_bounds__(LT_GRID) k_lt_build(SppmBufs b, const DevCtr* __restrict__ ctr) {
    // every operation IEEE-rounded and none fused (the _rn intrinsics): the map is a function of the integer counts
    // alone, the same bits as the oracle's sequential f32 build of them
    __shared__ float rowW[LT_GRID], rowP[LT_GRID];
    __shared__ float total;
    const uint32_t k = ctr->sample;
    if (k == 0u || (k & 3u) != 0u) return;                           // every fourth sample
    const uint32_t r = threadIdx.x, base = r * LT_GRID;
    const float keep = 1.f - LT_FLOOR, rfloor = LT_FLOOR / (float)LT_GRID, cfloor = LT_FLOOR / (float)LT_CELLS;
    float sum = 0.f;
    for (uint32_t c = 0; c < LT_GRID; c++) {
        const uint32_t e = b.lt_emit[base + c], h = b.lt_hit[base + c];
        const float w = e > 0u ? __fdiv_rn((float)h, (float)e) : 0.f;
        b.lt_cdf[base + c] = w;                                      // scratch: the raw worth
        sum = __fadd_rn(sum, w);
        b.lt_emit[base + c] = e / 2u;                                // forget half
        b.lt_hit[base + c] = h / 2u;
    }
    rowW[r] = sum;
    __syncthreads();
    if (r == 0) {
        float t = 0.f;
        for (uint32_t q = 0; q < LT_GRID; q++) t = __fadd_rn(t, rowW[q]);
        total = t;
    }
    __syncthreads();
    const float T = total;
    const bool learned = T > 0.f;
    const float Tm = fmaxf(T, 1e-30f);
    const float rp = learned ? __fadd_rn(__fdiv_rn(__fmul_rn(keep, rowW[r]), Tm), rfloor) : 1.f / (float)LT_GRID;
    rowP[r] = rp;
    float acc = 0.f;
    for (uint32_t c = 0; c < LT_GRID; c++) {
        const float p = learned ? __fadd_rn(__fdiv_rn(__fmul_rn(keep, b.lt_cdf[base + c]), Tm), cfloor)
                                : 1.f / (float)LT_CELLS;
        acc = __fadd_rn(acc, p);
        b.lt_cdf[base + c] = __fdiv_rn(acc, rp);                      // conditional on the row
    }
    b.lt_cdf[base + LT_GRID - 1u] = 1.f;
    __syncthreads();
    if (r == 0) {
        float racc = 0.f;
        for (uint32_t q = 0; q < LT_GRID; q++) {
            racc = __fadd_rn(racc, rowP[q]);
            b.lt_cdf[LT_CELLS + q] = racc;
        }
        b.lt_cdf[LT_CELLS + LT_GRID - 1u] = 1.f;
    }
}

// THE SUN'S PHOTONS (wavefront.js:596-626): a direction in the sun's cone, a point uniform over the square of half
// width sppm_half across the sun's direction (the reference's learned 128^2 map at its uniform start), the photon
// started back along its line at the scene's radius, its flux L_disc cos Omega / (N pdf_area)
__global__ void __launch_bounds__(256) k_genphotons(WaveArgs a, uint32_t first, uint32_t n) {
    const Uni& u = a.u;
    const uint4 ps = photon_seed(u, a.ctr->sample);
    const f3 s = u.sun_dir;
    const f3 t = fabsf(s.x) > 0.9f ? mk(0, 1, 0) : mk(1, 0, 0);
    const f3 b1 = normalize(cross(t, s));
    const f3 b2 = cross(s, b1);
    const float R = u.sppm_half;
    const float n_sun = (float)max(u.sppm_n - u.lt_emit_n, 1u);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t id = first + i;
        Rng rng = path_rng(ps, id, PHOTON_GEN_SALT);
        const float4 r0 = rng.next();
        if (id < u.lt_emit_n) {
            // AN EMITTER PROBE (wavefront.js:552-588): a listed box by its probability, a direction w uniform on the
            // sphere, a point uniform on the disc across the box's bounding sphere perpendicular to w -- a uniformly
            // random line through the sphere -- started at the line's far end, heading back (-w), its chord its length;
            // nothing listed yet: a probe that finds nothing
            const EmitDev* ed = a.em.dev;
            const uint32_t K = ed ? min(ed->count, EMIT_MAX) : 0u;
            f3 org = mk(0.f), dir = mk(0.f, 0.f, 1.f);
            float len = -1.f;
            if (K > 0u) {
                const float4 r1 = rng.next();
                const uint32_t b = emit_pick(ed, r0.x);
                const float4 bx = ed->box[b];
                const float z = 1.f - 2.f * r0.y, rz = sqrtf(fmaxf(0.f, 1.f - z * z));
                float sw, cw;
                sincosf(2.f * ST_PI * r0.z, &sw, &cw);
                const f3 w = mk(rz * cw, rz * sw, z);
                const f3 ta = fabsf(w.x) > 0.9f ? mk(0.f, 1.f, 0.f) : mk(1.f, 0.f, 0.f);
                const f3 e1 = normalize(cross(ta, w));
                const f3 e2 = cross(w, e1);
                const float rho = bx.w * sqrtf(r0.w);
                float sd, cd;
                sincosf(2.f * ST_PI * r1.x, &sd, &cd);
                const f3 q = mk(bx.x, bx.y, bx.z) + e1 * (rho * cd) + e2 * (rho * sd);
                const float hl = sqrtf(fmaxf(bx.w * bx.w - rho * rho, 0.f));
                org = q + w * hl;
                dir = -w;
                len = 2.f * hl;
            }
            a.pb.pos[i] = make_float4(org.x, org.y, org.z, 0.f);
            a.pb.dir[i] = make_float4(dir.x, dir.y, dir.z, 1.f);
            a.pb.beta[i] = make_float4(1.f, 1.f, 1.f, 1.f);
            a.pb.rad[i] = make_float4(0.f, 0.f, 0.f, len);                 // w: its length along the line
            a.pb.meta[i] = make_uint4(id, meta_y(0, 0, RAY_ACTIVE) | META_PROBE, 0u, __float_as_uint(0.f));
            a.pb.lam[i] = 0.f;
            a.pb.lprev[i] = make_float2(__uint_as_float(0xffffffffu), 0.f);
            a.q.ray[0][i] = i;
            continue;
        }
        const f3 w = sample_sun_cone(u, r0.x, r0.y);
        float x, y, area;                                                // the point, and 1 / its density
        uint32_t cell = 0xffffffffu;
        if (u.sppm_learn) {                                              // a cell by the map, a point in it
            const float4 r1 = rng.next();
            const uint32_t row = lt_search(a.sp.lt_cdf + LT_CELLS, r0.z);
            const uint32_t col = lt_search(a.sp.lt_cdf + row * LT_GRID, r0.w);
            const float pCell = lt_mass(a.sp.lt_cdf + LT_CELLS, row) * lt_mass(a.sp.lt_cdf + row * LT_GRID, col);
            const float csz = 2.f * R / (float)LT_GRID;
            x = -R + ((float)col + r1.x) * csz;
            y = -R + ((float)row + r1.y) * csz;
            area = csz * csz / fmaxf(pCell, 1e-30f);
            cell = row * LT_GRID + col;
            atomicAdd(&a.sp.lt_emit[cell], 1u);
        } else {                                                         // the square, uniform
            x = -R + 2.f * R * r0.z;
            y = -R + 2.f * R * r0.w;
            area = 4.f * R * R;
        }
        const float cosW = fmaxf(dot(w, s), 1e-4f);
        const f3 q = b1 * x + b2 * y;
        const f3 org = q + w * ((u.envR - dot(q, s)) / cosW);
        const f3 disc = u.sun_on ? env_radiance(u, w) : mk(0.f);
        const f3 flux = disc * (cosW * u.sun_omega * area / n_sun);
        a.pb.pos[i] = make_float4(org.x, org.y, org.z, 0.f);
        a.pb.dir[i] = make_float4(-w.x, -w.y, -w.z, 1.f);
        a.pb.beta[i] = make_float4(1.f, 1.f, 1.f, 1.f);
        a.pb.rad[i] = make_float4(flux.x, flux.y, flux.z, 0.f);          // a photon's radiance field is its flux
        a.pb.meta[i] = make_uint4(id, meta_y(0, 0, RAY_ACTIVE), 0u, __float_as_uint(0.f));   // w: absLtot (haze.js)
        a.pb.lam[i] = 0.f;
        a.pb.lprev[i] = make_float2(__uint_as_float(cell), 0.f);        // its emission cell
        a.q.ray[0][i] = i;
    }
}

// A PHOTON'S CONNECTION TO THE CAMERA (materials_pbr.js:672-830 ltConnect, :598-612 camFootprint, lens.js lensDisc /
// lensImage; haze.js:404-460 ltConnectMedium). From the point P to the camera -- to a point of the thin lens's disc
// drawn uniformly from the photon's own stream, or the pinhole -- for the pixel the line lands on: phi f G / A_px, A_px
// a pixel's area on the image plane at unit distance, f the camera's lobes evaluated for the photon's direction (the
// evaluable ones, glossy from LT_MIN_ALPHA up) or, in the haze, the phase function; G = |n.v| dist / z^3 at a surface
// and dist / z^3 in the air (perspective; |n.fwd| and 1 orthographic). False where nothing connects: behind the
// camera, off the picture, the camera on the surface's other side, no evaluable lobe, no light. The haze the line
// crosses is put on what it carries (haze.js:463-481 hazeShadow).
struct LtConn { f3 org, dir, c; float len; uint32_t pix; };
struct LtView { f3 cam, v; float dist, gm; uint32_t pix; };
__device__ __forceinline__ bool lt_view(const Uni& u, f3 P, const uint4& ps, uint32_t id, LtView& o) {
    f3 off = mk(0.f);
    const float R = u.camtype == 0u ? u.lens_r : 0.f;
    if (R > 0.f) {
        Rng rl = path_rng(ps, id, LT_LENS_SALT);
        const float4 ul = rl.next();
        const float r = R * sqrtf(ul.x);
        float sp, cp;
        sincosf(6.28318530718f * ul.y, &sp, &cp);
        off = u.right * (r * cp) + u.up * (r * sp);
    }
    o.cam = u.cam + off;
    const f3 d = o.cam - P;
    float xx, yy;
    if (u.camtype == 0u) {
        o.dist = length(d);
        const float z = dot(d, u.fwd);                                // depth in front of the camera
        if (z <= 1e-4f || o.dist <= 1e-4f) return false;
        o.v = d * (1.f / o.dist);
        if (R > 0.f) {                                                // where the lens point's ray meets the picture
            const float c = dot(o.v, u.fwd);
            const f3 F = off + (-o.v) * (u.lens_f / fmaxf(c, 1e-30f));
            xx = dot(F, u.right) / (u.lens_f * u.fx);
            yy = dot(F, u.up) / (u.lens_f * u.fy);
        } else {
            xx = -dot(d, u.right) / (z * u.fx);
            yy = -dot(d, u.up) / (z * u.fy);
        }
        o.gm = o.dist / (z * z * z);
    } else {
        o.dist = dot(d, u.fwd);                                       // to the camera plane along the view axis
        if (o.dist <= 1e-4f) return false;
        o.v = u.fwd;
        xx = -dot(d, u.right) / u.fx;
        yy = -dot(d, u.up) / u.fy;
        o.gm = 1.f;
    }
    if (fabsf(xx) >= 1.f || fabsf(yy) >= 1.f) return false;           // off the picture
    const float px = clampf((xx + 1.f) * 0.5f * (float)u.W, 0.f, (float)u.W - 1.f);
    const float py = clampf((yy + 1.f) * 0.5f * (float)u.H, 0.f, (float)u.H - 1.f);
    o.pix = (uint32_t)px + (uint32_t)py * u.W;
    return true;
}
__device__ __forceinline__ float lt_apx(const Uni& u) { return 4.f * u.fx * u.fy / ((float)u.W * (float)u.H); }
__device__ __forceinline__ void lt_haze(const Uni& u, f3 P, float h, LtConn& out) {
    if (!u.haze_on) return;
    const f3 e = out.org + out.dir * (out.len + h) - P;               // the true segment, to the camera
    const float el = length(e);
    out.c = out.c * haze_tr(u, P, e * (1.f / fmaxf(el, 1e-30f)), el);
}
// at a surface (in air, nrm turned to the photon, which arrives along din with flux phi): the shadow ray starts on the
// camera's line of sight to P, as far along it as lifts it 2 offsets off the surface (at grazing views at most 4 such
// lengths, the rest along the normal, re-aimed at the camera), and stops that height short of the camera
__device__ __forceinline__ bool lt_connect(const Uni& u, const st_material& m, const MfTab& tab, f3 P, f3 nrm, f3 din,
                                           f3 phi, float lam, const uint4& ps, uint32_t id, LtConn& out) {
    LtView w;
    if (!lt_view(u, P, ps, id, w)) return false;
    if (lobes_none(m, m.transmission, m.haze)) return false;
    const f3 v = w.v;
    const float cv = dot(nrm, v);
    if (cv <= 0.f) return false;                                      // the camera on the surface's other side
    // the camera's own lobes at this vertex, seen along v, in air (the interface air to the material's index); a
    // coating's pick keeps the even weights, the camera's first vertex's (its beta is white)
    const Lobes lb = make_lobes(nrm, v, m, 1.f / fmaxf(m.ior, 1.f), tab, m.transmission, m.specular, m.haze, 1.f, false,
                                lam);
    const f3 f = lobes_eval(lb, tab, -din, LT_MIN_ALPHA);
    out.c = phi * f * (cv * w.gm / lt_apx(u));
    if (!(luma(out.c) > 0.f)) return false;
    out.pix = w.pix;
    const float h = 20.f * march_tol(P, u.tol);                       // offsetTol(P) * 2
    const bool grazing = cv < 0.25f;
    const float sl = h / fmaxf(cv, 0.25f);
    const float lift = grazing ? h - sl * cv : 0.f;
    out.org = P + v * sl + nrm * lift;
    out.dir = v;
    out.len = w.dist - sl - cv * lift - h;
    if (grazing && u.camtype == 0u) {
        const f3 toCam = w.cam - out.org;
        const float l = length(toCam);
        out.dir = toCam * (1.f / fmaxf(l, 1e-30f));
        out.len = l - h;
    }
    lt_haze(u, P, h, out);
    return out.len > 0.f;
}
// in the haze (a collision; the photon arrives along din with flux phi, its albedo in it): no surface, so no side and
// no lift -- the shadow ray starts at the point and stops 2 offsets short of the camera
__device__ __forceinline__ bool lt_connect_medium(const Uni& u, f3 P, f3 din, f3 phi, const uint4& ps, uint32_t id,
                                                  LtConn& out) {
    LtView w;
    if (!lt_view(u, P, ps, id, w)) return false;
    const float ph = hg_eval(dot(din, w.v), clampf(u.hg, -0.95f, 0.95f));
    out.c = phi * (ph * w.gm / lt_apx(u));
    if (!(luma(out.c) > 0.f)) return false;
    out.pix = w.pix;
    const float h = 20.f * march_tol(P, u.tol);
    out.org = P;
    out.dir = w.v;
    out.len = w.dist - h;
    lt_haze(u, P, h, out);
    return out.len > 0.f;
}

// A PHOTON'S HIT (prog_sppm's store, then pathBegin..pathEnd for a photon): with light tracing on, connected to the
// camera first (pathMiddle: once it has passed a delta event, in air, within the bounce cap); then stored where it
// may be, else bounced -- no light sampling; a delta lobe keeps it in the class, anything else ends it. Connections go
// to the shadow side `side`, which the occlusion pass after this kernel traces.
__global__ void __launch_bounds__(256) k_photon_shade(WaveArgs a, int nxt, int last, int side) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    const Uni& u = a.u;
    st_material* sm = reinterpret_cast<st_material*>(smem);
    if (!stage_table(sm, a.mats, u.n_mats * (uint32_t)sizeof(st_material), &mbar, a.ctr)) return;
    const uint32_t count = a.ctr->hitCount;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t nrounds = (count + stride - 1) / stride;
    uint32_t* __restrict__ outq = nxt ? a.q.ray[1] : a.q.ray[0];
    uint32_t* outc = nxt ? &a.ctr->rayCount[1] : &a.ctr->rayCount[0];
    const uint4 ps = photon_seed(u, a.ctr->sample);
    SppmDev* d = a.sp.dev;
    for (uint32_t r = 0; r < nrounds; r++) {
        const uint32_t q = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool cont = false, store = false;
        uint32_t slot = 0;
        f3 pos = mk(0.f), dir = mk(0.f), beta = mk(0.f), rad = mk(0.f), nrm = mk(0.f);
        float ltot = 0.f, n = 1.f, lam = 0.f;
        uint4 m4 = make_uint4(0, 0, 0, 0);
        uint32_t bounces = 0, sub = 0;
        bool conn = false;
        LtConn lc;
        if (q < count) {
            slot = a.q.hit[q];
            const float dh = a.q.hitd[q];
            const float4 p4 = a.pb.pos[slot], d4 = a.pb.dir[slot], b4 = a.pb.beta[slot], r4 = a.pb.rad[slot];
            m4 = a.pb.meta[slot];
            pos = xyz(p4); ltot = p4.w; dir = xyz(d4); n = d4.w; beta = xyz(b4); rad = xyz(r4);
            bounces = m4.y & 0xffu;
            const uint32_t state = (m4.y >> 16) & 0xffu;
            const uint32_t cell = __float_as_uint(a.pb.lprev[slot].x);    // its emission cell
            if (m4.y & META_PROBE) {
                // THE PROBE (tracebasics.js:782-831): past its chord, out of the scene or out of steps it found
                // nothing; an emissive surface seen from outside starts its photon, leaving along the line with the
                // emission over the probes and the line density there (Crofton: |n.w| dA dw / (4 pi^2 r^2) a box, the
                // Lambertian emission's own measure); anything else it passes through
                const float4 r4 = a.pb.rad[slot];
                if (state == RAY_ACTIVE && ltot <= r4.w) {
                    const float4 sf = a.q.hsurf[q];
                    const uint32_t ids = __float_as_uint(sf.w);
                    const float otol = 10.f * march_tol(pos, u.tol);
                    const st_material* m = ids != SURF_LEAVING ? &sm[ids & 0xffffu] : nullptr;
                    const f3 nn = xyz(sf);
                    const bool outside = m && dh >= 0.f && dot(nn, -dir) > 0.f;
                    const f3 le = m ? mk(m->emissive[0], m->emissive[1], m->emissive[2]) : mk(0.f);
                    if (outside && max3(le) > 0.f) {
                        const EmitDev* ed = a.em.dev;
                        const uint32_t K = min(ed->count, EMIT_MAX);
                        float dens = 0.f;
                        for (uint32_t b = 0; b < K; b++) {
                            const float4 bx = ed->box[b];
                            const f3 d = pos - mk(bx.x, bx.y, bx.z);
                            if (dot(d, d) < bx.w * bx.w) dens += ed->pc[b].x / (4.f * ST_PI * ST_PI * bx.w * bx.w);
                        }
                        if (dens > 0.f) {
                            pos = pos + nn * (2.f * otol);
                            dir = -dir;
                            rad = le * (emit_beam(m->beam_cos, dot(dir, nn)) / ((float)u.lt_emit_n * dens));
                            beta = mk(1.f);
                            ltot = 0.f;
                            n = 1.f;
                            bounces = 0;
                            m4.y = meta_y(0, 0, RAY_ACTIVE);              // a photon now, its own flags clear
                            m4.w = __float_as_uint(0.f);
                            a.pb.rad[slot] = make_float4(rad.x, rad.y, rad.z, 0.f);
                            cont = !last && luma(rad) > 0.f;
                        }
                    } else {
                        const f3 off = dir * (2.f * otol);
                        pos = pos + off; ltot += length(off);
                        cont = !last;
                    }
                }
            } else if (state == RAY_SCATTER) {
                // A COLLISION IN THE AIR (haze.js:491-545 mediumVertex, a photon's): the albedo on its weight; once it
                // has passed a delta event, its connection through the phase function (ltConnectMedium); then its end
                bounces += 1;
                beta = beta * u.halb;
                if (u.lt_on && (m4.y & META_PASSED) != 0u && bounces <= u.maxbounce) {
                    conn = lt_connect_medium(u, pos, dir, rad * beta, ps, m4.x, lc);
                    if (conn && u.sppm_learn && cell < LT_CELLS) atomicAdd(&a.sp.lt_hit[cell], 1u);
                }
            } else if (state == RAY_ACTIVE) {
                const float4 sf = a.q.hsurf[q];
                const uint32_t ids = __float_as_uint(sf.w);
                const f3 nn = xyz(sf);
                nrm = dh < 0.f ? -nn : nn;
                const float eps = march_tol(pos, u.tol), otol = 10.f * eps;
                if (ids == SURF_LEAVING) {                            // seen from behind: moved on, no event
                    const f3 off = dir * otol;
                    pos = pos + off; ltot += length(off) * n;
                    cont = !last;
                } else {
                    const st_material& m = sm[ids & 0xffffu];
                    const bool emissive = fmaxf(fmaxf(m.emissive[0], m.emissive[1]), m.emissive[2]) > 0.f;
                    const bool passed = (m4.y & META_PASSED) != 0u;
                    if (u.lt_on && !emissive && passed && fabsf(n - 1.f) <= 1e-3f && bounces + 1u <= u.maxbounce) {
                        conn = lt_connect(u, m, a.tab, pos, nrm, dir, rad * beta, a.pb.lam[slot], ps, m4.x, lc);
                        // teach the emission map: this cell's photon reached the camera (ltConnect's learn)
                        if (conn && u.sppm_learn && cell < LT_CELLS) atomicAdd(&a.sp.lt_hit[cell], 1u);
                    }
                    if (emissive) {
                    } else if (passed && sppm_evaluable(m, false)) {
                        // STORED (sppm.js sppmStores / sppmStore): within the cap a gather can accept
                        if (u.sppm_on && bounces + 2u <= u.maxbounce && luma(rad * beta) > 0.f) {
                            Rng rs = path_rng(ps, m4.x, SPPM_STORE_SALT);
                            const float4 us = rs.next();
                            sub = min((uint32_t)(us.y * (float)SPPM_SUBS), SPPM_SUBS - 1u);
                            store = true;
                        }
                    } else {
                        lam = a.pb.lam[slot];
                        bounces += 1;
                        m4.w = __float_as_uint(ltot);                        // absLtot: the ltot on arrival here
                        uint32_t seg = (m4.y >> 8) & 0xffu;
                        Rng rng = path_rng(ps, m4.x, 1u + seg);
                        seg += 1;
                        const bool inside = dh < 0.f;
                        float n0 = n, n1d = fmaxf(m.ior, n0), v1 = 0.f;
                        if ((ids >> 16) != SURF_NONE) { n1d = sm[ids >> 16].ior; v1 = sm[ids >> 16].abbe; }
                        const float lam0 = lam;
                        const float n1 = lam0 > 0.f ? cauchy_n(n1d, v1, lam0) : n1d;
                        const bool draw = v1 > 0.f && lam0 == 0.f;
                        SpecDraw spec;
                        float nT = n1;
                        if (draw) {
                            const float4 rl = rng.next();
                            spec = spec_draw(a.spec, rl.x);
                            spec.lam = lambda_coded(spec.lam);
                            nT = cauchy_n(n1d, v1, spec.lam);
                        }
                        const float pG = refract_share_of(m.transmission, m.haze);
                        float trans = m.transmission, specv = m.specular, hz = m.haze;
                        bool diffFace = pG <= 0.f && m.transmission > 0.f;
                        if (inside && pG > 0.f && pG < 1.f) {
                            const float k = mixf(2.f * m.specular, 1.f, pG);
                            const float4 rp = rng.next();
                            if (rp.x < pG) { trans = 1.f; hz = 0.f; }
                            else {
                                trans = sat(sat(m.transmission) * sat(m.haze) / fmaxf(1.f - pG, 1e-6f));
                                hz = 1.f; specv = 0.5f * k; diffFace = true;
                            }
                        }
                        const float etaFace = diffFace ? fminf(n0, n1) / fmaxf(n0, n1) : n0 / n1;
                        Lobes lb = make_lobes(nrm, -dir, m, etaFace, a.tab, trans, specv, hz, n0, inside, lam0);
                        lb.etaT = n0 / nT;
                        coat_pick(lb, beta);
                        const LobeSample smp = lobes_sample(lb, a.tab, rng.next());
                        dir = smp.dir;
                        beta = beta * smp.w;
                        if (smp.transmitted) {
                            n = nT;
                            if (draw) { beta = beta * spec.w; lam = spec.lam; }
                            // the medium it is in now, the one beyond the face (tracebasics.js enterMedium)
                            const uint32_t med = (ids >> 16) != SURF_NONE ? (ids >> 16)
                                                                          : (inside ? 0u : (ids & 0xffffu));
                            if (a.u.scatter_on) m4.z = (m4.z & META_STEPS) | (min(med, 255u) << MEDIUM_SHIFT);
                        }
                        const f3 off = dir * otol;
                        pos = pos + off; ltot += length(off) * n;
                        // a delta event keeps it in the class (TAG_PASSED); anything else is its D: nothing more
                        // can store it, so it ends here (the reference's photon goes on for light tracing only)
                        bool alive = max3(smp.w) > 0.f && smp.ev == EV_DELTA && bounces <= u.maxbounce;
                        if (alive && u.rr != 0u && bounces >= 3u) {
                            const float p = clampf(max3(beta), 0.1f, 0.95f);
                            const float4 rr = rng.next();
                            if (rr.x > p) alive = false;
                            else beta = beta / p;
                        }
                        m4.y = meta_y(bounces, seg, RAY_ACTIVE) | (m4.y & ~META_LOW) | META_PASSED;
                        cont = alive && !last;
                    }
                }
            }
        }
        const uint32_t at = warp_append(&d->count, store);
        if (store) {
            if (at < d->cap) {
                const f3 pw = rad * beta;
                a.sp.pos[at] = make_float4(pos.x, pos.y, pos.z, 0.f);
                a.sp.power[at] = make_float4(pw.x, pw.y, pw.z, 0.f);
                a.sp.dir_oct[at] = oct_word(-dir);
                a.sp.nrm_oct[at] = oct_word(nrm);
                a.sp.flags[at] = (bounces + 1u) | (sub << SPPM_SUB_SHIFT);
                // teach the map: this cell paid (with light tracing on, its connections teach it instead)
                const uint32_t cell = __float_as_uint(a.pb.lprev[slot].x);
                if (!u.lt_on && cell < LT_CELLS) atomicAdd(&a.sp.lt_hit[cell], 1u);
            } else {
                atomicAdd(&d->dropped, 1u);
            }
        }
        if (u.lt_on) {
            // the connection: a shadow ray of its length (it arrives when ltot, started at minus that, reaches 0)
            const uint32_t cq = warp_append(&a.ctr->shadowCount[side], conn);
            if (conn) {
                if (cq < a.q.scap) {
                    a.q.s_org[side][cq] = f4(lc.org, -lc.len);
                    a.q.s_dir[side][cq] = make_float4(lc.dir.x, lc.dir.y, lc.dir.z, __uint_as_float(lc.pix));
                    a.q.s_rad[side][cq] = make_float4(lc.c.x, lc.c.y, lc.c.z, 1.f);
                    a.q.s_steps[side][cq] = SHADOW_FACE | SHADOW_CONN;
                } else {
                    atomicAdd(&a.ctr->shadowdrop, 1u);
                }
            }
        }
        const uint32_t rq = warp_append(outc, cont);
        if (cont) {
            a.pb.pos[slot] = f4(pos, ltot);
            a.pb.dir[slot] = f4(dir, n);
            a.pb.beta[slot] = make_float4(beta.x, beta.y, beta.z, 1.f);
            // a new leg: its collision drawn afresh, in the haze or a scattering material (a probe's is its chord, kept)
            if ((u.haze_on || u.scatter_on) && !(m4.y & META_PROBE)) a.pb.rad[slot].w = 0.f;
            a.pb.meta[slot] = m4;
            if (lam != 0.f) a.pb.lam[slot] = lam;
            outq[rq] = slot;
        }
    }
}

// THE GATHER (sppm.js:475-494 sppmGather, wavefront.js:1196-1212): a camera ray with delta events only since the
// eye (its lens field 1) -- or at the eye's first surface: the class light -> delta+ -> D -> eye, which the
// reference hands to its light tracer (CLS_CAND | CLS_SPEC) and this build, which has none, to the map -- on an
// evaluable surface facing it, takes sum f(l_p -> v) Phi_p / (pi r^2) over the records within r on a facing surface
// inside the bounce cap, over n^2, times its throughput, into its radiance; the eight cells, each cell's records
// whole within its share of the budget, else m of its sub-lists from a drawn start, each record found weighing 32 / m;
// a gather stops at the hard cap, counting the records in walk order.
//
// A query walks 9 to 10 records on average (up to the cap at a caustic's focus), so its time is memory latency: the
// eight cells' ranges, then the records. Here each lane sets up one query (its lobes, its cell coordinates) and loads
// its eight cells' ranges at once from the per-hash heads (4 MB, resident in L2); the warp then walks the records of
// all its queries whose cells are whole and within the cap as one list, 32 records a pass, each lane finding its
// record's query and cell in shared memory, the sums segmented by query across the lanes in a fixed order. A query
// with a cell past its share (sub-lists drawn, the cap possible) is walked by the whole warp in the reference's
// order, cell by cell: the cell's drawn sub-lists' ranges loaded at once, one a lane, and walked as one list.
struct GatherQuery {
    Lobes lb;
    f3 x, nrm;
    float scale;          // 1 / (pi r^2 n^2)
    uint32_t slot, my;    // the path's slot and meta word
    int32_t c0[3];
    uint32_t side;        // bit k: the neighbour along axis k is on the + side
    uint32_t a0[8];       // each cell's first record
    uint32_t pre[9];      // the records of the cells before each; pre[8] their total
    uint32_t pad;         // to an odd number of words
};
// an odd number of words, so lanes reading one field of 32 different queries meet 32 different banks
static_assert(sizeof(GatherQuery) % 8 == 4, "GatherQuery: an odd word stride");

__device__ __forceinline__ void gather_cell(const GatherQuery& g, uint32_t k, int32_t& cx, int32_t& cy, int32_t& cz) {
    cx = g.c0[0] + ((k & 1) ? ((g.side & 1) ? 1 : -1) : 0);
    cy = g.c0[1] + ((k & 2) ? ((g.side & 2) ? 1 : -1) : 0);
    cz = g.c0[2] + ((k & 4) ? ((g.side & 4) ? 1 : -1) : 0);
}
// one record's share f(l_p -> v) Phi_p, or 0 where it is of another cell with the hash, past r, past the bounce cap,
// or on a surface facing away (the radius and normal tests in IEEE f32, unfused, as the reference's)
__device__ __forceinline__ f3 gather_record(const WaveArgs& a, const GatherQuery& g, uint32_t rec, int32_t cx,
                                            int32_t cy, int32_t cz, float cellsz, float r2) {
    const float4 pp = a.sp.spos[rec];
    if (cell_of(pp.x, cellsz) != cx || cell_of(pp.y, cellsz) != cy || cell_of(pp.z, cellsz) != cz) return mk(0.f);
    const float dx = __fsub_rn(pp.x, g.x.x), dy = __fsub_rn(pp.y, g.x.y), dz = __fsub_rn(pp.z, g.x.z);
    const float dd = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    if (dd > r2) return mk(0.f);
    const uint32_t b = a.sp.sflags[rec];
    if (b & SPPM_VOL) return mk(0.f);                               // a record in a volume is the volume's gather's
    if ((g.my & 0xffu) + 1u + (b & SPPM_B_MASK) > a.u.maxbounce + 1u) return mk(0.f);
    const f3 pn = unoct(a.sp.snrm[rec]);
    const float nd = __fadd_rn(__fadd_rn(__fmul_rn(pn.x, g.nrm.x), __fmul_rn(pn.y, g.nrm.y)), __fmul_rn(pn.z, g.nrm.z));
    if (nd < SPPM_NORMAL_DOT) return mk(0.f);
    return lobes_eval(g.lb, a.tab, unoct(a.sp.sdir[rec]), LT_MIN_ALPHA) * xyz(a.sp.spow[rec]);
}
__device__ __forceinline__ void gather_add(const WaveArgs& a, uint32_t slot, f3 L) {
    if (luma(L) == 0.f) return;
    const float4 r4 = a.pb.rad[slot];
    const f3 b = xyz(a.pb.beta[slot]);
    a.pb.rad[slot] = make_float4(r4.x + b.x * L.x, r4.y + b.y * L.y, r4.z + b.z * L.z, r4.w);
}

__global__ void __launch_bounds__(256, 2) k_gather(WaveArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t qpre_all[8][33];
    __shared__ float acc_all[8][32][3];
    const Uni& u = a.u;
    st_material* sm = reinterpret_cast<st_material*>(smem);
    const uint32_t mat_bytes = u.n_mats * (uint32_t)sizeof(st_material);
    if (!stage_table(sm, a.mats, mat_bytes, &mbar, a.ctr)) return;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    GatherQuery* gq = reinterpret_cast<GatherQuery*>(smem + ((mat_bytes + 15u) & ~15u)) + warp * 32u;
    uint32_t* qpre = qpre_all[warp];
    float(*acc)[3] = acc_all[warp];
    const uint32_t count = a.ctr->hitCount;
    const SppmDev* d = a.sp.dev;
    const float cellsz = d->cell, r2 = d->r2, inv_area = d->inv_area;
    const uint32_t nrec = min(d->count, d->cap);
    if (nrec == 0u) return;
    const uint32_t share = max(1u, u.sppm_budget / 8u);
    const uint32_t hard = SPPM_VISIT_HARD * u.sppm_budget;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long walked = 0;
    uint32_t gathers = 0;
    for (uint32_t q0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32u; q0 < count; q0 += nwarps * 32u) {
        // 1. each lane's query: the eye's first surface, or delta events only since the eye (lens field 1), on an
        // evaluable surface that does not emit; its setup and its cells' ranges into shared memory
        const uint32_t q = q0 + lane;
        bool take = false, fast = false;
        uint32_t T = 0;
        if (q < count) {
            const uint32_t slot = a.q.hit[q];
            const uint32_t my = a.pb.meta[slot].y;
            const float4 sf = a.q.hsurf[q];
            const uint32_t ids = __float_as_uint(sf.w);
            // (at the eye's first surface too, unless light tracing runs: that class is its)
            if (((my >> 16) & 0xffu) == RAY_ACTIVE &&
                (((my & 0xffu) == 0u && !a.u.lt_on) || ((my >> META_LENS_SHIFT) & 3u) == 1u) &&
                ids != SURF_LEAVING) {
                const st_material& m = sm[ids & 0xffffu];
                take = fmaxf(fmaxf(m.emissive[0], m.emissive[1]), m.emissive[2]) <= 0.f && sppm_evaluable(m, true);
                if (take) {
                    GatherQuery& g = gq[lane];
                    const float dh = a.q.hitd[q];
                    const f3 nrm = dh < 0.f ? -xyz(sf) : xyz(sf);
                    const float4 p4 = a.pb.pos[slot], d4 = a.pb.dir[slot];
                    const f3 x = xyz(p4);
                    const float n0 = d4.w;
                    g.lb = make_lobes(nrm, -xyz(d4), m, n0 / fmaxf(m.ior, n0), a.tab, m.transmission, m.specular,
                                      m.haze, n0, false, a.pb.lam[slot]);
                    g.x = x;
                    g.nrm = nrm;
                    g.scale = inv_area / (n0 * n0);
                    g.slot = slot;
                    g.my = my;
                    const float gx[3] = {__fdiv_rn(x.x, cellsz), __fdiv_rn(x.y, cellsz), __fdiv_rn(x.z, cellsz)};
                    uint32_t side = 0;
                    int32_t c0[3];
                    for (int k = 0; k < 3; k++) {
                        c0[k] = (int32_t)floorf(gx[k]);
                        g.c0[k] = c0[k];
                        if (__fsub_rn(gx[k], floorf(gx[k])) >= 0.5f) side |= 1u << k;
                    }
                    g.side = side;
                    uint32_t a0[8], a1[8];
#pragma unroll
                    for (uint32_t k = 0; k < 8; k++) {
                        const int32_t cx = c0[0] + ((k & 1) ? ((side & 1) ? 1 : -1) : 0),
                                      cy = c0[1] + ((k & 2) ? ((side & 2) ? 1 : -1) : 0),
                                      cz = c0[2] + ((k & 4) ? ((side & 4) ? 1 : -1) : 0);
                        const uint32_t h = sppm_hash(cx, cy, cz);
                        a0[k] = __ldg(&a.sp.heads[h]);
                        a1[k] = __ldg(&a.sp.heads[h + 1]);
                    }
                    bool whole = true;
#pragma unroll
                    for (uint32_t k = 0; k < 8; k++) {
                        g.a0[k] = a0[k];
                        g.pre[k] = T;
                        whole = whole && a1[k] - a0[k] <= share;
                        T += a1[k] - a0[k];
                    }
                    g.pre[8] = T;
                    fast = whole && T <= hard;
                }
            }
        }
        const uint32_t taken = __ballot_sync(FULL_MASK, take);
        const uint32_t slow = __ballot_sync(FULL_MASK, take && !fast);
        gathers += __popc(taken);
        // 2. the whole-cell queries' records as one list over the lanes: each query's first item, their total
        const uint32_t t = fast ? T : 0u;
        uint32_t incl = t;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(FULL_MASK, incl, o);
            if ((int)lane >= o) incl += v;
        }
        qpre[lane] = incl - t;
        if (lane == 31u) qpre[32] = incl;
        acc[lane][0] = acc[lane][1] = acc[lane][2] = 0.f;
        walked += t;
        __syncwarp();
        const uint32_t total = qpre[32];
        for (uint32_t base = 0; base < total; base += 32u) {
            const uint32_t i = base + lane;
            uint32_t s = 32u;                                   // no query: past the list's end
            f3 v = mk(0.f);
            if (i < total) {
                // the item's query: the last whose first item is at or before it (the ones with none are passed)
                s = 0;
#pragma unroll
                for (uint32_t st = 16; st > 0; st >>= 1)
                    if (qpre[s + st] <= i) s += st;
                const GatherQuery& g = gq[s];
                const uint32_t r = i - qpre[s];
                uint32_t k = 0;
#pragma unroll
                for (uint32_t st = 4; st > 0; st >>= 1)
                    if (g.pre[k + st] <= r) k += st;
                int32_t cx, cy, cz;
                gather_cell(g, k, cx, cy, cz);
                v = gather_record(a, g, g.a0[k] + (r - g.pre[k]), cx, cy, cz, cellsz, r2);
            }
            // the sums segmented by query (the items lie in query order), each segment's added by its last lane
            for (int o = 1; o < 32; o <<= 1) {
                const float vx = __shfl_up_sync(FULL_MASK, v.x, o), vy = __shfl_up_sync(FULL_MASK, v.y, o),
                            vz = __shfl_up_sync(FULL_MASK, v.z, o);
                const uint32_t so = __shfl_up_sync(FULL_MASK, s, o);
                if ((int)lane >= o && so == s) { v.x += vx; v.y += vy; v.z += vz; }
            }
            const uint32_t sn = __shfl_down_sync(FULL_MASK, s, 1);
            if (s < 32u && (lane == 31u || sn != s)) {
                acc[s][0] += v.x;
                acc[s][1] += v.y;
                acc[s][2] += v.z;
            }
            __syncwarp();
        }
        if (fast && T > 0u) gather_add(a, gq[lane].slot, mk(acc[lane][0], acc[lane][1], acc[lane][2]) * gq[lane].scale);
        // 3. the others, one at a time by the whole warp, in the reference's order: per cell, its whole range on lane
        // 0 or its drawn sub-lists' ranges on lanes 0..m-1 (loaded at once), walked as one list 32 records a pass
        for (uint32_t todo = slow; todo != 0u; todo &= todo - 1u) {
            const GatherQuery& g = gq[__ffs(todo) - 1];
            const uint32_t tile = g.slot % u.P, j = slot_sample(u, g.slot), seg = (g.my >> 8) & 0xffu;
            Rng rng = path_rng(sample_seed(u.seed, a.ctr->sample + j), tile, SPPM_STORE_SALT + seg);
            f3 sum = mk(0.f);
            uint32_t visits = 0;
            for (uint32_t k = 0; k < 8; k++) {
                int32_t cx, cy, cz;
                gather_cell(g, k, cx, cy, cz);
                const uint32_t h = sppm_hash(cx, cy, cz);
                const uint32_t a0 = g.a0[k], cnt = g.pre[k + 1] - g.pre[k];
                const bool whole = cnt <= share;
                const uint32_t subs = whole ? 1u : max(1u, (SPPM_SUBS * share) / max(cnt, 1u));
                const float w = whole ? 1.f : (float)SPPM_SUBS / (float)subs;
                const float4 rk = rng.next();
                const uint32_t st0 = min((uint32_t)(rk.x * (float)SPPM_SUBS), SPPM_SUBS - 1);
                uint32_t lo = 0, len = 0;
                if (whole) {
                    if (lane == 0u) { lo = a0; len = cnt; }
                } else if (lane < subs) {
                    const uint32_t sl = (st0 + lane) % SPPM_SUBS;
                    lo = __ldg(&a.sp.start[h * SPPM_SUBS + sl]);
                    len = __ldg(&a.sp.start[h * SPPM_SUBS + sl + 1]) - lo;
                }
                uint32_t incl = len;
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t v = __shfl_up_sync(FULL_MASK, incl, o);
                    if ((int)lane >= o) incl += v;
                }
                const uint32_t off = incl - len;
                uint32_t n = __shfl_sync(FULL_MASK, incl, 31);
                // the hard cap, in walk order: the records past it are not met, nor the cells after
                const bool cut = visits + n > hard;
                if (cut) n = hard - visits;
                visits += n;
                for (uint32_t base = 0; base < n; base += 32u) {
                    const uint32_t i = base + lane;
                    // the lane whose range holds item i: the last whose offset is at or before it
                    uint32_t src = 0;
#pragma unroll
                    for (uint32_t st = 16; st > 0; st >>= 1)
                        if (__shfl_sync(FULL_MASK, off, src + st) <= i) src += st;
                    const uint32_t lo_s = __shfl_sync(FULL_MASK, lo, src), off_s = __shfl_sync(FULL_MASK, off, src);
                    if (i < n) sum = sum + gather_record(a, g, lo_s + (i - off_s), cx, cy, cz, cellsz, r2) * w;
                }
                if (cut) break;
            }
            for (int o = 16; o > 0; o >>= 1) {
                sum.x += __shfl_xor_sync(FULL_MASK, sum.x, o);
                sum.y += __shfl_xor_sync(FULL_MASK, sum.y, o);
                sum.z += __shfl_xor_sync(FULL_MASK, sum.z, o);
            }
            if (lane == 0u) {
                gather_add(a, g.slot, sum * g.scale);
                walked += visits;
            }
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) walked += __shfl_down_sync(FULL_MASK, walked, o);
    if (lane == 0u && walked) atomicAdd(&a.sp.dev->visits, walked);
    if (lane == 0u && gathers) atomicAdd(&a.sp.dev->gathers, gathers);
}

cudaError_t launch_sppm_begin(const WaveArgs& a, cudaStream_t s) {
    k_sppm_begin<<<1, 32, 0, s>>>(a.sp.dev, a.ctr, a.u.sppm_r1, a.u.sppm_alpha, a.sp.cap, a.u.sppm_r1v);
    return cudaGetLastError();
}
cudaError_t launch_lt_build(const WaveArgs& a, cudaStream_t s) {
    k_lt_build<<<1, LT_GRID, 0, s>>>(a.sp, a.ctr);
    return cudaGetLastError();
}
cudaError_t launch_genphotons(const WaveArgs& a, uint32_t first, uint32_t n, int sms, cudaStream_t s) {
    k_genphotons<<<std::min((n + 255u) / 256u, (uint32_t)sms * 8u), 256, 0, s>>>(a, first, n);
    return cudaGetLastError();
}
cudaError_t launch_photon_shade(const WaveArgs& a, int nxt, int last, int side, int sms, cudaStream_t s) {
    const size_t smem = a.u.n_mats * sizeof(st_material);
    k_photon_shade<<<sms * 4, 256, smem, s>>>(a, nxt, last, side);
    return cudaGetLastError();
}
cudaError_t launch_gather(const WaveArgs& a, int sms, cudaStream_t s) {
    const size_t smem = ((a.u.n_mats * sizeof(st_material) + 15) & ~(size_t)15) + 256 * sizeof(GatherQuery);
    cudaFuncSetAttribute(k_gather, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gather, 256, smem);
    k_gather<<<sms * (nb > 0 ? nb : 1), 256, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace st
