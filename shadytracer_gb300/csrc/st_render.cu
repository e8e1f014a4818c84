// st_render.cu -- the wavefront kernels of the rendering hot path, for sm_103a.
//
//   k_mf_lut, k_mf_avg   the GGX albedo tables, once at init            core/microfacet.js:245-330
//   k_genrays            one camera ray per path of the wave             core/genrays.js:36-107
//   k_iter_begin         a wavefront iteration's counters                core/wavefront.js:333-387 (prog_flip)
//   k_march              sphere tracing, persistent with refill          core/wavefront.js:834-1005 (prog_march)
//   k_shade              surface answers + BSDF + light sample + deposit core/wavefront.js:1037-1147 (prog_surface),
//                                                                        :1244-1442 (prog_shade)
//   k_occlude            shadow rays, persistent with refill             core/wavefront.js:1481-1692 (prog_occlude)
//   k_resolve            the sample into the FP64 mean and error bar     core/wavefront.js:414-494 (prog_resolve)
//
// GB300 shape of it. The path state lives in HBM by slot as structure-of-arrays float4s; the queues hold slots,
// appended with one atomic per warp (ballot + popc). The march and the occlusion pass are persistent: a grid of a
// few CTAs per SM whose warps claim the queue 64 entries at a time and refill a lane the moment its ray ends, so a
// warp keeps 32 rays in flight however uneven their step counts. The scene's primitive table is staged into
// shared memory by one bulk copy (cp.async.bulk + mbarrier) per CTA and read as broadcasts. Nothing is read back
// by the host inside a sample: every kernel sizes itself from the device counters.
#include "st_emit.cuh"
#include "st_light.cuh"
#include "st_guide.cuh"
#include "st_kernels.cuh"
#include "st_scene_kernels.cuh"

namespace st {


// ------------------------------------------------------------------------------------------------------------
// THE ALBEDO TABLES (microfacet.js:245-330), the isotropic part: one thread per entry, a 32 x 32 stratified grid
// warped toward the visible cap's rim.
// ------------------------------------------------------------------------------------------------------------
__global__ void k_mf_lut(float* ec, float* e1) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t NEC = MF_NIOR * MF_NR * MF_NMU, NE1 = MF_NR * MF_NMU;
    if (e >= NEC + NE1) return;
    float ior = 1.f;
    uint32_t k, j;
    bool isE1 = false;
    if (e < NEC) {
        ior = 1.f + 2.f * float(e / (MF_NR * MF_NMU)) / float(MF_NIOR - 1);
        k = (e / MF_NMU) % MF_NR; j = e % MF_NMU;
    } else {
        uint32_t t = e - NEC;
        isE1 = true; k = t / MF_NMU; j = t % MF_NMU;
    }
    float r = float(k) / float(MF_NR - 1);
    float mu = (float(j) + 0.5f) / float(MF_NMU);
    float st = sqrtf(fmaxf(0.f, 1.f - mu * mu));
    float a = fmaxf(r * r, MF_ALPHA_MIN);
    f3 o = mk(st, 0.f, mu);
    float acc = 0.f;
    for (int sy = 0; sy < 32; sy++)
        for (int sx = 0; sx < 32; sx++) {
            float vx = (float(sx) + 0.5f) / 32.f, vy = (float(sy) + 0.5f) / 32.f;
            float ux = vx, uy = 1.f - (1.f - vy) * (1.f - vy);
            f3 h = mf_sample_vndf(o, a, ux, uy);
            f3 i3 = reflectv(-o, h);
            if (i3.z > 0.f) {
                float fr = isE1 ? 1.f : fresnel_dielectric(dot(o, h), 1.f / ior);
                acc += 2.f * (1.f - vy) * fr * mf_g2(o, i3, a) / mf_g1(o, a);
            }
        }
    acc = acc / 1024.f;
    if (e < NEC) ec[e] = acc; else e1[e - NEC] = acc;
}
__global__ void k_mf_avg(const float* ec, float* ecavg) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= MF_NIOR * MF_NR) return;
    float acc = 0.f;
    for (int j = 0; j < MF_NMU; j++) {
        float mu = (float(j) + 0.5f) / float(MF_NMU);
        acc += 2.f * ec[e * MF_NMU + j] * mu / float(MF_NMU);
    }
    ecavg[e] = acc;
}

// ------------------------------------------------------------------------------------------------------------
// GENRAYS (genrays.js:36-107): slot i is path (tile = i mod P) of sample (first + i / P)
// ------------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_genrays(WaveArgs a) {
    const Uni& u = a.u;
    const uint32_t first = a.ctr->sample;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.slots; i += gridDim.x * blockDim.x) {
        uint32_t tile = i % u.P, j = slot_sample(u, i);
        // the slot's camera: its view's (many views in the wave), else the one
        f3 ucam = u.cam, uright = u.right, uup = u.up, ufwd = u.fwd;
        float ufx = u.fx, ufy = u.fy, ulens_r = u.lens_r, ulens_f = u.lens_f;
        uint32_t ucamtype = u.camtype;
        if (u.views) {
            const float4* vw = u.views + (size_t)slot_view(u, i) * VIEW_F4;
            const float4 v0 = vw[0], v1 = vw[1], v2 = vw[2], v3 = vw[3], v4 = vw[4];
            ucam = xyz(v0); ucamtype = __float_as_uint(v0.w);
            uright = xyz(v1); ufx = v1.w;
            uup = xyz(v2); ufy = v2.w;
            ufwd = xyz(v3); ulens_r = v3.w;
            ulens_f = v4.x;
        }
        Rng rng = path_rng(sample_seed(u.seed, first + j), tile, 0);
        float cx = float(tile % u.tilesX), cy = float(tile / u.tilesX);
        float uv0x = (cx + 0.5f) * u.invTX, uv0y = (cy + 0.5f) * u.invTY;
        float4 rnd = rng.next();
        float ux = clampf(uv0x + (rnd.x - 0.5f) * u.invTX, 0.f, 1.f);
        float uy = clampf(uv0y + (rnd.y - 0.5f) * u.invTY, 0.f, 1.f);
        float xx = ux * 2.f - 1.f, yy = uy * 2.f - 1.f;
        f3 pos, dir;
        if (ucamtype == 0) {
            f3 dc = mk(xx * ufx, yy * ufy, -1.f);
            dir = normalize(uright * dc.x + uup * dc.y + ufwd * dc.z);
            pos = ucam;
            // THROUGH THE LENS (genrays.js:80-87, lens.js lensDisc): from a point of its disc (the same draw's zw),
            // at the point the pinhole's ray meets the focus plane
            if (ulens_r > 0.f) {
                const float r = ulens_r * sqrtf(rnd.z);
                float sp, cp;
                sincosf(6.28318530718f * rnd.w, &sp, &cp);
                const f3 off = uright * (r * cp) + uup * (r * sp);
                pos = ucam + off;
                dir = normalize((uright * dc.x + uup * dc.y + ufwd * dc.z) * ulens_f - off);
            }
        } else {
            pos = ucam + uright * (xx * ufx) + uup * (yy * ufy);
            dir = -ufwd;
        }
        dir = normalize(dir);
        float px = clampf(ux * float(u.W), 0.f, float(u.W) - 1.f), py = clampf(uy * float(u.H), 0.f, float(u.H) - 1.f);
        uint32_t pix = (uint32_t)px + (uint32_t)py * u.W;
        a.pb.pos[i] = make_float4(pos.x, pos.y, pos.z, 0.f);
        a.pb.dir[i] = make_float4(dir.x, dir.y, dir.z, 1.f);
        a.pb.beta[i] = make_float4(1.f, 1.f, 1.f, 1.f);
        a.pb.rad[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.pb.meta[i] = make_uint4(pix, RAY_ACTIVE << 16, 0u, __float_as_uint(0.f));
        a.pb.lam[i] = 0.f;
        if (a.em.w) a.em.w[i] = 1.f;                                  // a camera ray: no light sample to weigh against
        a.q.ray[0][i] = i;
    }
}

// a wavefront iteration's start: the queues it fills emptied (prog_flip, wavefront.js:368-387)
__global__ void k_iter_begin(DevCtr* ctr, int it, int nxt, uint32_t slots, int first) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (first) { ctr->rayCount[0] = slots; ctr->shadowCount[0] = 0u; }
        ctr->rayCount[nxt] = 0u;
        ctr->hitCount = 0u;
        ctr->shadowCount[(it + 1) & 1] = 0u;
        ctr->marchHead = 0u;
        ctr->occHead = 0u;
        ctr->emitHits = 0u;
    }
}

// ------------------------------------------------------------------------------------------------------------
// THE MARCH (wavefront.js:866-947), persistent. Each warp claims CLAIM queue entries at a time; a lane whose ray
// ended takes the next one at once. A step: the scene's distance, the hit test against marchTol, lmax and
// maxiter, the escape test; then the step of ea * stepscale. On the haze's collision (haze.js:280-288) the ray is
// moved back to it and handed to shade as RAY_SCATTER. A ray still marching after MARCH_CHUNK evaluations goes on
// in the next iteration (the reference's 32-step dispatches, wavefront.js:870); the last iteration's launch
// marches every ray to its end.
// ------------------------------------------------------------------------------------------------------------
// ------------------------------------------------------------------------------------------------------------
// THE MARCH QUEUE IN SPACE ORDER. The fold skips a primitive by its bounding sphere per lane, but a warp issues a
// primitive's evaluation whenever any of its 32 rays needs it, so rays far apart in one warp pay for the union of
// their neighbourhoods. Before each march the queue is put in the order of a counting sort on (cell of a
// SORT_G^3 grid over the primitives' bounds, direction octant): one atomic per ray for its rank in its bucket, a
// one-block scan of the buckets, a scatter. Each ray's answer is its own (its random numbers come from its path),
// so the order changes only which rays share a warp.
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t sort_bucket(f3 glo, f3 ginv, f3 p, f3 d) {
    const float fx = (p.x - glo.x) * ginv.x, fy = (p.y - glo.y) * ginv.y, fz = (p.z - glo.z) * ginv.z;
    const uint32_t ix = (uint32_t)fminf(fmaxf(fx, 0.f), (float)(SORT_G - 1));
    const uint32_t iy = (uint32_t)fminf(fmaxf(fy, 0.f), (float)(SORT_G - 1));
    const uint32_t iz = (uint32_t)fminf(fmaxf(fz, 0.f), (float)(SORT_G - 1));
    const uint32_t oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
    return ((iz * SORT_G + iy) * SORT_G + ix) * 8u + oct;
}
// each entry's bucket and rank: entry i is the ray at pos / dir [inq ? inq[i] : i]. The lanes of a warp that share
// a bucket take their ranks with one atomic (coherent rays share buckets, and one counter taking a million atomics
// one at a time serialises the launch), in lane order, so the queue's order survives within a bucket.
__global__ void __launch_bounds__(256) k_sort_key(const uint32_t* __restrict__ countp, uint32_t cap,
                                                  const uint32_t* __restrict__ inq, const float4* __restrict__ pos,
                                                  const float4* __restrict__ dir, f3 glo, f3 ginv,
                                                  uint32_t* __restrict__ key, uint32_t* __restrict__ rank,
                                                  uint32_t* __restrict__ bcnt) {
    const uint32_t count = min(*countp, cap);
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < count; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + lane;
        const bool ok = i < count;
        uint32_t b = 0xffffffffu;
        if (ok) {
            const uint32_t at = inq ? inq[i] : i;
            b = sort_bucket(glo, ginv, xyz(pos[at]), xyz(dir[at]));
            key[i] = b;
        }
        const uint32_t peers = __match_any_sync(FULL_MASK, b);
        const uint32_t leader = (uint32_t)__ffs(peers) - 1u;
        uint32_t base = 0;
        if (ok && lane == leader) base = atomicAdd(&bcnt[b], (uint32_t)__popc(peers));
        base = __shfl_sync(FULL_MASK, base, leader);
        if (ok) rank[i] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    }
}
__global__ void __launch_bounds__(1024) k_sort_scan(uint32_t* __restrict__ cnt, uint32_t* __restrict__ off) {
    constexpr uint32_t PER = SORT_BUCKETS / 1024u;
    __shared__ uint32_t wsum[32];
    uint32_t v[PER];
    uint4* c4 = reinterpret_cast<uint4*>(cnt + threadIdx.x * PER);
    uint32_t t = 0;
#pragma unroll
    for (uint32_t k = 0; k < PER / 4; k++) {
        uint4 q = c4[k];
        v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
        t += q.x + q.y + q.z + q.w;
        c4[k] = make_uint4(0u, 0u, 0u, 0u);
    }
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t incl = t;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31u) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t x = wsum[lane], xi = x;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(FULL_MASK, xi, o);
            if (lane >= (uint32_t)o) xi += y;
        }
        wsum[lane] = xi - x;
    }
    __syncthreads();
    uint32_t run = wsum[w] + incl - t;
    uint4* o4 = reinterpret_cast<uint4*>(off + threadIdx.x * PER);
#pragma unroll
    for (uint32_t k = 0; k < PER / 4; k++) {
        uint4 q;
        q.x = run; run += v[4 * k];
        q.y = run; run += v[4 * k + 1];
        q.z = run; run += v[4 * k + 2];
        q.w = run; run += v[4 * k + 3];
        o4[k] = q;
    }
}
__global__ void __launch_bounds__(256) k_sort_scatter(const uint32_t* __restrict__ countp, uint32_t cap,
                                                      const uint32_t* __restrict__ inq,
                                                      const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
                                                      const uint32_t* __restrict__ boff, uint32_t* __restrict__ out) {
    const uint32_t count = min(*countp, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[boff[key[i]] + rank[i]] = inq ? inq[i] : i;
}


// ------------------------------------------------------------------------------------------------------------
// SHADE: what prog_surface asks the scene (the normal by three forward differences at normalTol, the material, the
// medium beyond) and what prog_shade does with it (pathBegin..pathEnd, processMaterial_advanced's light sample and
// lobe draw, the MIS weights, the bounce cap and roulette); an escaped ray's environment; a point in the haze
// (haze.js:493-596 mediumVertex); the deposit of a path that ends. One thread per shade-queue entry.
// ------------------------------------------------------------------------------------------------------------
struct ShadowOut { bool valid, emit, face; f3 org, dir, rad; float n, dist; };

// THE GATHER IN A VOLUME (sppm.js:497-511 sppmGatherVolume through sppmWalk :305-360): at a camera ray's collision in a
// scattering material, the records photons stored at their own collisions (SPPM_VOL) within R in the eight cells of
// the volume's grid round x, each through the phase function from the way it came to the way to the camera,
// sum p(l . v) Phi / (sigma 4/3 pi R^3); a cell's records whole while their count is within its share of the budget,
// else m of its sub-lists from a drawn start, each record then weighing 32 / m; the walk cut at the hard cap.
#define SPPM_GATHER_SALT 0x53505031u            // the map's own stream (wavefront.js:1186): shade's draws do not move
__device__ __forceinline__ f3 volume_gather(const WaveArgs& a, f3 x, f3 v, uint32_t bc, float g, float sigma, Rng& rng) {
    const SppmDev* d = a.sp.dev;
    const uint32_t nrec = min(d->count, d->cap);
    if (nrec == 0u || !(sigma > 0.f)) return mk(0.f);
    const float csz = d->vcell, r2 = d->vr2;
    const float gx[3] = {__fdiv_rn(x.x, csz), __fdiv_rn(x.y, csz), __fdiv_rn(x.z, csz)};
    int32_t c0[3], sd[3];
    for (int k = 0; k < 3; k++) {
        c0[k] = (int32_t)floorf(gx[k]);
        sd[k] = __fsub_rn(gx[k], floorf(gx[k])) >= 0.5f ? 1 : -1;
    }
    const uint32_t budget = a.u.sppm_budget, share = max(1u, budget / 8u), hard = SPPM_VISIT_HARD * budget;
    f3 sum = mk(0.f);
    uint32_t visits = 0;
    bool cut = false;
    for (uint32_t k = 0; k < 8u && !cut; k++) {
        const int32_t cx = c0[0] + ((k & 1u) ? sd[0] : 0), cy = c0[1] + ((k & 2u) ? sd[1] : 0),
                      cz = c0[2] + ((k & 4u) ? sd[2] : 0);
        const uint32_t h = sppm_hash(cx, cy, cz);
        const uint32_t a0 = __ldg(&a.sp.heads[h]), a1 = __ldg(&a.sp.heads[h + 1u]), cnt = a1 - a0;
        const bool whole = cnt <= share;
        const uint32_t subs = whole ? 1u : max(1u, (SPPM_SUBS * share) / max(cnt, 1u));
        const float w = whole ? 1.f : (float)SPPM_SUBS / (float)subs;
        const uint32_t start = min((uint32_t)(rng.next().x * (float)SPPM_SUBS), SPPM_SUBS - 1u);
        for (uint32_t j = 0; j < subs && !cut; j++) {
            const uint32_t s = (start + j) % SPPM_SUBS;
            const uint32_t lo = whole ? a0 : __ldg(&a.sp.start[h * SPPM_SUBS + s]);
            const uint32_t hi = whole ? a1 : __ldg(&a.sp.start[h * SPPM_SUBS + s + 1u]);
            for (uint32_t q = lo; q < hi; q++) {
                if (visits >= hard) { cut = true; break; }
                visits++;
                const uint32_t b = a.sp.sflags[q];
                if (!(b & SPPM_VOL) || bc + (b & SPPM_B_MASK) > a.u.maxbounce + 1u) continue;
                const float4 pp = a.sp.spos[q];
                if (cell_of(pp.x, csz) != cx || cell_of(pp.y, csz) != cy || cell_of(pp.z, csz) != cz) continue;
                const float dx = __fsub_rn(pp.x, x.x), dy = __fsub_rn(pp.y, x.y), dz = __fsub_rn(pp.z, x.z);
                if (__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)) > r2) continue;
                sum = sum + xyz(a.sp.spow[q]) * (w * hg_eval(dot(unoct(a.sp.sdir[q]), v), g));
            }
        }
    }
    return sum * (d->inv_vol / sigma);
}

template <bool GUIDE>
__device__ __forceinline__ void shade_surface(const WaveArgs& a, const st_material* sm, float4 surf,
                                              f3& pos, f3& dir, float& ltot, float& n, f3& beta, float& sunmis,
                                              f3& rad, uint32_t& bounces, uint32_t& state, float& lam,
                                              uint32_t& lens, float dh, Rng& rng, bool last, ShadowOut& sh,
                                              uint32_t q, uint32_t& my, uint32_t gpix, float& emw, float2& lp,
                                              float& absL, uint32_t& mz) {
    const Uni& u = a.u;
    float eps = march_tol(pos, u.tol);
    const uint32_t ids = __float_as_uint(surf.w);
    f3 nn = xyz(surf);                                                // k_surface: the normal, the material
    bool inside = dh < 0.f;
    f3 nrm = inside ? -nn : nn;                                       // pathFacing (scene_api.js:127-135)
    float otol = 10.f * eps;                                          // offsetTol
    if (ids == SURF_LEAVING) {                                        // leaving: moved on along its way, no bounce
        f3 off = dir * otol;
        pos = pos + off; ltot += length(off) * n;
        return;
    }
    bounces += 1;
    const st_material& m = sm[ids & 0xffffu];
    // ABSORPTION INSIDE (tracebasics.js absorbAlong; materials.js:125-133 mediumMu): a ray met from inside crossed this
    // material's volume from where it arrived last (absL): exp(-mu d) a channel, mu = -ln(base) / attenuationDistance
    if (inside && m.attenuation > 0.f) {
        const float d = fmaxf(ltot - absL, 0.f) / fmaxf(n, 1e-4f);
        const float ia = 1.f / m.attenuation;
        beta = beta * mk(__expf(logf(fminf(fmaxf(m.base[0], 1e-6f), 1.f)) * ia * d),
                         __expf(logf(fminf(fmaxf(m.base[1], 1e-6f), 1.f)) * ia * d),
                         __expf(logf(fminf(fmaxf(m.base[2], 1e-6f), 1.f)) * ia * d));
    }
    absL = ltot;                                                      // absorbAlong: arrival here
    const uint32_t fid = a.lf.n ? (uint32_t)a.lf.of[ids & 0xffu] : 0u;
    if (fid) {                                                        // a light's face (codegen LIGHTS)
        // its luminance at this angle from its own normal over n^2 of the medium met in, weighed past the first
        // surface against the faces' light sample the last vertex could have drawn this point with (:826-834)
        const Face f = face_at(a.lf, fid - 1u);
        const float cosY = -dot(dir, f.n);
        float w = 1.f;
        if (bounces >= 2u && lp.x >= 0.f) {
            const float pl = face_density(FACE_SHARE, a.lf.n, f, fmaxf(ltot - lp.y, 0.f) / fmaxf(n, 1e-4f), cosY);
            const float a2 = lp.x * lp.x;
            w = a2 / fmaxf(a2 + pl * pl, 1e-20f);
        }
        rad = rad + beta * f.le * (face_beam(f, cosY) / fmaxf(n * n, 1.f) * w);
        state = RAY_SOURCE;
        f3 off = dir * (otol * 2.f);
        pos = pos + off; ltot += length(off) * n;
        return;
    }
    f3 emis = mk(m.emissive[0], m.emissive[1], m.emissive[2]);
    if (max3(emis) > 0.f) {                                           // emitterHit (materials_pbr.js:1014-1075)
        // weighed against the light sample the last vertex could have drawn this direction with (emw, set there),
        // and discovered: its place and brightness into the emitter grid. A path in light tracing's class (or the
        // map's) leaves it to the emitter photons where a probe could have started one (materials_pbr.js:1044-1047)
        float w = emw;
        if (u.lt_emit_n && ((my & (META_CAND | META_SPEC)) == (META_CAND | META_SPEC) || (u.sppm_on && lens == 3u)) &&
            emit_covers(a.em.dev, pos))
            w = 0.f;
        rad = rad + beta * emis * (w * emit_beam(m.beam_cos, -dot(dir, nn)));
        if (a.em.on) emit_deposit(a.em, pos, emis);
        state = RAY_SOURCE;
        f3 off = dir * (otol * 2.f);
        pos = pos + off; ltot += length(off) * n;
        return;
    }
    float n0 = n;
    float n1d = fmaxf(m.ior, n0), v1 = 0.f;                           // ownMedium
    if ((ids >> 16) != SURF_NONE) {                                   // asksMedium -> mediumBeyond: index, Abbe
        n1d = sm[ids >> 16].ior;
        v1 = sm[ids >> 16].abbe;
    }
    // DISPERSION (materials_pbr.js:1116-1139): a ray with a wavelength meets the medium beyond at n(its wavelength);
    // one without, at a dispersive medium, draws one (the camera's table), used only if it refracts -- the reflect-
    // or-refract pick and its Fresnel stay the d line's
    const float lam0 = lam;
    const float n1 = lam0 > 0.f ? cauchy_n(n1d, v1, lam0) : n1d;
    const bool draw = v1 > 0.f && lam0 == 0.f;
    SpecDraw spec;
    float nT = n1;
    if (draw) {
        float4 r4 = rng.next();
        spec = spec_draw(a.spec, r4.x);
        spec.lam = lambda_coded(spec.lam);
        nT = cauchy_n(n1d, v1, spec.lam);
    }
    // a face that both refracts and diffuses, seen from inside (materials_pbr.js:1141-1165): the area mix, one part
    // drawn -- clear glass with the share that refracts, else the diffuse face, the same surface from either side
    const float pG = refract_share_of(m.transmission, m.haze);
    float trans = m.transmission, specv = m.specular, hz = m.haze;
    bool diffFace = pG <= 0.f && m.transmission > 0.f;               // haze 1: the diffuse face alone
    if (inside && pG > 0.f && pG < 1.f) {
        float k = mixf(2.f * m.specular, 1.f, pG);
        float4 r4 = rng.next();
        if (r4.x < pG) { trans = 1.f; hz = 0.f; }
        else { trans = sat(sat(m.transmission) * sat(m.haze) / fmaxf(1.f - pG, 1e-6f)); hz = 1.f; specv = 0.5f * k; diffFace = true; }
    }
    float etaFace = diffFace ? fminf(n0, n1) / fmaxf(n0, n1) : n0 / n1;
    Lobes lb = make_lobes(nrm, -dir, m, etaFace, a.tab, trans, specv, hz, n0, inside, lam0);
    lb.etaT = n0 / nT;
    coat_pick(lb, beta);
    // THE SIDE BEYOND, LIT (materials_pbr.js:1176-1190): light sampling may aim through this face where what it
    // transmits by can be evaluated and the medium beyond is air; the sky's cosine draw then comes from the far side
    const bool throughLit = fabsf(n1 - 1.f) <= 1e-3f && through_evaluable(m, trans, hz);
    lb.through = throughLit;
    const float qf = throughLit ? 1.f : 0.f;
    // THE LEARNED PROPOSAL (st_guide.cuh): at an evaluable opaque vertex met from outside, the direction is drawn from
    // the network's mixture with probability alpha, else from the BSDF, and weighed by f cos / (alpha q + (1 - alpha)
    // p_bsdf) -- one-sample MIS, so the estimator stays unbiased whatever the network says; the environment's MIS
    // weights take the same combined density on both sides
    const uint32_t gpx = GUIDE ? guide_pixel(u, gpix, gpix % u.P) : 0u;
    const bool guided = GUIDE && a.gd.on != 0u && !last && !inside && bounces == 1u && guide_vertex(m) &&
                        a.gd.stamp[gpx] != 0u;                        // (its pixel's mixture inferred this wave)
    const uint2* __restrict__ gmix = a.gd.mix + (size_t)gpx * GUIDE_LOBES;
    const float galpha = guided ? guide_share(a.gd.alpha, &a.gd.dev->step, a.gd.train) : 0.f;
    // the discovered emitters' share of the light samples (materials_pbr.js:1216-1330): 0 while nothing is listed,
    // when the environment's draw is the one it always was
    const float es = (a.em.on && u.nee != 0u && !last) ? emit_share(a.em) : 0.f;
    // ...and before them the lights' faces' (lightFaceShare): half the samples when there are faces
    const float fs = (a.lf.n && u.nee != 0u && !last) ? FACE_SHARE : 0.f;
    const float rs = 1.f - fs;                                        // the rest's: emitters, then the environment
    if (u.nee != 0u && !last) {                                       // light sampling (materials_pbr.js:1196-1330)
        float4 u0 = rng.next();
        float4 u1 = rng.next();
        if (!lobes_none(m, trans, hz)) {
            f3 L = mk(0.f, 0.f, 1.f);
            float pS = 0.f, fdist = 0.f;
            bool toEmit = false, toFace = false;
            f3 fle = mk(0.f);
            const float pick0 = (u0.x - fs) / fmaxf(rs, 1e-6f);      // the rest's own draw, when it is theirs
            if (u0.x < fs) {                                          // a face: one of them, a point uniform on it
                const Face f = face_at(a.lf, min((uint32_t)(u0.y * (float)a.lf.n), a.lf.n - 1u));
                const f3 dy = face_point(f, u1.x, u1.y) - pos;
                fdist = length(dy);
                L = dy * (1.f / fmaxf(fdist, 1e-20f));
                const float cosY = -dot(f.n, L);
                if (fdist > 0.f && cosY > 1e-6f) {
                    pS = face_density(fs, a.lf.n, f, fdist, cosY);
                    const float nSide = dot(nrm, L) < 0.f ? n1 : n;   // the far side's is air
                    fle = f.le * (face_beam(f, cosY) / fmaxf(nSide * nSide, 1.f));
                    toFace = true;
                }
            } else if (pick0 < es) {                                  // an emitter: a box, a direction into its cone
                const uint32_t b = emit_pick(a.em.dev, pick0 / es);
                if (emit_sample(a.em.dev, b, pos, u1.x, u1.y, L)) {
                    pS = rs * es * emit_cone_pdf(a.em.dev, pos, L);   // the whole mixture's density, not the box's
                    toEmit = true;
                }
            } else {                                                  // the environment: sun disc or sky
                L = env_sample_dir_q(u, nrm, es > 0.f ? (pick0 - es) / (1.f - es) : pick0, u1.x, u1.y, qf);
                pS = rs * (1.f - es) * env_pdf_q(u, L, nrm, qf);
            }
            float NoL = dot(nrm, L);
            if ((NoL > 0.f || (throughLit && NoL < 0.f)) && pS > 0.f) {  // sideLit
                // an emitter's radiance is the occlusion pass's to multiply in, where its ray stops
                f3 le = toEmit ? mk(1.f) : (toFace ? fle : env_radiance(u, L));
                f3 f = lobes_eval(lb, a.tab, L, 0.f);
                float pB = lobes_pdf(lb, L);
                if (guided) pB = galpha * guide_pdf(gmix, L) + (1.f - galpha) * pB;
                float w = mis_weight(pS, pB);
                f3 contrib = beta * f * le * (fabsf(NoL) * (w / pS));
                if (max3(contrib) > (toEmit ? 1e-9f : 1e-7f)) {
                    const float nS = NoL < 0.f ? n1 : n;                 // the medium the shadow ray crosses
                    float tr = 1.f;
                    if (!toEmit && u.haze_on && fabsf(nS - 1.f) <= 1e-3f)
                        tr = haze_tr(u, pos, L, toFace ? fdist : 2.f * u.envR + length(pos));
                    sh.valid = true;
                    sh.emit = toEmit;
                    sh.face = toFace;
                    sh.dist = fdist;
                    sh.org = pos + nrm * (NoL < 0.f ? -otol * 2.f : otol * 2.f);
                    sh.dir = L;
                    sh.rad = contrib * tr;
                    sh.n = nS;
                }
            }
        }
    }
    LobeSample smp;                                                   // the bounce
    float pGuided = 0.f;
    if (guided) {
        const float4 rg = rng.next();
        if (rg.x < galpha) {
            smp.dir = guide_sample(gmix, rg.y, rg.z, rg.w);
        } else {
            smp = lobes_sample(lb, a.tab, rng.next());
        }
        const float c = dot(nrm, smp.dir);
        pGuided = galpha * guide_pdf(gmix, smp.dir) + (1.f - galpha) * lobes_pdf(lb, smp.dir);
        smp.w = (c > 0.f && pGuided > 0.f) ? lobes_eval(lb, a.tab, smp.dir, 0.f) * (c / pGuided) : mk(0.f);
        smp.ev = EV_EVAL;
        smp.isDelta = false;
        smp.transmitted = false;
        // the path's first guided vertex keeps a training record: where, the direction and its density, the
        // throughput reaching the vertex and the radiance before it (the light found after it is summed into acc)
        if (GUIDE && a.gd.train && !(my & META_TRAIN) && max3(smp.w) > 0.f) {
            GuideRec rc;
            rc.a = make_float4(pos.x, pos.y, pos.z, pGuided);
            rc.b = make_float4(__uint_as_float(guide_oct16(nrm)), __uint_as_float(guide_oct16(smp.dir)),
                               luma(beta), luma(rad));
            a.gd.rec[gpix] = rc;
            my |= META_TRAIN;
        }
    } else {
        smp = lobes_sample(lb, a.tab, rng.next());
    }
    dir = smp.dir;
    beta = beta * smp.w;
    if (smp.transmitted) {
        n = nT;                                                       // n(lambda) where the ray has a wavelength
        if (draw) { beta = beta * spec.w; lam = spec.lam; }           // ...and the one it was refracted at, kept
        // ...and the medium it is in now, the one beyond the face (tracebasics.js:522-530 enterMedium), where a
        // material scatters inside: the march reads it there alone, and elsewhere meta.z stays the steps it was
        const uint32_t med = (ids >> 16) != SURF_NONE ? (ids >> 16) : (inside ? 0u : (ids & 0xffffu));
        if (a.u.scatter_on) mz = (mz & META_STEPS) | (min(med, 255u) << MEDIUM_SHIFT);
    }
    if (u.sppm_on) {                                                  // materials_pbr.js:862-873 lensStep
        const bool delta = smp.ev == EV_DELTA;
        // the first surface: 1 through a delta; a D there was gathered, so 2 -- unless light tracing runs, whose
        // class that is (the reference's split: 0)
        if (bounces == 1u) lens = delta ? 1u : ((smp.ev == EV_EVAL && !u.lt_on) ? 2u : 0u);
        else if (lens == 1u) lens = delta ? 1u : (smp.ev == EV_EVAL ? 2u : 0u);
        else lens = ((lens == 2u || lens == 3u) && delta) ? 3u : 0u;
    }
    if (u.lt_on) {
        // LIGHT TRACING'S CLASS (tracebasics.js:995-1011): a first vertex drawn from an evaluable lobe, then delta
        // events only; the first other event takes the path out for good
        if (bounces == 1u) my = (my & ~(META_CAND | META_SPEC)) | (smp.ev == EV_EVAL ? META_CAND : 0u);
        else if (my & META_CAND) my = smp.ev == EV_DELTA ? (my | META_SPEC) : (my & ~(META_CAND | META_SPEC));
    }
    if (max3(smp.w) <= 0.f) state = RAY_ABSORBED;
    if (u.nee != 0u && !last) {                                       // the other half of MIS (:1370-1395)
        const float cO = dot(nrm, dir);
        bool above = (cO > 0.f || (throughLit && cO < 0.f)) && !smp.isDelta;   // sideLit: what light sampling draws
        float pOut = smp.isDelta ? 0.f : (guided ? pGuided : lobes_pdf(lb, smp.dir));
        float pLout = above ? rs * (1.f - es) * env_pdf_q(u, dir, nrm, qf) : 0.f;
        sunmis = pLout <= 0.f ? 1.f : mis_weight(pOut, pLout);
        // an emitter this bounce meets is weighed against the list's density for the direction, from here
        const float pEout = (above && es > 0.f) ? rs * es * emit_cone_pdf(a.em.dev, pos, dir) : 0.f;
        emw = pEout <= 0.f ? 1.f : mis_weight(pOut, pEout);
        // a face it meets, against the faces' density there (prevPdf, vtxLtot): only what light sampling could draw
        lp = make_float2((above && fs > 0.f && !lobes_none(m, trans, hz)) ? pOut : -1.f, ltot);
    } else {
        sunmis = 1.f;
        emw = 1.f;
        lp = make_float2(-1.f, ltot);
    }
    f3 off = dir * otol;
    pos = pos + off; ltot += length(off) * n;
    if (bounces > u.maxbounce) state = RAY_TERMINATED;                // pathEnd's tail (tracebasics.js:1040-1103)
    if (u.rr != 0u && bounces >= 3u && state == RAY_ACTIVE) {
        float p = clampf(max3(beta), 0.1f, 0.95f);
        float4 r4 = rng.next();
        if (r4.x > p) state = RAY_TERMINATED;
        else beta = beta / p;
    }
}

__device__ __forceinline__ void shade_medium(const WaveArgs& a, f3& pos, f3& dir, f3& beta, float& sunmis,
                                             uint32_t& bounces, uint32_t& state, float n, Rng& rng, bool last,
                                             ShadowOut& sh, float& emw, float ltot, float2& lp) {
    const Uni& u = a.u;
    state = RAY_ACTIVE;
    bounces += 1;
    float g = clampf(u.hg, -0.95f, 0.95f);
    f3 din = dir;
    beta = beta * u.halb;
    // the discovered emitters' share of the air's light samples (haze.js:324-370), as at a surface
    const float es = (a.em.on && u.nee != 0u && !last) ? emit_share(a.em) : 0.f;
    const float fs = (a.lf.n && u.nee != 0u && !last) ? FACE_SHARE : 0.f;   // the faces' share (haze.js:315-350)
    const float rs = 1.f - fs;
    if (u.nee != 0u && !last) {                                       // mediumNee (haze.js:318-405)
        float4 u0 = rng.next();
        float4 u1 = rng.next();
        f3 L = mk(0.f, 0.f, 1.f);
        float pS = 0.f, fdist = 0.f;
        bool toEmit = false, toFace = false;
        f3 fle = mk(0.f);
        const float pick0 = (u0.x - fs) / fmaxf(rs, 1e-6f);
        if (u0.x < fs) {                                              // a face: no vertex normal, the face's side
            const Face f = face_at(a.lf, min((uint32_t)(u0.y * (float)a.lf.n), a.lf.n - 1u));
            const f3 dy = face_point(f, u1.x, u1.y) - pos;
            fdist = length(dy);
            L = dy * (1.f / fmaxf(fdist, 1e-20f));
            const float cosY = -dot(f.n, L);
            if (fdist > 0.f && cosY > 1e-6f) {
                pS = face_density(fs, a.lf.n, f, fdist, cosY);
                fle = f.le * face_beam(f, cosY);                      // in air: over n^2 = 1
                toFace = true;
            }
        } else if (pick0 < es) {
            const uint32_t b = emit_pick(a.em.dev, pick0 / es);
            if (emit_sample(a.em.dev, b, pos, u1.x, u1.y, L)) {
                pS = rs * es * emit_cone_pdf(a.em.dev, pos, L);
                toEmit = true;
            }
        } else {
            L = env_sample_dir_m(u, es > 0.f ? (pick0 - es) / (1.f - es) : pick0, u1.x, u1.y);
            pS = rs * (1.f - es) * env_pdf_m(u, L);
        }
        if (pS > 0.f) {
            float ph = hg_eval(dot(din, L), g);
            float w = mis_weight(pS, ph);
            f3 le = toEmit ? mk(1.f) : (toFace ? fle : env_radiance(u, L));
            f3 contrib = beta * le * (ph * w / pS);
            if (max3(contrib) > (toEmit ? 1e-9f : 1e-7f)) {
                // an emitter's ray takes the haze from where it starts to where it stops, at its resolve
                float tr = toEmit ? 1.f : haze_tr(u, pos, L, toFace ? fdist : 2.f * u.envR + length(pos));
                sh.valid = true; sh.emit = toEmit; sh.face = toFace; sh.dist = fdist;
                sh.org = pos; sh.dir = L; sh.rad = contrib * tr; sh.n = n;
            }
        }
    }
    float4 r2 = rng.next();
    f3 dout = hg_sample(din, g, r2.x, r2.y);
    dir = dout;
    if (u.nee != 0u && !last) {
        float pB = hg_eval(dot(din, dout), g);
        float pL = rs * (1.f - es) * env_pdf_m(u, dout);
        sunmis = pL <= 0.f ? 1.f : mis_weight(pB, pL);
        const float pE = es > 0.f ? rs * es * emit_cone_pdf(a.em.dev, pos, dout) : 0.f;
        emw = pE <= 0.f ? 1.f : mis_weight(pB, pE);
        lp = make_float2(fs > 0.f ? pB : -1.f, ltot);
    } else {
        sunmis = 1.f;
        emw = 1.f;
        lp = make_float2(-1.f, ltot);
    }
    if (bounces > u.maxbounce) state = RAY_TERMINATED;
}

// GUIDE: the variant with the learned proposal (its sampling, records and their light), kept apart so the plain
// kernel's registers stay as they were
template <bool GUIDE>
__global__ void __launch_bounds__(256) k_shade(WaveArgs a, int nxt, int side, int last) {
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
    float4* s_org = side ? a.q.s_org[1] : a.q.s_org[0];
    float4* s_dir = side ? a.q.s_dir[1] : a.q.s_dir[0];
    float4* s_rad = side ? a.q.s_rad[1] : a.q.s_rad[0];
    uint32_t* s_steps = side ? a.q.s_steps[1] : a.q.s_steps[0];
    uint32_t* s_cnt = side ? &a.ctr->shadowCount[1] : &a.ctr->shadowCount[0];
    unsigned long long paths = 0;
    uint32_t flushed = 0, dropped = 0;
    for (uint32_t r = 0; r < nrounds; r++) {
        uint32_t q = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool valid = q < count;
        bool cont = false;
        ShadowOut sh; sh.valid = false; sh.emit = false; sh.face = false; sh.dist = 0.f;
        uint32_t slot = 0, pix = 0, gpix = 0;
        f3 pos, dir, beta, rad;
        float ltot = 0.f, n = 1.f, sunmis = 1.f, tmax = 0.f;
        uint4 m4 = make_uint4(0, 0, 0, 0);
        uint32_t bounces = 0, seg = 0, state = RAY_TERMINATED;
        float lam = 0.f, emw = 1.f;
        float2 lp = make_float2(-1.f, 0.f);
        bool train_nee = false;
        if (valid) {
            slot = a.q.hit[q];
            float dh = a.q.hitd[q];
            float4 p4 = a.pb.pos[slot], d4 = a.pb.dir[slot], b4 = a.pb.beta[slot], r4 = a.pb.rad[slot];
            m4 = a.pb.meta[slot];
            pos = xyz(p4); ltot = p4.w; dir = xyz(d4); n = d4.w; beta = xyz(b4); sunmis = b4.w;
            rad = xyz(r4); tmax = r4.w;
            pix = m4.x; bounces = m4.y & 0xffu; seg = (m4.y >> 8) & 0xffu; state = (m4.y >> 16) & 0xffu;
            gpix = (slot / u.P) * u.P + pix;                          // the pixel in the wave's frames
            if (state == RAY_ESCAPED) {
                // wavefront.js:1292-1310: a path the photon map owns (its lens field 3: delta events only since
                // its D), or light tracing (its class: an evaluable first vertex, delta events since), takes the sky
                // but not the disc, where the sun's photons were drawn along its line
                const bool owned = ((u.sppm_on && ((m4.y >> META_LENS_SHIFT) & 3u) == 3u) ||
                                    (u.lt_on && (m4.y & (META_CAND | META_SPEC)) == (META_CAND | META_SPEC))) &&
                                   sppm_covers(u, pos, dir);
                rad = rad + beta * (owned ? env_sky(u, dir) : env_radiance(u, dir)) * sunmis;
            } else if (state == RAY_ACTIVE || state == RAY_SCATTER || state == RAY_GATHER) {
                train_nee = GUIDE && (m4.y & META_TRAIN) != 0u;       // light found past a record's vertex counts
                if (a.em.on) emw = a.em.w[slot];
                if (a.lf.n) lp = a.pb.lprev[slot];
                uint32_t tile = slot % u.P, j = slot_sample(u, slot);
                Rng rng = path_rng(sample_seed(u.seed, a.ctr->sample + j), tile, 1u + seg);
                seg += 1;
                float absL = __uint_as_float(m4.w);                   // absorbAlong: ltot on arrival at the last vertex
                if (state == RAY_GATHER) {
                    // THE MAP GATHERED AT A COLLISION (haze.js:692-707 mediumGathered; wavefront.js:1179-1183): the
                    // throughput absorbed to here, the photons' in-scattered light over n^2, then turned there as the
                    // march would have -- a vertex now, the map's D: a bounce, its lens field moved on, light sampling's
                    // MIS halves cleared, its next flight drawn from here
                    const uint32_t med = m4.z >> MEDIUM_SHIFT;
                    const st_material& mm = sm[min(med, u.n_mats - 1u)];
                    const float sd = mm.scatter_distance, sig = sd > 0.f ? 1.f / sd : 0.f;
                    const float g = clampf(mm.scatter_g, -0.95f, 0.95f);
                    if (mm.attenuation > 0.f) {
                        const float dl = fmaxf(ltot - absL, 0.f) / fmaxf(n, 1e-4f) / mm.attenuation;
                        beta = beta * mk(__expf(logf(fminf(fmaxf(mm.base[0], 1e-6f), 1.f)) * dl),
                                         __expf(logf(fminf(fmaxf(mm.base[1], 1e-6f), 1.f)) * dl),
                                         __expf(logf(fminf(fmaxf(mm.base[2], 1e-6f), 1.f)) * dl));
                    }
                    m4.w = __float_as_uint(ltot);
                    Rng grng = path_rng(sample_seed(u.seed, a.ctr->sample + j), tile, SPPM_GATHER_SALT + (seg - 1u));
                    const f3 Lv = volume_gather(a, pos, dir, bounces + 1u, g, sig, grng);
                    rad = rad + beta * Lv * (1.f / fmaxf(n * n, 1e-8f));
                    if (Lv.x != 0.f || Lv.y != 0.f || Lv.z != 0.f) atomicAdd(&a.sp.dev->vgathers, 1u);
                    state = RAY_ACTIVE;
                    bounces += 1;
                    m4.y = (m4.y & ~((3u << META_LENS_SHIFT) | META_CAND | META_SPEC)) | (2u << META_LENS_SHIFT);
                    const float4 rh = rng.next();
                    dir = hg_sample(dir, g, rh.x, rh.y);
                    sunmis = 1.f;
                    emw = 1.f;
                    lp = make_float2(-1.f, ltot);
                    if (last || bounces > u.maxbounce) state = RAY_TERMINATED;
                } else if (state == RAY_SCATTER) {
                    m4.w = __float_as_uint(ltot);
                    shade_medium(a, pos, dir, beta, sunmis, bounces, state, n, rng, last != 0, sh, emw, ltot, lp);
                    // haze.js:539: the air is no delta event (out of the map's class); light tracing's class begins
                    // at a first vertex in the air, as at an evaluable surface, and any later one ends it (:550-553)
                    m4.y &= ~((3u << META_LENS_SHIFT) | META_CAND | META_SPEC);
                    if (u.lt_on && bounces == 1u) m4.y |= META_CAND;
                }
                else
                {
                    lam = a.pb.lam[slot];
                    uint32_t lens = (m4.y >> META_LENS_SHIFT) & 3u;
                    shade_surface<GUIDE>(a, sm, a.q.hsurf[q], pos, dir, ltot, n, beta, sunmis, rad, bounces, state,
                                         lam, lens, dh, rng, last != 0, sh, q, m4.y, gpix, emw, lp, absL, m4.z);
                    m4.w = __float_as_uint(absL);                     // kept where a leaving face moved the ray on
                    m4.y = (m4.y & ~(3u << META_LENS_SHIFT)) | (lens << META_LENS_SHIFT);
                }
                if (state == RAY_ACTIVE) {
                    tmax = 0.f;                                       // a new leg
                    if (last) { state = RAY_MAXITER; flushed++; }     // THE FLUSH
                    else cont = true;
                }
            }
        }
        // the shadow ray, the ray on, the path's end: one append per warp each
        uint32_t sq = warp_append(s_cnt, sh.valid);
        if (sh.valid) {
            if (sq < a.q.scap) {
                // a face's ray starts at minus the way to the face, less four offsets: it arrives at ltot 0
                s_org[sq] = f4(sh.org, sh.face ? -fmaxf(sh.dist - 40.f * march_tol(sh.org, u.tol), 0.f) * sh.n : 0.f);
                s_dir[sq] = f4(sh.dir, __uint_as_float(gpix));
                s_rad[sq] = f4(sh.rad, train_nee ? -sh.n : sh.n);    // a negative index: counted for a record
                s_steps[sq] = sh.emit ? SHADOW_EMIT : (sh.face ? SHADOW_FACE : 0u);
            } else {
                dropped++;
            }
        }
        uint32_t rq = warp_append(outc, cont);
        if (cont) {
            a.pb.pos[slot] = f4(pos, ltot);
            a.pb.dir[slot] = f4(dir, n);
            a.pb.beta[slot] = f4(beta, sunmis);
            a.pb.rad[slot] = f4(rad, tmax);
            if (lam != 0.f) a.pb.lam[slot] = lam;
            if (a.em.on) a.em.w[slot] = emw;
            if (a.lf.n) a.pb.lprev[slot] = lp;
            m4.y = meta_y(bounces, seg, RAY_ACTIVE) | (m4.y & ~META_LOW);
            a.pb.meta[slot] = m4;
            outq[rq] = slot;
        } else if (valid) {
            // THE PATH IS OVER (wavefront.js:1400-1425): its radiance into this sample's (and view's) frame, once
            uint32_t k = slot / u.P;
            float4* fr = a.frame + (size_t)k * u.P;
            deposit(fr, pix, rad, a.ctr);
            atomicAdd(&fr[pix].w, 1.f);
            paths++;
            if (GUIDE && a.gd.train && (m4.y & META_TRAIN))
                atomicAdd(&a.gd.acc[gpix], luma(rad) - a.gd.rec[gpix].b.w);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        paths += __shfl_down_sync(FULL_MASK, paths, o);
        flushed += __shfl_down_sync(FULL_MASK, flushed, o);
        dropped += __shfl_down_sync(FULL_MASK, dropped, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (paths) atomicAdd(&a.ctr->paths, paths);
        if (flushed) atomicAdd(&a.ctr->flushed, flushed);
        if (dropped) atomicAdd(&a.ctr->shadowdrop, dropped);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&a.ctr->segments, (unsigned long long)count);
}


// ------------------------------------------------------------------------------------------------------------
// RESOLVE (wavefront.js:414-494; measure.js:36-51), in FP64: each sample of the wave in order folded into the mean
// and the error bar's moments, the frame taken and cleared in the same pass.
// ------------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_resolve(WaveArgs a) {
    const Uni& u = a.u;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;                 // view i / P's pixel i % P
    if (i == 0) atomicAdd(&a.ctr->sample, a.spw);
    const uint32_t nv = max(u.nv, 1u);
    if (i >= nv * u.P) return;
    const uint32_t view = i / u.P, pix = i % u.P;
    Acc4 acc = a.acc[i];
    double2 mo = a.mom[i];
    // light tracing's estimate for the pixel (one sample a wave while it runs), taken and cleared first: added as it
    // is, not averaged with the pixel's paths (wavefront.js:425-433, :459-462)
    float4 lt = make_float4(0.f, 0.f, 0.f, 0.f);
    if (u.lt_on && view == 0u) {                                      // one view while light tracing runs
        lt = a.splat[i];
        a.splat[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (uint32_t j = 0; j < a.spw; j++) {
        const size_t fi = (size_t)(j * nv + view) * u.P + pix;
        float4 f = a.frame[fi];
        a.frame[fi] = make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t n = (uint32_t)f.w;
        if (n == 0u) continue;
        double sx = double(f.x) / n + lt.x, sy = double(f.y) / n + lt.y, sz = double(f.z) / n + lt.z;
        double prevn = u.maxaverages ? fmin(acc.w, double(u.maxaverages)) : acc.w;
        double cnt = prevn + 1.0;
        double px = fmin(fmax(acc.x, -1e20), 1e20), py = fmin(fmax(acc.y, -1e20), 1e20), pz = fmin(fmax(acc.z, -1e20), 1e20);
        acc.x = (px * prevn + sx) / cnt;
        acc.y = (py * prevn + sy) / cnt;
        acc.z = (pz * prevn + sz) / cnt;
        acc.w = cnt;
        double y = sx * 0.2126 + sy * 0.7152 + sz * 0.0722;
        double w = 1.0 / cnt;
        double d = prevn > 0 ? y - (px * 0.2126 + py * 0.7152 + pz * 0.0722) : 0.0;
        double v0 = fmin(fmax(mo.x, 0.0), 1e300), s0 = fmin(fmax(mo.y, 0.0), 1.0);
        mo.x = (1 - w) * (v0 + w * d * d);
        mo.y = (1 - w) * (1 - w) * s0 + w * w;
    }
    a.acc[i] = acc;
    a.mom[i] = mo;
}

// ------------------------------------------------------------------------------------------------------------
// launch wrappers
// ------------------------------------------------------------------------------------------------------------
static int g_occ_march = 0, g_occ_occl = 0, g_occ_shade = 0, g_occ_shade_g = 0, g_occ_surf = 0;

cudaError_t launch_mf_tables(float* ec, float* ecavg, float* e1, cudaStream_t s) {
    const uint32_t N = MF_NIOR * MF_NR * MF_NMU + MF_NR * MF_NMU;
    k_mf_lut<<<(N + 127) / 128, 128, 0, s>>>(ec, e1);
    k_mf_avg<<<(MF_NIOR * MF_NR + 127) / 128, 128, 0, s>>>(ec, ecavg);
    return cudaGetLastError();
}
cudaError_t launch_genrays(const WaveArgs& a, int sms, cudaStream_t s) {
    uint32_t blocks = min((a.slots + 255) / 256, (uint32_t)sms * 8u);
    k_genrays<<<blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_iter_begin(const WaveArgs& a, int it, int nxt, int first, cudaStream_t s) {
    k_iter_begin<<<1, 32, 0, s>>>(a.ctr, it, nxt, a.slots, first);
    return cudaGetLastError();
}
static int occupancy(const void* fn, size_t smem) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 256, smem);
    return nb > 0 ? nb : 1;
}
template <bool MEDIA, bool INST, bool COUNT>
static void march_variant(const WaveArgs& a, int cur, int nxt, int last, int sms, cudaStream_t s, int* occ_cache) {
    size_t smem = a.u.n_prims * sizeof(DPrim);
    auto fn = k_march<TableScene, MEDIA, INST, COUNT>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = occ_cache && *occ_cache ? *occ_cache : occupancy((const void*)fn, smem);
    if (occ_cache) *occ_cache = nb;
    fn<<<sms * nb, 256, smem, s>>>(a, cur, nxt, last);
}
// a kernel of the scene's own compiled code (st_scene_rtc.cu): a persistent grid at its occupancy (occ non-null), or
// grid_per_sm CTAs an SM
static cudaError_t code_launch(const void* fn, int* occ, unsigned grid_per_sm, int sms, size_t smem, cudaStream_t s,
                               void** args) {
    if (!fn) return cudaErrorInvalidDeviceFunction;
    if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    unsigned per_sm = grid_per_sm;
    if (occ) {
        if (!*occ) *occ = occupancy(fn, smem);
        per_sm = (unsigned)*occ;
    }
    return cudaLaunchKernel(fn, dim3((unsigned)sms * per_sm), dim3(256), args, smem, s);
}
cudaError_t launch_march(const WaveArgs& a, int cur, int nxt, int last, int sms, cudaStream_t s) {
    const bool media = a.u.haze_on || a.u.scatter_on;        // a haze box or a material that scatters inside
    if (a.code && !a.inst_range) {
        const int med = media ? 1 : 0, count = a.u.count_work ? 1 : 0;
        void* args[] = {(void*)&a, &cur, &nxt, &last};
        return code_launch(a.code->march[med][count], &a.code->occ_march[med][count], 0, sms, 0, s, args);
    }
    if (a.inst_range) march_variant<false, true, false>(a, cur, nxt, last, sms, s, nullptr);
    else if (a.u.count_work && media) march_variant<true, false, true>(a, cur, nxt, last, sms, s, nullptr);
    else if (a.u.count_work) march_variant<false, false, true>(a, cur, nxt, last, sms, s, nullptr);
    else if (media) march_variant<true, false, false>(a, cur, nxt, last, sms, s, nullptr);
    else march_variant<false, false, false>(a, cur, nxt, last, sms, s, &g_occ_march);
    return cudaGetLastError();
}
// THE MAP'S BAKE (envmap.js:100-150 prog_envbake): one thread a texel of the equal-area map, the environment's own
// light (no gains) at 2 x 2 stratified points in it, the sun's cone left out where there is one; its mean luminance
__global__ void __launch_bounds__(256) k_env_bake(Uni u, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint32_t)(ENV_MW * ENV_MH)) return;
    const float x = (float)(i % ENV_MW), y = (float)(i / ENV_MW);
    f3 acc = mk(0.f);
    for (int sy = 0; sy < 2; sy++)
        for (int sx = 0; sx < 2; sx++) {
            const float ux = (x + ((float)sx + 0.5f) * 0.5f) / (float)ENV_MW;
            const float uy = (y + ((float)sy + 0.5f) * 0.5f) / (float)ENV_MH;
            const float z = 1.f - 2.f * uy, sz = sqrtf(fmaxf(0.f, 1.f - z * z));
            float sp, cp;
            sincosf(2.f * ST_PI * ux, &sp, &cp);
            const f3 d = mk(sz * cp, sz * sp, z);
            if (!(u.sun_on && in_sun_disc(u, d))) acc = acc + env_base(u, d);
        }
    out[i] = luma(acc * 0.25f);
}
cudaError_t launch_sc_fill(const DPrim* prims, uint32_t n_prims, f3 lo, float cs, uint32_t dx, uint32_t dy, uint32_t dz,
                           float* out, int sms, cudaStream_t s, const SceneCode* code) {
    if (code) {
        void* args[] = {(void*)&prims, &n_prims, &lo, &cs, &dx, &dy, &dz, &out};
        return code_launch(code->sc_fill, nullptr, 8, sms, 0, s, args);
    }
    k_sc_fill<TableScene><<<sms * 8, 256, 0, s>>>(prims, n_prims, lo, cs, dx, dy, dz, out);
    return cudaGetLastError();
}
// THE ENVIRONMENT'S TEXTURE (envmap.js:186-202 ENV_CACHE_MAIN): a texel the preset's light averaged over 2 x 2 points
// even in azimuth and angle, the sun's cone left out (there the preset itself is asked)
__global__ void __launch_bounds__(256) k_env_cache(Uni u, float4* __restrict__ out, uint32_t w, uint32_t h) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w * h) return;
    const float x = (float)(i % w), y = (float)(i / w);
    f3 acc = mk(0.f);
    float n = 0.f;
    for (int sy = 0; sy < 2; sy++)
        for (int sx = 0; sx < 2; sx++) {
            const float uu = (x + ((float)sx + 0.5f) * 0.5f) / (float)w, vv = (y + ((float)sy + 0.5f) * 0.5f) / (float)h;
            float sp, cp, st, ct;
            sincosf(2.f * ST_PI * uu, &sp, &cp);
            sincosf(ST_PI * vv, &st, &ct);
            const f3 d = mk(st * cp, st * sp, ct);
            if (!(u.sun_on && in_sun_disc(u, d))) { acc = acc + env_base(u, d); n += 1.f; }
        }
    acc = acc * (1.f / fmaxf(n, 1.f));
    out[i] = make_float4(acc.x, acc.y, acc.z, 1.f);
}
cudaError_t launch_env_cache(const Uni& u, float4* out, uint32_t w, uint32_t h, cudaStream_t s) {
    k_env_cache<<<(w * h + 255) / 256, 256, 0, s>>>(u, out, w, h);
    return cudaGetLastError();
}
cudaError_t launch_env_bake(const Uni& u, float* out, cudaStream_t s) {
    k_env_bake<<<(ENV_MW * ENV_MH + 255) / 256, 256, 0, s>>>(u, out);
    return cudaGetLastError();
}
cudaError_t launch_eval_sdf(const DPrim* prims, uint32_t n_prims, const float* pts, uint32_t n, float* out,
                            cudaStream_t s, const SceneCode* code) {
    const unsigned blocks = std::min((n + 255u) / 256u, 4096u);
    if (code) {
        if (!code->eval_sdf) return cudaErrorInvalidDeviceFunction;
        void* args[] = {(void*)&prims, &n_prims, (void*)&pts, &n, &out};
        return cudaLaunchKernel(code->eval_sdf, dim3(blocks), dim3(256), args, 0, s);
    }
    k_eval_sdf<TableScene><<<blocks, 256, 0, s>>>(prims, n_prims, pts, n, out);
    return cudaGetLastError();
}
cudaError_t launch_sort(const WaveArgs& a, int cur, int sms, cudaStream_t s) {
    if (!a.u.sort_on) return cudaSuccess;
    const uint32_t* cnt = &a.ctr->rayCount[cur];
    const uint32_t* inq = cur ? a.q.ray[1] : a.q.ray[0];
    k_sort_key<<<sms * 8, 256, 0, s>>>(cnt, a.q.cap, inq, a.pb.pos, a.pb.dir, a.u.glo, a.u.ginv, a.q.skey, a.q.srank,
                                       a.q.bcnt);
    k_sort_scan<<<1, 1024, 0, s>>>(a.q.bcnt, a.q.boff);
    k_sort_scatter<<<sms * 8, 256, 0, s>>>(cnt, a.q.cap, inq, a.q.skey, a.q.srank, a.q.boff, a.q.sorted);
    return cudaGetLastError();
}
cudaError_t launch_sort_shadow(const WaveArgs& a, int side, int sms, cudaStream_t s) {
    if (!a.u.sort_on) return cudaSuccess;
    const uint32_t* cnt = &a.ctr->shadowCount[side];
    k_sort_key<<<sms * 8, 256, 0, s>>>(cnt, a.q.scap, nullptr, a.q.s_org[side], a.q.s_dir[side], a.u.glo, a.u.ginv,
                                       a.q.sskey, a.q.ssrank, a.q.bcnt);
    k_sort_scan<<<1, 1024, 0, s>>>(a.q.bcnt, a.q.boff);
    k_sort_scatter<<<sms * 8, 256, 0, s>>>(cnt, a.q.scap, nullptr, a.q.sskey, a.q.ssrank, a.q.boff, a.q.ssorted);
    return cudaGetLastError();
}
cudaError_t launch_surface(const WaveArgs& a, int sms, cudaStream_t s) {
    if (a.code && !a.inst_range) {
        const size_t smem = a.u.n_mats * sizeof(st_material);
        void* args[] = {(void*)&a};
        return code_launch(a.code->surface, &a.code->occ_surface, 0, sms, smem, s, args);
    }
    size_t smem = a.u.n_prims * sizeof(DPrim) + a.u.n_mats * sizeof(st_material);
    auto fn = k_surface<TableScene>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!g_occ_surf) g_occ_surf = occupancy((const void*)fn, smem);
    fn<<<sms * g_occ_surf, 256, smem, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_shade(const WaveArgs& a, int nxt, int side, int last, int sms, cudaStream_t s) {
    size_t smem = a.u.n_mats * sizeof(st_material);
    if (a.gd.on) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(k_shade<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (!g_occ_shade_g) g_occ_shade_g = occupancy((const void*)k_shade<true>, smem);
        k_shade<true><<<sms * g_occ_shade_g, 256, smem, s>>>(a, nxt, side, last);
        return cudaGetLastError();
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_shade<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!g_occ_shade) g_occ_shade = occupancy((const void*)k_shade<false>, smem);
    k_shade<false><<<sms * g_occ_shade, 256, smem, s>>>(a, nxt, side, last);
    return cudaGetLastError();
}
template <int SIDE>
static void occlude_side(const WaveArgs& a, int last, int sms, cudaStream_t s) {
    size_t smem = a.u.n_prims * sizeof(DPrim);
    auto fn = k_occlude<TableScene, SIDE>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!g_occ_occl) g_occ_occl = occupancy((const void*)fn, smem);
    fn<<<sms * g_occ_occl, 256, smem, s>>>(a, last);
}
cudaError_t launch_occlude(const WaveArgs& a, int side, int last, int sms, cudaStream_t s) {
    if (a.code && !a.inst_range) {
        void* args[] = {(void*)&a, &last};
        return code_launch(a.code->occlude[side ? 1 : 0], &a.code->occ_occlude, 0, sms, 0, s, args);
    }
    if (side) occlude_side<1>(a, last, sms, s);
    else occlude_side<0>(a, last, sms, s);
    return cudaGetLastError();
}
cudaError_t launch_resolve(const WaveArgs& a, cudaStream_t s) {
    k_resolve<<<((a.u.nv ? a.u.nv : 1u) * a.u.P + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace st
