// st_scene_kernels.cuh -- the kernels that ask the scene its distance or its full answer, written once for both
// forms a scene takes:
//
//   a TABLE of primitives (the scene as data, builder/scenedata.js; st_device.cuh scene_dist / scene_full), staged
//   into shared memory by a bulk copy and folded by a loop -- TableScene, instantiated in st_render.cu; and
//   CODE (the builder's shape-as-code contract, builder/codegen.js:974-1060 generate; lib/pathtracer/README.md:126-145),
//   the scene's own __device__ functions st_scene_dist / st_scene_full compiled with these kernels by NVRTC for
//   sm_103a when the scene is set -- the CodeScene policy of st_scene_rtc.cu, which needs no table in shared memory.
//
//   k_march         sphere tracing, persistent with refill          core/wavefront.js:834-1005 (prog_march)
//   k_surface       the hit's normal, material, medium beyond      core/wavefront.js:1037-1147 (prog_surface)
//   k_occlude       shadow rays, persistent with refill            core/wavefront.js:1481-1692 (prog_occlude)
//   k_emit_resolve  what an emitter's shadow ray met               core/wavefront.js:1694-1749 (prog_occlude_emit)
//   k_sc_fill       the step cache's cells                          core/wavefront.js:119-147 (prog_stepcache_fill)
//   k_eval_sdf      the distance at given points (st_eval_sdf)
//
// A policy SC gives kTable (whether the kernel stages the table) and dist<COUNT>(sp, n, p, wc) / dist(sp, n, p) /
// full(sp, n, p); the code policy ignores sp and n.
#pragma once
#include "st_emit.cuh"
#include "st_kernels.cuh"
#include "st_sppm_dev.cuh"

namespace st {

// THE TABLE AS THE SCENE: the fold of st_device.cuh over the table in shared memory (or, for the kernels that do not
// stage it, in global memory)
struct TableScene {
    static constexpr bool kTable = true;
    template <bool COUNT>
    __device__ static __forceinline__ float dist(const DPrim* sp, uint32_t n, f3 p, uint32_t* wc) {
        return scene_dist<COUNT>(sp, n, p, wc);
    }
    __device__ static __forceinline__ float dist(const DPrim* sp, uint32_t n, f3 p) { return scene_dist(sp, n, p); }
    __device__ static __forceinline__ SceneHit full(const DPrim* sp, uint32_t n, f3 p) { return scene_full(sp, n, p); }
};

#define ST_SALT_VOL_STORE 0x564F4C53u      // a photon's record in a volume: its sub-list (haze.js mediumStore)
#define ST_SALT_VOL_KEEP 0x4B454550u       // ...and whether the sample's thinning keeps it
// a scattering material's walk draws from the path's own streams (a photon's from its id), by the path's steps so far
__device__ __forceinline__ Rng walk_rng(const WaveArgs& a, uint32_t slot, uint32_t id, uint32_t salt) {
    const Uni& u = a.u;
    return u.photon_pass ? path_rng(photon_seed_of(u.seed, a.ctr->sample), id, salt)
                         : path_rng(sample_seed(u.seed, a.ctr->sample + slot_sample(u, slot)), slot % u.P, salt);
}

// ------------------------------------------------------------------------------------------------------------
// THE MARCH (wavefront.js:834-1005): persistent -- a few CTAs an SM whose warps claim CLAIM queue entries at a time
// (the autotuner's claim) and refill a lane the moment its ray ends; a ray marches at most MARCH_CHUNK evaluations (the
// autotuner's chunk) a launch (the last
// iteration's launch to its end) and goes to the hit queue or the next iteration's march queue.
// MEDIA: compiled in for a scene with a haze box or a material that scatters inside. In the haze a leg's collision ends
// the march (a vertex: haze.js mediumVertex); in a scattering material the march itself turns the ray at each collision
// and marches on (haze.js:574-650 THE MEDIUM'S WALK): a free flight -ln(1 - u) / sigma drawn as a leg starts, from its
// vertex, each collision taken back to along the line the ray came, turned by Henyey-Greenstein and given its next
// flight, a march step against maxiter; a surface met first ends the leg as it would have.
// ------------------------------------------------------------------------------------------------------------
template <class SC, bool MEDIA, bool INST, bool COUNT>
__global__ void __launch_bounds__(256, 4) k_march(WaveArgs a, int cur, int nxt, int last) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t wc[COUNT ? WC_N : 1];
    DPrim* sp = reinterpret_cast<DPrim*>(smem);
    const uint32_t n_prims = a.u.n_prims;
    if (COUNT)
        for (uint32_t k = threadIdx.x; k < WC_N; k += blockDim.x) wc[k] = 0u;
    if (SC::kTable && !stage_table(sp, a.prims, n_prims * (uint32_t)sizeof(DPrim), &mbar, a.ctr)) return;
    const uint32_t count = a.ctr->rayCount[cur];
    const uint32_t* __restrict__ inq = a.u.sort_on ? a.q.sorted : (cur ? a.q.ray[1] : a.q.ray[0]);
    uint32_t* __restrict__ outq = nxt ? a.q.ray[1] : a.q.ray[0];
    uint32_t* outc = nxt ? &a.ctr->rayCount[1] : &a.ctr->rayCount[0];
    const float tol = a.u.tol, stepscale = a.u.stepscale, envR2 = a.u.envR2;
    const uint32_t maxiter = a.u.maxiter;
    const uint32_t chunk = last ? 0xffffffffu : (a.u.chunk ? a.u.chunk : MARCH_CHUNK);
    const uint32_t claim = a.u.claim ? a.u.claim : CLAIM;
    const int lane = threadIdx.x & 31;

    uint32_t slot = INVALID_SLOT;
    f3 pos = mk(0.f), dir = mk(0.f);
    float ltot = 0.f, n = 1.f, tmax = 0.f;
    float wsig = 0.f, wg = 0.f;                     // the walk's medium: its scattering coefficient (0: none) and g
    uint32_t wid = 0, wmed = 0;
    uint32_t wmap = 0;                              // the photon map in the volume: 1 a photon that stores at its
                                                    // collisions, 2 a camera ray that gathers at its first
    float wabs = 0.f;                               // absLtot: where the ray arrived last (its absorption since)
    bool walked = false;                            // a collision turned the ray in this launch
    uint32_t steps = 0, evals_here = 0;
    uint32_t wpos = 0, wend = 0;
    bool exhausted = false;
    unsigned long long evals = 0;
    uint32_t pfirst = 0, pcount = n_prims;          // the primitives this ray sees: its instance's, in a batch

    for (;;) {
        // ---- refill: idle lanes take the warp's next claimed entries ----
        uint32_t idle = __ballot_sync(FULL_MASK, slot == INVALID_SLOT);
        if (idle && !exhausted) {
            if (wpos >= wend) {
                uint32_t b = 0;
                if (lane == 0) b = atomicAdd(&a.ctr->marchHead, claim);
                b = __shfl_sync(FULL_MASK, b, 0);
                if (b >= count) exhausted = true;
                else { wpos = b; wend = min(b + claim, count); }
            }
            if (!exhausted) {
                uint32_t avail = wend - wpos;
                uint32_t rank = __popc(idle & lanemask_lt());
                if (slot == INVALID_SLOT && rank < avail) {
                    slot = inq[wpos + rank];
                    float4 p4 = a.pb.pos[slot], d4 = a.pb.dir[slot];
                    pos = xyz(p4); ltot = p4.w; dir = xyz(d4); n = d4.w;
                    uint4 m4 = a.pb.meta[slot];
                    steps = m4.z & META_STEPS;
                    evals_here = 0;
                    if (INST) { uint2 rg = a.inst_range[m4.w]; pfirst = rg.x; pcount = rg.y; }
                    tmax = MEDIA ? a.pb.rad[slot].w : 0.f;
                    wsig = 0.f;
                    walked = false;
                    wid = m4.x;
                    wmap = 0u;
                    if (MEDIA && a.u.scatter_on) {                    // the medium the ray is in, if it scatters
                        const uint32_t med = m4.z >> MEDIUM_SHIFT;
                        if (med != 0u && med < a.u.n_mats && (m4.y & META_PROBE) == 0u) {
                            const float sd = a.mats[med].scatter_distance;
                            if (sd > 0.f) { wsig = 1.f / sd; wg = clampf(a.mats[med].scatter_g, -0.95f, 0.95f); }
                        }
                        wmed = med;
                        wabs = __uint_as_float(m4.w);
                        // the map in the volume (haze.js:651-690): a photon past a delta event stores at its collisions
                        // within the bounce cap a gather can accept; a camera ray that came in by delta events alone
                        // (its lens field 1) gathers at its first
                        if (wsig > 0.f && a.u.sppm_on) {
                            if (a.u.photon_pass)
                                wmap = ((m4.y & META_PASSED) && (m4.y & 0xffu) + 2u <= a.u.maxbounce) ? 1u : 0u;
                            else
                                wmap = ((m4.y >> META_LENS_SHIFT) & 3u) == 1u ? 2u : 0u;
                        }
                    }
                    if (MEDIA && wsig > 0.f && tmax == 0.f) {
                        // THE LEG'S FLIGHT (haze.js:598-618 mediumDraw), from its vertex (absLtot): a collision the
                        // step off the surface already passed is taken back to below
                        Rng wr = walk_rng(a, slot, m4.x, ST_SALT_WALK + steps);
                        const float4 r4 = wr.next();
                        tmax = fmaxf(fminf(__uint_as_float(m4.w), ltot) - logf(1.f - r4.x) / wsig * n, 1e-30f);
                    } else if (MEDIA && a.u.haze_on && wsig == 0.f && tmax == 0.f) {
                        // THE LEG'S COLLISION, drawn as it starts (haze.js:255-273 hazeDraw)
                        const Uni& u = a.u;
                        tmax = -1.f;
                        if (fabsf(n - 1.f) <= 1e-3f) {
                            float absL = __uint_as_float(m4.w);
                            f3 A = pos - dir * (fmaxf(ltot - absL, 0.f) / fmaxf(n, 1e-4f));
                            float t0, t1;
                            haze_span(u, A, dir, 1e30f, t0, t1);
                            if (t1 > t0) {
                                uint32_t tile = slot % u.P, j = slot_sample(u, slot), seg = (m4.y >> 8) & 0xffu;
                                // a photon's from its own stream (its id), a camera path's from its path's
                                Rng hr = u.photon_pass
                                             ? path_rng(photon_seed_of(u.seed, a.ctr->sample), m4.x, ST_SALT_HAZE + seg)
                                             : path_rng(sample_seed(u.seed, a.ctr->sample + j), tile, ST_SALT_HAZE + seg);
                                float4 r4 = hr.next();
                                float t = t0 - logf(1.f - r4.x) / u.hsig;
                                if (t < t1) tmax = fmaxf(absL + t * n, 1e-30f);
                            }
                        }
                    }
                }
                wpos += min((uint32_t)__popc(idle), avail);
            }
        }
        if (__ballot_sync(FULL_MASK, slot != INVALID_SLOT) == 0) break;

        // ---- one step ----
        bool fin = false, more = false, vstore = false;
        uint32_t state = RAY_ACTIVE;
        float dh = 0.f;
        f3 vin = dir;
        if (slot != INVALID_SLOT && MEDIA && wsig > 0.f && ltot >= tmax) {
            // A COLLISION IN THE MATERIAL (haze.js:619-650 mediumArrived, mediumBack, mediumCollide): back to it along
            // the line the ray came, turned by the phase function, its next flight drawn
            pos = pos - dir * ((ltot - tmax) / fmaxf(n, 1e-4f));
            ltot = tmax;
            if (wmap == 2u) {
                // handed to shade, where the map gathers and the ray is turned (wavefront.js:881-892, RAY_GATHER)
                state = RAY_GATHER;
                fin = true;
                dh = 1e7f;
            } else {
                Rng wr = walk_rng(a, slot, wid, ST_SALT_WALK_HIT + steps);
                const float4 r4 = wr.next();
                vstore = wmap == 1u;                              // a photon's record where it collided
                dir = hg_sample(dir, wg, r4.x, r4.y);
                tmax = fmaxf(ltot - logf(1.f - r4.z) / wsig * n, 1e-30f);
                steps += 1;
                evals_here += 1;
                walked = true;
                if (steps > maxiter) { state = RAY_MAXITER; fin = true; dh = 1e7f; }
                else if (evals_here >= chunk) more = true;
            }
        } else if (slot != INVALID_SLOT) {
            // THE STEP CACHE (wavefront.js:901-912): a ball that holds the ray far enough moves it with no distance;
            // a step that carries it past its collision in the haze is taken back to it below, as a distance step's
            // is. Up to SC_BURST balls in a row: a lane in empty space goes on while its warp's others ask the scene,
            // then asks it too where no ball holds it, so the warp's distance pass is not spent waiting on it
            uint32_t burst = 0;
            if (!INST && a.u.sc_looks) {
                while (burst < SC_BURST && !(MEDIA && tmax > 0.f && ltot >= tmax)) {
                    const float sc = sc_step(a.u, pos, dir);
                    if (!(sc > 0.f)) break;
                    steps += 1;
                    f3 off = dir * (sc * stepscale);
                    pos = pos + off;
                    ltot += length(off) * n;
                    burst++;
                }
                evals_here += burst;
            }
            // (a ray in a scattering material that passed its collision takes it on its next step, above)
            const bool hz = MEDIA && wsig == 0.f;
            if (burst == SC_BURST || (burst && evals_here >= chunk)) {
                if (hz && tmax > 0.f && ltot >= tmax) { state = RAY_SCATTER; fin = true; }
                else if (evals_here >= chunk) more = true;
            } else if (hz && tmax > 0.f && ltot >= tmax) {
                state = RAY_SCATTER;
                fin = true;
            } else {
                float d = SC::template dist<COUNT>(sp + pfirst, pcount, pos, wc);
                evals++;
                evals_here++;
                float ea = fabsf(d);
                float eps = march_tol(pos, tol);
                if (ltot > 1000.f || steps > maxiter) state = RAY_MAXITER;
                if (dot(pos, dir) > 0.f && dot(pos, pos) > envR2) state = RAY_ESCAPED;
                if (ea < eps || state != RAY_ACTIVE) {
                    fin = true;
                    dh = d;
                } else {
                    steps += 1;
                    f3 off = dir * (ea * stepscale);
                    pos = pos + off;
                    ltot += length(off) * n;
                    if (hz && tmax > 0.f && ltot >= tmax) { state = RAY_SCATTER; fin = true; }
                    else if (evals_here >= chunk) more = true;
                }
            }
            if (state == RAY_SCATTER) {                                 // hazeAt: back to the collision
                pos = pos - dir * ((ltot - tmax) / fmaxf(n, 1e-4f));
                ltot = tmax;
            }
        }
        if (MEDIA && a.u.sppm_on && a.u.photon_pass && a.u.scatter_on) {
            // THE RECORD (haze.js:680-690 mediumStore, sppm.js sppmPut): its point, the way it came, its power with
            // the absorption since its vertex, its bounce, the volume's flag and a sub-list
            SppmDev* d = a.sp.dev;
            warp_append(&d->vdemand, vstore);                            // the collisions that would store
            if (vstore) {                                                // ...each kept with the sample's share
                Rng kr = walk_rng(a, slot, wid, ST_SALT_VOL_KEEP + steps);
                vstore = kr.next().x < d->vkeep;
            }
            const uint32_t at = warp_append(&d->count, vstore);
            if (vstore) {
                if (at < d->cap) {
                    const st_material& mm = a.mats[wmed];
                    f3 pw = xyz(a.pb.rad[slot]) * xyz(a.pb.beta[slot]) * (1.f / d->vkeep);
                    if (mm.attenuation > 0.f) {
                        const float dl = fmaxf(ltot - wabs, 0.f) / fmaxf(n, 1e-4f) / mm.attenuation;
                        pw = pw * mk(__expf(logf(fminf(fmaxf(mm.base[0], 1e-6f), 1.f)) * dl),
                                     __expf(logf(fminf(fmaxf(mm.base[1], 1e-6f), 1.f)) * dl),
                                     __expf(logf(fminf(fmaxf(mm.base[2], 1e-6f), 1.f)) * dl));
                    }
                    Rng sr = walk_rng(a, slot, wid, ST_SALT_VOL_STORE + steps);
                    const uint32_t sub = min((uint32_t)(sr.next().y * (float)SPPM_SUBS), SPPM_SUBS - 1u);
                    a.sp.pos[at] = make_float4(pos.x, pos.y, pos.z, 0.f);
                    a.sp.power[at] = make_float4(pw.x, pw.y, pw.z, 0.f);
                    a.sp.dir_oct[at] = oct_word(-vin);
                    a.sp.nrm_oct[at] = 0u;
                    a.sp.flags[at] = ((a.pb.meta[slot].y & 0xffu) + 1u) | (sub << SPPM_SUB_SHIFT) | SPPM_VOL;
                    atomicAdd(&d->vstores, 1u);
                } else {
                    atomicAdd(&d->dropped, 1u);
                }
            }
        }
        uint32_t qp = warp_append(&a.ctr->hitCount, fin);
        uint32_t cp = warp_append(outc, more);
        if (fin || more) {
            a.pb.pos[slot] = make_float4(pos.x, pos.y, pos.z, ltot);
            uint4 m = a.pb.meta[slot];
            m.y = (m.y & ~0x00ff0000u) | (state << 16);               // the classes above it kept
            m.z = (m.z & ~META_STEPS) | min(steps, META_STEPS);        // the medium above it kept
            a.pb.meta[slot] = m;
            if (MEDIA) a.pb.rad[slot].w = tmax;
            if (MEDIA && walked) {
                a.pb.dir[slot] = make_float4(dir.x, dir.y, dir.z, n);
                // a path that collided goes on as one light sampling could not have made (prevPdf -1, sunmis 1): the
                // light it meets takes its whole weight (a photon's fields there are its own)
                if (!a.u.photon_pass) {
                    reinterpret_cast<float*>(&a.pb.beta[slot])[3] = 1.f;
                    if (a.em.on) a.em.w[slot] = 1.f;
                    if (a.lf.n) a.pb.lprev[slot].x = -1.f;
                }
            }
            if (fin) { a.q.hit[qp] = slot; a.q.hitd[qp] = dh; }
            else outq[cp] = slot;
            slot = INVALID_SLOT;
        }
    }
    // the steps taken, one atomic per warp
    for (int o = 16; o > 0; o >>= 1) evals += __shfl_down_sync(FULL_MASK, evals, o);
    if (lane == 0 && evals) atomicAdd(&a.ctr->march_steps, evals);
    if (COUNT) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < WC_N; k += blockDim.x)
            if (wc[k]) atomicAdd(&a.ctr->work[k], (unsigned long long)wc[k]);
    }
}

// THE SURFACE: the geometric half of prog_surface (wavefront.js:1037-1147) -- what a hit asks the scene: the
// normal by three forward differences at normalTol (tracebasics.js:164-165), whether the ray meets it from behind
// (pathFacing, scene_api.js:127-135), the material there and, for a transmissive one, the medium beyond it
// (mediumBeyond, two offset tolerances inside). One thread per shade-queue entry, written to hsurf for k_shade,
// so the shading kernel carries no distance function and the distance work runs at the march's occupancy.
template <class SC>
__global__ void __launch_bounds__(256, 3) k_surface(WaveArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ __align__(8) uint64_t mbar2;
    const Uni& u = a.u;
    DPrim* sp = reinterpret_cast<DPrim*>(smem);
    st_material* sm = reinterpret_cast<st_material*>(smem + (SC::kTable ? u.n_prims * sizeof(DPrim) : 0));
    if (SC::kTable && !stage_table(sp, a.prims, u.n_prims * (uint32_t)sizeof(DPrim), &mbar, a.ctr)) return;
    if (!stage_table(sm, a.mats, u.n_mats * (uint32_t)sizeof(st_material), &mbar2, a.ctr)) return;
    const uint32_t count = a.ctr->hitCount;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x) {
        const uint32_t slot = a.q.hit[q];
        const uint4 m4 = a.pb.meta[slot];
        if (((m4.y >> 16) & 0xffu) != RAY_ACTIVE) continue;          // escaped, out of steps, a haze collision
        const float dh = a.q.hitd[q];
        const f3 pos = xyz(a.pb.pos[slot]);
        const f3 dir = xyz(a.pb.dir[slot]);
        float eps = march_tol(pos, u.tol);
        float gx = SC::dist(sp, u.n_prims, mk(pos.x + eps, pos.y, pos.z)) - dh;
        float gy = SC::dist(sp, u.n_prims, mk(pos.x, pos.y + eps, pos.z)) - dh;
        float gz = SC::dist(sp, u.n_prims, mk(pos.x, pos.y, pos.z + eps)) - dh;
        f3 nn = normalize(mk(gx, gy, gz));
        f3 nrm = dh < 0.f ? -nn : nn;
        uint32_t ids = SURF_LEAVING;
        if (!(dot(-dir, nrm) < 0.f)) {
            SceneHit h = SC::full(sp, u.n_prims, pos);
            const uint32_t mi = min(h.m, u.n_mats - 1);
            const st_material& m = sm[mi];
            uint32_t med = SURF_NONE;
            if (m.transmission > 0.f && m.metallic < 1.f) {
                SceneHit mb = SC::full(sp, u.n_prims, pos + (-nrm) * (10.f * eps * 2.f));
                med = min(mb.a, u.n_mats - 1);
            }
            ids = mi | (med << 16);
        }
        a.q.hsurf[q] = make_float4(nn.x, nn.y, nn.z, __uint_as_float(ids));
    }
}

// ------------------------------------------------------------------------------------------------------------
// THE OCCLUSION PASS (wavefront.js:1481-1692), distance only, persistent with refill like the march: any surface
// blocks; leaving the scene, lmax or maxiter reaches (maxiter counted in shadowcut); a ray that reaches deposits.
// A ray still going after MARCH_CHUNK evaluations is queued for the next iteration's pass on the other side; the
// last iteration's pass runs every ray to its end (the reference's extra rounds on the last pass,
// raytrace_main.js THE LAST PASS'S SHADOW ROUNDS).
// ------------------------------------------------------------------------------------------------------------
template <class SC, int SIDE>
__global__ void __launch_bounds__(256, 4) k_occlude(WaveArgs a, int last) {
    constexpr int side = SIDE;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    DPrim* sp = reinterpret_cast<DPrim*>(smem);
    const uint32_t n_prims = a.u.n_prims;
    if (SC::kTable && !stage_table(sp, a.prims, n_prims * (uint32_t)sizeof(DPrim), &mbar, a.ctr)) return;
    const uint32_t count = min(side ? a.ctr->shadowCount[1] : a.ctr->shadowCount[0], a.q.scap);
    const float4* __restrict__ i_org = side ? a.q.s_org[1] : a.q.s_org[0];
    const float4* __restrict__ i_dir = side ? a.q.s_dir[1] : a.q.s_dir[0];
    const float4* __restrict__ i_rad = side ? a.q.s_rad[1] : a.q.s_rad[0];
    const uint32_t* __restrict__ i_steps = side ? a.q.s_steps[1] : a.q.s_steps[0];
    float4* o_org = side ? a.q.s_org[0] : a.q.s_org[1];
    float4* o_dir = side ? a.q.s_dir[0] : a.q.s_dir[1];
    float4* o_rad = side ? a.q.s_rad[0] : a.q.s_rad[1];
    uint32_t* o_steps = side ? a.q.s_steps[0] : a.q.s_steps[1];
    uint32_t* o_cnt = side ? &a.ctr->shadowCount[0] : &a.ctr->shadowCount[1];
    const float tol = a.u.tol, stepscale = a.u.stepscale, envR2 = a.u.envR2;
    const uint32_t maxiter = a.u.maxiter;
    const uint32_t chunk = last ? 0xffffffffu : (a.u.chunk ? a.u.chunk : MARCH_CHUNK);
    const uint32_t claim = a.u.claim ? a.u.claim : CLAIM;
    const int lane = threadIdx.x & 31;
    uint32_t idx = INVALID_SLOT;
    f3 pos = mk(0.f), dir = mk(0.f);
    float ltot = 0.f, n = 1.f;
    uint32_t steps = 0, evals_here = 0, sflag = 0;
    uint32_t wpos = 0, wend = 0;
    bool exhausted = false;
    unsigned long long evals = 0, rays = 0;
    uint32_t cuts = 0, dropped = 0;
    for (;;) {
        uint32_t idle = __ballot_sync(FULL_MASK, idx == INVALID_SLOT);
        if (idle && !exhausted) {
            if (wpos >= wend) {
                uint32_t b = 0;
                if (lane == 0) b = atomicAdd(&a.ctr->occHead, claim);
                b = __shfl_sync(FULL_MASK, b, 0);
                if (b >= count) exhausted = true;
                else { wpos = b; wend = min(b + claim, count); }
            }
            if (!exhausted) {
                uint32_t avail = wend - wpos;
                uint32_t rank = __popc(idle & lanemask_lt());
                if (idx == INVALID_SLOT && rank < avail) {
                    idx = a.u.sort_on ? a.q.ssorted[wpos + rank] : wpos + rank;
                    float4 o4 = i_org[idx], d4 = i_dir[idx];
                    pos = xyz(o4); ltot = o4.w; dir = xyz(d4); n = fabsf(i_rad[idx].w);
                    steps = i_steps[idx];
                    sflag = steps & SHADOW_FLAGS;                     // aimed at an emitter (TAG_EMIT), a face,
                                                                      // the camera (a photon's connection)
                    steps &= ~SHADOW_FLAGS;
                    evals_here = 0;
                    if (steps == 0u) rays++;
                }
                wpos += min((uint32_t)__popc(idle), avail);
            }
        }
        if (__ballot_sync(FULL_MASK, idx != INVALID_SLOT) == 0) break;
        bool reached = false, done = false, more = false;
        // the step cache (wavefront.js:1536-1546): balls that hold the ray far enough move it with no distance, up to
        // SC_BURST in a row, then the distance where none does (as in the march)
        uint32_t burst = 0;
        if (idx != INVALID_SLOT && a.u.sc_looks) {
            while (burst < SC_BURST && !((sflag & SHADOW_FACE) && ltot >= 0.f)) {
                const float sc = sc_step(a.u, pos, dir);
                if (!(sc > 0.f)) break;
                steps += 1;
                f3 off = dir * (sc * stepscale);
                pos = pos + off;
                ltot += length(off) * n;
                burst++;
            }
            evals_here += burst;
        }
        if (burst == SC_BURST || (burst && evals_here >= chunk)) {
            if (evals_here >= chunk) more = true;
        } else if (idx != INVALID_SLOT) {
            float d = SC::dist(sp, n_prims, pos);
            evals++;
            evals_here++;
            float ea = fabsf(d);
            float eps = march_tol(pos, tol);
            if ((sflag & SHADOW_FACE) && ltot >= 0.f) { reached = true; done = true; }   // at the face (TAG_FNEE)
            else if (ea < eps) done = true;                           // blocked
            else if (dot(pos, dir) > 0.f && dot(pos, pos) > envR2) { reached = true; done = true; }
            else {
                steps += 1;
                if (ltot > 1000.f || steps > maxiter) {
                    reached = true; done = true;
                    if (steps > maxiter) cuts++;
                } else {
                    f3 off = dir * (ea * stepscale);
                    pos = pos + off;
                    ltot += length(off) * n;
                    if (evals_here >= chunk) more = true;
                }
            }
        }
        uint32_t cp = warp_append(o_cnt, more);
        // an emitter's ray asks what it stopped at (wavefront.js:1694-1749): handed to k_emit_resolve; it finds
        // nothing where it leaves the scene
        const bool met = done && !reached && (sflag & SHADOW_EMIT) != 0u;
        const uint32_t ep = a.em.on ? warp_append(&a.ctr->emitHits, met) : 0u;
        if (met && ep < a.q.scap) {
            a.em.hpos[ep] = f4(pos, ltot);
            a.em.hdir[ep] = i_dir[idx];
            a.em.hrad[ep] = i_rad[idx];
        }
        if (reached && (sflag & SHADOW_CONN)) {
            // a photon's connection (wavefront.js:1649-1661): to the splat buffer, added to its pixel as it is
            // (resolve does not average it with the pixel's paths); the connections counted per pixel
            const uint32_t pix = __float_as_uint(i_dir[idx].w);
            deposit(a.splat, pix, xyz(i_rad[idx]), a.ctr);
            atomicAdd(&a.ltcount[pix], 1u);
        } else if (reached && (sflag & SHADOW_EMIT) == 0u) {
            float4 r4 = i_rad[idx];
            uint32_t gpix = __float_as_uint(i_dir[idx].w);          // the pixel in the wave's frames
            deposit(a.frame, gpix, xyz(r4), a.ctr);
            if (r4.w < 0.f && a.gd.train) atomicAdd(&a.gd.acc[gpix], luma(xyz(r4)));
        }
        if (more) {
            if (cp < a.q.scap) {
                o_org[cp] = f4(pos, ltot);
                o_dir[cp] = i_dir[idx];
                o_rad[cp] = i_rad[idx];
                o_steps[cp] = steps | sflag;
            } else {
                dropped++;
            }
        }
        if (done || more) idx = INVALID_SLOT;
    }
    for (int o = 16; o > 0; o >>= 1) {
        evals += __shfl_down_sync(FULL_MASK, evals, o);
        rays += __shfl_down_sync(FULL_MASK, rays, o);
        cuts += __shfl_down_sync(FULL_MASK, cuts, o);
        dropped += __shfl_down_sync(FULL_MASK, dropped, o);
    }
    if (lane == 0) {
        if (evals) atomicAdd(&a.ctr->shadow_steps, evals);
        if (rays) atomicAdd(&a.ctr->shadow_rays, rays);
        if (cuts) atomicAdd(&a.ctr->shadowcut, cuts);
        if (dropped) atomicAdd(&a.ctr->shadowdrop, dropped);
    }
}

// THE EMITTER RAYS THAT MET SOMETHING (wavefront.js:1694-1749): the material where each stopped, its emission
// times what the ray carries, into the pixel; through the haze in air from where the ray started
template <class SC>
__global__ void __launch_bounds__(256) k_emit_resolve(WaveArgs a) {
    const uint32_t count = min(a.ctr->emitHits, a.q.scap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float4 p4 = a.em.hpos[i], d4 = a.em.hdir[i], r4 = a.em.hrad[i];
        const f3 p = xyz(p4);
        const SceneHit H = SC::full(a.prims, a.u.n_prims, p);
        const st_material& m = a.mats[H.m];
        const f3 le = mk(m.emissive[0], m.emissive[1], m.emissive[2]);
        if (max3(le) <= 0.f) continue;
        f3 c = xyz(r4) * le;
        if (m.beam_cos > 0.f) {                       // a beam: the outward normal there (three differences)
            const float eps = march_tol(p, a.u.tol);
            const float dh = SC::dist(a.prims, a.u.n_prims, p);
            const f3 nn = normalize(mk(SC::dist(a.prims, a.u.n_prims, mk(p.x + eps, p.y, p.z)) - dh,
                                       SC::dist(a.prims, a.u.n_prims, mk(p.x, p.y + eps, p.z)) - dh,
                                       SC::dist(a.prims, a.u.n_prims, mk(p.x, p.y, p.z + eps)) - dh));
            c = c * emit_beam(m.beam_cos, -dot(xyz(d4), nn));
        }
        const float n = fabsf(r4.w);
        if (a.u.haze_on && fabsf(n - 1.f) <= 1e-3f) {
            const float hl = fmaxf(p4.w, 0.f) / fmaxf(n, 1e-4f);
            c = c * haze_tr(a.u, p - xyz(d4) * hl, xyz(d4), hl);
        }
        const uint32_t gpix = __float_as_uint(d4.w);
        deposit(a.frame, gpix, c, a.ctr);
        if (r4.w < 0.f && a.gd.train) atomicAdd(&a.gd.acc[gpix], luma(c));
    }
}

// the scene's distance at given points, as the march folds the table (st_eval_sdf)
template <class SC>
__global__ void __launch_bounds__(256) k_eval_sdf(const DPrim* __restrict__ pr, uint32_t n_prims,
                                                  const float* __restrict__ pts, uint32_t n, float* __restrict__ out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = SC::dist(pr, n_prims, mk(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
}
// THE STEP CACHE'S CELLS (wavefront.js:119-147 prog_stepcache_fill): one thread a cell, the scene's distance at its
// centre, its magnitude held to [1e-6, 1e18]
template <class SC>
__global__ void __launch_bounds__(256) k_sc_fill(const DPrim* __restrict__ prims, uint32_t n_prims, f3 lo, float cs,
                                                 uint32_t dx, uint32_t dy, uint32_t dz, float* __restrict__ out) {
    const uint64_t n = (uint64_t)dx * dy * dz;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(k % dx), y = (uint32_t)((k / dx) % dy), z = (uint32_t)(k / ((uint64_t)dx * dy));
        const f3 c = lo + mk((float)x + 0.5f, (float)y + 0.5f, (float)z + 0.5f) * cs;
        out[k] = fminf(fmaxf(fabsf(SC::dist(prims, n_prims, c)), 1e-6f), 1e18f);
    }
}

}  // namespace st
