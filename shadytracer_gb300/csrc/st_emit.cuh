// st_emit.cuh -- the emitter list's device helpers: a camera path's emitter hit into the discovery grid
// (materials_pbr.js:887-905 emitDeposit), the brightness code (tracebasics.js:62-76 LUM_CODE), and light sampling's
// questions of the list (tracebasics.js:1148-1210: emitPick, coneOneMinusCos, emitConePdf).
#pragma once
#include "st_internal.h"

namespace st {

#define EMIT_LUM_K 209715.2f              // 2^24 / 80 codes a stop: 80 stops (2^-40 .. 2^40 cd/m^2) in 24 bits
#define EMIT_LUM_DECAY 31877u             // x 0.9 a rebuild, in the log code: round(-log2(0.9) * EMIT_LUM_K)
#define EMIT_Q 16777215.f                 // the bounds' quantisation over +-half: 24 bits an axis

__host__ __device__ __forceinline__ uint32_t emit_lum_code(float lum) {
    return (uint32_t)(fminf(fmaxf(log2f(fmaxf(lum, 1e-30f)) + 40.f, 0.f), 80.f) * EMIT_LUM_K) + 1u;
}
__host__ __device__ __forceinline__ float emit_lum_decode(uint32_t q) {
    return q ? exp2f((float)(q - 1u) / EMIT_LUM_K - 40.f) : 0.f;
}
// where a camera path met an emitter, and how bright it is: the voxel's tight bounds (24-bit over +-half), its
// brightest emission (not a sum, which a screen-filling emitter would wrap) and its hit count
__device__ __forceinline__ void emit_deposit(const EmitBufs& em, f3 p, f3 le) {
    const float R = em.half;
    const float ux = (p.x + R) / (2.f * R), uy = (p.y + R) / (2.f * R), uz = (p.z + R) / (2.f * R);
    if (ux < 0.f || uy < 0.f || uz < 0.f || ux >= 1.f || uy >= 1.f || uz >= 1.f) return;
    const uint32_t cell = (uint32_t)(ux * (float)EMIT_G) + EMIT_G * ((uint32_t)(uy * (float)EMIT_G) +
                                                                      EMIT_G * (uint32_t)(uz * (float)EMIT_G));
    uint32_t* g = em.grid + (size_t)cell * 8u;
    const uint32_t qx = (uint32_t)(ux * EMIT_Q), qy = (uint32_t)(uy * EMIT_Q), qz = (uint32_t)(uz * EMIT_Q);
    atomicMin(&g[0], qx); atomicMin(&g[1], qy); atomicMin(&g[2], qz);
    atomicMax(&g[3], qx); atomicMax(&g[4], qy); atomicMax(&g[5], qz);
    atomicMax(&g[6], emit_lum_code(luma(le)));
    atomicAdd(&g[7], 1u);
}
// an emitter's emission leaving it at cosT from its outward normal, over its luminance straight out
// (builder/lights.js:221-228 beamShape, a cosine light, n = 1): within its beam's cone 1, else 0; a glowing surface
// (no beam) 1 every way
__host__ __device__ __forceinline__ float emit_beam(float beam_cos, float cosT) {
    return beam_cos > 0.f ? (cosT >= beam_cos ? 1.f : 0.f) : 1.f;
}
// 1 - cos of the cone a sphere of radius r subtends at squared distance d2, as sin^2 / (1 + cos)
__device__ __forceinline__ float cone_omc(float r, float d2) {
    const float s2 = r * r / d2;
    return s2 / (1.f + sqrtf(fmaxf(0.f, 1.f - s2)));
}
// the share of light samples that aim at the list: 0 with nothing listed, so an emitter-free picture samples as
// it always did
__device__ __forceinline__ float emit_share(const EmitBufs& em) {
    return (em.nee && em.dev->count > 0u) ? fminf(fmaxf(em.share, 0.05f), 0.95f) : 0.f;
}
// whether a probe could have started a photon at y (tracebasics.js:1187-1195 emitCovers): inside a listed sphere
__device__ __forceinline__ bool emit_covers(const EmitDev* d, f3 y) {
    const uint32_t K = min(d->count, EMIT_MAX);
    for (uint32_t b = 0; b < K; b++) {
        const float4 bx = d->box[b];
        const f3 dc = mk(y.x - bx.x, y.y - bx.y, y.z - bx.z);
        if (dot(dc, dc) < bx.w * bx.w) return true;
    }
    return false;
}
// a box by its cumulative probability (linear: at most EMIT_MAX)
__device__ __forceinline__ uint32_t emit_pick(const EmitDev* d, float u) {
    const uint32_t K = min(d->count, EMIT_MAX);
    for (uint32_t b = 0; b < K; b++)
        if (u < d->pc[b].y) return b;
    return K ? K - 1u : 0u;
}
// the density light sampling draws w with from x: the mixture over the boxes x is outside of whose cone holds w
__device__ __forceinline__ float emit_cone_pdf(const EmitDev* d, f3 x, f3 w) {
    const uint32_t K = min(d->count, EMIT_MAX);
    float p = 0.f;
    for (uint32_t b = 0; b < K; b++) {
        const float4 bx = d->box[b];
        const f3 dc = mk(bx.x - x.x, bx.y - x.y, bx.z - x.z);
        const float d2 = dot(dc, dc);
        if (d2 <= bx.w * bx.w) continue;
        const float omc = cone_omc(bx.w, d2);
        if (dot(w, dc) >= (1.f - omc) * sqrtf(d2)) p += d->pc[b].x / (2.f * ST_PI * omc);
    }
    return p;
}
// a direction into box b's cone, uniform in solid angle, from the numbers (u1, u2); false if x is inside its sphere
__device__ __forceinline__ bool emit_sample(const EmitDev* d, uint32_t b, f3 x, float u1, float u2, f3& w) {
    const float4 bx = d->box[b];
    const f3 dc = mk(bx.x - x.x, bx.y - x.y, bx.z - x.z);
    const float d2 = dot(dc, dc);
    if (d2 <= bx.w * bx.w) return false;
    const float dd = sqrtf(d2);
    const f3 axis = dc / dd;
    const float omc = cone_omc(bx.w, d2);
    const float cosT = 1.f - u1 * omc;
    const float sinT = sqrtf(fmaxf(0.f, 1.f - cosT * cosT));
    float sp, cp;
    sincosf(2.f * ST_PI * u2, &sp, &cp);
    const f3 tt = fabsf(axis.x) > 0.9f ? mk(0.f, 1.f, 0.f) : mk(1.f, 0.f, 0.f);
    const f3 b1 = normalize(cross(tt, axis));
    const f3 b2 = cross(axis, b1);
    w = normalize(b1 * (cp * sinT) + b2 * (sp * sinT) + axis * cosT);
    return true;
}

}  // namespace st
