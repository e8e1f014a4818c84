// st_sppm_dev.cuh -- the photon map's device helpers, shared by the grid (st_sppm.cu) and the wavefront's store and
// gather (st_photons.cu): its constants (core/sppm.js:82-135), the cell and its hash (sppm.js:194-198, :381-386), and
// a direction in 32 bits (sppm.js:366-379 sppmOct / sppmUnoct), each rounded as the reference's arithmetic rounds
// (IEEE intrinsics: the grid must agree with it bit for bit whatever the compiler's fast-math flags).
#pragma once
#include "st_device.cuh"

#define SPPM_HEADS (1u << 20)
#define SPPM_SUBS 32u
#define SPPM_BUCKETS (SPPM_HEADS * SPPM_SUBS)
#define SPPM_VISIT_HARD 8u
#define SPPM_SUB_SHIFT 16u
#define SPPM_B_MASK 0xFFFFu
#define SPPM_NORMAL_DOT 0.9f
#define SPPM_VOL 0x40000000u              // a record stored where a photon collided inside a medium (sppm.js:93-95)
#define SPPM_BUDGET 512u                  // records a gather may walk before it subsamples (sppm.js SPPM_VISIT)
#define LT_MIN_ALPHA 0.05f                // from it up a glossy lobe is evaluable (tracebasics.js:299)

namespace st {

// the cell's hash (sppm.js:383-386 sppmHash): 32-bit wrapping multiplies of the cell's coordinates
__device__ __forceinline__ uint32_t sppm_hash(int32_t x, int32_t y, int32_t z) {
    return (((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349663u) ^ ((uint32_t)z * 83492791u)) & (SPPM_HEADS - 1);
}
__device__ __forceinline__ int32_t cell_of(float p, float c) { return (int32_t)floorf(__fdiv_rn(p, c)); }

// pack2x16snorm: clamp to [-1, 1], times 32767, to the nearest integer
__device__ __forceinline__ uint32_t snorm16(float v) {
    const float c = fminf(fmaxf(v, -1.f), 1.f);
    return (uint32_t)(uint16_t)(int16_t)__float2int_rn(__fmul_rn(c, 32767.f));
}
__device__ __forceinline__ uint32_t oct_word(f3 v) {
    const float s = __fadd_rn(__fadd_rn(fabsf(v.x), fabsf(v.y)), fabsf(v.z));
    const float ax = __fdiv_rn(v.x, s), ay = __fdiv_rn(v.y, s), az = __fdiv_rn(v.z, s);
    float ex = ax, ey = ay;
    if (az < 0.f) {
        ex = __fmul_rn(__fsub_rn(1.f, fabsf(ay)), ax >= 0.f ? 1.f : -1.f);
        ey = __fmul_rn(__fsub_rn(1.f, fabsf(ax)), ay >= 0.f ? 1.f : -1.f);
    }
    return snorm16(ex) | (snorm16(ey) << 16);
}
__device__ __forceinline__ float unsnorm16(uint32_t w) {
    int16_t q = (int16_t)(uint16_t)(w & 0xFFFFu);
    return fmaxf(__fdiv_rn((float)q, 32767.f), -1.f);
}
__device__ __forceinline__ f3 unoct(uint32_t w) {
    float ex = unsnorm16(w), ey = unsnorm16(w >> 16);
    float vx = ex, vy = ey, vz = __fsub_rn(__fsub_rn(1.f, fabsf(ex)), fabsf(ey));
    if (vz < 0.f) {
        float nx = __fmul_rn(__fsub_rn(1.f, fabsf(vy)), vx >= 0.f ? 1.f : -1.f);
        float ny = __fmul_rn(__fsub_rn(1.f, fabsf(vx)), vy >= 0.f ? 1.f : -1.f);
        vx = nx; vy = ny;
    }
    float l = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz)));
    return mk(__fdiv_rn(vx, l), __fdiv_rn(vy, l), __fdiv_rn(vz, l));
}

}  // namespace st
