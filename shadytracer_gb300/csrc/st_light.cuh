// st_light.cuh -- the lights' faces as light sampling and a BSDF's hit see them (core/scene_api.js:259-289
// lightFaceArea, lightFaceShare, lightFaceDensity; tracebasics.js:1268 lightFaceLe; builder/lights.js:209-228
// beamOf / beamShape; materials_pbr.js:1244-1268 the point aimed at). The two sides compute the density alike, so
// the MIS weights of a face's light sample and of a BSDF's hit of it sum to one.
#pragma once
#include "st_internal.h"

namespace st {

#define FACE_SHARE 0.5f                   // the share of a vertex's light samples that go to the faces (FACE_NEE_SHARE)

struct Face {
    f3 c, u, v, n, le;
    float hw, hh, beam_cos, expo;         // expo: the cos^n exponent, or < 0 for even intensity
    uint32_t shape;
};

__device__ __forceinline__ Face face_at(const LightBufs& lf, uint32_t i) {
    const float4* f = lf.face + (size_t)i * FACE_F4;
    const float4 a = f[0], b = f[1], c = f[2], d = f[3], e = f[4];
    Face r;
    r.c = mk(a.x, a.y, a.z); r.hw = a.w;
    r.u = mk(b.x, b.y, b.z); r.hh = b.w;
    r.v = mk(c.x, c.y, c.z); r.shape = (uint32_t)c.w;
    r.n = mk(d.x, d.y, d.z); r.beam_cos = d.w;
    r.le = mk(e.x, e.y, e.z); r.expo = e.w;
    return r;
}
__host__ __device__ __forceinline__ float face_area(uint32_t shape, float hw, float hh) {
    return shape == ST_LIGHT_DISC ? 3.14159265359f * hw * hw : 4.f * hw * hh;
}
// the face's radiance at cosT from its normal over its luminance straight out (lightBeam): 0 outside the cone (and
// behind the face); even intensity, 1 / cos; cos^n intensity, cos^(n-1)
__device__ __forceinline__ float face_beam(const Face& f, float cosT) {
    if (cosT < f.beam_cos || cosT <= 0.f) return 0.f;
    const float c = fmaxf(cosT, 1e-4f);
    if (f.expo < 0.f) return 1.f / c;
    return f.expo == 1.f ? 1.f : __powf(c, f.expo - 1.f);
}
// the density, in solid angle, of light sampling with the faces' share picking the direction to a point of a face
// dist away seen at cosY from its normal: the share, the face's pick (1 of n), 1 / area, area to solid angle
__device__ __forceinline__ float face_density(float share, uint32_t nf, const Face& f, float dist, float cosY) {
    if (share <= 0.f || nf == 0u) return 0.f;
    return share / (float)nf * dist * dist / fmaxf(face_area(f.shape, f.hw, f.hh) * fabsf(cosY), 1e-20f);
}
// a point uniform on the face (a disc: r = R sqrt(u), an angle 2 pi u'; a rectangle: each axis uniform)
__device__ __forceinline__ f3 face_point(const Face& f, float ux, float uy) {
    if (f.shape == ST_LIGHT_DISC) {
        const float rr = f.hw * sqrtf(ux), ph = 6.28318530718f * uy;
        float sp, cp;
        __sincosf(ph, &sp, &cp);
        return f.c + (f.u * cp + f.v * sp) * rr;
    }
    return f.c + f.u * ((2.f * ux - 1.f) * f.hw) + f.v * ((2.f * uy - 1.f) * f.hh);
}

}  // namespace st
