// TEST INFRASTRUCTURE ONLY -- the oracle. A CPU restatement of lampmaker/ShadyTracer's rendering hot path
// (v0.88.0), used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as the checker; never by the
// product. Every function names the reference file:line whose arithmetic it restates. The reference itself is
// JavaScript + WGSL with no JS runtime or WebGPU in this environment, so its results are pinned through the
// known answers its own tests assert (core/test/*.test.mjs, optics/test/*.test.mjs) -- see tests/test_oracle_*.py.
//
// Templated on the arithmetic type: T = float is the reference-equivalent mode (the WGSL computes in f32), T =
// double the accuracy oracle.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>

namespace sto {

template <class T> struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit V3(T a) : x(a), y(a), z(a) {}
    V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3 operator*(const V3& o) const { return V3(x * o.x, y * o.y, z * o.z); }
    V3 operator/(const V3& o) const { return V3(x / o.x, y / o.y, z / o.z); }
    V3 operator*(T s) const { return V3(x * s, y * s, z * s); }
    V3 operator/(T s) const { return V3(x / s, y / s, z / s); }
    V3 operator-() const { return V3(-x, -y, -z); }
    V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator*=(const V3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
};
template <class T> inline T dot(const V3<T>& a, const V3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(const V3<T>& a, const V3<T>& b) {
    return V3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> inline T length(const V3<T>& a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(const V3<T>& a) { return a / length(a); }
template <class T> inline T max3(const V3<T>& a) { return std::max(a.x, std::max(a.y, a.z)); }
template <class T> inline V3<T> vmin(const V3<T>& a, T s) { return V3<T>(std::min(a.x, s), std::min(a.y, s), std::min(a.z, s)); }
template <class T> inline V3<T> vmax(const V3<T>& a, T s) { return V3<T>(std::max(a.x, s), std::max(a.y, s), std::max(a.z, s)); }
template <class T> inline T clampT(T x, T lo, T hi) { return std::min(std::max(x, lo), hi); }
template <class T> inline T sat(T x) { return clampT(x, T(0), T(1)); }
template <class T> inline T mixT(T a, T b, T t) { return a * (T(1) - t) + b * t; }
template <class T> inline V3<T> reflectv(const V3<T>& I, const V3<T>& N) { return I - N * (T(2) * dot(N, I)); }
// WGSL refract(e1, e2, e3): k = 1 - e3^2 (1 - dot(e2, e1)^2); 0 if k < 0, else e3 e1 - (e3 dot(e2, e1) + sqrt(k)) e2
template <class T> inline V3<T> refractv(const V3<T>& I, const V3<T>& N, T eta) {
    T d = dot(N, I);
    T k = T(1) - eta * eta * (T(1) - d * d);
    if (k < T(0)) return V3<T>(0);
    return I * eta - N * (eta * d + std::sqrt(k));
}

const double PI_D = 3.14159265358979323846;
// Rec.709 luminance weights: core/photometry.js:31
const double LUMA_R = 0.2126, LUMA_G = 0.7152, LUMA_B = 0.0722;
template <class T> inline T luma(const V3<T>& c) { return c.x * T(LUMA_R) + c.y * T(LUMA_G) + c.z * T(LUMA_B); }

// ------------------------------------------------------------------------------------------------------------
// PCG4D -- core/tracebasics.js:330-380 (SEED_u32, pcg4d, PRNG: the top 24 bits of each lane)
// ------------------------------------------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };
inline U4 pcg4d(U4 v) {
    v.x = v.x * 1664525u + 1013904223u; v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u; v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    v.x ^= v.x >> 16; v.y ^= v.y >> 16; v.z ^= v.z >> 16; v.w ^= v.w >> 16;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    return v;
}
struct Rng {
    U4 h;
    // SEED_u32: NOISE_H = (NOISE_H.yzwx ^ v) * NOISE_HX   (tracebasics.js:337)
    void seed_u32(uint32_t v) {
        U4 o = h;
        h.x = (o.y ^ v) * 2313257647u; h.y = (o.z ^ v) * 2700274807u;
        h.z = (o.w ^ v) * 3152041561u; h.w = (o.x ^ v) * 3679390633u;
    }
    template <class T> void next4(T out[4]) {
        h = pcg4d(h);
        const T s = T(1.0 / 16777216.0);
        out[0] = T(h.x >> 8) * s; out[1] = T(h.y >> 8) * s; out[2] = T(h.z >> 8) * s; out[3] = T(h.w >> 8) * s;
    }
};
// THE SEEDS. The reference seeds each kernel invocation from the iteration's seed and the ray's SLOT in its queue
// (wavefront.js:856-858), which is the order atomics ran in; its optics shade seeds by the ray's own id and bounce
// instead (optics/kernels.js:598-606, "SEEDED BY THE RAY, not by its slot"). Both sides of this build seed by the
// path: a sample's seed from the base seed, then the path's id, then the event (0 the camera ray, 1 + i the shade
// of the path's i-th segment, SEED_SALT_* for the rest).
inline U4 sample_seed(uint32_t base, uint32_t sample) {
    U4 s = {base, sample, 0xA53B3F17u, 0xC0FFEE42u};
    return pcg4d(pcg4d(s));
}
inline Rng path_rng(U4 sseed, uint32_t path, uint32_t event) {
    Rng r; r.h = sseed; r.seed_u32(path); r.seed_u32(event); return r;
}

}  // namespace sto
