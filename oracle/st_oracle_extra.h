// TEST INFRASTRUCTURE ONLY -- the oracle's haze box (core/haze.js), Henyey-Greenstein, and the medium's light
// sampling. Restated from the reference; never part of the product.
#pragma once
#include "st_oracle_render.h"

namespace sto {

const uint32_t SEED_SALT_HAZE = 0x48410000u;   // the haze's own draws (haze.js:266 seeds a constant of its own)

// Henyey-Greenstein (haze.js:191-211 HG_WGSL)
template <class T> inline T hg_eval(T cosT, T g) {
    T d = T(1) + g * g - T(2) * g * cosT;
    return (T(1) - g * g) / (T(4) * T(PI_D) * std::pow(std::max(d, T(1e-12)), T(1.5)));
}
template <class T> inline V3<T> hg_sample(const V3<T>& d, T g, T u0, T u1) {
    T c = T(1) - T(2) * u0;
    if (std::fabs(g) >= T(1e-3)) {
        T s = (T(1) - g * g) / (T(1) - g + T(2) * g * u0);
        c = clampT((T(1) + g * g - s * s) / (T(2) * g), T(-1), T(1));
    }
    T sn = std::sqrt(std::max(T(0), T(1) - c * c));
    T ph = T(2) * T(PI_D) * u1;
    V3<T> t = std::fabs(d.x) > T(0.9) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
    V3<T> b1 = normalize(cross(t, d));
    V3<T> b2 = cross(d, b1);
    return normalize(b1 * (std::cos(ph) * sn) + b2 * (std::sin(ph) * sn) + d * c);
}

// the environment from a point in the air (haze.js:296-310 envSampleDirM / envPdfM): the sun's cone, else the sphere
template <class T> inline V3<T> env_sample_dir_m(const Env<T>& e, T pick, T u0, T u1) {
    if (pick < e.pick) return e.sample_sun_cone(u0, u1);
    if (e.mshare > T(0) && (pick - e.pick) / std::max(T(1) - e.pick, T(1e-6)) < e.mshare) return e.map_sample(u0, u1);
    T z = T(1) - T(2) * u0;
    T s = std::sqrt(std::max(T(0), T(1) - z * z));
    T ph = T(2) * T(PI_D) * u1;
    return V3<T>(s * std::cos(ph), s * std::sin(ph), z);
}
template <class T> inline T env_pdf_m(const Env<T>& e, const V3<T>& L) {
    T pSun = e.in_sun_disc(L) ? T(1) / e.sun_omega : T(0);
    const T pm = e.mshare > T(0) ? e.mshare * e.map_pdf(L) : T(0);
    return e.pick * pSun + (T(1) - e.pick) * (pm + (T(1) - e.mshare) / (T(4) * T(PI_D)));
}

// THE BOX (haze.js:64-80 hazeUniforms, :222-252 hazeSlab / hazeSpan / hazeTr, :255-273 hazeDraw)
template <class T> struct HazeBox {
    bool on = false;
    V3<T> c, u, v, w, albedo;
    T hu, hv, hw, sigma, g;
    void init(const st_scene_desc& s) {
        on = s.haze_sigma_t > 0;
        c = V3<T>(T(s.haze_centre[0]), T(s.haze_centre[1]), T(s.haze_centre[2]));
        u = V3<T>(T(s.haze_axes[0]), T(s.haze_axes[1]), T(s.haze_axes[2]));
        v = V3<T>(T(s.haze_axes[3]), T(s.haze_axes[4]), T(s.haze_axes[5]));
        w = V3<T>(T(s.haze_axes[6]), T(s.haze_axes[7]), T(s.haze_axes[8]));
        hu = T(s.haze_half[0]); hv = T(s.haze_half[1]); hw = T(s.haze_half[2]);
        sigma = T(s.haze_sigma_t);
        albedo = V3<T>(T(sat(s.haze_albedo[0])), T(sat(s.haze_albedo[1])), T(sat(s.haze_albedo[2])));
        g = clampT(T(s.haze_g), T(-0.95), T(0.95));
    }
    static void slab(T o, T dd, T h, T& t0, T& t1) {
        if (std::fabs(dd) < T(1e-12)) { if (std::fabs(o) > h) { t0 = T(1); t1 = T(0); } return; }
        T a = (-h - o) / dd, b = (h - o) / dd;
        t0 = std::max(t0, std::min(a, b));
        t1 = std::min(t1, std::max(a, b));
    }
    // [t0, t1] of A + d t, t in [0, len], inside the box and the scene's radius R; t1 <= t0 when none
    void span(const V3<T>& A, const V3<T>& d, T len, T R, T& t0, T& t1) const {
        V3<T> o = A - c;
        t0 = T(0); t1 = len;
        slab(dot(o, u), dot(d, u), hu, t0, t1);
        slab(dot(o, v), dot(d, v), hv, t0, t1);
        slab(dot(o, w), dot(d, w), hw, t0, t1);
        T b = dot(A, d);
        T disc = b * b - (dot(A, A) - R * R);
        if (disc <= T(0)) { t0 = T(1); t1 = T(0); return; }
        T s = std::sqrt(disc);
        t0 = std::max(t0, -b - s);
        t1 = std::min(t1, -b + s);
    }
    T transmittance(const V3<T>& A, const V3<T>& d, T len, T R) const {
        if (!on) return T(1);
        T t0, t1;
        span(A, d, len, R, t0, t1);
        if (t1 <= t0) return T(1);
        return std::exp(-sigma * (t1 - t0));
    }
    // the leg's collision as it starts (hazeDraw), the leg from A (its vertex, where ltot was absLtot): the ltot at
    // which it meets a particle, or -1 for none on this leg
    T draw(const V3<T>& A, const V3<T>& dir, T absLtot, T n, T R, Rng& rng) const {
        if (!on || std::fabs(n - T(1)) > T(1e-3)) return T(-1);
        T t0, t1;
        span(A, dir, T(1e30), R, t0, t1);
        if (t1 <= t0) return T(-1);
        T u[4]; rng.next4(u);
        T t = t0 - std::log(T(1) - u[0]) / sigma;
        return t < t1 ? std::max(absLtot + t * n, T(1e-30)) : T(-1);
    }
};
template <class T> inline bool haze_arrived(T tmax, T ltot) { return tmax > T(0) && ltot >= tmax; }

}  // namespace sto
