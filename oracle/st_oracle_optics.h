// TEST INFRASTRUCTURE ONLY -- the oracle's optics bench (optics/kernels.js, optics/farfield.js, optics/illum.js):
// source sampling, the trace's per-interaction tallies, the far field's binning and its intensity, the lux plane.
// Restated from the reference; never part of the product.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>
#include "st_oracle_render.h"

namespace sto {

// THE FAR FIELD'S BIN (kernels.js:251-272 optFarAdd, farfield.js:45-54 farBin), in f32 as the kernel bins it:
// gamma from the axis, C about it from c0, counter-clockwise seen from where the light shines; nG gamma bins centred
// on 0 .. 180 degrees, nC C bins centred on 0, 360/nC, ...
inline uint32_t far_bin(const float* d, const float* ax, const float* c0, uint32_t nC, uint32_t nG) {
    float c90[3] = {ax[1] * c0[2] - ax[2] * c0[1], ax[2] * c0[0] - ax[0] * c0[2], ax[0] * c0[1] - ax[1] * c0[0]};
    float l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    float dn[3] = {d[0] / l, d[1] / l, d[2] / l};
    float ca = dn[0] * ax[0] + dn[1] * ax[1] + dn[2] * ax[2];
    float g = std::acos(std::min(1.f, std::max(-1.f, ca)));
    float c = std::atan2(dn[0] * c90[0] + dn[1] * c90[1] + dn[2] * c90[2], dn[0] * c0[0] + dn[1] * c0[1] + dn[2] * c0[2]);
    if (c < 0.f) c += 6.28318530718f;
    uint32_t ig = std::min((uint32_t)(g / 3.14159265359f * (float)(nG - 1) + 0.5f), nG - 1);
    uint32_t ic = (uint32_t)(c / 6.28318530718f * (float)nC + 0.5f) % nC;
    return ig * nC + ic;
}
// each gamma row's solid angle per C bin (farfield.js:33-41 farGeometry)
inline void far_geometry(uint32_t nC, uint32_t nG, double* omega) {
    const double RAD = PI_D / 180, dG = 180.0 / (nG - 1);
    for (uint32_t j = 0; j < nG; j++) {
        double lo = std::max(0.0, (j - 0.5) * dG) * RAD, hi = std::min(180.0, (j + 0.5) * dG) * RAD;
        omega[j] = (2 * PI_D / nC) * (std::cos(lo) - std::cos(hi));
    }
}
// luminous intensity per bin (farfield.js:63-85 intensity, symmetry 'none'): flux over the bin's solid angle, the
// two caps pooled over every C
inline void far_intensity(const double* flux, uint32_t nC, uint32_t nG, double* I) {
    std::vector<double> om(nG);
    far_geometry(nC, nG, om.data());
    for (uint32_t j = 0; j < nG; j++) {
        if (j == 0 || j == nG - 1) {
            double f = 0;
            for (uint32_t i = 0; i < nC; i++) f += flux[j * nC + i];
            for (uint32_t i = 0; i < nC; i++) I[j * nC + i] = f / (om[j] * nC);
        } else {
            for (uint32_t i = 0; i < nC; i++) I[j * nC + i] = flux[j * nC + i] / om[j];
        }
    }
}

// A SOURCE'S RAY (kernels.js:299-408 optSourceRay): the source by flux, a point on it, the side, the direction from
// the distribution, stepped two march tolerances off the sheet when the source is geometry. `cdf` is each source's
// cumulative share. Returns the ray's origin and direction.
// the ray table a ray set reads (8 floats a ray: position, weight, direction, wavelength), for the runs that follow
inline std::vector<float>& optics_rays() { static std::vector<float> r; return r; }
template <class T>
inline void source_ray(const st_optics_source* src, const float* cdf, uint32_t nsrc, Rng& rng, T tol,
                       V3<T>& org, V3<T>& dir, uint32_t& which, T& w) {
    T pick[4]; rng.next4(pick);
    uint32_t k = 0;
    for (uint32_t i = 0; i < nsrc; i++) { k = i; if (pick[0] <= T(cdf[i])) break; }
    which = k;
    const st_optics_source& s = src[k];
    w = T(1);
    if (s.shape == 3) {                                     // a ray set (kernels.js:320-336): one of its rays, weighted
        const std::vector<float>& R = optics_rays();
        const uint32_t cnt = std::max(s.ray_count, 1u);
        T u[4]; rng.next4(u);
        const uint32_t j = s.ray_first + std::min((uint32_t)(float)(u[0] * T(cnt)), cnt - 1u);
        const float* r = &R[(size_t)j * 8];
        org = V3<T>(T(r[0]), T(r[1]), T(r[2]));
        dir = normalize(V3<T>(T(r[4]), T(r[5]), T(r[6])));
        w = T(r[3]);
        return;
    }
    V3<T> front = normalize(V3<T>(T(s.axis[0]), T(s.axis[1]), T(s.axis[2])));
    V3<T> t0(T(s.tangent[0]), T(s.tangent[1]), T(s.tangent[2]));
    V3<T> tu = normalize(t0 - front * dot(t0, front));
    V3<T> tv = cross(front, tu);
    T u[4]; rng.next4(u);
    V3<T> p(T(s.centre[0]), T(s.centre[1]), T(s.centre[2]));
    if (s.shape == 1) {
        T r = T(s.size_x) * std::sqrt(u[0]);
        T ph = T(6.28318530718) * u[1];
        p += (tu * std::cos(ph) + tv * std::sin(ph)) * r;
    } else if (s.shape == 2) {
        p += tu * ((T(2) * u[0] - T(1)) * T(s.size_x)) + tv * ((T(2) * u[1] - T(1)) * T(s.size_y));
    }
    V3<T> axis = front;
    if (s.two_sided && pick[1] < T(0.5)) axis = -front;
    T u2[4]; rng.next4(u2);
    T c = T(1);
    if (s.dist == 1) c = T(1) - u2[0] * (T(1) - T(s.cos_half));
    else if (s.dist == 2) {
        T e = T(s.n_exp) + T(1);
        T lo = std::pow(std::max(T(s.cos_half), T(0)), e);
        c = std::pow(T(1) - u2[0] * (T(1) - lo), T(1) / e);
    }
    T sn = std::sqrt(std::max(T(0), T(1) - c * c));
    T ph2 = T(6.28318530718) * u2[1];
    dir = normalize(tu * (sn * std::cos(ph2)) + tv * (sn * std::sin(ph2)) + axis * c);
    T off = s.on_surface ? T(2) * march_tol(p, tol) : T(0);
    org = p + axis * off;
}

}  // namespace sto
