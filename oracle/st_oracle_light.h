// TEST INFRASTRUCTURE ONLY -- the oracle's restatement of the lights' faces (builder/lights.js, the builder's light
// object; core/scene_api.js:259-289 lightFaceArea, lightFaceShare, lightFaceDensity; tracebasics.js:1268
// lightFaceLe; lights.js:209-228 beamOf / beamShape; materials_pbr.js:1244-1268 the point aimed at; haze.js:315-350
// from the air; builder/codegen.js:795-836 a face's hit and its MIS weight). In double where the library computes in
// float; the faces' frames made orthonormal and drawn as sheets appended to the primitives, as the library does.
#pragma once
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../include/shadytracer.h"

namespace sto {

const double FACE_SHARE = 0.5;            // FACE_NEE_SHARE (tracebasics.js:279)

struct OFace {
    double c[3], u[3], v[3], n[3], le[3];
    double hw, hh, beam_cos, expo;        // expo < 0: even intensity
    uint32_t shape;
};

// the faces of a scene and the sheets that draw them (a rectangle a box of no thickness, a disc a cylinder of none,
// their rotation rows u, v, n); false with a reason for a face the library would refuse
inline bool build_faces(const st_scene_desc& s, std::vector<st_prim>& prims, std::vector<OFace>& faces,
                        uint8_t* face_of, std::string& why) {
    for (int i = 0; i < ST_MAX_MATERIALS; i++) face_of[i] = 0;
    const uint32_t nl = s.lights ? s.n_lights : 0u;
    if (nl > ST_MAX_LIGHTS || prims.size() + nl > ST_MAX_PRIMS) { why = "too many lights"; return false; }
    for (uint32_t i = 0; i < nl; i++) {
        const st_light& L = s.lights[i];
        if ((L.shape != ST_LIGHT_DISC && L.shape != ST_LIGHT_RECTANGLE) || L.material == 0 ||
            L.material >= s.n_materials || face_of[L.material] || !(L.half_w > 0.f) ||
            (L.shape == ST_LIGHT_RECTANGLE && !(L.half_h > 0.f))) { why = "bad light"; return false; }
        OFace f;
        double lu = 0, lv = 0, uv = 0;
        for (int k = 0; k < 3; k++) { f.u[k] = L.u[k]; lu += f.u[k] * f.u[k]; }
        lu = std::sqrt(lu);
        for (int k = 0; k < 3; k++) { f.u[k] /= lu; uv += f.u[k] * L.v[k]; }
        for (int k = 0; k < 3; k++) { f.v[k] = L.v[k] - uv * f.u[k]; lv += f.v[k] * f.v[k]; }
        lv = std::sqrt(lv);
        for (int k = 0; k < 3; k++) f.v[k] /= lv;
        f.n[0] = f.u[1] * f.v[2] - f.u[2] * f.v[1];
        f.n[1] = f.u[2] * f.v[0] - f.u[0] * f.v[2];
        f.n[2] = f.u[0] * f.v[1] - f.u[1] * f.v[0];
        for (int k = 0; k < 3; k++) { f.c[k] = L.centre[k]; f.le[k] = L.le[k]; }
        f.hw = L.half_w;
        f.hh = L.shape == ST_LIGHT_DISC ? L.half_w : L.half_h;
        f.beam_cos = L.beam_cos;
        f.expo = L.dist == ST_LIGHT_UNIFORM ? -1.0 : (double)L.n;
        f.shape = L.shape;
        faces.push_back(f);
        face_of[L.material] = (uint8_t)(i + 1);
        st_prim p{};
        p.type = L.shape == ST_LIGHT_DISC ? ST_PRIM_CYLINDER : ST_PRIM_BOX;
        p.op = ST_OP_ITEM;
        p.material = L.material;
        for (int k = 0; k < 3; k++) {
            p.pos[k] = L.centre[k];
            p.rot[k] = (float)f.u[k]; p.rot[3 + k] = (float)f.v[k]; p.rot[6 + k] = (float)f.n[k];
        }
        if (L.shape == ST_LIGHT_DISC) { p.p[0] = 0.f; p.p[1] = L.half_w; }
        else { p.p[0] = L.half_w; p.p[1] = L.half_h; p.p[2] = 0.f; }
        prims.push_back(p);
    }
    return true;
}

inline double face_area(const OFace& f) { return f.shape == ST_LIGHT_DISC ? M_PI * f.hw * f.hw : 4.0 * f.hw * f.hh; }
// lightBeam: the radiance at cosT from the face's normal over its luminance straight out
inline double face_beam(const OFace& f, double cosT) {
    if (cosT < f.beam_cos || cosT <= 0.0) return 0.0;
    const double c = std::max(cosT, 1e-4);
    if (f.expo < 0.0) return 1.0 / c;
    return f.expo == 1.0 ? 1.0 : std::pow(c, f.expo - 1.0);
}
// lightFaceDensity: the share, 1 / n faces, 1 / area, area to solid angle
inline double face_density(double share, size_t nf, const OFace& f, double dist, double cosY) {
    if (share <= 0.0 || nf == 0) return 0.0;
    return share / (double)nf * dist * dist / std::max(face_area(f) * std::fabs(cosY), 1e-20);
}
inline void face_point(const OFace& f, double ux, double uy, double* out) {
    if (f.shape == ST_LIGHT_DISC) {
        const double rr = f.hw * std::sqrt(ux), ph = 2.0 * M_PI * uy;
        for (int k = 0; k < 3; k++) out[k] = f.c[k] + (f.u[k] * std::cos(ph) + f.v[k] * std::sin(ph)) * rr;
        return;
    }
    for (int k = 0; k < 3; k++) out[k] = f.c[k] + f.u[k] * ((2.0 * ux - 1.0) * f.hw) + f.v[k] * ((2.0 * uy - 1.0) * f.hh);
}

}  // namespace sto
