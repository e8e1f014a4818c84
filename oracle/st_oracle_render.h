// TEST INFRASTRUCTURE ONLY -- the oracle's path tracer: scene SDF fold, environment, GGX/Fresnel lobes, next-event
// estimation with MIS, march, occlusion, resolve. Restates the reference (lampmaker/ShadyTracer v0.88.0) file:line
// by file:line; the product never includes or links this.
#pragma once
#include "st_oracle_core.h"
#include "st_oracle_spectral.h"
#include "../include/shadytracer.h"

namespace sto {

// ------------------------------------------------------------------------------------------------------------
// DERIVED UNIFORMS in double precision -- core/photometry.js:55-73 sunCone/discLuminance, :182-237 derive
// ------------------------------------------------------------------------------------------------------------
// THE ENVIRONMENT IMAGE (envimage.js) and the map light sampling draws from (envmap.js), set for every render that
// follows (sto_set_env_image): the pixels (rgb, top row first), the cd/m^2 of a unit, the turn, the map's tables
const int ENV_MW = 512, ENV_MH = 256;
struct EnvImage {
    std::vector<float> rgb;
    uint32_t w = 0, h = 0;
    double lum = 179.0, turn = 0.0;
    std::vector<float> tex;                 // ENV_MW x ENV_MH x 4, as the library's
    bool on() const { return w > 0; }
};
inline EnvImage& env_image_state() { static EnvImage e; return e; }
// envImage (envimage.js:33-52 and its JS twin envImageAt): bilinear, wrapping across the seam, clamped at the poles
inline void env_image_at(const EnvImage& im, double dx, double dy, double dz, double* out) {
    const double n = std::sqrt(dx * dx + dy * dy + dz * dz);
    dx /= n; dy /= n; dz /= n;
    const int w = (int)im.w, h = (int)im.h;
    double a = 0.5 - std::atan2(dy, dx) / (2.0 * PI_D) + im.turn / 360.0;
    a -= std::floor(a);
    const double u = a * w - 0.5, v = std::acos(std::min(1.0, std::max(-1.0, dz))) / PI_D * h - 0.5;
    const double x0 = std::floor(u), y0 = std::floor(v), fx = u - x0, fy = v - y0;
    const int xa = (((int)x0 % w) + w) % w, xb = (xa + 1) % w;
    const int ya = std::min(std::max((int)y0, 0), h - 1), yb = std::min(std::max((int)y0 + 1, 0), h - 1);
    for (int c = 0; c < 3; c++) {
        auto px = [&](int x, int y) { return (double)im.rgb[((size_t)y * w + x) * 3 + c]; };
        const double top = px(xa, ya) * (1 - fx) + px(xb, ya) * fx, bot = px(xa, yb) * (1 - fx) + px(xb, yb) * fx;
        out[c] = std::max(0.0, top * (1 - fy) + bot * fy) * im.lum;
    }
}
// envSampling (envmap.js:215-260): the texels' weights (luminance plus a floor of 1e-3 of the mean), the CDFs
inline void env_tables(const std::vector<double>& lum, std::vector<float>& tex) {
    const int W = ENV_MW, H = ENV_MH, N = W * H;
    double sum = 0;
    for (int i = 0; i < N; i++) sum += (lum[i] > 0 && std::isfinite(lum[i])) ? lum[i] : 0.0;
    const double mean = sum / N, fl = mean > 0 ? 1e-3 * mean : 1.0;
    std::vector<double> w(N);
    double total = 0;
    for (int i = 0; i < N; i++) { w[i] = ((lum[i] > 0 && std::isfinite(lum[i])) ? lum[i] : 0.0) + fl; total += w[i]; }
    tex.assign((size_t)N * 4, 0.f);
    double below = 0;
    for (int row = 0; row < H; row++) {
        double rs = 0, along = 0;
        for (int x = 0; x < W; x++) rs += w[row * W + x];
        const double rc = row == H - 1 ? 1.0 : (below + rs) / total;
        for (int x = 0; x < W; x++) {
            const int i = row * W + x;
            along += w[i];
            tex[4 * i] = x == W - 1 ? 1.f : (float)(along / rs);
            tex[4 * i + 1] = (float)(w[i] / total * (N / (4.0 * PI_D)));
            tex[4 * i + 2] = (float)rc;
        }
        below += rs;
    }
}

// THE SUN AND SKY'S BANDS (environment.js SKY_BAND_TABLE), in double: 16 bands of 380-730 nm sampled at every
// nanometre from each band's start, sunlight above the air (Planck, 5778 K) times the CIE 1931 functions (the
// Wyman-Sloan-Shirley fit, as the spectral table's) to linear Rec.709, the sixteen scaled to luminance 1 together;
// each band's middle (weighted by x + y + z), its Rayleigh depth there (Hansen & Travis 1974 eq. 2.29), Angstrom's
// aerosol factor (l / 550)^-1.3 and the ozone's depth (the Chappuis band's 223 K cross-section, 300 Dobson units)
struct SkyBand { double tauR, haze, ozone, nm, rgb[3]; };
inline std::vector<SkyBand> sky_bands_build() {
    std::vector<SkyBand> bands;
    static const double sigma[16] = {6.2648e-24, 3.1169e-23, 1.0195e-22, 2.4886e-22, 5.4883e-22, 1.1517e-21, 2.0211e-21,
                                     3.0497e-21, 4.2480e-21, 4.5252e-21, 4.7153e-21, 3.4726e-21, 2.3885e-21, 1.5936e-21,
                                     9.8370e-22, 6.3061e-22};
    auto lobe = [](double l, double mu, double lo, double hi) {
        const double t = (l - mu) / (l < mu ? lo : hi);
        return std::exp(-0.5 * t * t);
    };
    const double step = 350.0 / 16.0;
    double tot[3] = {0, 0, 0};
    for (int k = 0; k < 16; k++) {
        double X = 0, Y = 0, Z = 0, wl = 0, ws = 0;
        for (double l = 380.0 + k * step; l < 380.0 + (k + 1) * step; l += 1.0) {
            const double li = std::round(l), m = l * 1e-9;
            const double w = 1.0 / (std::pow(m, 5) * (std::exp(1.438776877e-2 / (m * 5778.0)) - 1.0));
            const double x = 1.056 * lobe(li, 599.8, 37.9, 31.0) + 0.362 * lobe(li, 442.0, 16.0, 26.7) -
                             0.065 * lobe(li, 501.1, 20.4, 26.2);
            const double y = 0.821 * lobe(li, 568.8, 46.9, 40.5) + 0.286 * lobe(li, 530.9, 16.3, 31.1);
            const double z = 1.217 * lobe(li, 437.0, 11.8, 36.0) + 0.681 * lobe(li, 459.0, 26.0, 13.8);
            X += w * x; Y += w * y; Z += w * z;
            wl += w * (x + y + z) * l; ws += w * (x + y + z);
        }
        SkyBand b;
        b.nm = wl / ws;
        const double um = b.nm / 1000.0;
        b.tauR = 0.008569 * std::pow(um, -4.0) * (1 + 0.0113 * std::pow(um, -2.0) + 0.00013 * std::pow(um, -4.0));
        b.haze = std::pow(b.nm / 550.0, -1.3);
        b.ozone = sigma[k] * 300.0 * 2.6867e16;
        b.rgb[0] = 3.2404542 * X - 1.5371385 * Y - 0.4985314 * Z;
        b.rgb[1] = -0.9692660 * X + 1.8760108 * Y + 0.0415560 * Z;
        b.rgb[2] = 0.0556434 * X - 0.2040259 * Y + 1.0572252 * Z;
        for (int c = 0; c < 3; c++) tot[c] += b.rgb[c];
        bands.push_back(b);
    }
    const double Yt = LUMA_R * tot[0] + LUMA_G * tot[1] + LUMA_B * tot[2];
    for (auto& b : bands)
        for (int c = 0; c < 3; c++) b.rgb[c] /= Yt;
    return bands;
}
// built once, by whichever thread asks first (a function-local static is initialised exactly once, under a lock: the
// presets' texture asks from many threads at once)
inline const std::vector<SkyBand>& sky_bands() {
    static const std::vector<SkyBand> bands = sky_bands_build();
    return bands;
}
// Kasten-Young relative air mass (sdf.js:96-100)
inline double air_mass(double cz) {
    const double c = std::min(std::max(cz, 0.0), 1.0);
    const double zdeg = std::acos(c) * 180.0 / PI_D;
    return 1.0 / (c + 0.15 * std::pow(std::max(93.885 - zdeg, 0.1), -1.253));
}

struct Derived {
    double sun_half, sun_omc, sun_sin2, sun_omega, disc_lum;
    double sun_tint[3];
    double sun_dir[3];
    int sun_on;
    uint32_t env_mode;
    double nee_sun_pick;
    double tol_setting;        // tolSetting(): eps, else the scene's
    double env_radius;
};
inline Derived derive(const st_params& p, const st_scene_desc& s) {
    Derived d;
    double half = std::max((double)p.sun_diameter, 1e-3) * PI_D / 360.0;         // photometry.js:56
    double sh = std::sin(half / 2);
    d.sun_half = half;
    d.sun_omc = 2 * sh * sh;                                                       // 1 - cos via 2 sin^2(h/2)
    d.sun_sin2 = std::sin(half) * std::sin(half);
    d.sun_omega = 2 * PI_D * d.sun_omc;
    d.disc_lum = (double)p.sun_illuminance / (PI_D * std::sin(half) * std::sin(half));   // photometry.js:73
    const double raw[3] = {1.0, 0.96, 0.9};                                        // photometry.js:43-44 SUN_TINT
    double y = raw[0] * LUMA_R + raw[1] * LUMA_G + raw[2] * LUMA_B;
    for (int i = 0; i < 3; i++) d.sun_tint[i] = raw[i] / y;
    bool furnace = p.env_uniform > 0;
    // the presets (environment.js): an image or the furnace replaces them; the studio has no sun to aim at
    d.env_mode = (furnace || env_image_state().on() || p.env_mode > 2) ? 0u : p.env_mode;
    d.sun_on = (p.sun_hint != 0 && p.sun_elevation * PI_D / 180.0 + half > 0 && !furnace &&          // photometry.js:194
                !env_image_state().on() && d.env_mode != 2) ? 1 : 0;                              // an image: no sun
    d.nee_sun_pick = (d.sun_on && p.env_sun_gain > 0) ? p.nee_sun_pick : 0.0;                        // photometry.js:226
    d.tol_setting = p.eps > 0 ? p.eps : (s.tolerance > 0 ? s.tolerance : 1e-3);                     // photometry.js:141-150
    d.env_radius = s.env_radius > 0 ? s.env_radius : 400.0;                                          // photometry.js:158
    double e = p.sun_elevation * PI_D / 180.0, a = p.sun_azimuth * PI_D / 180.0;                      // sdf.js:74-78
    d.sun_dir[0] = std::cos(e) * std::sin(a); d.sun_dir[1] = std::cos(e) * std::cos(a); d.sun_dir[2] = std::sin(e);
    return d;
}

// ------------------------------------------------------------------------------------------------------------
// THE TOLERANCE -- core/tolerances.js:27-37 marchTol; tracebasics.js:164-165 normalTol, offsetTol
// ------------------------------------------------------------------------------------------------------------
template <class T> inline T march_tol(const V3<T>& p, T setting) {
    T f = T(128.0) * T(1.1920928955078125e-7) * std::max(std::fabs(p.x), std::max(std::fabs(p.y), std::fabs(p.z)));
    return std::max(std::max(setting, T(1e-9)), f);
}

// ------------------------------------------------------------------------------------------------------------
// PRIMITIVES -- core/sdf.js:214-256, :602 Ntorus; core/shapes.js:266-287 prism, :621-660 aspheric lens, :717 extrude
// ------------------------------------------------------------------------------------------------------------
template <class T> inline T sd_box(const V3<T>& p, const V3<T>& b) {
    V3<T> q(std::fabs(p.x) - b.x, std::fabs(p.y) - b.y, std::fabs(p.z) - b.z);
    return length(vmax(q, T(0))) + std::min(std::max(q.x, std::max(q.y, q.z)), T(0));
}
// g2RegularPolygon (shapes.js:266-283): the signed distance in the plane; only .z (the distance) is used here
template <class T> inline T g2_regular_polygon(T qx, T qy, T sides, T R0) {
    const T PI = T(PI_D);
    T n = clampT(std::nearbyint(sides), T(3), T(64));
    T R = std::max(R0, T(0));
    T an = PI / n;
    T a = R * std::cos(an), he = R * std::sin(an);
    T k = std::nearbyint((std::atan2(qy, qx) + T(0.5) * PI) / (T(2) * an));
    T phi = T(-0.5) * PI + T(2) * an * k;
    T nkx = std::cos(phi), nky = std::sin(phi);
    T tkx = -nky, tky = nkx;
    T u = qx * nkx + qy * nky, v = qx * tkx + qy * tky;
    if (u <= a) return u - a;
    T ex = u - a, ey = v - clampT(v, -he, he);
    return std::sqrt(ex * ex + ey * ey);
}
// g2Extrude's distance (shapes.js:717-726)
template <class T> inline T g2_extrude(T pz, T gz, T h) {
    T wz = std::fabs(pz) - h;
    if (gz > T(0) && wz > T(0)) return std::sqrt(gz * gz + wz * wz);
    if (gz > wz) return gz;
    return wz;
}
// the aspheric lens (shapes.js:629-660), its distance bound
template <class T> inline void asph_sag(T r, T c, T k, T a4, T a6, T& sag, T& slope) {
    T r2 = r * r;
    T w = T(1) - (T(1) + k) * c * c * r2;
    T u = std::sqrt(std::max(w, T(1e-4)));
    T poly = r2 * r2 * (a4 + r2 * a6);
    T dpoly = r * r2 * (T(4) * a4 + r2 * (T(6) * a6));
    sag = c * r2 / (T(1) + u) + poly;
    slope = (w >= T(1e-4) ? c * r / u : T(2) * c * r / (T(1) + u)) + dpoly;
}
template <class T> inline T asph_slope_max(T rho, T c, T k, T a4, T a6) {
    T r2 = rho * rho;
    T u = std::sqrt(std::max(T(1) - (T(1) + k) * c * c * r2, T(1e-4)));
    T poly = rho * r2 * (T(4) * std::fabs(a4) + r2 * (T(6) * std::fabs(a6)));
    return std::fabs(c) * rho / u + poly;
}
template <class T> inline T asph_face(const V3<T>& p, T l, T rho, T ht, T R, T k, T a4, T a6, T s) {
    T c = std::fabs(R) > T(1e-9) ? T(1) / R : T(0);
    T sag, slope;
    asph_sag(std::min(l, rho), c, k, a4, a6, sag, slope);
    T m = asph_slope_max(rho, c, k, a4, a6);
    return (s * p.z - ht + sag) / std::sqrt(T(1) + m * m);
}
template <class T> inline T sd_asphere(const V3<T>& p, const float* q) {
    T rho = std::max(T(0.5) * T(q[0]), T(1e-6));
    T l = std::sqrt(p.x * p.x + p.y * p.y);
    T d = l - rho;
    T top = asph_face(p, l, rho, T(0.5) * T(q[1]), T(q[2]), T(q[3]), T(q[4]), T(q[5]), T(1));
    if (top > d) d = top;
    T bot = asph_face(p, l, rho, T(0.5) * T(q[1]), T(q[6]), T(q[7]), T(q[8]), T(q[9]), T(-1));
    if (bot > d) d = bot;
    return d;
}

template <class T> inline T prim_sdf(const st_prim& pr, const V3<T>& pw) {
    V3<T> d = pw - V3<T>(T(pr.pos[0]), T(pr.pos[1]), T(pr.pos[2]));
    V3<T> q(T(pr.rot[0]) * d.x + T(pr.rot[1]) * d.y + T(pr.rot[2]) * d.z,
            T(pr.rot[3]) * d.x + T(pr.rot[4]) * d.y + T(pr.rot[5]) * d.z,
            T(pr.rot[6]) * d.x + T(pr.rot[7]) * d.y + T(pr.rot[8]) * d.z);
    const float* p = pr.p;
    switch (pr.type) {
        case ST_PRIM_PLANE: return q.z;
        case ST_PRIM_SPHERE: return length(q) - T(p[0]);                                            // sdf.js:217
        case ST_PRIM_BOX: return sd_box(q, V3<T>(T(p[0]), T(p[1]), T(p[2])));                       // sdf.js:220
        case ST_PRIM_ROUNDBOX: return sd_box(q, V3<T>(T(p[0]), T(p[1]), T(p[2]))) - T(p[3]);       // sdf.js:224
        case ST_PRIM_TORUS: {                                                                        // sdf.js:602
            T lxy = std::sqrt(q.x * q.x + q.y * q.y);
            T a = lxy - T(p[0]);
            return std::sqrt(a * a + q.z * q.z) - T(p[1]);
        }
        case ST_PRIM_PRISM: {                                                                        // shapes.js:285
            T g = g2_regular_polygon(q.x, q.y, T(p[0]), T(p[1]));
            return g2_extrude(q.z, g, std::max(T(0.5) * T(p[2]), T(0))) - T(p[3]);
        }
        case ST_PRIM_ASPHERE: return sd_asphere(q, p);                                               // shapes.js:651
        case ST_PRIM_CYLINDER: {                                                                     // sdf.js:228
            T lx = std::sqrt(q.x * q.x + q.y * q.y) - T(p[1]);
            T lz = std::fabs(q.z) - T(p[0]);
            T ox = std::max(lx, T(0)), oz = std::max(lz, T(0));
            return std::min(std::max(lx, lz), T(0)) + std::sqrt(ox * ox + oz * oz);
        }
    }
    return T(1e7);
}

// opSmoothUnion (sdf.js:252-256)
template <class T> inline T smooth_union(T d1, T d2, T k) {
    if (!(k > T(0))) return std::min(d1, d2);
    T h = clampT(T(0.5) + T(0.5) * (d2 - d1) / k, T(0), T(1));
    return mixT(d2, d1, h) - k * h * (T(1) - h);
}

// THE FOLD (core/scene_api.js:28-80 add_new / fold; emptyHit :93): the surface is the item of least |d|, the
// medium the item the point is least deep inside (material 0 -- the air -- when none).
template <class T> struct SceneHit { T d; uint32_t m; uint32_t a; T insideW; uint32_t item; };
// item: the first primitive of the item the surface answered from (the object, the optics tallies' tag)
template <class T> inline SceneHit<T> scene_eval(const st_scene_desc& s, const V3<T>& p) {
    SceneHit<T> H{T(1e7), 0u, 0u, T(-1e7), 0u};
    uint32_t i = 0;
    while (i < s.n_prims) {
        const st_prim& pi = s.prims[i];
        T di = prim_sdf(pi, p);
        uint32_t mat = pi.material;
        T near = std::fabs(di);
        uint32_t j = i + 1;
        while (j < s.n_prims && s.prims[j].op != ST_OP_ITEM) {
            const st_prim& pj = s.prims[j];
            T dj = prim_sdf(pj, p);
            if (pj.op == ST_OP_SMOOTH) di = smooth_union(di, dj, T(pj.k));
            else if (pj.op == ST_OP_UNION) di = std::min(di, dj);
            else di = std::max(di, -dj);
            if (pj.op != ST_OP_SUB && std::fabs(dj) < near) { near = std::fabs(dj); mat = pj.material; }
            j++;
        }
        if (di < T(0) && di > H.insideW) { H.insideW = di; H.a = mat; }
        if (std::fabs(di) < std::fabs(H.d)) { H.d = di; H.m = mat; H.item = i; }
        i = j;
    }
    return H;
}

// BOUNDING-BOX CULLING AT THE ROOT (builder/codegen.js:2141-2193, ONLY THE DEAR ONES; scene_api.js:288-305 cullDist,
// cullMargin): each top-level node that is not one plain shape -- here an item with a CSG chain -- is first measured
// against its box; farther than the margin (ten surface tolerances), the box's distance stands in for it as a lower
// bound (CULL, the nearest skipped box) and it is not evaluated; the fold's |d| is then held to CULL
// (codegen.js:2350). A plain shape (an item of one primitive) is never boxed: its box test costs what it does. The
// box: the members' bounding spheres (a subtraction adds nothing), widened by the largest smooth-union radius / 4
// (the most a polynomial smooth union bulges past its members); none where a member has no bound (a plane, a lens).
struct CullBox { uint32_t first, end; bool boxed; double lo[3], hi[3]; };
inline std::vector<CullBox> cull_boxes(const st_scene_desc& s) {
    std::vector<CullBox> out;
    uint32_t i = 0;
    while (i < s.n_prims) {
        CullBox b{i, i + 1, false, {1e300, 1e300, 1e300}, {-1e300, -1e300, -1e300}};
        while (b.end < s.n_prims && s.prims[b.end].op != ST_OP_ITEM) b.end++;
        bool bounded = true;
        double kmax = 0.0;
        for (uint32_t j = b.first; j < b.end; j++) {
            const st_prim& q = s.prims[j];
            if (j > b.first && q.op == ST_OP_SUB) continue;
            if (q.op == ST_OP_SMOOTH) kmax = std::max(kmax, (double)q.k);
            const float* r = q.p;
            double R;
            switch (q.type) {
                case ST_PRIM_SPHERE: R = std::fabs(r[0]); break;
                case ST_PRIM_BOX: R = std::sqrt(double(r[0]) * r[0] + double(r[1]) * r[1] + double(r[2]) * r[2]); break;
                case ST_PRIM_ROUNDBOX:
                    R = std::sqrt(double(r[0]) * r[0] + double(r[1]) * r[1] + double(r[2]) * r[2]) + std::fabs(r[3]);
                    break;
                case ST_PRIM_TORUS: R = std::fabs(r[0]) + std::fabs(r[1]); break;
                case ST_PRIM_PRISM: R = std::sqrt(double(r[1]) * r[1] + 0.25 * double(r[2]) * r[2]) + std::fabs(r[3]); break;
                case ST_PRIM_CYLINDER: R = std::sqrt(double(r[0]) * r[0] + double(r[1]) * r[1]); break;
                default: R = -1.0;
            }
            if (R < 0.0) { bounded = false; break; }
            for (int k = 0; k < 3; k++) {
                b.lo[k] = std::min(b.lo[k], (double)q.pos[k] - R);
                b.hi[k] = std::max(b.hi[k], (double)q.pos[k] + R);
            }
        }
        b.boxed = bounded && b.end - b.first > 1;
        for (int k = 0; k < 3; k++) { b.lo[k] -= 0.25 * kmax + 1e-6; b.hi[k] += 0.25 * kmax + 1e-6; }
        out.push_back(b);
        i = b.end;
    }
    return out;
}
// the distance alone, as the reference's culled render copy folds it (the march's and the shadow rays' question)
template <class T> inline T scene_dist_culled(const st_scene_desc& s, const std::vector<CullBox>& boxes, const V3<T>& p,
                                              T margin) {
    T best = T(1e7), cull = T(1e7);
    for (const CullBox& b : boxes) {
        if (b.boxed) {                                                      // cullDist (scene_api.js:297-301)
            const T cx = T(0.5) * (T(b.lo[0]) + T(b.hi[0])), cy = T(0.5) * (T(b.lo[1]) + T(b.hi[1]));
            const T cz = T(0.5) * (T(b.lo[2]) + T(b.hi[2]));
            const T dx = std::fabs(p.x - cx) - T(0.5) * (T(b.hi[0]) - T(b.lo[0]));
            const T dy = std::fabs(p.y - cy) - T(0.5) * (T(b.hi[1]) - T(b.lo[1]));
            const T dz = std::fabs(p.z - cz) - T(0.5) * (T(b.hi[2]) - T(b.lo[2]));
            const T ox = std::max(dx, T(0)), oy = std::max(dy, T(0)), oz = std::max(dz, T(0));
            const T bd = std::sqrt(ox * ox + oy * oy + oz * oz) + std::min(std::max(dx, std::max(dy, dz)), T(0));
            if (bd > margin) { cull = std::min(cull, bd); continue; }
        }
        T di = prim_sdf(s.prims[b.first], p);
        for (uint32_t j = b.first + 1; j < b.end; j++) {
            const st_prim& pj = s.prims[j];
            T dj = prim_sdf(pj, p);
            if (pj.op == ST_OP_SMOOTH) di = smooth_union(di, dj, T(pj.k));
            else if (pj.op == ST_OP_UNION) di = std::min(di, dj);
            else di = std::max(di, -dj);
        }
        if (std::fabs(di) < std::fabs(best)) best = di;
    }
    if (cull < std::fabs(best)) best = cull;
    return best;
}

// ------------------------------------------------------------------------------------------------------------
// THE ENVIRONMENT -- core/sdf.js:70-160 (inSunDisc, envBase, skyRadiance, sampleSunCone, envRadiance,
// skyLuminance). The environment's code (core/environment.js: "THE ENVIRONMENT IS CODE") is the scene's: here a
// sun disc of the set illuminance (photometry.js discLuminance, SUN_TINT) over a uniform sky above the horizon and
// a uniform ground below it; env_uniform > 0 is the white-furnace environment (sdf.js:124-127).
// ------------------------------------------------------------------------------------------------------------
template <class T> struct Env {
    V3<T> sun_dir; T sun_sin2, sun_omc, sun_omega; int sun_on; T pick;
    V3<T> disc; T sky, ground, uniform, sun_gain, sky_gain;
    const EnvImage* img = nullptr;          // the environment image, and its map's share of the samples
    const std::vector<float>* tex = nullptr; // the map's tables: the image's, or a preset's
    const std::vector<float>* cache = nullptr;   // a preset in a texture (envCache): rgb, cache_w x cache_h
    uint32_t cache_w = 0, cache_h = 0;
    T mshare = 0;
    // the presets: the mode, the sun and sky's light above the air and aerosol depth at 550 nm; the studio's L0, top
    // and colour
    uint32_t mode = 0;
    double sun_outside = 128000.0, aerosol = 0.12, st_l0 = 0.0, st_top = 0.0, st_tint[3] = {1, 1, 1};
    void init(const st_params& p, const Derived& d, const std::vector<float>* preset_tex = nullptr) {
        const EnvImage& im = env_image_state();
        img = im.on() ? &im : nullptr;
        mode = d.env_mode;
        sun_outside = p.sun_outside > 0.f ? p.sun_outside : 128000.0;
        aerosol = 0.05 + 0.1 * std::max(0.0, (double)p.sky_turbidity);
        st_top = std::min(std::max((double)p.studio_top, 0.0), 1.0);
        double c[3] = {std::max(0.0, (double)p.studio_color[0]), std::max(0.0, (double)p.studio_color[1]),
                       std::max(0.0, (double)p.studio_color[2])};
        const double yc = std::max(c[0] * LUMA_R + c[1] * LUMA_G + c[2] * LUMA_B, 1e-6);
        for (int k = 0; k < 3; k++) st_tint[k] = c[k] / yc;
        st_l0 = std::max(0.0, (double)p.studio_illuminance) / (PI_D * (1.0 + 2.0 * st_top / 3.0));
        tex = img ? &im.tex : (mode != 0 ? preset_tex : nullptr);
        mshare = (tex && !p.env_map_off) ? T(0.5) : T(0);
        sun_dir = V3<T>(T(d.sun_dir[0]), T(d.sun_dir[1]), T(d.sun_dir[2]));
        sun_sin2 = T(d.sun_sin2); sun_omc = T(d.sun_omc); sun_omega = T(d.sun_omega); sun_on = d.sun_on;
        pick = T(d.nee_sun_pick);
        disc = V3<T>(T(d.disc_lum * d.sun_tint[0]), T(d.disc_lum * d.sun_tint[1]), T(d.disc_lum * d.sun_tint[2]));
        sky = T(p.sky_luminance); ground = T(p.ground_luminance); uniform = T(p.env_uniform);
        sun_gain = T(std::max(0.f, p.env_sun_gain)); sky_gain = T(std::max(0.f, p.env_sky_gain));
    }
    V3<T> sky_only(const V3<T>& dir) const {                        // sdf.js skyRadiance: nothing in the cone
        if (sun_on && in_sun_disc(dir)) return V3<T>(0);
        return base(dir) * sky_gain;
    }
    // THE SUN AND SKY, PHYSICALLY (environment.js SUNSKY_FN), in double
    V3<T> sun_sky(const V3<T>& d) const {
        const double sz = (double)sun_dir.z, dz = (double)d.z;
        const double mv = air_mass(std::max(dz, 0.0)), ms = air_mass(std::max(sz, 0.0));
        const bool disc_in = in_sun_disc(d) && sz > -std::sqrt((double)sun_sin2);
        const double c = (double)dot(d, sun_dir), g = 0.7;
        const double phR = 3.0 / (16.0 * PI_D) * (1.0 + c * c);
        const double phM = (1.0 - g * g) / (4.0 * PI_D * std::pow(1.0 + g * g - 2.0 * g * c, 1.5));
        const double up = std::min(std::max((sz + 0.05) / 0.05, 0.0), 1.0);
        const double dm = mv - ms;
        double L[3] = {0, 0, 0};
        for (const SkyBand& b : sky_bands()) {
            const double tr = b.tauR, ta = aerosol * b.haze, tau = tr + ta + b.ozone;
            double v;
            if (disc_in) v = std::exp(-tau * ms) / (PI_D * (double)sun_sin2);
            else {
                const double k1 = std::fabs(dm) < 1e-3 ? tau * mv * std::exp(-tau * mv)
                                                       : mv * (std::exp(-tau * ms) - std::exp(-tau * mv)) / dm;
                v = (tr * phR + 0.9 * ta * phM) / tau * k1 * up;
            }
            for (int k = 0; k < 3; k++) L[k] += b.rgb[k] * v;
        }
        return V3<T>(T(std::max(L[0], 0.0) * sun_outside), T(std::max(L[1], 0.0) * sun_outside),
                     T(std::max(L[2], 0.0) * sun_outside));
    }
    // THE STUDIO (environment.js STUDIO_FN)
    V3<T> studio(const V3<T>& d) const {
        const double v = st_l0 * std::max(1.0 + st_top * (double)d.z, 0.0);
        return V3<T>(T(st_tint[0] * v), T(st_tint[1] * v), T(st_tint[2] * v));
    }
    bool in_sun_disc(const V3<T>& dir) const {                       // sdf.js:91-96
        V3<T> L = normalize(dir);
        V3<T> c = cross(L, sun_dir);
        return dot(L, sun_dir) > T(0) && dot(c, c) <= sun_sin2;
    }
    bool in_sun_cone(const V3<T>& dir) const { return sun_on && in_sun_disc(dir); }
    V3<T> background(const V3<T>& dir) const {
        if (in_sun_disc(dir)) return disc;
        return V3<T>(dir.z > T(0) ? sky : ground);
    }
    V3<T> image(const V3<T>& dir) const {
        double c[3];
        env_image_at(*img, (double)dir.x, (double)dir.y, (double)dir.z, c);
        return V3<T>(T(c[0]), T(c[1]), T(c[2]));
    }
    // envMapSample / envMapPdf (envmap.js:54-98): a row down column 0's CDF, a column along the row's, a point uniform
    // in (azimuth, z) inside the texel
    V3<T> map_sample(T ux, T uy) const {
        const std::vector<float>& m = *tex;
        auto at = [&](int x, int y, int c) { return (T)m[4 * ((size_t)y * ENV_MW + x) + c]; };
        int lo = 0, hi = ENV_MH - 1;
        while (lo < hi) { int mid = (lo + hi) / 2; if (ux < at(0, mid, 2)) hi = mid; else lo = mid + 1; }
        const int row = lo;
        const T r0 = row > 0 ? at(0, row - 1, 2) : T(0), r1 = at(0, row, 2);
        const T fy = std::min(std::max((ux - r0) / std::max(r1 - r0, T(1e-12)), T(0)), T(0.999999));
        lo = 0; hi = ENV_MW - 1;
        while (lo < hi) { int mid = (lo + hi) / 2; if (uy < at(mid, row, 0)) hi = mid; else lo = mid + 1; }
        const int col = lo;
        const T c0 = col > 0 ? at(col - 1, row, 0) : T(0), c1 = at(col, row, 0);
        const T fx = std::min(std::max((uy - c0) / std::max(c1 - c0, T(1e-12)), T(0)), T(0.999999));
        const T z = T(1) - T(2) * (T(row) + fy) / T(ENV_MH);
        const T phi = T(2) * T(PI_D) * (T(col) + fx) / T(ENV_MW);
        const T sz = std::sqrt(std::max(T(0), T(1) - z * z));
        return V3<T>(sz * std::cos(phi), sz * std::sin(phi), z);
    }
    T map_pdf(const V3<T>& L) const {
        const V3<T> d = normalize(L);
        T a = std::atan2(d.y, d.x) / (T(2) * T(PI_D));
        a -= std::floor(a);
        const int col = std::min(std::max((int)(a * T(ENV_MW)), 0), ENV_MW - 1);
        const int row = std::min(std::max((int)((T(1) - d.z) * T(0.5) * T(ENV_MH)), 0), ENV_MH - 1);
        return (T)(*tex)[4 * ((size_t)row * ENV_MW + col) + 1];
    }
    // THE ENVIRONMENT FROM ITS TEXTURE (envmap.js:162-182 envCacheAt): bilinear, wrapping, clamped at the poles
    V3<T> cache_at(const V3<T>& d) const {
        const int w = (int)cache_w, h = (int)cache_h;
        double a = std::atan2((double)d.y, (double)d.x) / (2.0 * PI_D);
        a -= std::floor(a);
        const double u = a * w - 0.5, v = std::acos(std::min(1.0, std::max(-1.0, (double)d.z))) / PI_D * h - 0.5;
        const double x0 = std::floor(u), y0 = std::floor(v), fx = u - x0, fy = v - y0;
        const int xa = (((int)x0 % w) + w) % w, xb = (xa + 1) % w;
        const int ya = std::min(std::max((int)y0, 0), h - 1), yb = std::min(std::max((int)y0 + 1, 0), h - 1);
        double c[3];
        for (int k = 0; k < 3; k++) {
            auto px = [&](int x, int y) { return (double)(*cache)[((size_t)y * w + x) * 3 + k]; };
            c[k] = (px(xa, ya) * (1 - fx) + px(xb, ya) * fx) * (1 - fy) + (px(xa, yb) * (1 - fx) + px(xb, yb) * fx) * fy;
        }
        return V3<T>(T(c[0]), T(c[1]), T(c[2]));
    }
    V3<T> base(const V3<T>& dir) const {                             // sdf.js:121-130 envBase
        if (img) return image(dir);
        if (uniform > T(0)) return V3<T>(uniform);
        if (cache && !(sun_on && in_sun_disc(dir))) return cache_at(normalize(dir));
        if (mode == 1) return sun_sky(normalize(dir));
        if (mode == 2) return studio(normalize(dir));
        V3<T> c = background(normalize(dir));
        return vmax(c, T(0));
    }
    V3<T> radiance(const V3<T>& dir) const {                         // sdf.js:180-182 envRadiance
        return base(dir) * (in_sun_cone(dir) ? sun_gain : sky_gain);
    }
    V3<T> sample_sun_cone(T u0, T u1) const {                        // sdf.js:149-160
        const V3<T>& sd = sun_dir;
        T omc = u0 * sun_omc;
        T cosT = T(1) - omc;
        T sinT = std::sqrt(std::max(T(0), omc * (T(2) - omc)));
        T phi = T(2) * T(PI_D) * u1;
        V3<T> t = std::fabs(sd.x) > T(0.9) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
        V3<T> b1 = normalize(cross(t, sd));
        V3<T> b2 = cross(sd, b1);
        return normalize(b1 * (std::cos(phi) * sinT) + b2 * (std::sin(phi) * sinT) + sd * cosT);
    }
};
// A PRESET'S MAP (envmap.js:100-150 prog_envbake, as the library bakes it): per texel of the equal-area map the
// environment's own light at 2 x 2 stratified points, the sun's cone left out where there is one, its mean luminance;
// then the tables
// A PRESET'S TEXTURE (envmap.js:186-202 ENV_CACHE_MAIN): a texel the preset's light over 2 x 2 points even in azimuth
// and angle, the sun's cone left out
template <class T> inline std::vector<float> preset_texture(const Env<T>& e, uint32_t w, uint32_t h) {
    std::vector<float> out((size_t)w * h * 3);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)w * h; i++) {
        const double x = (double)(i % w), y = (double)(i / w);
        double acc[3] = {0, 0, 0}, n = 0;
        for (int sy = 0; sy < 2; sy++)
            for (int sx = 0; sx < 2; sx++) {
                const double u = (x + (sx + 0.5) * 0.5) / w, v = (y + (sy + 0.5) * 0.5) / h;
                const double ph = 2 * PI_D * u, th = PI_D * v;
                const V3<T> d(T(std::sin(th) * std::cos(ph)), T(std::sin(th) * std::sin(ph)), T(std::cos(th)));
                if (e.sun_on && e.in_sun_disc(d)) continue;
                const V3<T> c = e.base(d);
                acc[0] += (double)c.x; acc[1] += (double)c.y; acc[2] += (double)c.z; n += 1;
            }
        for (int k = 0; k < 3; k++) out[(size_t)i * 3 + k] = (float)(acc[k] / std::max(n, 1.0));
    }
    return out;
}
template <class T> inline std::vector<float> preset_map(const Env<T>& e) {
    std::vector<double> lum((size_t)ENV_MW * ENV_MH);
    for (int i = 0; i < ENV_MW * ENV_MH; i++) {
        const int x = i % ENV_MW, y = i / ENV_MW;
        double acc = 0;
        for (int sy = 0; sy < 2; sy++)
            for (int sx = 0; sx < 2; sx++) {
                const double ux = (x + (sx + 0.5) * 0.5) / ENV_MW, uy = (y + (sy + 0.5) * 0.5) / ENV_MH;
                const double z = 1 - 2 * uy, sz = std::sqrt(std::max(0.0, 1 - z * z)), ph = 2 * PI_D * ux;
                const V3<T> d(T(sz * std::cos(ph)), T(sz * std::sin(ph)), T(z));
                if (e.sun_on && e.in_sun_disc(d)) continue;
                const V3<T> c = e.base(d);
                acc += LUMA_R * (double)c.x + LUMA_G * (double)c.y + LUMA_B * (double)c.z;
            }
        lum[i] = 0.25 * acc;
    }
    std::vector<float> tex;
    env_tables(lum, tex);
    return tex;
}
// sampleCosineHemi (tracebasics.js:655-665)
template <class T> inline V3<T> sample_cosine_hemi(const V3<T>& n, T u0, T u1) {
    T r = std::sqrt(u0);
    T phi = T(2) * T(PI_D) * u1;
    V3<T> t = std::fabs(n.x) > T(0.9) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
    V3<T> b1 = normalize(cross(t, n));
    V3<T> b2 = cross(n, b1);
    return normalize(b1 * (r * std::cos(phi)) + b2 * (r * std::sin(phi)) + n * std::sqrt(std::max(T(0), T(1) - u0)));
}
// envSampleDir / envPdf (tracebasics.js:670-692), no environment map (envMapShare 0)
template <class T> inline V3<T> env_sample_dir(const Env<T>& e, const V3<T>& n, T pick, T u0, T u1) {
    if (pick < e.pick) return e.sample_sun_cone(u0, u1);
    if (e.mshare > T(0) && (pick - e.pick) / std::max(T(1) - e.pick, T(1e-6)) < e.mshare) return e.map_sample(u0, u1);
    return sample_cosine_hemi(n, u0, u1);
}
template <class T> inline T env_pdf(const Env<T>& e, const V3<T>& L, const V3<T>& n) {
    T pSun = e.in_sun_disc(L) ? T(1) / e.sun_omega : T(0);
    T pCos = std::max(dot(L, n), T(0)) / T(PI_D);
    const T pm = e.mshare > T(0) ? e.mshare * e.map_pdf(L) : T(0);
    return e.pick * pSun + (T(1) - e.pick) * (pm + (T(1) - e.mshare) * pCos);
}
// envSampleDirQ / envPdfQ (materials_pbr.js:1089-1105): a share q of the sky's cosine draw from the far hemisphere
template <class T> inline V3<T> env_sample_dir_q(const Env<T>& e, const V3<T>& n, T pick, T u0, T u1, T q) {
    if (q <= T(0) || pick < e.pick) return env_sample_dir(e, n, pick, u0, u1);
    const T rest = (pick - e.pick) / std::max(T(1) - e.pick, T(1e-6));
    if (rest < e.mshare) return e.map_sample(u0, u1);
    const T pc = (rest - e.mshare) / std::max(T(1) - e.mshare, T(1e-6));
    return sample_cosine_hemi(pc < q ? n * T(-1) : n, u0, u1);
}
template <class T> inline T env_pdf_q(const Env<T>& e, const V3<T>& L, const V3<T>& n, T q) {
    if (q <= T(0)) return env_pdf(e, L, n);
    const T pSun = e.in_sun_disc(L) ? T(1) / e.sun_omega : T(0);
    const T c = dot(L, n);
    const T pCos = ((T(1) - q) * std::max(c, T(0)) + q * std::max(-c, T(0))) / T(PI_D);
    const T pm = e.mshare > T(0) ? e.mshare * e.map_pdf(L) : T(0);
    return e.pick * pSun + (T(1) - e.pick) * (pm + (T(1) - e.mshare) * pCos);
}
// power heuristic (tracebasics.js:695-699)
template <class T> inline T mis_weight(T a, T b) { T a2 = a * a, b2 = b * b; return a2 / std::max(a2 + b2, T(1e-20)); }

// ------------------------------------------------------------------------------------------------------------
// MICROFACET -- core/microfacet.js:72-140 (GGX, Smith, VNDF by spherical caps, exact Fresnel, Schlick) and the
// albedo tables, :143-330 (prog_mf_lut, prog_mf_lut_avg, the isotropic Ec / Ec_avg / E1 and their reads)
// ------------------------------------------------------------------------------------------------------------
const int MF_NMU = 32, MF_NR = 32, MF_NIOR = 16, MF_SQRT_SAMPLES = 32;
const double ALPHA_MIN = 1e-3;
// the two alphas along the local x and y (microfacet.js mfAnisoAlpha); equal, the isotropic formulas exactly
template <class T> struct A2 { T x, y; };
template <class T> inline T mf_lambda(const V3<T>& w, A2<T> a) {
    T z2 = std::max(w.z * w.z, T(1e-12));
    T t2 = (a.x * a.x * w.x * w.x + a.y * a.y * w.y * w.y) / z2;
    return T(0.5) * (T(-1) + std::sqrt(T(1) + t2));
}
template <class T> inline T mf_g1(const V3<T>& w, A2<T> a) { return T(1) / (T(1) + mf_lambda(w, a)); }
template <class T> inline T mf_g2(const V3<T>& o, const V3<T>& i, A2<T> a) { return T(1) / (T(1) + mf_lambda(o, a) + mf_lambda(i, a)); }
template <class T> inline T mf_d(const V3<T>& h, A2<T> a) {
    if (h.z <= T(0)) return T(0);
    T t = (h.x * h.x) / (a.x * a.x) + (h.y * h.y) / (a.y * a.y) + h.z * h.z;
    return T(1) / (T(PI_D) * a.x * a.y * t * t);
}
template <class T> inline V3<T> mf_sample_vndf(const V3<T>& o, A2<T> a, T u0, T u1) {
    V3<T> os = normalize(V3<T>(o.x * a.x, o.y * a.y, o.z));
    T phi = T(2) * T(PI_D) * u0;
    T z = (T(1) - u1) * (T(1) + os.z) - os.z;
    T sinT = std::sqrt(clampT(T(1) - z * z, T(0), T(1)));
    V3<T> c(sinT * std::cos(phi), sinT * std::sin(phi), z);
    V3<T> hs = c + os;
    return normalize(V3<T>(hs.x * a.x, hs.y * a.y, std::max(hs.z, T(1e-7))));
}
template <class T> inline T mf_pdf_reflect(const V3<T>& o, const V3<T>& i, A2<T> a) {
    if (o.z <= T(0) || i.z <= T(0)) return T(0);
    V3<T> h = normalize(o + i);
    return mf_g1(o, a) * mf_d(h, a) / (T(4) * o.z);
}
template <class T> inline T mf_lambda(const V3<T>& w, T a) { return mf_lambda(w, A2<T>{a, a}); }
template <class T> inline T mf_g1(const V3<T>& w, T a) { return mf_g1(w, A2<T>{a, a}); }
template <class T> inline T mf_g2(const V3<T>& o, const V3<T>& i, T a) { return mf_g2(o, i, A2<T>{a, a}); }
template <class T> inline T mf_d(const V3<T>& h, T a) { return mf_d(h, A2<T>{a, a}); }
template <class T> inline V3<T> mf_sample_vndf(const V3<T>& o, T a, T u0, T u1) { return mf_sample_vndf(o, A2<T>{a, a}, u0, u1); }
template <class T> inline T mf_pdf_reflect(const V3<T>& o, const V3<T>& i, T a) { return mf_pdf_reflect(o, i, A2<T>{a, a}); }
template <class T> inline T fresnel_dielectric(T cosI_in, T eta) {
    T cosI = clampT(cosI_in, T(0), T(1));
    T sin2T = eta * eta * (T(1) - cosI * cosI);
    if (sin2T >= T(1)) return T(1);
    T cosT = std::sqrt(T(1) - sin2T);
    T rs = (eta * cosI - cosT) / (eta * cosI + cosT);
    T rp = (cosI - eta * cosT) / (cosI + eta * cosT);
    return T(0.5) * (rs * rs + rp * rp);
}
template <class T> inline V3<T> fresnel_schlick3(T cosI, const V3<T>& f0) {
    T m = T(1) - clampT(cosI, T(0), T(1));
    T m5 = m * m * m * m * m;
    return f0 + (V3<T>(1) - f0) * m5;
}

struct MfTables {
    std::vector<float> ec, ecavg, e1;   // [ior][r][mu], [ior][r], [r][mu]
};
// prog_mf_lut / prog_mf_lut_avg (microfacet.js:245-330), isotropic part, one entry at a time in T precision
template <class T> inline MfTables build_mf_tables() {
    MfTables t;
    t.ec.resize(MF_NIOR * MF_NR * MF_NMU); t.ecavg.resize(MF_NIOR * MF_NR); t.e1.resize(MF_NR * MF_NMU);
    auto entry = [](T ior, int k, int j, bool isE1) -> T {
        T r = T(k) / T(MF_NR - 1);
        T mu = (T(j) + T(0.5)) / T(MF_NMU);
        T st = std::sqrt(std::max(T(0), T(1) - mu * mu));
        T a = std::max(r * r, T(ALPHA_MIN));
        V3<T> o(st, 0, mu);
        T acc = 0;
        for (int sy = 0; sy < MF_SQRT_SAMPLES; sy++)
            for (int sx = 0; sx < MF_SQRT_SAMPLES; sx++) {
                T vx = (T(sx) + T(0.5)) / T(MF_SQRT_SAMPLES), vy = (T(sy) + T(0.5)) / T(MF_SQRT_SAMPLES);
                T ux = vx, uy = T(1) - (T(1) - vy) * (T(1) - vy);
                V3<T> h = mf_sample_vndf(o, a, ux, uy);
                V3<T> i3 = reflectv(-o, h);
                if (i3.z > T(0)) {
                    T fr = isE1 ? T(1) : fresnel_dielectric(dot(o, h), T(1) / ior);
                    acc += T(2) * (T(1) - vy) * fr * mf_g2(o, i3, a) / mf_g1(o, a);
                }
            }
        return acc / T(MF_SQRT_SAMPLES * MF_SQRT_SAMPLES);
    };
    for (int e = 0; e < MF_NIOR * MF_NR * MF_NMU; e++) {
        T ior = T(1) + T(2) * T(e / (MF_NR * MF_NMU)) / T(MF_NIOR - 1);
        t.ec[e] = (float)entry(ior, (e / MF_NMU) % MF_NR, e % MF_NMU, false);
    }
    for (int e = 0; e < MF_NR * MF_NMU; e++) t.e1[e] = (float)entry(T(1), e / MF_NMU, e % MF_NMU, true);
    for (int e = 0; e < MF_NIOR * MF_NR; e++) {
        T acc = 0;
        for (int j = 0; j < MF_NMU; j++) {
            T mu = (T(j) + T(0.5)) / T(MF_NMU);
            acc += T(2) * T(t.ec[e * MF_NMU + j]) * mu / T(MF_NMU);
        }
        t.ecavg[e] = (float)acc;
    }
    return t;
}
// the reads (microfacet.js:152-240): linear in every axis, clamped at the ends
template <class T> inline void mf_axis(T x, int n, T& i0, T& f) {
    T c = clampT(x, T(0), T(n - 1));
    i0 = std::min(std::floor(c), T(n - 2));
    f = c - i0;
}
template <class T> inline T mf_ec(const MfTables& tb, T mu, T r, T n) {
    T m0, mf, r0, rf, n0, nf;
    mf_axis(mu * T(MF_NMU) - T(0.5), MF_NMU, m0, mf);
    mf_axis(r * T(MF_NR - 1), MF_NR, r0, rf);
    mf_axis((n - T(1)) * T(MF_NIOR - 1) / T(2), MF_NIOR, n0, nf);
    T acc = 0;
    for (int c = 0; c < 8; c++) {
        int di = c & 1, dk = (c >> 1) & 1, dj = (c >> 2) & 1;
        T w = (di ? nf : T(1) - nf) * (dk ? rf : T(1) - rf) * (dj ? mf : T(1) - mf);
        int idx = (((int)n0 + di) * MF_NR + (int)r0 + dk) * MF_NMU + (int)m0 + dj;
        acc += w * T(tb.ec[idx]);
    }
    return acc;
}
template <class T> inline T mf_ecavg(const MfTables& tb, T r, T n) {
    T r0, rf, n0, nf;
    mf_axis(r * T(MF_NR - 1), MF_NR, r0, rf);
    mf_axis((n - T(1)) * T(MF_NIOR - 1) / T(2), MF_NIOR, n0, nf);
    T acc = 0;
    for (int c = 0; c < 4; c++) {
        int di = c & 1, dk = (c >> 1) & 1;
        T w = (di ? nf : T(1) - nf) * (dk ? rf : T(1) - rf);
        acc += w * T(tb.ecavg[((int)n0 + di) * MF_NR + (int)r0 + dk]);
    }
    return acc;
}
template <class T> inline T mf_e1(const MfTables& tb, T mu, T r) {
    T m0, mf, r0, rf;
    mf_axis(mu * T(MF_NMU) - T(0.5), MF_NMU, m0, mf);
    mf_axis(r * T(MF_NR - 1), MF_NR, r0, rf);
    T acc = 0;
    for (int c = 0; c < 4; c++) {
        int dk = c & 1, dj = (c >> 1) & 1;
        T w = (dk ? rf : T(1) - rf) * (dj ? mf : T(1) - mf);
        acc += w * T(tb.e1[((int)r0 + dk) * MF_NMU + (int)m0 + dj]);
    }
    return acc;
}

// ------------------------------------------------------------------------------------------------------------
// THE LOBES -- core/materials_pbr.js:164-275 makeLobes, :296-350 lobesEval/lobesPdf, :352-358 interfaceReflectP,
// :450-596 lobesSample; :379-432 THE SIDE BEYOND (the translucent base, rough refraction's value and density below
// the surface); isotropic, uncoated: what the hot path's materials use.
// ------------------------------------------------------------------------------------------------------------
const uint32_t EV_NONE = 0, EV_DELTA = 1, EV_EVAL = 2, EV_OTHER = 3;
const double LT_MIN_ALPHA = 0.05;
// a coating over a metal (materials_pbr.js:114-136 metalFresnel, coatOverMetal): the stack's R and the metal's F as
// intensities, R + (1 - R)^2 F (1 + R F + (R F)^2 + ...) = 1 - (1 - R)(1 - F) / (1 - R F), F held to [0, 1]
template <class T> inline V3<T> coat_over_metal(const V3<T>& r, const V3<T>& f) {
    const V3<T> fc(sat(f.x), sat(f.y), sat(f.z));
    const V3<T> one(1);
    const V3<T> den = vmax(one - r * fc, T(1e-6));
    return one - (one - r) * (one - fc) / den;
}
template <class T> struct Lobes {
    V3<T> tX, tY, nZ, o, base, transTint, coatK, cm, ecO, ecAvg;
    V3<T> coatR{T(0)};                      // a coating's reflectance per channel at the view (0: anti-reflective)
    V3<T> pw{T(1) / T(3)};                  // the channels' weights in a coated reflect-or-pass pick (coatPick)
    T ax, ay;                               // the alphas along tX and tY (tX the rough axis)
    T aMin, r, metallic, trans, transl, eta, etaT, nrel, ps;
    bool isDelta;
    bool coated = false;                    // a coating is the interface: coatR, not coatK x the Fresnel
    bool through = false;                   // the side beyond lit: the lobes below the surface evaluated
    const MfTables* tb;
    A2<T> al() const { return A2<T>{ax, ay}; }
    V3<T> to_local(const V3<T>& w) const { return V3<T>(dot(w, tX), dot(w, tY), dot(w, nZ)); }
    V3<T> to_world(const V3<T>& w) const { return normalize(tX * w.x + tY * w.y + nZ * w.z); }
    // materials_pbr.js:106-113 coatFresnel: a coating's R at every facet, total past the critical angle
    V3<T> coat_fresnel(T cosI) const {
        const T f = fresnel_dielectric(cosI, eta);
        if (coated) return f >= T(1) ? V3<T>(1) : coatR;
        return vmin(coatK * f, T(1));
    }
    V3<T> metal_fresnel(T cosI) const {
        const V3<T> f = fresnel_schlick3(cosI, base);
        return coated ? coat_over_metal(coatR, f) : f;
    }
    // materials_pbr.js:137-142 reflectPick: the largest channel, or under a coating the channels weighed by the ray
    T reflect_pick(const V3<T>& c) const { return coated ? dot(c, pw) : max3(c); }
    V3<T> coat_albedo(const V3<T>& w) const {
        if (coated) return coatR;           // materials_pbr.js:151-153: the coating's at the view, at every angle
        return vmin(coatK * mf_ec(*tb, w.z, r, nrel), T(1));
    }
    // coatPs (materials_pbr.js:274-279)
    T coat_ps() const {
        return std::min(reflect_pick(coat_fresnel(o.z)), fresnel_dielectric(o.z, eta) >= T(1) ? T(1) : T(0.999));
    }
};
// coatPick (materials_pbr.js:280-291): a coated lobe's pick weighed by the shares of |beta| the ray carries
template <class T> inline void coat_pick(Lobes<T>& lb, const V3<T>& beta) {
    if (!lb.coated) return;
    const V3<T> a(std::fabs(beta.x), std::fabs(beta.y), std::fabs(beta.z));
    const T t = a.x + a.y + a.z;
    lb.pw = t > T(0) ? a * (T(1) / t) : V3<T>(T(1) / T(3));
    lb.ps = lb.coat_ps();
}
// refractShare (materials.js:123): T (1 - H)
template <class T> inline T refract_share_of(T transmission, T haze) { return sat(transmission) * (T(1) - sat(haze)); }
template <class T> inline T refract_share(const st_material& m) { return refract_share_of(T(m.transmission), T(m.haze)); }
template <class T> inline Lobes<T> make_lobes(const V3<T>& n, const V3<T>& v, const st_material& m, T eta,
                                              const MfTables* tb, T transmission_override = T(-1), T specular_override = T(-1),
                                              T haze_override = T(-1), T n0 = T(1), bool inside = false, T lam = T(0)) {
    Lobes<T> lb;
    lb.tb = tb;
    // mtlOrthonormalBasis (materials_pbr.js:13-19)
    V3<T> s = std::fabs(n.z) < T(0.999) ? normalize(cross(n, V3<T>(0, 0, 1))) : normalize(cross(n, V3<T>(0, 1, 0)));
    V3<T> t = cross(s, n);
    lb.tX = s; lb.tY = t; lb.nZ = n;
    lb.o = V3<T>(dot(v, lb.tX), dot(v, lb.tY), std::max(dot(v, n), T(1e-4)));
    lb.r = clampT(T(m.roughness), T(0), T(1));
    T aIso = lb.r * lb.r;
    lb.isDelta = aIso < T(ALPHA_MIN);
    // anisotropy without a grain (microfacet.js mfAnisoAlpha): x the rough axis, ratio 1 / (1 - 0.9 |anisotropy|)
    const T sa = std::sqrt(T(1) - T(0.9) * std::min(std::fabs(T(m.anisotropy)), T(1)));
    const T ax = aIso / sa, ay = aIso * sa;
    lb.aMin = std::min(ax, ay);
    lb.ax = clampT(ax, T(ALPHA_MIN), T(1));
    lb.ay = clampT(ay, T(ALPHA_MIN), T(1));
    lb.metallic = sat(T(m.metallic));
    T transm = transmission_override >= T(0) ? transmission_override : T(m.transmission);
    T spec = specular_override >= T(0) ? specular_override : T(m.specular);
    T hz = haze_override >= T(0) ? haze_override : T(m.haze);
    lb.trans = refract_share_of(transm, hz);                                   // materials_pbr.js:196-204
    lb.transl = T(1) - lb.trans > T(1e-6) ? sat(sat(transm) * sat(hz) / std::max(T(1) - lb.trans, T(1e-6))) : T(0);
    lb.base = V3<T>(T(m.base[0]), T(m.base[1]), T(m.base[2]));
    lb.transTint = m.attenuation > 0 ? V3<T>(1) : lb.base;
    T lum = max3(lb.base);
    V3<T> tint = lum > T(0) ? lb.base / std::max(lum, T(1e-6)) : V3<T>(1);
    T st = T(m.specular_tint);
    V3<T> tintMix = V3<T>(1) * (T(1) - st) + tint * st;
    lb.coatK = tintMix * mixT(T(2) * spec, T(1), lb.trans);
    lb.eta = eta; lb.etaT = eta;
    lb.nrel = clampT(T(1) / eta, T(1), T(3));
    // A COATING (materials_pbr.js:220-245): the interface on the faces light enters by; on the faces it leaves by,
    // anti-reflective (coat 1), the bare interface (2) or the coating again (3); its R at the view's angle, the edge
    // moved by the invariant n0 sin(theta0) through the stack's effective index; a ray with a wavelength takes R there
    const uint32_t coat = std::min(m.coat, 3u);
    if (coat != 0u) {
        if (!inside || coat == 3u) {
            const double sin0 = std::sqrt(std::max(0.0, 1.0 - (double)lb.o.z * (double)lb.o.z));
            const double lo = std::min(std::max((double)m.coat_lo, 0.0), 1.0);
            const double hi = std::min(std::max((double)m.coat_hi, 0.0), 1.0);
            const double w = std::max((double)m.coat_width, 0.0);
            const double edge = coat_edge_at((double)m.coat_edge, (double)n0 * sin0, std::max((double)m.coat_index, 1.0));
            if (lam > T(0)) {
                lb.coatR = V3<T>(T(coat_edge_at_lambda(lo, hi, edge, w, (double)lam)));
            } else {
                double c[3];
                coat_edge_rgb(lo, hi, edge, w, c);
                lb.coatR = V3<T>(T(c[0]), T(c[1]), T(c[2]));
            }
            lb.coated = true;
        } else if (coat == 1u) {
            lb.coated = true;
        }
    }
    lb.ps = lb.coat_ps();
    lb.ecO = lb.coat_albedo(lb.o);
    T e1 = lb.metallic > T(0) ? mf_e1(*tb, lb.o.z, lb.r) : T(1);
    lb.ecAvg = lb.coated ? lb.coatR : vmin(lb.coatK * mf_ecavg(*tb, lb.r, lb.nrel), T(1));
    // Turquin's factor from F0: the metal's colour, or under a coating what the two reflect head-on
    const V3<T> f0 = lb.coated ? coat_over_metal(lb.coatR, lb.base) : lb.base;
    lb.cm = V3<T>(1) + f0 * (T(1) / std::max(e1, T(1e-3)) - T(1));
    return lb;
}
template <class T> inline V3<T> lobes_through_eval(const Lobes<T>& lb, const V3<T>& i, T minAlpha);
template <class T> inline V3<T> lobes_eval(const Lobes<T>& lb, const V3<T>& l, T minAlpha) {
    V3<T> i = lb.to_local(l);
    if (lb.through && i.z < T(0)) return lobes_through_eval(lb, i, minAlpha);
    if (i.z <= T(0)) return V3<T>(0);
    V3<T> f(0);
    if (!lb.isDelta && lb.aMin >= minAlpha) {
        V3<T> h = normalize(lb.o + i);
        T spec = mf_d(h, lb.al()) * mf_g2(lb.o, i, lb.al()) / (T(4) * lb.o.z * i.z);
        T oh = dot(lb.o, h);
        f += lb.cm * lb.metal_fresnel(oh) * (lb.metallic * spec);
        f += lb.coat_fresnel(oh) * ((T(1) - lb.metallic) * spec);
    }
    T wDiff = (T(1) - lb.metallic) * (T(1) - lb.trans) * (T(1) - lb.transl);
    if (wDiff > T(0)) {
        V3<T> ecI = lb.coat_albedo(i);
        V3<T> den = vmax(V3<T>(1) - lb.ecAvg, T(1e-4)) * T(PI_D);
        f += lb.base * (V3<T>(1) - lb.ecO) * (V3<T>(1) - ecI) / den * wDiff;
    }
    return f;
}
template <class T> inline T interface_reflect_p(const Lobes<T>& lb, T oh) {
    T fh = lb.reflect_pick(lb.coat_fresnel(oh));
    T den = fh + (T(1) - fh) * lb.trans;
    return den > T(1e-6) ? fh / den : T(1);
}
// throughHalf (materials_pbr.js:385-396): the refraction's generalised half vector, turned to the view's side
template <class T> inline bool through_half(const Lobes<T>& lb, const V3<T>& i, V3<T>& h) {
    h = (lb.o * lb.etaT + i) * T(-1);
    const T hl = length(h);
    if (hl < T(1e-12)) return false;
    h = h * (T(1) / hl);
    if (h.z < T(0)) h = h * T(-1);
    return dot(lb.o, h) > T(0) && dot(i, h) < T(0);
}
// lobesThroughEval / lobesThroughPdf (materials_pbr.js:397-432)
template <class T> inline V3<T> lobes_through_eval(const Lobes<T>& lb, const V3<T>& i, T minAlpha) {
    const T wd = T(1) - lb.metallic;
    V3<T> f(0);
    const T wT = wd * (T(1) - lb.trans) * lb.transl;
    if (wT > T(0)) {
        const V3<T> ecI = lb.coat_albedo(V3<T>(i.x, i.y, -i.z));
        f = lb.base * (V3<T>(1) - lb.ecO) * (V3<T>(1) - ecI) / (vmax(V3<T>(1) - lb.ecAvg, T(1e-4)) * T(PI_D)) * wT;
    }
    if (wd <= T(0) || lb.trans <= T(0) || lb.isDelta || lb.aMin < minAlpha) return f;
    V3<T> h;
    if (!through_half(lb, i, h)) return f;
    const T oh = dot(lb.o, h), ih = dot(i, h), den = lb.etaT * oh + ih;
    const V3<T> fc = lb.coat_fresnel(oh);
    return f + (V3<T>(1) - fc) * lb.transTint *
               (wd * lb.trans * mf_d(h, lb.al()) * mf_g2(lb.o, i, lb.al()) * oh * (-ih) / (lb.o.z * (-i.z) * std::max(den * den, T(1e-20))));
}
template <class T> inline T lobes_through_pdf(const Lobes<T>& lb, const V3<T>& i) {
    const T wd = T(1) - lb.metallic;
    const T pd = (T(1) - lb.ps) * (T(1) - lb.trans);
    const T p = wd * pd * lb.transl * (-i.z) / T(PI_D);
    if (wd <= T(0) || lb.trans <= T(0) || lb.isDelta) return p;
    V3<T> h;
    if (!through_half(lb, i, h)) return p;
    const T oh = dot(lb.o, h), ih = dot(i, h), den = lb.etaT * oh + ih;
    return p + wd * (T(1) - pd) * (T(1) - interface_reflect_p(lb, oh)) * mf_g1(lb.o, lb.al()) * mf_d(h, lb.al()) * oh / lb.o.z *
                   (-ih) / std::max(den * den, T(1e-20));
}
template <class T> inline T lobes_pdf(const Lobes<T>& lb, const V3<T>& l) {
    V3<T> i = lb.to_local(l);
    if (lb.through && i.z < T(0)) return lobes_through_pdf(lb, i);
    if (i.z <= T(0)) return T(0);
    T wd = T(1) - lb.metallic;
    T pd = (T(1) - lb.ps) * (T(1) - lb.trans);
    T p = wd * pd * (T(1) - lb.transl) * i.z / T(PI_D);
    if (!lb.isDelta) {
        T pr = mf_pdf_reflect(lb.o, i, lb.al());
        p += (lb.metallic + wd * (T(1) - pd) * interface_reflect_p(lb, dot(lb.o, normalize(lb.o + i)))) * pr;
    }
    return p;
}
// lobesNone (materials_pbr.js:325-328)
template <class T> inline bool lobes_none(const st_material& m, T transmission, T haze) {
    T r = clampT(T(m.roughness), T(0), T(1));
    return r * r < T(ALPHA_MIN) && (T(1) - sat(T(m.metallic))) * (T(1) - refract_share_of(transmission, haze)) <= T(0);
}
// throughEvaluable (materials_pbr.js:379-384)
template <class T> inline bool through_evaluable(const st_material& m, T transmission, T haze) {
    const T r = clampT(T(m.roughness), T(0), T(1)), wd = T(1) - sat(T(m.metallic));
    return (wd * refract_share_of(transmission, haze) > T(0) && r * r >= T(ALPHA_MIN)) || wd * sat(transmission) * sat(haze) > T(0);
}
template <class T> struct LobeSample { V3<T> dir, w; uint32_t ev; bool isDelta, transmitted; };
template <class T> inline LobeSample<T> lobes_sample(const Lobes<T>& lb, const T rnd[4]) {
    LobeSample<T> s;
    s.w = V3<T>(0); s.ev = EV_OTHER; s.isDelta = false; s.transmitted = false;
    V3<T> i(0, 0, 1);
    uint32_t glossyEv = lb.aMin >= T(LT_MIN_ALPHA) ? EV_EVAL : EV_OTHER;
    T wd = T(1) - lb.metallic;
    T pick = rnd[0];
    if (pick < lb.metallic) {                                                  // metal
        if (lb.isDelta) {
            i = V3<T>(-lb.o.x, -lb.o.y, lb.o.z);
            s.w = lb.metal_fresnel(lb.o.z) * lb.cm;
            s.ev = EV_DELTA; s.isDelta = true;
        } else {
            V3<T> h = mf_sample_vndf(lb.o, lb.al(), rnd[1], rnd[2]);
            i = reflectv(-lb.o, h);
            if (i.z > T(0)) s.w = lb.cm * lb.metal_fresnel(dot(lb.o, h)) * (mf_g2(lb.o, i, lb.al()) / mf_g1(lb.o, lb.al()));
            s.ev = glossyEv;
        }
    } else {
        pick = (pick - lb.metallic) / std::max(wd, T(1e-6));
        T pd = (T(1) - lb.ps) * (T(1) - lb.trans);
        if (pick < T(1) - pd) {
            T sub = pick / std::max(T(1) - pd, T(1e-6));
            if (lb.isDelta) {
                if (sub < lb.ps / std::max(T(1) - pd, T(1e-6))) {                    // mirror coat
                    i = V3<T>(-lb.o.x, -lb.o.y, lb.o.z);
                    s.w = lb.coat_fresnel(lb.o.z) / lb.ps;
                } else {                                                             // clear refraction
                    s.transmitted = true;
                    i = refractv(-lb.o, V3<T>(0, 0, 1), lb.etaT);
                    if (i.z < T(0)) s.w = (V3<T>(1) - lb.coat_fresnel(lb.o.z)) * lb.transTint / (T(1) - lb.ps);
                }
                s.ev = EV_DELTA; s.isDelta = true;
            } else {
                V3<T> h = mf_sample_vndf(lb.o, lb.al(), rnd[1], rnd[2]);
                T oh = dot(lb.o, h);
                V3<T> fc = lb.coat_fresnel(oh);
                T r = interface_reflect_p(lb, oh);
                if (sub < r) {                                                       // glossy coat
                    i = reflectv(-lb.o, h);
                    if (i.z > T(0)) s.w = fc * (mf_g2(lb.o, i, lb.al()) / mf_g1(lb.o, lb.al()) / ((T(1) - pd) * r));
                    s.ev = glossyEv;
                } else {                                                             // rough refraction
                    s.transmitted = true;
                    i = refractv(-lb.o, h, lb.etaT);
                    if (i.z < T(0))
                        s.w = (V3<T>(1) - fc) * lb.transTint *
                              (lb.trans * mf_g2(lb.o, i, lb.al()) / mf_g1(lb.o, lb.al()) / ((T(1) - pd) * (T(1) - r)));
                    s.ev = lb.aMin >= T(LT_MIN_ALPHA) ? EV_EVAL : EV_OTHER;
                }
            }
        } else {                                                                     // diffuse base
            T r = std::sqrt(rnd[1]);
            T phi = T(2) * T(PI_D) * rnd[2];
            const T z = std::sqrt(std::max(T(0), T(1) - rnd[1]));
            i = V3<T>(r * std::cos(phi), r * std::sin(phi), z);
            V3<T> ecI = lb.coat_albedo(i);
            s.w = lb.base * (V3<T>(1) - lb.ecO) * (V3<T>(1) - ecI) / vmax(V3<T>(1) - lb.ecAvg, T(1e-4)) / (T(1) - lb.ps);
            s.ev = EV_EVAL;
            if (rnd[3] < lb.transl) { i.z = -z; s.transmitted = true; }              // the translucent base (B1)
        }
    }
    s.dir = lb.to_world(i);
    return s;
}

}  // namespace sto
