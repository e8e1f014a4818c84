// TEST INFRASTRUCTURE ONLY -- the oracle's entry points (extern "C", loaded by oracle/oracle.py through ctypes).
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg call these, as the checker and the CPU
// baseline; the product (libshadytracer.so) never links or runs any of it.
//
// The path tracer restates, for one path at a time, what the reference's wavefront does to it:
//   genrays            core/genrays.js:36-97
//   march              core/wavefront.js:834-1005 (sphere tracing, marchTol hit test, escape test, lmax, maxiter)
//   shade              core/wavefront.js:1244-1442, core/tracebasics.js:834-1100 (pathBegin..pathEnd),
//                      core/materials_pbr.js:1110-1440 (processMaterial_advanced: NEE + MIS + the lobe draw)
//   occlude            core/wavefront.js:1481-1692
//   deposit            core/wavefront.js:162-245 (refused: NaN, inf, negative luminance)
//   resolve            core/wavefront.js:414-494 and core/measure.js:36-51 (EMA mean, V and S moments), in FP64
// A wavefront processes every live path one segment per iteration, so "the i-th iteration" is the path's i-th
// segment here too; the last iteration takes no light sample (UB.lastpass) and ends what is left (THE FLUSH).
#include "st_oracle_render.h"
#include "st_oracle_extra.h"
#include "st_oracle_optics.h"
#include "st_oracle_sppm.h"
#include "st_oracle_spectral.h"
#include "st_oracle_guide.h"
#include "st_oracle_light.h"
#ifdef _OPENMP
#include <omp.h>
#endif
#include <atomic>
#include <map>

using namespace sto;

namespace {

// the most SDF evaluations a ray takes in one iteration's march (the product's MARCH_CHUNK)
const uint32_t MARCH_CHUNK = 48;
const uint32_t RAY_ACTIVE = 0, RAY_ABSORBED = 1, RAY_ESCAPED = 2, RAY_MAXITER = 4, RAY_SOURCE = 5,
               RAY_TERMINATED = 8, RAY_SCATTER = 9, RAY_GATHER = 10;

struct Stats {
    std::atomic<uint64_t> paths{0}, segments{0}, march_steps{0}, shadow_rays{0}, shadow_steps{0};
    std::atomic<uint32_t> nonfinite{0}, flushed{0}, shadowcut{0};
};

// THE EMITTER LIST (wavefront.js:715-815 prog_emit_collect / publish; tracebasics.js:1148-1210 EMIT_LIST;
// materials_pbr.js:887-905 emitDeposit): the discovery grid the camera paths' emitter hits go into (a copy a thread,
// merged after each sample), and the list built from it between samples, every EMIT_EPOCH -- in voxel order, as the
// product builds it
const uint32_t EMIT_G = 16, EMIT_CELLS = EMIT_G * EMIT_G * EMIT_G, EMIT_MAX = 64, EMIT_EPOCH = 2;
const float EMIT_Q = 16777215.f, EMIT_LUM_K = 209715.2f;
const uint32_t EMIT_LUM_DECAY = 31877u;
struct EmitList {
    uint32_t count = 0, last = 0;
    float box[EMIT_MAX][4];           // centre, radius
    float pc[EMIT_MAX][2];            // probability, running sum
};
inline uint32_t emit_lum_code(float lum) {
    return (uint32_t)(std::fmin(std::fmax(std::log2(std::fmax(lum, 1e-30f)) + 40.f, 0.f), 80.f) * EMIT_LUM_K) + 1u;
}
inline float emit_lum_decode(uint32_t q) { return q ? std::exp2((float)(q - 1u) / EMIT_LUM_K - 40.f) : 0.f; }
inline void emit_grid_init(uint32_t* g) {
    for (uint32_t i = 0; i < EMIT_CELLS * 8; i++) g[i] = (i & 7u) < 3u ? 0xFFFFFFFFu : 0u;
}

template <class T> struct Ctx {
    const st_scene_desc* s;
    st_params p;
    Derived d;
    Env<T> env;
    const MfTables* tb;
    T tol, envR2, stepscale;
    uint32_t budget;
    HazeBox<T> haze;
    bool scatter_on = false;                // a material that scatters inside: the march walks it (haze.js:574-650)
    // the photon map of the sample being traced (sppm.js): on, its grid, radius, cell, 1 / (pi r^2), the photons'
    // square, the gather's budget
    bool sppm = false;
    const SppmGrid* grid = nullptr;
    float sp_r2 = 0, sp_cell = 0, sp_half = 0;
    double sp_inv_area = 0;
    float sp_vr2 = 0, sp_vcell = 0;                 // in the volume (sppmRadiusVolume): R^2, the records' cell 2R
    double sp_inv_vol = 0;                          // 3 / (4 pi R^3)
    uint32_t sp_budget = 512;
    // the learned emission map (wavefront.js:628-711): on, the photons sent and stored per cell, the CDF
    bool sp_learn = false;
    uint32_t* lt_emit = nullptr;
    uint32_t* lt_hit = nullptr;
    const float* lt_cdf = nullptr;
    // the emitter list: on in a scene with emitters; light sampling aims at it (nee) with this share; the grid's half
    bool em_on = false, em_nee = false;
    float em_share = 0.5f, em_half = 15.f;
    const EmitList* em = nullptr;
    std::vector<std::vector<uint32_t>>* em_grids = nullptr;     // a discovery grid a thread
    // the lights' faces and the material -> face map (its index + 1, 0 none)
    const std::vector<OFace>* faces = nullptr;
    uint8_t face_of[ST_MAX_MATERIALS] = {};
    // the reference's bounding-box culling at the root (a timing mode: the CPU baseline does the reference's work)
    const std::vector<CullBox>* cull = nullptr;
    // light tracing to the camera (materials_pbr.js ltConnect): on, the camera, the sample's splat buffer (rgb a
    // pixel, added to the pixel as it is) and the connections that reached each pixel
    bool lt = false;
    uint32_t lt_emit_n = 0;                 // of a sample's photons, the first this many are emitter probes
    const st_view* view = nullptr;
    std::vector<double>* splat = nullptr;
    std::vector<uint32_t>* ltcount = nullptr;
};
// the march's and the shadow rays' distance: the fold, or the reference's culled render copy of it
template <class T> inline T march_dist(const Ctx<T>& C, const V3<T>& p) {
    if (C.cull) return scene_dist_culled(*C.s, *C.cull, p, T(10) * march_tol(p, C.tol));
    return scene_eval(*C.s, p).d;
}
const uint32_t LT_G = 128, LT_N = LT_G * LT_G;
const float LT_FLOOR_F = 0.2f;
// ltSearch / ltMass (wavefront.js:520-536)
inline uint32_t lt_search(const float* cdf, float u) {
    uint32_t lo = 0, hi = LT_G - 1;
    while (lo < hi) { uint32_t mid = (lo + hi) / 2; if (u < cdf[mid]) hi = mid; else lo = mid + 1; }
    return lo;
}
inline float lt_mass(const float* cdf, uint32_t i) { return std::max(cdf[i] - (i ? cdf[i - 1] : 0.f), 0.f); }
// prog_lt_build (wavefront.js:628-711): worth = stores / sent per cell, both halved; the floor mixed in; row CDF and
// per-row conditional CDFs, in f32 as the kernel sums them
inline void lt_build(uint32_t* emit, uint32_t* hit, float* cdf) {
    std::vector<float> rowW(LT_G), rowP(LT_G);
    for (uint32_t r = 0; r < LT_G; r++) {
        float sum = 0.f;
        for (uint32_t c = 0; c < LT_G; c++) {
            uint32_t e = emit[r * LT_G + c], h = hit[r * LT_G + c];
            float w = e > 0 ? (float)h / (float)e : 0.f;
            cdf[r * LT_G + c] = w;
            sum += w;
            emit[r * LT_G + c] = e / 2;
            hit[r * LT_G + c] = h / 2;
        }
        rowW[r] = sum;
    }
    float T = 0.f;
    for (uint32_t r = 0; r < LT_G; r++) T += rowW[r];
    const bool learned = T > 0.f;
    for (uint32_t r = 0; r < LT_G; r++) {
        float rp = learned ? (1.f - LT_FLOOR_F) * rowW[r] / std::max(T, 1e-30f) + LT_FLOOR_F / (float)LT_G : 1.f / (float)LT_G;
        rowP[r] = rp;
        float acc = 0.f;
        for (uint32_t c = 0; c < LT_G; c++) {
            float p = learned ? (1.f - LT_FLOOR_F) * cdf[r * LT_G + c] / std::max(T, 1e-30f) + LT_FLOOR_F / (float)LT_N
                              : 1.f / (float)LT_N;
            acc += p;
            cdf[r * LT_G + c] = acc / rp;
        }
        cdf[r * LT_G + LT_G - 1] = 1.f;
    }
    float racc = 0.f;
    for (uint32_t r = 0; r < LT_G; r++) { racc += rowP[r]; cdf[LT_N + r] = racc; }
    cdf[LT_N + LT_G - 1] = 1.f;
}
// the last render's learned emission map as it ended (photons sent, stored, the CDF), for the tests to read
std::vector<uint32_t> g_lt_emit, g_lt_hit;
std::vector<uint32_t> g_lt_count;               // light tracing's connections per pixel, over the last render call
std::vector<float> g_lt_cdf;
inline void lt_uniform(float* cdf) {
    for (uint32_t r = 0; r < LT_G; r++)
        for (uint32_t c = 0; c < LT_G; c++) cdf[r * LT_G + c] = c + 1 == LT_G ? 1.f : (float)(c + 1) / LT_G;
    for (uint32_t r = 0; r < LT_G; r++) cdf[LT_N + r] = r + 1 == LT_G ? 1.f : (float)(r + 1) / LT_G;
}

template <class T> struct Ray {
    V3<T> pos, dir, beta, rad;
    T ltot, n, sunmis, tmax, absLtot;
    T lam = T(0);                           // the wavelength a dispersive refraction gave it (nm, as coded), 0 none
    T emw = T(1);                           // an emitter hit's MIS weight against the last vertex's light sample
    T lpx = T(-1), lpy = T(0);              // the last vertex's density for the direction sent (< 0: no weight
                                            // against the faces) and ltot there (prevPdf, vtxLtot)
    uint32_t lens = 0;                      // a camera path's lens field (materials_pbr.js lensField): 1 delta only
                                            // since the eye, 2 at its D, 3 delta only since its D
    bool passed = false;                    // a photon that has passed a delta event (TAG_PASSED)
    uint32_t cls = 0;                       // light tracing's class (CLS_CAND 1, CLS_SPEC 2): a first vertex drawn
                                            // from an evaluable lobe, then delta events only
    uint32_t medium = 0;                    // the material whose volume holds the ray, 0 none (tracebasics.js md0-2)
    uint32_t bounces, steps, state, pix;
};

struct PhotonRec { float pos[3], power[3]; uint32_t dir, nrm, flags; };
// a walk's seed and what it does with the photon map in the volume: 1 a photon that stores where it collides, 2 a
// camera ray handed to the gather at its first collision
struct WalkIO { U4 ps; uint32_t id; int map; std::vector<PhotonRec>* out; };

template <class T> inline void move_by(Ray<T>& r, const V3<T>& off) {       // tracebasics.js:562-567 moveBy
    r.pos += off;
    r.ltot += length(off) * r.n;
}

// badDeposit (wavefront.js:181-188): NaN or inf in a channel, or negative luminance
template <class T> inline bool bad_deposit(const V3<T>& c) {
    return !std::isfinite(c.x) || !std::isfinite(c.y) || !std::isfinite(c.z) || luma(c) < T(0);
}

template <class T> struct Frame {
    std::vector<double> rgb;   // per sample: the deposits (the reference's f32 frame; summed in double here)
    std::vector<uint32_t> cnt;
};

template <class T> inline void deposit(Frame<T>& f, uint32_t pix, const V3<T>& c, Stats& st) {
    if (bad_deposit(c)) { st.nonfinite++; return; }
#pragma omp atomic
    f.rgb[pix * 3 + 0] += (double)c.x;
#pragma omp atomic
    f.rgb[pix * 3 + 1] += (double)c.y;
#pragma omp atomic
    f.rgb[pix * 3 + 2] += (double)c.z;
}

// the march (wavefront.js:866-947): to the surface, the sky, lmax or maxiter. With a walk's seed (wps: the path's
// sample seed and its tile, or a photon's seed and id), a ray in a material that scatters inside walks it (haze.js:574-650
// THE MEDIUM'S WALK): a free flight -ln(1 - u) / sigma drawn as its leg starts, from its vertex; at each collision
// taken back to it, turned by Henyey-Greenstein, its next flight drawn, a march step; what it meets after that takes
// its whole weight (prevPdf -1, sunmis 1). A collision counts as an evaluation in the chunks an iteration marches.
const uint32_t SEED_SALT_WALK = 0x57410000u, SEED_SALT_WALK_HIT = 0x57480000u, SEED_SALT_VOL_STORE = 0x564F4C53u;
// whether the ray is in a material that scatters inside (the haze's draw is then not its)
template <class T> inline bool walks(const Ctx<T>& C, const Ray<T>& r) {
    return C.scatter_on && r.medium != 0 && r.medium < C.s->n_materials && C.s->materials[r.medium].scatter_distance > 0.f;
}
template <class T> inline T march(const Ctx<T>& C, Ray<T>& r, Stats& st, bool use_haze, uint32_t& evals_out,
                                  const WalkIO* wio = nullptr) {
    uint64_t steps = 0;
    T dh = T(1e7);
    T wsig = T(0), wg = T(0);
    if (wio && C.scatter_on && r.medium != 0 && r.medium < C.s->n_materials) {
        const st_material& mm = C.s->materials[r.medium];
        if (mm.scatter_distance > 0.f) {
            wsig = T(1) / T(mm.scatter_distance);
            wg = clampT(T(mm.scatter_g), T(-0.95), T(0.95));
        }
    }
    if (wsig > T(0) && r.tmax == T(0)) {                                       // haze.js:598-618 mediumDraw
        Rng wr = path_rng(wio->ps, wio->id, SEED_SALT_WALK + r.steps);
        T u[4]; wr.next4(u);
        r.tmax = std::max(std::min(r.absLtot, r.ltot) - std::log(T(1) - u[0]) / wsig * r.n, T(1e-30));
    }
    for (;;) {
        if (wsig > T(0) && r.ltot >= r.tmax) {                                // haze.js:619-650 mediumCollide
            r.pos = r.pos - r.dir * ((r.ltot - r.tmax) / std::max(r.n, T(1e-4)));
            r.ltot = r.tmax;
            if (wio->map == 2) { r.state = RAY_GATHER; break; }          // the map gathers here (RAY_GATHER)
            Rng wr = path_rng(wio->ps, wio->id, SEED_SALT_WALK_HIT + r.steps);
            T u[4]; wr.next4(u);
            const V3<T> din = r.dir;
            r.dir = hg_sample(r.dir, wg, u[0], u[1]);
            r.tmax = std::max(r.ltot - std::log(T(1) - u[2]) / wsig * r.n, T(1e-30));
            r.steps += 1;
            steps++;
            r.sunmis = T(1); r.emw = T(1); r.lpx = T(-1);
            if (wio->map == 1) {                                               // haze.js:680-690 mediumStore
                const st_material& mm = C.s->materials[r.medium];
                V3<T> pw = r.rad * r.beta;
                if (mm.attenuation > 0.f) {
                    const T dl = std::max(r.ltot - r.absLtot, T(0)) / std::max(r.n, T(1e-4)) / T(mm.attenuation);
                    pw.x *= std::exp(std::log(std::min(std::max(T(mm.base[0]), T(1e-6)), T(1))) * dl);
                    pw.y *= std::exp(std::log(std::min(std::max(T(mm.base[1]), T(1e-6)), T(1))) * dl);
                    pw.z *= std::exp(std::log(std::min(std::max(T(mm.base[2]), T(1e-6)), T(1))) * dl);
                }
                Rng sr = path_rng(wio->ps, wio->id, SEED_SALT_VOL_STORE + r.steps);
                T us[4]; sr.next4(us);
                const uint32_t sub = std::min((uint32_t)(us[1] * T(SPPM_SUBS)), SPPM_SUBS - 1);
                PhotonRec rec;
                rec.pos[0] = (float)r.pos.x; rec.pos[1] = (float)r.pos.y; rec.pos[2] = (float)r.pos.z;
                rec.power[0] = (float)pw.x; rec.power[1] = (float)pw.y; rec.power[2] = (float)pw.z;
                const float dv[3] = {(float)-din.x, (float)-din.y, (float)-din.z};
                rec.dir = sppm_oct(dv);
                rec.nrm = 0;
                rec.flags = (r.bounces + 1) | (sub << SPPM_SUB_SHIFT) | SPPM_VOL;
                wio->out->push_back(rec);
            }
            if (r.steps > C.p.maxiter) { r.state = RAY_MAXITER; break; }
            continue;
        }
        if (use_haze && wsig == T(0) && haze_arrived(r.tmax, r.ltot)) {      // haze.js:280-288 hazeArrived / hazeAt
            r.pos = r.pos - r.dir * ((r.ltot - r.tmax) / std::max(r.n, T(1e-4)));
            r.ltot = r.tmax;
            r.state = RAY_SCATTER;
            break;
        }
        const T hd = march_dist(C, r.pos);
        T ea = std::fabs(hd);
        T eps = march_tol(r.pos, C.tol);
        steps++;
        if (r.ltot > T(1000) || r.steps > C.p.maxiter) r.state = RAY_MAXITER;
        if (dot(r.pos, r.dir) > T(0) && dot(r.pos, r.pos) > C.envR2) r.state = RAY_ESCAPED;
        if (ea < eps || r.state != RAY_ACTIVE) { dh = hd; break; }
        r.steps += 1;
        T d = ea * C.stepscale;
        move_by(r, r.dir * d);
    }
    st.march_steps += steps;
    evals_out = (uint32_t)steps;
    return dh;
}

// the occlusion pass (wavefront.js:1481-1692), distance only: true when the shadow ray reaches the light
template <class T> inline bool occlude(const Ctx<T>& C, V3<T> pos, const V3<T>& dir, T n, Stats& st,
                                      V3<T>* stop = nullptr, T* stop_ltot = nullptr, bool face = false, T ltot0 = T(0)) {
    T ltot = ltot0;                         // a face's ray: minus the way to it, less four offsets (TAG_FNEE)
    uint32_t steps = 0;
    bool reached = false, cut = false;
    uint64_t evals = 0;
    for (;;) {
        const T hd = march_dist(C, pos);
        evals++;
        T ea = std::fabs(hd);
        T eps = march_tol(pos, C.tol);
        if (face && ltot >= T(0)) { reached = true; break; }                           // at the face
        if (ea < eps) break;                                                           // blocked
        if (dot(pos, dir) > T(0) && dot(pos, pos) > C.envR2) { reached = true; break; }
        steps += 1;
        if (ltot > T(1000) || steps > C.p.maxiter) { reached = true; cut = steps > C.p.maxiter; break; }
        T step = ea * C.stepscale;
        V3<T> off = dir * step;
        pos += off;
        ltot += length(off) * n;
    }
    st.shadow_rays++;
    st.shadow_steps += evals;
    if (cut) st.shadowcut++;
    if (stop) *stop = pos;
    if (stop_ltot) *stop_ltot = ltot;
    return reached;
}

// the list's questions (tracebasics.js:1148-1210): a box by its running sum, 1 - cos of a sphere's cone, the
// mixture's density of a direction, a direction into a box's cone
inline uint32_t emit_pick(const EmitList& L, float u) {
    for (uint32_t b = 0; b < L.count; b++)
        if (u < L.pc[b][1]) return b;
    return L.count ? L.count - 1 : 0;
}
template <class T> inline T cone_omc(T r, T d2) {
    const T s2 = r * r / d2;
    return s2 / (T(1) + std::sqrt(std::max(T(0), T(1) - s2)));
}
// tracebasics.js:1187-1195 emitCovers: inside a listed sphere
template <class T> inline bool emit_covers(const EmitList& L, const V3<T>& y) {
    for (uint32_t b = 0; b < L.count; b++) {
        const V3<T> d(y.x - T(L.box[b][0]), y.y - T(L.box[b][1]), y.z - T(L.box[b][2]));
        if (dot(d, d) < T(L.box[b][3]) * T(L.box[b][3])) return true;
    }
    return false;
}
template <class T> inline T emit_cone_pdf(const EmitList& L, const V3<T>& x, const V3<T>& w) {
    T p = 0;
    for (uint32_t b = 0; b < L.count; b++) {
        const V3<T> dc(T(L.box[b][0]) - x.x, T(L.box[b][1]) - x.y, T(L.box[b][2]) - x.z);
        const T d2 = dot(dc, dc), r = T(L.box[b][3]);
        if (d2 <= r * r) continue;
        const T omc = cone_omc(r, d2);
        if (dot(w, dc) >= (T(1) - omc) * std::sqrt(d2)) p += T(L.pc[b][0]) / (T(2) * T(PI_D) * omc);
    }
    return p;
}
template <class T> inline bool emit_sample(const EmitList& L, uint32_t b, const V3<T>& x, T u1, T u2, V3<T>& w) {
    const V3<T> dc(T(L.box[b][0]) - x.x, T(L.box[b][1]) - x.y, T(L.box[b][2]) - x.z);
    const T d2 = dot(dc, dc), r = T(L.box[b][3]);
    if (d2 <= r * r) return false;
    const T d = std::sqrt(d2);
    const V3<T> axis = dc * (T(1) / d);
    const T omc = cone_omc(r, d2);
    const T cosT = T(1) - u1 * omc;
    const T sinT = std::sqrt(std::max(T(0), T(1) - cosT * cosT));
    const T ph = T(2) * T(PI_D) * u2;
    const V3<T> tt = std::fabs(axis.x) > T(0.9) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
    const V3<T> b1 = normalize(cross(tt, axis));
    const V3<T> b2 = cross(axis, b1);
    w = normalize(b1 * (std::cos(ph) * sinT) + b2 * (std::sin(ph) * sinT) + axis * cosT);
    return true;
}
// a camera path's emitter hit into this thread's grid (materials_pbr.js:887-905 emitDeposit)
template <class T> inline void emit_deposit(const Ctx<T>& C, const V3<T>& p, const V3<T>& le) {
    const float R = C.em_half;
    const float ux = ((float)p.x + R) / (2.f * R), uy = ((float)p.y + R) / (2.f * R), uz = ((float)p.z + R) / (2.f * R);
    if (ux < 0.f || uy < 0.f || uz < 0.f || ux >= 1.f || uy >= 1.f || uz >= 1.f) return;
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    uint32_t* g = (*C.em_grids)[tid].data() +
                  8 * ((uint32_t)(ux * EMIT_G) + EMIT_G * ((uint32_t)(uy * EMIT_G) + EMIT_G * (uint32_t)(uz * EMIT_G)));
    const uint32_t q[3] = {(uint32_t)(ux * EMIT_Q), (uint32_t)(uy * EMIT_Q), (uint32_t)(uz * EMIT_Q)};
    for (int k = 0; k < 3; k++) { g[k] = std::min(g[k], q[k]); g[3 + k] = std::max(g[3 + k], q[k]); }
    g[6] = std::max(g[6], emit_lum_code((float)luma(le)));
    g[7] += 1;
}
// the list from the grid (prog_emit_collect + publish): each voxel with hits a box, its hits and brightness fading
// by a tenth; at most EMIT_MAX, in voxel order; probabilities by brightness x size^2
inline void emit_build(uint32_t* g, EmitList& L, float half, float tol_setting) {
    const float R = half;
    std::vector<float> score;
    uint32_t K = 0;
    for (uint32_t cell = 0; cell < EMIT_CELLS; cell++) {
        uint32_t* v = g + 8 * cell;
        const uint32_t w = v[6], n = v[7];
        if (n == 0) continue;
        const uint32_t n2 = n - n / 10u, w2 = std::max(w, EMIT_LUM_DECAY + 1u) - EMIT_LUM_DECAY;
        v[6] = w2; v[7] = n2;
        if (n2 == 0) { v[0] = v[1] = v[2] = 0xFFFFFFFFu; v[3] = v[4] = v[5] = 0; continue; }
        float mn[3], mx[3], c[3];
        for (int k = 0; k < 3; k++) {
            mn[k] = (float)v[k] / EMIT_Q * (2.f * R) - R;
            mx[k] = (float)v[3 + k] / EMIT_Q * (2.f * R) - R;
            c[k] = (mn[k] + mx[k]) * 0.5f;
        }
        const float pad = 10.f * march_tol(V3<float>(c[0], c[1], c[2]), tol_setting);
        const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        const float r = std::sqrt(dx * dx + dy * dy + dz * dz) * 0.5f * 1.05f + pad + 4.f * (2.f * R) / EMIT_Q;
        if (K < EMIT_MAX) {
            L.box[K][0] = c[0]; L.box[K][1] = c[1]; L.box[K][2] = c[2]; L.box[K][3] = r;
            score.push_back(emit_lum_decode(w2) * r * r);
        }
        K++;
    }
    K = std::min(K, EMIT_MAX);
    float tot = 0.f;
    for (uint32_t b = 0; b < K; b++) tot += score[b];
    float acc = 0.f;
    for (uint32_t b = 0; b < K; b++) {
        const float P = tot > 0.f ? score[b] / tot : 1.f / (float)K;
        acc += P;
        L.pc[b][0] = P;
        L.pc[b][1] = b + 1 == K ? 1.f : acc;
    }
    L.count = K;
}

// the normal by three forward differences at normalTol (tracebasics.js:1310-1322 calcNormals_fast)
template <class T> inline V3<T> hit_normal(const Ctx<T>& C, const V3<T>& p, T d) {
    T eps = march_tol(p, C.tol);
    T gx = scene_eval(*C.s, V3<T>(p.x + eps, p.y, p.z)).d - d;
    T gy = scene_eval(*C.s, V3<T>(p.x, p.y + eps, p.z)).d - d;
    T gz = scene_eval(*C.s, V3<T>(p.x, p.y, p.z + eps)).d - d;
    return normalize(V3<T>(gx, gy, gz));
}

const uint32_t SPPM_STORE_SALT = 0x53505031u;   // a store's and a gather's own stream (wavefront.js:1186)
const uint32_t PHOTON_SEED_SALT = 0x50484F54u;  // the photons' sample seed: the picture's seed xor this
const uint32_t PHOTON_GEN_SALT = 0x5A17u;       // their draw at the source (wavefront.js:594)

// sppmEvaluable (wavefront.js prog_sppm): a diffuse base, or gloss rough enough (LT_MIN_ALPHA 0.05 for a photon's
// store, ALPHA_MIN 1e-3 for a camera's gather)
inline bool sppm_evaluable(const st_material& m, bool all) {
    float r = std::min(std::max(m.roughness, 0.f), 1.f);
    float rs = std::min(std::max(m.transmission, 0.f), 1.f);
    return (1.f - m.metallic) * (1.f - rs) > 0.f || r * r >= (all ? 1e-3f : 0.05f);
}
// THE GATHER at a camera vertex (sppm.js:475-494 sppmGather through sppmWalk): the eight cells, each cell's whole list
// within its share of the budget, else m of its sub-lists from a drawn start, each record weighing SUBS / m; records of
// another cell, past r, facing away or past the bounce cap passed by; f over the evaluable lobes (from LT_MIN_ALPHA)
template <class T>
inline V3<T> sppm_gather_lobes(const Ctx<T>& C, const V3<T>& X, const V3<T>& nrm, const Lobes<T>& lb, uint32_t bc,
                               Rng& rng) {
    const SppmGrid& g = *C.grid;
    const float csz = g.cell;
    const float x[3] = {(float)X.x, (float)X.y, (float)X.z};
    const float nq[3] = {(float)nrm.x, (float)nrm.y, (float)nrm.z};
    float gx[3] = {x[0] / csz, x[1] / csz, x[2] / csz};
    int32_t c0[3], side[3];
    for (int a = 0; a < 3; a++) {
        c0[a] = (int32_t)std::floor(gx[a]);
        side[a] = (gx[a] - std::floor(gx[a]) >= 0.5f) ? 1 : -1;
    }
    const uint32_t share = std::max(1u, C.sp_budget / 8);
    const uint64_t hard = (uint64_t)SPPM_VISIT_HARD * C.sp_budget;
    uint64_t visits = 0;
    bool cut = false;
    V3<T> sum(T(0));
    for (uint32_t k = 0; k < 8 && !cut; k++) {
        int32_t cell[3] = {c0[0] + ((k & 1) ? side[0] : 0), c0[1] + ((k & 2) ? side[1] : 0), c0[2] + ((k & 4) ? side[2] : 0)};
        uint32_t h = sppm_hash(cell[0], cell[1], cell[2]);
        const std::vector<uint32_t>& L = g.lists[h];
        uint32_t count = (uint32_t)L.size();
        bool whole = count <= share;
        uint32_t subs = whole ? 1 : std::max(1u, (SPPM_SUBS * share) / std::max(count, 1u));
        T w = whole ? T(1) : T(SPPM_SUBS) / T(subs);
        float u4[4];
        rng.next4(u4);
        uint32_t start = std::min((uint32_t)(u4[0] * (float)SPPM_SUBS), SPPM_SUBS - 1);
        for (uint32_t j = 0; j < subs && !cut; j++) {
            uint32_t s = (start + j) % SPPM_SUBS;
            for (uint32_t idx : L) {
                uint32_t b = g.flags[idx];
                if (!whole && ((b >> SPPM_SUB_SHIFT) & (SPPM_SUBS - 1)) != s) continue;
                if (visits >= hard) { cut = true; break; }
                visits++;
                if (b & SPPM_VOL) continue;                                     // the volume's gather's
                const float* p = &g.pos[3 * idx];
                int32_t pc[3];
                sppm_cell(p, csz, pc);
                if (pc[0] != cell[0] || pc[1] != cell[1] || pc[2] != cell[2]) continue;
                float d[3] = {p[0] - x[0], p[1] - x[1], p[2] - x[2]};
                float dd = d[0] * d[0] + d[1] * d[1];
                dd = dd + d[2] * d[2];
                if (dd > C.sp_r2) continue;
                if (bc + (b & SPPM_B_MASK) > C.p.maxbounce + 1) continue;
                float pn[3];
                sppm_unoct(g.nrm[idx], pn);
                float nd = pn[0] * nq[0] + pn[1] * nq[1];
                nd = nd + pn[2] * nq[2];
                if (nd < SPPM_NORMAL_DOT) continue;
                float l[3];
                sppm_unoct(g.dir[idx], l);
                V3<T> f = lobes_eval(lb, V3<T>(T(l[0]), T(l[1]), T(l[2])), T(0.05));
                sum += f * V3<T>(T(g.power[3 * idx]), T(g.power[3 * idx + 1]), T(g.power[3 * idx + 2])) * w;
            }
        }
    }
    return sum;
}
// lensStep (materials_pbr.js:862-873), a camera path's: at its first surface 1 for a delta event, 2 for an
// evaluable one (the map gathers there: light -> delta+ -> D -> eye, the reference's light tracer's class, is the
// map's in this build), else 0; 1 stays 1 through a delta and goes to 2 at an evaluable event; 2 or 3 go to 3
// through a delta; anything else to 0
// (with light tracing on, a D at the first surface is its class, and the reference's 0)
inline uint32_t lens_step(uint32_t lens, uint32_t bounces, uint32_t ev, bool lt) {
    const bool delta = ev == EV_DELTA;
    if (bounces == 1) return delta ? 1u : ((ev == EV_EVAL && !lt) ? 2u : 0u);   // a D at the eye's first surface
    if (lens == 1) return delta ? 1u : (ev == EV_EVAL ? 2u : 0u);
    return ((lens == 2 || lens == 3) && delta) ? 3u : 0u;
}
// sdf.js ltCovers: whether the sun's photons were drawn along this line (it crosses their square)
template <class T> inline void sun_frame(const Env<T>& e, V3<T>& b1, V3<T>& b2) {
    const V3<T> s = e.sun_dir;
    const V3<T> t = std::fabs(s.x) > T(0.9) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
    b1 = normalize(cross(t, s));
    b2 = cross(s, b1);
}
template <class T> inline bool sppm_covers(const Ctx<T>& C, const V3<T>& p, const V3<T>& d) {
    const V3<T> s = C.env.sun_dir;
    const T ds = dot(d, s);
    if (!(ds > T(0))) return false;
    const V3<T> x = p - d * (dot(p, s) / ds);
    V3<T> b1, b2;
    sun_frame(C.env, b1, b2);
    return std::fabs(dot(x, b1)) <= T(C.sp_half) && std::fabs(dot(x, b2)) <= T(C.sp_half);
}

// a path's hit, shaded: pathBegin..pathEnd (tracebasics.js:834-1100) with processMaterial_advanced
// (materials_pbr.js:1110-1440). The light sample's shadow ray is traced here and its deposit made at once.
template <class T>
inline void shade_hit(const Ctx<T>& C, Ray<T>& r, T dhit, Rng& rng, Rng& grng, bool last, Frame<T>& fr, Stats& st) {
    V3<T> n = hit_normal(C, r.pos, dhit);
    bool inside = dhit < T(0);
    V3<T> nrm = inside ? -n : n;                                                   // scene_api.js:127-135 pathFacing
    T otol = T(10) * march_tol(r.pos, C.tol);                                      // offsetTol
    if (dot(-r.dir, nrm) < T(0)) {                                                 // leaving: moved on, no bounce
        move_by(r, r.dir * otol);
        return;
    }
    SceneHit<T> h = scene_eval(*C.s, r.pos);
    const st_material& m = C.s->materials[std::min(h.m, C.s->n_materials - 1)];
    // ABSORPTION INSIDE (tracebasics.js absorbAlong; materials.js:125-133 mediumMu): met from inside, the ray crossed
    // this material from its last arrival: exp(-mu d) a channel, mu = -ln(base) / attenuationDistance
    if (inside && m.attenuation > 0.f) {
        const T d = std::max(r.ltot - r.absLtot, T(0)) / std::max(r.n, T(1e-4));
        const T ia = T(1) / T(m.attenuation);
        V3<T> tr;
        tr.x = std::exp(std::log(std::min(std::max(T(m.base[0]), T(1e-6)), T(1))) * ia * d);
        tr.y = std::exp(std::log(std::min(std::max(T(m.base[1]), T(1e-6)), T(1))) * ia * d);
        tr.z = std::exp(std::log(std::min(std::max(T(m.base[2]), T(1e-6)), T(1))) * ia * d);
        r.beta = r.beta * tr;
    }
    r.absLtot = r.ltot;                                                            // absorbAlong: arrival here
    V3<T> emis(T(m.emissive[0]), T(m.emissive[1]), T(m.emissive[2]));
    // THE PHOTON MAP'S GATHER (wavefront.js:1196-1212), before the shading: a camera ray with delta events only since
    // the eye, on an evaluable surface, takes sum f Phi / (pi r^2) / n^2 into its radiance
    if (C.sppm && ((r.bounces == 0 && !C.lt) || r.lens == 1) && !(max3(emis) > T(0)) && sppm_evaluable(m, true)) {
        T n0g = r.n;
        Lobes<T> lg = make_lobes(nrm, -r.dir, m, n0g / std::max(T(m.ior), n0g), C.tb, T(m.transmission), T(m.specular),
                                 T(m.haze), n0g, false, r.lam);
        V3<T> L = sppm_gather_lobes(C, r.pos, nrm, lg, r.bounces + 1, grng) * T(C.sp_inv_area / ((double)n0g * n0g));
        r.rad += r.beta * L;
    }
    r.bounces += 1;
    const uint32_t fid = C.faces ? C.face_of[std::min(h.m, C.s->n_materials - 1)] : 0u;
    if (fid) {                                                                     // a light's face (codegen.js:795-836)
        const OFace& f = (*C.faces)[fid - 1];
        const T cosY = -(r.dir.x * T(f.n[0]) + r.dir.y * T(f.n[1]) + r.dir.z * T(f.n[2]));
        T w = T(1);
        if (r.bounces >= 2 && r.lpx >= T(0)) {
            const T pl = T(face_density(FACE_SHARE, C.faces->size(), f,
                                        (double)(std::max(r.ltot - r.lpy, T(0)) / std::max(r.n, T(1e-4))), (double)cosY));
            const T a2 = r.lpx * r.lpx;
            w = a2 / std::max(a2 + pl * pl, T(1e-20));
        }
        r.rad += r.beta * V3<T>(T(f.le[0]), T(f.le[1]), T(f.le[2])) *
                 (T(face_beam(f, (double)cosY)) / std::max(r.n * r.n, T(1)) * w);
        r.state = RAY_SOURCE;
        move_by(r, r.dir * (otol * T(2)));
        return;
    }
    if (max3(emis) > T(0)) {                                                       // materials_pbr.js:1014-1075 emitterHit
        const T beam = m.beam_cos > 0.f ? (-dot(r.dir, n) >= T(m.beam_cos) ? T(1) : T(0)) : T(1);   // lights.js beamShape
        // weighed against the last vertex's emitter light sample; left to the emitter photons by a path in light
        // tracing's class (or the map's) where a probe could have started one (materials_pbr.js:1044-1047)
        T w = r.emw;
        if (C.lt_emit_n && (r.cls == 3u || (C.sppm && r.lens == 3)) && emit_covers(*C.em, r.pos)) w = T(0);
        r.rad += r.beta * emis * (w * beam);
        if (C.em_on) emit_deposit(C, r.pos, emis);  // and discovered
        r.state = RAY_SOURCE;
        move_by(r, r.dir * (otol * T(2)));
        return;
    }
    T n0 = r.n;
    T n1d = std::max(T(m.ior), n0);                                                // ownMedium (materials_pbr.js:1080)
    T v1 = T(0);
    uint32_t beyond = inside ? 0u : std::min(h.m, C.s->n_materials - 1);          // the medium a refraction enters
    if (m.transmission > 0 && m.metallic < 1) {                                    // asksMedium (materials.js:114)
        SceneHit<T> mb = scene_eval(*C.s, r.pos + (-nrm) * (otol * T(2)));         // mediumBeyond (tracebasics.js:1332)
        beyond = std::min(mb.a, C.s->n_materials - 1);
        const st_material& mm = C.s->materials[beyond];
        n1d = T(mm.ior);
        v1 = T(mm.abbe);
    }
    // DISPERSION (materials_pbr.js:1116-1139): the medium beyond at the ray's own wavelength, if it has one; a ray
    // without one, at a dispersive medium beyond, draws one, used only if it refracts
    const T lam0 = r.lam;
    const T n1 = lam0 > T(0) ? cauchy_n(n1d, v1, lam0) : n1d;
    const bool draw = v1 > T(0) && lam0 == T(0);
    T nT = n1, lamD = T(0);
    V3<T> specW(T(1), T(1), T(1));
    if (draw) {
        T ul[4]; rng.next4(ul);
        lamD = lambda_coded(spec_draw(ul[0], specW));
        nT = cauchy_n(n1d, v1, lamD);
    }
    // A FACE THAT BOTH REFRACTS AND DIFFUSES, SEEN FROM INSIDE (materials_pbr.js:1150-1165): one part drawn
    T pG = refract_share<T>(m);
    T trans = T(m.transmission), specv = T(m.specular), hz = T(m.haze);
    bool diffFace = pG <= T(0) && m.transmission > 0.f;                          // haze 1: the diffuse face alone
    if (inside && pG > T(0) && pG < T(1)) {
        T k = mixT(T(2) * T(m.specular), T(1), pG);
        T u4[4]; rng.next4(u4);
        if (u4[0] < pG) { trans = T(1); hz = T(0); }
        else {
            trans = sat(sat(T(m.transmission)) * sat(T(m.haze)) / std::max(T(1) - pG, T(1e-6)));
            hz = T(1); specv = T(0.5) * k; diffFace = true;
        }
    }
    T etaFace = diffFace ? std::min(n0, n1) / std::max(n0, n1) : n0 / n1;
    Lobes<T> lb = make_lobes(nrm, -r.dir, m, etaFace, C.tb, trans, specv, hz, n0, inside, lam0);
    lb.etaT = n0 / nT;
    coat_pick(lb, r.beta);
    // THE SIDE BEYOND, LIT (materials_pbr.js:1176-1190): through this face where the medium beyond is air
    const bool throughLit = std::fabs(n1 - T(1)) <= T(1e-3) && through_evaluable<T>(m, trans, hz);
    lb.through = throughLit;
    const T qf = throughLit ? T(1) : T(0);

    // LIGHT SAMPLING (materials_pbr.js:1196-1330): the lights' faces with their share (lightFaceShare), then of the
    // rest the discovered emitters with theirs (0 while nothing is listed), else the environment -- with no face and
    // nothing listed, the environment's draw is what it always was
    const T es = (C.em_on && C.em_nee && C.p.nee != 0 && !last && C.em->count > 0)
                     ? T(std::min(std::max(C.em_share, 0.05f), 0.95f)) : T(0);
    const T fs = (C.faces && !C.faces->empty() && C.p.nee != 0 && !last) ? T(FACE_SHARE) : T(0);
    const T rs = T(1) - fs;
    if (C.p.nee != 0 && !last) {
        T u0[4], u1[4];
        rng.next4(u0);                                                             // pick00
        rng.next4(u1);                                                             // uL
        if (!lobes_none<T>(m, trans, hz)) {
            V3<T> L(0, 0, 1);
            T pS = 0, fdist = 0;
            bool toEmit = false, toFace = false;
            V3<T> fle(0, 0, 0);
            const T pick0 = (u0[0] - fs) / std::max(rs, T(1e-6));
            if (u0[0] < fs) {                                                      // a face, a point uniform on it
                const size_t nf = C.faces->size();
                const OFace& f = (*C.faces)[std::min((size_t)(u0[1] * T(nf)), nf - 1)];
                double y[3];
                face_point(f, (double)u1[0], (double)u1[1], y);
                const V3<T> dy = V3<T>(T(y[0]), T(y[1]), T(y[2])) - r.pos;
                fdist = length(dy);
                L = dy * (T(1) / std::max(fdist, T(1e-20)));
                const T cosY = -(L.x * T(f.n[0]) + L.y * T(f.n[1]) + L.z * T(f.n[2]));
                if (fdist > T(0) && cosY > T(1e-6)) {
                    pS = T(face_density((double)fs, nf, f, (double)fdist, (double)cosY));
                    const T nSide = dot(nrm, L) < T(0) ? n1 : r.n;                       // the far side's is air
                    fle = V3<T>(T(f.le[0]), T(f.le[1]), T(f.le[2])) *
                          (T(face_beam(f, (double)cosY)) / std::max(nSide * nSide, T(1)));
                    toFace = true;
                }
            } else if (pick0 < es) {
                const uint32_t b = emit_pick(*C.em, (float)(pick0 / es));
                if (emit_sample(*C.em, b, r.pos, u1[0], u1[1], L)) {
                    pS = rs * es * emit_cone_pdf(*C.em, r.pos, L);
                    toEmit = true;
                }
            } else {
                T pick = es > T(0) ? (pick0 - es) / (T(1) - es) : pick0;
                L = env_sample_dir_q(C.env, nrm, pick, u1[0], u1[1], qf);
                pS = rs * (T(1) - es) * env_pdf_q(C.env, L, nrm, qf);
            }
            T NoL = dot(nrm, L);
            if ((NoL > T(0) || (throughLit && NoL < T(0))) && pS > T(0)) {              // sideLit
                V3<T> le = toEmit ? V3<T>(1, 1, 1) : (toFace ? fle : C.env.radiance(L));
                V3<T> f = lobes_eval(lb, L, T(0));
                T pB = lobes_pdf(lb, L);
                T w = mis_weight(pS, pB);
                V3<T> contrib = r.beta * f * le * (std::fabs(NoL) * (w / pS));
                if (max3(contrib) > (toEmit ? T(1e-9) : T(1e-7))) {
                    const T nS = NoL < T(0) ? n1 : r.n;                                // the medium the ray crosses
                    V3<T> o = r.pos + nrm * (NoL < T(0) ? -otol * T(2) : otol * T(2));
                    T tr = T(1);
                    const bool air = C.haze.on && std::fabs(nS - T(1)) <= T(1e-3);
                    T R = T(C.d.env_radius);
                    if (toFace) {
                        // the face's ray aims at the point and arrives just short of it (TAG_FNEE)
                        if (air) tr = C.haze.transmittance(r.pos, L, fdist, R);
                        const T l0 = -std::max(fdist - T(40) * march_tol(o, C.tol), T(0)) * nS;
                        if (occlude(C, o, L, nS, st, (V3<T>*)nullptr, (T*)nullptr, true, l0)) deposit(fr, r.pix, contrib * tr, st);
                    } else if (!toEmit) {
                        if (air) tr = C.haze.transmittance(r.pos, L, T(2) * R + length(r.pos), R);   // haze.js:472-485
                        if (occlude(C, o, L, nS, st)) deposit(fr, r.pix, contrib * tr, st);
                    } else {
                        // an emitter's ray counts the emission of whatever it stops at (wavefront.js:1694-1749)
                        V3<T> hp;
                        T hl = 0;
                        if (!occlude(C, o, L, nS, st, &hp, &hl)) {
                            SceneHit<T> hh = scene_eval(*C.s, hp);
                            const st_material& me = C.s->materials[std::min(hh.m, C.s->n_materials - 1)];
                            V3<T> ee(T(me.emissive[0]), T(me.emissive[1]), T(me.emissive[2]));
                            if (me.beam_cos > 0.f && max3(ee) > T(0)) {                        // lights.js beamShape
                                const V3<T> nh = hit_normal(C, hp, hh.d);
                                if (!(-dot(L, nh) >= T(me.beam_cos))) ee = V3<T>(0, 0, 0);
                            }
                            if (max3(ee) > T(0)) {
                                if (air) tr = C.haze.transmittance(o, L, std::max(hl, T(0)) / std::max(nS, T(1e-4)), R);
                                deposit(fr, r.pix, contrib * ee * tr, st);
                            }
                        }
                    }
                }
            }
        }
    }
    // THE BOUNCE (materials_pbr.js:1332-1345)
    T ur[4]; rng.next4(ur);
    LobeSample<T> smp = lobes_sample(lb, ur);
    r.dir = smp.dir;
    r.beta *= smp.w;
    if (smp.transmitted) {
        r.n = nT;                                                                  // n(lambda) where it has one
        if (draw) { r.beta *= specW; r.lam = lamD; }
        r.medium = beyond;                                                         // tracebasics.js:522-530 enterMedium
    }
    if (C.sppm) r.lens = lens_step(r.lens, r.bounces, smp.ev, C.lt);
    if (C.lt) {                                                                    // tracebasics.js:995-1011
        if (r.bounces == 1) r.cls = smp.ev == EV_EVAL ? 1u : 0u;
        else if (r.cls & 1u) r.cls = smp.ev == EV_DELTA ? 3u : 0u;
    }
    if (max3(smp.w) <= T(0)) r.state = RAY_ABSORBED;
    bool misOut = C.p.nee != 0 && !last;
    if (misOut) {                                                                  // materials_pbr.js:1370-1395
        const T cO = dot(nrm, r.dir);
        bool above = (cO > T(0) || (throughLit && cO < T(0))) && !smp.isDelta;      // sideLit
        T pOut = smp.isDelta ? T(0) : lobes_pdf(lb, smp.dir);
        T pLout = above ? rs * (T(1) - es) * env_pdf_q(C.env, r.dir, nrm, qf) : T(0);
        r.sunmis = pLout <= T(0) ? T(1) : mis_weight(pOut, pLout);
        const T pEout = (above && es > T(0)) ? rs * es * emit_cone_pdf(*C.em, r.pos, r.dir) : T(0);
        r.emw = pEout <= T(0) ? T(1) : mis_weight(pOut, pEout);
        r.lpx = (above && fs > T(0) && !lobes_none<T>(m, trans, hz)) ? pOut : T(-1);   // prevPdf, for a face it meets
    } else {
        r.sunmis = T(1);
        r.emw = T(1);
        r.lpx = T(-1);
    }
    r.lpy = r.ltot;                                                                // vtxLtot
    move_by(r, r.dir * otol);
    // pathEnd's tail (tracebasics.js:1040-1103): the bounce cap, Russian roulette
    if (r.bounces > C.p.maxbounce) r.state = RAY_TERMINATED;
    if (C.p.rr != 0 && r.bounces >= 3 && r.state == RAY_ACTIVE) {
        T p = clampT(max3(r.beta), T(0.1), T(0.95));
        T u[4]; rng.next4(u);
        if (u[0] > p) r.state = RAY_TERMINATED;
        else r.beta = r.beta / p;
    }
}

// A PHOTON'S HIT (an optics ray, TAG_PHOTON | TAG_OPTIC): pathBegin..pathEnd without light sampling -- a photon
// carries flux, it samples no light (materials_pbr.js:1196-1201) -- and without the photon's end at a scatter,
// since an optics ray walks through every event (tracebasics.js:1008-1022); the bounce cap stays.
template <class T>
inline void shade_photon(const Ctx<T>& C, Ray<T>& r, T dhit, Rng& rng) {
    V3<T> n = hit_normal(C, r.pos, dhit);
    bool inside = dhit < T(0);
    V3<T> nrm = inside ? -n : n;
    T otol = T(10) * march_tol(r.pos, C.tol);
    if (dot(-r.dir, nrm) < T(0)) { move_by(r, r.dir * otol); return; }
    r.bounces += 1;
    SceneHit<T> h = scene_eval(*C.s, r.pos);
    const st_material& m = C.s->materials[std::min(h.m, C.s->n_materials - 1)];
    T n0 = r.n;
    T n1 = std::max(T(m.ior), n0);
    if (m.transmission > 0 && m.metallic < 1) {
        SceneHit<T> mb = scene_eval(*C.s, r.pos + (-nrm) * (otol * T(2)));
        n1 = T(C.s->materials[std::min(mb.a, C.s->n_materials - 1)].ior);
    }
    T pG = refract_share<T>(m);
    T trans = T(m.transmission), specv = T(m.specular), hz = T(m.haze);
    bool diffFace = pG <= T(0) && m.transmission > 0.f;
    if (inside && pG > T(0) && pG < T(1)) {
        T k = mixT(T(2) * T(m.specular), T(1), pG);
        T u4[4]; rng.next4(u4);
        if (u4[0] < pG) { trans = T(1); hz = T(0); }
        else {
            trans = sat(sat(T(m.transmission)) * sat(T(m.haze)) / std::max(T(1) - pG, T(1e-6)));
            hz = T(1); specv = T(0.5) * k; diffFace = true;
        }
    }
    T etaFace = diffFace ? std::min(n0, n1) / std::max(n0, n1) : n0 / n1;
    Lobes<T> lb = make_lobes(nrm, -r.dir, m, etaFace, C.tb, trans, specv, hz, n0, inside, T(0));
    lb.etaT = n0 / n1;
    coat_pick(lb, r.beta);
    T ur[4]; rng.next4(ur);
    LobeSample<T> smp = lobes_sample(lb, ur);
    r.dir = smp.dir;
    r.beta *= smp.w;
    if (smp.transmitted) r.n = n1;
    if (max3(smp.w) <= T(0)) r.state = RAY_ABSORBED;
    r.sunmis = T(1);
    move_by(r, r.dir * otol);
    if (r.bounces > C.p.maxbounce) r.state = RAY_TERMINATED;
}

// ------------------------------------------------------------------------------------------------------------
// THE MEDIUM VERTEX -- core/haze.js:493-596 mediumVertex, mediumNee: a point in the dust, its light sample
// (sun's cone or the uniform sphere, power heuristic against the phase function) and its phase-function draw
// ------------------------------------------------------------------------------------------------------------
template <class T>
void medium_vertex(const Ctx<T>& C, Ray<T>& r, Rng& rng, bool last, Frame<T>& fr, Stats& st) {
    r.state = RAY_ACTIVE;
    r.bounces += 1;
    T g = clampT(C.haze.g, T(-0.95), T(0.95));
    V3<T> din = r.dir;
    r.beta = r.beta * C.haze.albedo;
    // the discovered emitters' share of the air's light samples (haze.js:324-370), as at a surface
    const T es = (C.em_on && C.em_nee && C.p.nee != 0 && !last && C.em->count > 0)
                     ? T(std::min(std::max(C.em_share, 0.05f), 0.95f)) : T(0);
    const T fs = (C.faces && !C.faces->empty() && C.p.nee != 0 && !last) ? T(FACE_SHARE) : T(0);   // haze.js:315-350
    const T rs = T(1) - fs;
    if (C.p.nee != 0 && !last) {
        T u0[4], u1[4];
        rng.next4(u0); rng.next4(u1);
        V3<T> L(0, 0, 1);
        T pS = 0, fdist = 0;
        bool toEmit = false, toFace = false;
        V3<T> fle(0, 0, 0);
        const T pick0 = (u0[0] - fs) / std::max(rs, T(1e-6));
        if (u0[0] < fs) {                                      // a face: no vertex normal, the face's own side
            const size_t nf = C.faces->size();
            const OFace& f = (*C.faces)[std::min((size_t)(u0[1] * T(nf)), nf - 1)];
            double y[3];
            face_point(f, (double)u1[0], (double)u1[1], y);
            const V3<T> dy = V3<T>(T(y[0]), T(y[1]), T(y[2])) - r.pos;
            fdist = length(dy);
            L = dy * (T(1) / std::max(fdist, T(1e-20)));
            const T cosY = -(L.x * T(f.n[0]) + L.y * T(f.n[1]) + L.z * T(f.n[2]));
            if (fdist > T(0) && cosY > T(1e-6)) {
                pS = T(face_density((double)fs, nf, f, (double)fdist, (double)cosY));
                fle = V3<T>(T(f.le[0]), T(f.le[1]), T(f.le[2])) * T(face_beam(f, (double)cosY));   // in air
                toFace = true;
            }
        } else if (pick0 < es) {
            const uint32_t b = emit_pick(*C.em, (float)(pick0 / es));
            if (emit_sample(*C.em, b, r.pos, u1[0], u1[1], L)) { pS = rs * es * emit_cone_pdf(*C.em, r.pos, L); toEmit = true; }
        } else {
            L = env_sample_dir_m(C.env, es > T(0) ? (pick0 - es) / (T(1) - es) : pick0, u1[0], u1[1]);
            pS = rs * (T(1) - es) * env_pdf_m(C.env, L);
        }
        if (pS > T(0)) {
            T ph = hg_eval(dot(din, L), g);
            T w = mis_weight(pS, ph);
            V3<T> le = toEmit ? V3<T>(1, 1, 1) : (toFace ? fle : C.env.radiance(L));
            V3<T> contrib = r.beta * le * (ph * w / pS);
            if (max3(contrib) > (toEmit ? T(1e-9) : T(1e-7))) {
                T R = T(C.d.env_radius);
                if (toFace) {
                    T tr = C.haze.transmittance(r.pos, L, fdist, R);
                    const T l0 = -std::max(fdist - T(40) * march_tol(r.pos, C.tol), T(0)) * r.n;
                    if (occlude(C, r.pos, L, r.n, st, (V3<T>*)nullptr, (T*)nullptr, true, l0)) deposit(fr, r.pix, contrib * tr, st);
                } else if (!toEmit) {
                    T tr = C.haze.transmittance(r.pos, L, T(2) * R + length(r.pos), R);   // haze.js:472-485 hazeShadow
                    if (occlude(C, r.pos, L, r.n, st)) deposit(fr, r.pix, contrib * tr, st);
                } else {
                    V3<T> hp;
                    T hl = 0;
                    if (!occlude(C, r.pos, L, r.n, st, &hp, &hl)) {
                        SceneHit<T> hh = scene_eval(*C.s, hp);
                        const st_material& me = C.s->materials[std::min(hh.m, C.s->n_materials - 1)];
                        V3<T> ee(T(me.emissive[0]), T(me.emissive[1]), T(me.emissive[2]));
                        if (me.beam_cos > 0.f && max3(ee) > T(0)) {                        // lights.js beamShape
                            const V3<T> nh = hit_normal(C, hp, hh.d);
                            if (!(-dot(L, nh) >= T(me.beam_cos))) ee = V3<T>(0, 0, 0);
                        }
                        if (max3(ee) > T(0)) {
                            T tr = T(1);
                            if (C.haze.on && std::fabs(r.n - T(1)) <= T(1e-3))
                                tr = C.haze.transmittance(r.pos, L, std::max(hl, T(0)) / std::max(r.n, T(1e-4)), R);
                            deposit(fr, r.pix, contrib * ee * tr, st);
                        }
                    }
                }
            }
        }
    }
    T u2[4]; rng.next4(u2);
    V3<T> dout = hg_sample(din, g, u2[0], u2[1]);
    r.dir = dout;
    bool misOut = C.p.nee != 0 && !last;
    if (misOut) {
        T pB = hg_eval(dot(din, dout), g);
        T pL = rs * (T(1) - es) * env_pdf_m(C.env, dout);
        r.sunmis = pL <= T(0) ? T(1) : mis_weight(pB, pL);
        const T pE = es > T(0) ? rs * es * emit_cone_pdf(*C.em, r.pos, dout) : T(0);
        r.emw = pE <= T(0) ? T(1) : mis_weight(pB, pE);
        r.lpx = fs > T(0) ? pB : T(-1);
    } else {
        r.sunmis = T(1);
        r.emw = T(1);
        r.lpx = T(-1);
    }
    r.lpy = r.ltot;
    if (r.bounces > C.p.maxbounce) r.state = RAY_TERMINATED;
}

// THE GATHER IN A VOLUME (sppm.js:497-511 sppmGatherVolume through sppmWalk :305-360): the records photons stored where
// they collided (SPPM_VOL) within R in the eight cells of the volume's grid round x, each through the phase function
// from the way it came to the way to the camera, sum p(l . v) Phi / (sigma 4/3 pi R^3); whole cells within their share
// of the budget, else m sub-lists from a drawn start weighing 32 / m; the walk cut at the hard cap
template <class T>
inline V3<T> sppm_gather_volume(const Ctx<T>& C, const V3<T>& X, const V3<T>& v, uint32_t bc, T g, T sigma, Rng& rng) {
    const SppmGrid& gr = *C.grid;
    if (!(sigma > T(0)) || gr.flags.empty()) return V3<T>(T(0));
    const float csz = gr.vcell;
    const float x[3] = {(float)X.x, (float)X.y, (float)X.z};
    int32_t c0[3], side[3];
    for (int a = 0; a < 3; a++) {
        const float gx = x[a] / csz;
        c0[a] = (int32_t)std::floor(gx);
        side[a] = (gx - std::floor(gx) >= 0.5f) ? 1 : -1;
    }
    const uint32_t share = std::max(1u, C.sp_budget / 8);
    const uint64_t hard = (uint64_t)SPPM_VISIT_HARD * C.sp_budget;
    uint64_t visits = 0;
    bool cut = false;
    V3<T> sum(T(0));
    for (uint32_t k = 0; k < 8 && !cut; k++) {
        const int32_t cell[3] = {c0[0] + ((k & 1) ? side[0] : 0), c0[1] + ((k & 2) ? side[1] : 0),
                                 c0[2] + ((k & 4) ? side[2] : 0)};
        const std::vector<uint32_t>& L = gr.lists[sppm_hash(cell[0], cell[1], cell[2])];
        const uint32_t count = (uint32_t)L.size();
        const bool whole = count <= share;
        const uint32_t subs = whole ? 1 : std::max(1u, (SPPM_SUBS * share) / std::max(count, 1u));
        const T w = whole ? T(1) : T(SPPM_SUBS) / T(subs);
        float u4[4];
        rng.next4(u4);
        const uint32_t start = std::min((uint32_t)(u4[0] * (float)SPPM_SUBS), SPPM_SUBS - 1);
        for (uint32_t j = 0; j < subs && !cut; j++) {
            const uint32_t s = (start + j) % SPPM_SUBS;
            for (uint32_t idx : L) {
                const uint32_t b = gr.flags[idx];
                if (!whole && ((b >> SPPM_SUB_SHIFT) & (SPPM_SUBS - 1)) != s) continue;
                if (visits >= hard) { cut = true; break; }
                visits++;
                if (!(b & SPPM_VOL) || bc + (b & SPPM_B_MASK) > C.p.maxbounce + 1) continue;
                const float* p = &gr.pos[3 * idx];
                int32_t pc[3];
                sppm_cell(p, csz, pc);
                if (pc[0] != cell[0] || pc[1] != cell[1] || pc[2] != cell[2]) continue;
                const float d[3] = {p[0] - x[0], p[1] - x[1], p[2] - x[2]};
                float dd = d[0] * d[0] + d[1] * d[1];
                dd = dd + d[2] * d[2];
                if (dd > C.sp_vr2) continue;
                float l[3];
                sppm_unoct(gr.dir[idx], l);
                const T f = hg_eval(T(l[0]) * v.x + T(l[1]) * v.y + T(l[2]) * v.z, g);
                sum += V3<T>(T(gr.power[3 * idx]), T(gr.power[3 * idx + 1]), T(gr.power[3 * idx + 2])) * (w * f);
            }
        }
    }
    return sum * T(C.sp_inv_vol / (double)sigma);
}
// THE MAP GATHERED AT A COLLISION (haze.js:692-707 mediumGathered): the throughput absorbed to here, the photons'
// in-scattered light over n^2, then the ray turned there -- a vertex, the map's D: a bounce, its lens field 2, light
// sampling's MIS halves cleared, its next flight drawn from here
template <class T> inline void medium_gathered(const Ctx<T>& C, Ray<T>& r, Rng& rng, Rng& grng, bool last) {
    const st_material& mm = C.s->materials[std::min(r.medium, C.s->n_materials - 1)];
    const T sig = mm.scatter_distance > 0.f ? T(1) / T(mm.scatter_distance) : T(0);
    const T g = clampT(T(mm.scatter_g), T(-0.95), T(0.95));
    if (mm.attenuation > 0.f) {
        const T dl = std::max(r.ltot - r.absLtot, T(0)) / std::max(r.n, T(1e-4)) / T(mm.attenuation);
        r.beta.x *= std::exp(std::log(std::min(std::max(T(mm.base[0]), T(1e-6)), T(1))) * dl);
        r.beta.y *= std::exp(std::log(std::min(std::max(T(mm.base[1]), T(1e-6)), T(1))) * dl);
        r.beta.z *= std::exp(std::log(std::min(std::max(T(mm.base[2]), T(1e-6)), T(1))) * dl);
    }
    r.absLtot = r.ltot;
    const V3<T> Lv = sppm_gather_volume(C, r.pos, r.dir, r.bounces + 1, g, sig, grng);
    r.rad += r.beta * Lv * (T(1) / std::max(r.n * r.n, T(1e-8)));
    r.state = RAY_ACTIVE;
    r.bounces += 1;
    r.lens = 2;
    r.cls = 0;
    T u[4]; rng.next4(u);
    r.dir = hg_sample(r.dir, g, u[0], u[1]);
    r.sunmis = T(1); r.emw = T(1); r.lpx = T(-1); r.lpy = r.ltot;
    if (last || r.bounces > C.p.maxbounce) r.state = RAY_TERMINATED;
}

template <class T>
void trace_path(const Ctx<T>& C, U4 sseed, uint32_t tile, const st_view& v, uint32_t W, uint32_t H,
                Frame<T>& fr, Stats& st) {
    // genrays (genrays.js:26-97): the tile grid, one jittered ray through the tile
    Rng rng0 = path_rng(sseed, tile, 0);
    const double N = double(W) * double(H);
    uint32_t tilesX = std::max<uint32_t>(1, (uint32_t)std::llround(std::sqrt(N * (double(W) / std::max<double>(1, H)))));
    uint32_t tilesY = std::max<uint32_t>(1, (uint32_t)std::ceil(N / tilesX));
    T invTX = T(float(1.0 / tilesX)), invTY = T(float(1.0 / tilesY));
    T cx = T(tile % tilesX), cy = T(tile / tilesX);
    T uv0x = (cx + T(0.5)) * invTX, uv0y = (cy + T(0.5)) * invTY;
    T rnd[4]; rng0.next4(rnd);
    T ux = clampT(uv0x + (rnd[0] - T(0.5)) * invTX, T(0), T(1));
    T uy = clampT(uv0y + (rnd[1] - T(0.5)) * invTY, T(0), T(1));
    T xx = ux * T(2) - T(1), yy = uy * T(2) - T(1);
    V3<T> right(T(v.right[0]), T(v.right[1]), T(v.right[2])), up(T(v.up[0]), T(v.up[1]), T(v.up[2])),
        fwd(T(v.fwd[0]), T(v.fwd[1]), T(v.fwd[2])), cam(T(v.cam_pos[0]), T(v.cam_pos[1]), T(v.cam_pos[2]));
    Ray<T> r;
    if (v.camtype == 0) {
        V3<T> dc(xx * T(v.fx), yy * T(v.fy), T(-1));
        r.dir = normalize(right * dc.x + up * dc.y + fwd * dc.z);
        r.pos = cam;
        if (v.lens_radius > 0.f) {                                                 // genrays.js:80-87, lens.js lensDisc
            const T rr = T(v.lens_radius) * std::sqrt(rnd[2]);
            const T ph = T(6.28318530718) * rnd[3];
            const V3<T> off = right * (rr * std::cos(ph)) + up * (rr * std::sin(ph));
            r.pos = cam + off;
            r.dir = normalize((right * dc.x + up * dc.y + fwd * dc.z) * T(v.focus_distance) - off);
        }
    } else {
        r.pos = cam + right * (xx * T(v.fx)) + up * (yy * T(v.fy));
        r.dir = -fwd;
    }
    r.dir = normalize(r.dir);                                                      // newRay (tracebasics.js:479-499)
    r.beta = V3<T>(1); r.rad = V3<T>(0);
    r.ltot = 0; r.n = 1; r.sunmis = 1; r.tmax = 0; r.absLtot = 0;
    r.bounces = 0; r.steps = 0; r.state = RAY_ACTIVE;
    T px = clampT(ux * T(W), T(0), T(W) - T(1)), py = clampT(uy * T(H), T(0), T(H) - T(1));
    r.pix = (uint32_t)px + (uint32_t)py * W;

    // The wavefront's iterations, as they pass this path: a segment is marched MARCH_CHUNK evaluations an iteration
    // (the reference's 32-step dispatches, wavefront.js:870; the last iteration marches to the end), then shaded in
    // the iteration its march ended. Its random numbers are seeded by how many times it has been shaded (seg).
    uint32_t it = 0, seg = 0;
    while (it < C.budget) {
        bool use_haze = C.haze.on;
        if (use_haze && r.tmax == T(0) && !walks(C, r)) {                          // haze.js:255-273 hazeDraw
            // from where the leg starts: the vertex, before the step off it (absLtot is the ltot on arrival there)
            V3<T> A = r.pos - r.dir * (std::max(r.ltot - r.absLtot, T(0)) / std::max(r.n, T(1e-4)));
            Rng hr = path_rng(sseed, tile, SEED_SALT_HAZE + seg);
            r.tmax = C.haze.draw(A, r.dir, r.absLtot, r.n, T(C.d.env_radius), hr);
        }
        uint32_t evals = 0;
        const WalkIO wio{sseed, tile, (C.sppm && r.lens == 1) ? 2 : 0, nullptr};
        T dh = march(C, r, st, use_haze, evals, &wio);
        uint32_t chunks = std::max(1u, (evals + MARCH_CHUNK - 1) / MARCH_CHUNK);
        it = std::min(it + chunks - 1, C.budget - 1);
        bool last = it + 1 == C.budget;
        st.segments++;
        if (r.state == RAY_ESCAPED) {                                              // wavefront.js:1292-1310
            // a path the photon map owns (lens field 3), or light tracing (its class), takes the sky but not the disc
            // where the photons were drawn
            bool owned = ((C.sppm && r.lens == 3) || (C.lt && r.cls == 3u)) && sppm_covers(C, r.pos, r.dir);
            r.rad += r.beta * (owned ? C.env.sky_only(r.dir) : C.env.radiance(r.dir)) * r.sunmis;
            break;
        }
        if (r.state != RAY_ACTIVE && r.state != RAY_SCATTER && r.state != RAY_GATHER) break;   // out of steps or length
        Rng rng = path_rng(sseed, tile, 1 + seg);
        Rng grng = path_rng(sseed, tile, SPPM_STORE_SALT + seg);                   // the gather's own stream
        seg++;
        if (r.state == RAY_GATHER) {
            medium_gathered(C, r, rng, grng, last);
        } else if (r.state == RAY_SCATTER) {
            r.absLtot = r.ltot;                                                    // absorbAlong on arrival
            medium_vertex(C, r, rng, last, fr, st);
            r.lens = 0;                                                            // haze.js:539
            r.cls = (C.lt && r.bounces == 1) ? 1u : 0u;                            // haze.js:550-553
        } else {
            shade_hit(C, r, dh, rng, grng, last, fr, st);
        }
        if (r.state != RAY_ACTIVE) break;
        r.tmax = T(0);                                                             // a new leg (wavefront.js:1375-1380)
        if (last) { r.state = RAY_MAXITER; st.flushed++; break; }                  // THE FLUSH (wavefront.js:949-968)
        it++;
    }
    // THE PATH IS OVER (wavefront.js:1400-1425): its radiance into the frame, and it counts once
    deposit(fr, r.pix, r.rad, st);
#pragma omp atomic
    fr.cnt[r.pix] += 1;
    st.paths++;
}

// ------------------------------------------------------------------------------------------------------------
// THE OPTICS TRACE, one ray (optics/kernels.js:429-438 the generator, :571-699 the shade): a photon that walks
// through every event (TAG_OPTIC) -- no light sampling, no end at a diffuse bounce -- until it escapes, is absorbed,
// is stopped by a detector or runs out of bounces or steps; what it carries, as luminance (optWeight), tallied per
// interaction. Seeded by its id at the source and by its id and bounces at each shade (kernels.js:602-606).
// ------------------------------------------------------------------------------------------------------------
struct OptTally {
    double escaped = 0, lost = 0, detected = 0, absorbed = 0, emitted = 0;
    uint64_t interactions = 0;
    std::vector<double> far, lux;
    // by object (the item's first primitive) and by material: weight incident, leaving, interactions
    // (kernels.js:651-681 O_TAG / O_MAT); the rays escaped, lost, detected, absorbed (O_COUNT); the detector hits
    // (optRecordHit: position, weight, direction, tag)
    std::vector<double> tag, mat;
    uint64_t n_escaped = 0, n_lost = 0, n_detected = 0, n_absorbed = 0;
    std::vector<float> hits;
};
struct OptFrame {
    float axis[3], c0[3], c90[3], origin[3];
    uint32_t nC, nG, cells;
    float half, height;
};

template <class T>
void optics_ray(const Ctx<T>& C, U4 bseed, uint32_t id, const st_optics_source* src, const float* cdf, uint32_t nsrc,
                const OptFrame& F, uint32_t maxbounce, OptTally& tl) {
    Rng r0; r0.h = bseed; r0.seed_u32(id); r0.seed_u32(0x9E3779B9u);
    V3<T> org, dir;
    uint32_t which;
    T w;
    source_ray(src, cdf, nsrc, r0, C.tol, org, dir, which, w);
    Ray<T> r;
    r.pos = org; r.dir = dir;
    r.beta = V3<T>(w); r.rad = V3<T>(1);
    r.ltot = 0; r.n = T(std::max(1.f, src[which].emit_n)); r.sunmis = 1; r.tmax = 0; r.absLtot = 0;
    r.bounces = 0; r.steps = 0; r.state = RAY_ACTIVE; r.pix = id;
    tl.emitted += (double)luma(r.beta * r.rad);
    Stats st;
    for (;;) {
        uint32_t evals = 0;
        T dh = march(C, r, st, false, evals);
        T wIn = luma(r.beta * r.rad);
        if (r.state == RAY_ESCAPED) {                                             // kernels.js:609-625
            tl.escaped += (double)wIn;
            tl.n_escaped++;
            float d[3] = {(float)r.dir.x, (float)r.dir.y, (float)r.dir.z};
            tl.far[far_bin(d, F.axis, F.c0, F.nC, F.nG)] += (double)wIn;
            // the lux plane: the escaping ray's line met at `height` along the axis (it crosses nothing more)
            T dn = r.dir.x * T(F.axis[0]) + r.dir.y * T(F.axis[1]) + r.dir.z * T(F.axis[2]);
            if (F.cells && dn > T(0)) {
                V3<T> rel = r.pos - V3<T>(T(F.origin[0]), T(F.origin[1]), T(F.origin[2]));
                T z = rel.x * T(F.axis[0]) + rel.y * T(F.axis[1]) + rel.z * T(F.axis[2]);
                T t = (T(F.height) - z) / dn;
                V3<T> h = rel + r.dir * t;
                T a = h.x * T(F.c0[0]) + h.y * T(F.c0[1]) + h.z * T(F.c0[2]);
                T b = h.x * T(F.c90[0]) + h.y * T(F.c90[1]) + h.z * T(F.c90[2]);
                T cell = T(2) * T(F.half) / T(F.cells);
                if (t >= T(0) && std::fabs(a) < T(F.half) && std::fabs(b) < T(F.half)) {
                    uint32_t ix = std::min((uint32_t)((a + T(F.half)) / cell), F.cells - 1);
                    uint32_t iy = std::min((uint32_t)((b + T(F.half)) / cell), F.cells - 1);
                    tl.lux[(size_t)iy * F.cells + ix] += (double)wIn;
                }
            }
            return;
        }
        if (r.state != RAY_ACTIVE) { tl.lost += (double)wIn; tl.n_lost++; return; }   // out of steps or length
        SceneHit<T> h = scene_eval(*C.s, r.pos);
        const uint32_t mi = std::min(h.m, C.s->n_materials - 1);
        const st_material& m = C.s->materials[mi];
        V3<T> nn = hit_normal(C, r.pos, dh);
        bool inside = dh < T(0);
        V3<T> nrm = inside ? -nn : nn;
        if (m.detector > 0.5f && dot(-r.dir, nrm) >= T(0)) {                      // kernels.js:660-672
            tl.detected += (double)wIn;
            tl.n_detected++;
            tl.interactions++;
            tl.tag[3 * h.item] += (double)wIn; tl.tag[3 * h.item + 2] += 1;
            tl.mat[3 * mi] += (double)wIn; tl.mat[3 * mi + 2] += 1;
            const float hit[12] = {(float)r.pos.x, (float)r.pos.y, (float)r.pos.z, (float)wIn, (float)r.dir.x,
                                   (float)r.dir.y, (float)r.dir.z, (float)h.item, 0.f, 0.f, 0.f, 0.f};
            tl.hits.insert(tl.hits.end(), hit, hit + 12);
            return;
        }
        uint32_t b0 = r.bounces;
        Rng rng; rng.h = bseed; rng.seed_u32(id); rng.seed_u32(r.bounces);
        shade_photon(C, r, dh, rng);
        if (r.bounces == b0) {                                                   // declined: not an interaction
            if (r.state == RAY_ACTIVE) continue;
            tl.lost += (double)wIn;
            tl.n_lost++;
            return;
        }
        tl.interactions++;
        bool goesOn = r.state == RAY_ACTIVE || r.state == RAY_TERMINATED;
        T wOut = goesOn ? luma(r.beta * r.rad) : T(0);
        tl.absorbed += (double)(wIn - wOut);
        if (!goesOn) tl.n_absorbed++;
        tl.tag[3 * h.item] += (double)wIn; tl.tag[3 * h.item + 1] += (double)wOut; tl.tag[3 * h.item + 2] += 1;
        tl.mat[3 * mi] += (double)wIn; tl.mat[3 * mi + 1] += (double)wOut; tl.mat[3 * mi + 2] += 1;
        if (r.state == RAY_TERMINATED) { tl.lost += (double)wOut; tl.n_lost++; return; }   // the bounce cap
        if (r.state != RAY_ACTIVE) return;
        (void)maxbounce;
    }
}
}  // namespace

// ------------------------------------------------------------------------------------------------------------
// ONE RESOLVE STEP of a pixel's luminance moments (measure.js:36-51 stepMoments): the new sample y joins prevn
// earlier ones (their count capped at the EMA window) at weight w = 1 / (prevn + 1); V is the weighted spread of the
// deviations from the previous mean, S the sum of the squared weights (S = 1/n for a true mean of n, 1/(2N+1) at an
// EMA window N). A first sample (prevn 0) leaves V = 0, S = 1.
inline void step_moments(double prevn, double y, double prev_y, double& V, double& S) {
    double w = 1.0 / (prevn + 1);
    double d = prevn > 0 ? y - prev_y : 0.0;
    double v0 = std::min(std::max(V, 0.0), 1e300), s0 = std::min(std::max(S, 0.0), 1.0);
    V = (1 - w) * (v0 + w * d * d);
    S = (1 - w) * (1 - w) * s0 + w * w;
}

// extern "C"
// ------------------------------------------------------------------------------------------------------------
static MfTables g_tb_f, g_tb_d;
static bool g_tb_f_ok = false, g_tb_d_ok = false;

template <class T> static const MfTables* tables();
template <> const MfTables* tables<float>() {
    if (!g_tb_f_ok) { g_tb_f = build_mf_tables<float>(); g_tb_f_ok = true; }
    return &g_tb_f;
}
template <> const MfTables* tables<double>() {
    if (!g_tb_d_ok) { g_tb_d = build_mf_tables<double>(); g_tb_d_ok = true; }
    return &g_tb_d;
}

// ONE SUN PHOTON (wavefront.js:596-626 prog_genphotons, then the wavefront's iterations with prog_sppm's store and a
// photon's shade): a direction in the sun's cone, a point uniform over the square of half width sp_half across the
// sun, flux L_disc cos Omega / (N pdf_area); at each hit stored where it has passed delta events only, at least one,
// on an evaluable surface within the cap, else bounced -- a delta lobe keeps it, anything else ends it
const uint32_t LT_LENS_SALT = 0x4C54434Eu;      // a connection's point of the lens, from the photon's own stream

// A PHOTON'S CONNECTION TO THE CAMERA (materials_pbr.js:672-830 ltConnect, :598-612 camFootprint, lens.js lensDisc,
// lensImage), traced and splatted: from P (in air, nrm turned to the photon, arriving along din with flux phi) to the
// camera, or a point of its lens drawn from the photon's stream, through the evaluable lobes; phi f G / A_px to the
// pixel the line lands on, if the shadow ray -- started on the line of sight as far along it as lifts it 2 offsets
// off the surface (at most 4 such lengths at grazing views, the rest along the normal, re-aimed), stopped that height
// short of the camera -- gets there
template <class T>
void lt_splat(const Ctx<T>& C, const V3<T>& P, const V3<T>& org, const V3<T>& dir, T len, T h, V3<T> c, uint32_t pix,
              uint32_t cell, Stats& st);
template <class T>
void lt_connect(const Ctx<T>& C, const st_material& m, const V3<T>& P, const V3<T>& nrm, const V3<T>& din,
                const V3<T>& phi, T lam, U4 ps, uint32_t id, uint32_t cell, Stats& st) {
    const st_view& vw = *C.view;
    const V3<T> right(T(vw.right[0]), T(vw.right[1]), T(vw.right[2])), up(T(vw.up[0]), T(vw.up[1]), T(vw.up[2]));
    const V3<T> fwd(T(vw.fwd[0]), T(vw.fwd[1]), T(vw.fwd[2])), cam0(T(vw.cam_pos[0]), T(vw.cam_pos[1]), T(vw.cam_pos[2]));
    const T fx = T(vw.fx), fy = T(vw.fy), F = T(vw.focus_distance);
    const uint32_t W = C.p.width, H = C.p.height;
    V3<T> off(T(0));
    const T R = vw.camtype == 0 ? T(vw.lens_radius) : T(0);
    if (R > T(0)) {
        Rng rl = path_rng(ps, id, LT_LENS_SALT);
        T ul[4]; rl.next4(ul);
        const T r = R * std::sqrt(ul[0]), ph = T(6.28318530718) * ul[1];
        off = right * (r * std::cos(ph)) + up * (r * std::sin(ph));
    }
    if (lobes_none(m, T(m.transmission), T(m.haze))) return;
    const V3<T> cam = cam0 + off, d = cam - P;
    const T apx = T(4) * fx * fy / (T(W) * T(H));
    V3<T> v;
    T dist, xx, yy, G;
    if (vw.camtype == 0) {
        dist = length(d);
        const T z = dot(d, fwd);
        if (z <= T(1e-4) || dist <= T(1e-4)) return;
        v = d / dist;
        if (R > T(0)) {
            const T c = dot(v, fwd);
            const V3<T> Fp = off + (-v) * (F / std::max(c, T(1e-30)));
            xx = dot(Fp, right) / (F * fx);
            yy = dot(Fp, up) / (F * fy);
        } else {
            xx = -dot(d, right) / (z * fx);
            yy = -dot(d, up) / (z * fy);
        }
        G = std::fabs(dot(nrm, v)) * dist / (z * z * z);
    } else {
        dist = dot(d, fwd);
        if (dist <= T(1e-4)) return;
        v = fwd;
        xx = -dot(d, right) / fx;
        yy = -dot(d, up) / fy;
        G = std::fabs(dot(nrm, fwd));
    }
    if (std::fabs(xx) >= T(1) || std::fabs(yy) >= T(1)) return;
    const T cv = dot(nrm, v);
    if (cv <= T(0)) return;
    // (a coating's pick keeps the even weights, the camera's first vertex's: its beta is white)
    Lobes<T> lb = make_lobes(nrm, v, m, T(1) / std::max(T(m.ior), T(1)), C.tb, T(m.transmission), T(m.specular), T(m.haze),
                             T(1), false, lam);
    const V3<T> f = lobes_eval(lb, -din, T(0.05));
    const V3<T> c = phi * f * (G / apx);
    if (!(luma(c) > T(0))) return;
    const T px = clampT((xx + T(1)) * T(0.5) * T(W), T(0), T(W) - T(1));
    const T py = clampT((yy + T(1)) * T(0.5) * T(H), T(0), T(H) - T(1));
    const uint32_t pix = (uint32_t)px + (uint32_t)py * W;
    const T h = T(20) * march_tol(P, C.tol);
    const bool grazing = cv < T(0.25);
    const T sl = h / std::max(cv, T(0.25));
    const T lift = grazing ? h - sl * cv : T(0);
    V3<T> org = P + v * sl + nrm * lift, dir = v;
    T len = dist - sl - cv * lift - h;
    if (grazing && vw.camtype == 0) {
        const V3<T> toCam = cam - org;
        const T l = length(toCam);
        dir = toCam / std::max(l, T(1e-30));
        len = l - h;
    }
    if (!(len > T(0))) return;
    lt_splat(C, P, org, dir, len, h, c, pix, cell, st);
}

// the connection's end: the emission map taught, the haze on the true segment (haze.js:463-481 hazeShadow), the
// shadow ray traced, what arrives splatted and counted
template <class T>
void lt_splat(const Ctx<T>& C, const V3<T>& P, const V3<T>& org, const V3<T>& dir, T len, T h, V3<T> c, uint32_t pix,
              uint32_t cell, Stats& st) {
    if (C.haze.on) {
        const V3<T> e = org + dir * (len + h) - P;
        const T el = length(e);
        c = c * C.haze.transmittance(P, e / std::max(el, T(1e-30)), el, T(C.d.env_radius));
    }
    if (C.sp_learn && cell < LT_N) {                                               // ltConnect's learn
#pragma omp atomic
        C.lt_hit[cell]++;
    }
    if (!occlude<T>(C, org, dir, T(1), st, nullptr, nullptr, true, -len)) return;
    if (bad_deposit(c)) { st.nonfinite++; return; }
#pragma omp atomic
    (*C.splat)[pix * 3 + 0] += (double)c.x;
#pragma omp atomic
    (*C.splat)[pix * 3 + 1] += (double)c.y;
#pragma omp atomic
    (*C.splat)[pix * 3 + 2] += (double)c.z;
#pragma omp atomic
    (*C.ltcount)[pix]++;
}
// A PHOTON SCATTERED IN THE HAZE, CONNECTED (haze.js:404-460 ltConnectMedium): the phase function for the lobes,
// dist / z^3 for the footprint (1 orthographic), from the point itself to 2 offsets short of the camera
template <class T>
void lt_connect_medium(const Ctx<T>& C, const V3<T>& P, const V3<T>& din, const V3<T>& phi, U4 ps, uint32_t id,
                       uint32_t cell, Stats& st) {
    const st_view& vw = *C.view;
    const V3<T> right(T(vw.right[0]), T(vw.right[1]), T(vw.right[2])), up(T(vw.up[0]), T(vw.up[1]), T(vw.up[2]));
    const V3<T> fwd(T(vw.fwd[0]), T(vw.fwd[1]), T(vw.fwd[2])), cam0(T(vw.cam_pos[0]), T(vw.cam_pos[1]), T(vw.cam_pos[2]));
    const T fx = T(vw.fx), fy = T(vw.fy), F = T(vw.focus_distance);
    const uint32_t W = C.p.width, H = C.p.height;
    V3<T> off(T(0));
    const T R = vw.camtype == 0 ? T(vw.lens_radius) : T(0);
    if (R > T(0)) {
        Rng rl = path_rng(ps, id, LT_LENS_SALT);
        T ul[4]; rl.next4(ul);
        const T r = R * std::sqrt(ul[0]), ph = T(6.28318530718) * ul[1];
        off = right * (r * std::cos(ph)) + up * (r * std::sin(ph));
    }
    const V3<T> cam = cam0 + off, d = cam - P;
    V3<T> v;
    T dist, xx, yy, gm;
    if (vw.camtype == 0) {
        dist = length(d);
        const T z = dot(d, fwd);
        if (z <= T(1e-4) || dist <= T(1e-4)) return;
        v = d / dist;
        if (R > T(0)) {
            const T c = dot(v, fwd);
            const V3<T> Fp = off + (-v) * (F / std::max(c, T(1e-30)));
            xx = dot(Fp, right) / (F * fx);
            yy = dot(Fp, up) / (F * fy);
        } else {
            xx = -dot(d, right) / (z * fx);
            yy = -dot(d, up) / (z * fy);
        }
        gm = dist / (z * z * z);
    } else {
        dist = dot(d, fwd);
        if (dist <= T(1e-4)) return;
        v = fwd;
        xx = -dot(d, right) / fx;
        yy = -dot(d, up) / fy;
        gm = T(1);
    }
    if (std::fabs(xx) >= T(1) || std::fabs(yy) >= T(1)) return;
    const T apx = T(4) * fx * fy / (T(W) * T(H));
    const V3<T> c = phi * (hg_eval(dot(din, v), clampT(C.haze.g, T(-0.95), T(0.95))) * gm / apx);
    if (!(luma(c) > T(0))) return;
    const T px = clampT((xx + T(1)) * T(0.5) * T(W), T(0), T(W) - T(1));
    const T py = clampT((yy + T(1)) * T(0.5) * T(H), T(0), T(H) - T(1));
    const uint32_t pix = (uint32_t)px + (uint32_t)py * W;
    const T h = T(20) * march_tol(P, C.tol);
    const T len = dist - h;
    if (!(len > T(0))) return;
    lt_splat(C, P, P, v, len, h, c, pix, cell, st);
}
// AN EMITTER PROBE (wavefront.js:552-588; tracebasics.js:782-831 THE PROBE): a listed box by its probability, a line
// uniformly random through its bounding sphere followed back from the far end, through everything but an emissive
// surface seen from outside, where it becomes a photon leaving along the line, its flux the emission over the probes
// and the line density there; false if it finds none (past its chord, out of the scene, out of steps or iterations)
template <class T>
bool probe_photon(const Ctx<T>& C, U4 ps, uint32_t id, Ray<T>& r, uint32_t& it, Stats& st) {
    const EmitList& L = *C.em;
    if (L.count == 0) return false;
    Rng r0 = path_rng(ps, id, PHOTON_GEN_SALT);
    T u[4], u2[4];
    r0.next4(u); r0.next4(u2);
    const uint32_t b = emit_pick(L, (float)u[0]);
    const V3<T> c(T(L.box[b][0]), T(L.box[b][1]), T(L.box[b][2]));
    const T rb = T(L.box[b][3]);
    const T z = T(1) - T(2) * u[1], rz = std::sqrt(std::max(T(0), T(1) - z * z)), ph = T(2) * T(PI_D) * u[2];
    const V3<T> w(rz * std::cos(ph), rz * std::sin(ph), z);
    const V3<T> ta = std::fabs(w.x) > T(0.9) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
    const V3<T> e1 = normalize(cross(ta, w)), e2 = cross(w, e1);
    const T rho = rb * std::sqrt(u[3]), pd = T(2) * T(PI_D) * u2[0];
    const V3<T> q = c + e1 * (rho * std::cos(pd)) + e2 * (rho * std::sin(pd));
    const T hl = std::sqrt(std::max(rb * rb - rho * rho, T(0)));
    r.pos = q + w * hl; r.dir = -w; r.beta = V3<T>(1); r.rad = V3<T>(0);
    r.ltot = 0; r.n = 1; r.sunmis = 1; r.tmax = 0; r.absLtot = 0;
    r.bounces = 0; r.steps = 0; r.state = RAY_ACTIVE; r.pix = id;
    const T len = T(2) * hl;
    while (it < C.budget) {
        uint32_t evals = 0;
        T dh = march(C, r, st, false, evals);
        uint32_t chunks = std::max(1u, (evals + MARCH_CHUNK - 1) / MARCH_CHUNK);
        it = std::min(it + chunks - 1, C.budget - 1);
        const bool last = it + 1 == C.budget;
        if (r.state != RAY_ACTIVE || r.ltot > len) return false;
        const V3<T> nn = hit_normal(C, r.pos, dh);
        const T otol = T(10) * march_tol(r.pos, C.tol);
        const bool outside = dh >= T(0) && dot(nn, -r.dir) > T(0);
        SceneHit<T> h = scene_eval(*C.s, r.pos);
        const st_material& m = C.s->materials[std::min(h.m, C.s->n_materials - 1)];
        const V3<T> le(T(m.emissive[0]), T(m.emissive[1]), T(m.emissive[2]));
        if (outside && max3(le) > T(0)) {
            T dens = 0;
            for (uint32_t k = 0; k < L.count; k++) {
                const V3<T> d = r.pos - V3<T>(T(L.box[k][0]), T(L.box[k][1]), T(L.box[k][2]));
                const T rk = T(L.box[k][3]);
                if (dot(d, d) < rk * rk) dens += T(L.pc[k][0]) / (T(4) * T(PI_D) * T(PI_D) * rk * rk);
            }
            if (!(dens > T(0))) return false;
            r.pos = r.pos + nn * (T(2) * otol);
            r.dir = -r.dir;
            const T beam = m.beam_cos > 0.f ? (dot(r.dir, nn) >= T(m.beam_cos) ? T(1) : T(0)) : T(1);
            r.rad = le * (beam / (T(C.lt_emit_n) * dens));
            r.ltot = 0; r.n = 1; r.absLtot = 0; r.tmax = 0; r.bounces = 0;
            if (last || !(luma(r.rad) > T(0))) return false;
            it++;
            return true;
        }
        move_by(r, r.dir * (T(2) * otol));                                        // through it, looking on
        if (last) return false;
        it++;
    }
    return false;
}

template <class T>
void photon_walk(const Ctx<T>& C, U4 ps, uint32_t id, Ray<T>& r, uint32_t it, uint32_t cell, std::vector<PhotonRec>& out,
                 Stats& st);
template <class T>
void trace_photon(const Ctx<T>& C, U4 ps, uint32_t id, uint32_t N, std::vector<PhotonRec>& out, Stats& st) {
    if (id < C.lt_emit_n) {
        Ray<T> r;
        uint32_t it = 0;
        if (probe_photon(C, ps, id, r, it, st)) photon_walk(C, ps, id, r, it, 0xffffffffu, out, st);
        return;
    }
    Rng r0 = path_rng(ps, id, PHOTON_GEN_SALT);
    T u[4]; r0.next4(u);
    V3<T> w = C.env.sample_sun_cone(u[0], u[1]);
    const V3<T> sdir = C.env.sun_dir;
    V3<T> b1, b2;
    sun_frame(C.env, b1, b2);
    const T R = T(C.sp_half);
    T x, y, area;
    uint32_t cell = 0xffffffffu;
    if (C.sp_learn) {                                                              // a cell by the map, a point in it
        T u2[4]; r0.next4(u2);
        const uint32_t row = lt_search(C.lt_cdf + LT_N, (float)u[2]);
        const uint32_t col = lt_search(C.lt_cdf + row * LT_G, (float)u[3]);
        const float pCell = lt_mass(C.lt_cdf + LT_N, row) * lt_mass(C.lt_cdf + row * LT_G, col);
        const T csz = T(2) * R / T(LT_G);
        x = -R + (T(col) + u2[0]) * csz;
        y = -R + (T(row) + u2[1]) * csz;
        area = csz * csz / T(std::max(pCell, 1e-30f));
        cell = row * LT_G + col;
#pragma omp atomic
        C.lt_emit[cell]++;
    } else {
        x = -R + T(2) * R * u[2];
        y = -R + T(2) * R * u[3];
        area = T(4) * R * R;
    }
    const T cosW = std::max(dot(w, sdir), T(1e-4));
    const V3<T> q = b1 * x + b2 * y;
    const T envR = T(C.d.env_radius);
    Ray<T> r;
    r.pos = q + w * ((envR - dot(q, sdir)) / cosW);
    r.dir = -w;
    r.beta = V3<T>(1);
    V3<T> disc = C.env.sun_on ? C.env.radiance(w) : V3<T>(0);
    r.rad = disc * (cosW * C.env.sun_omega * area / T(std::max(N - C.lt_emit_n, 1u)));
    r.ltot = 0; r.n = 1; r.sunmis = 1; r.tmax = 0; r.absLtot = 0;
    r.bounces = 0; r.steps = 0; r.state = RAY_ACTIVE; r.pix = id;
    photon_walk(C, ps, id, r, 0u, cell, out, st);
}

// a photon's walk from where it leaves its source: connected and stored past delta events, bounced through them
template <class T>
void photon_walk(const Ctx<T>& C, U4 ps, uint32_t id, Ray<T>& r, uint32_t it, uint32_t cell, std::vector<PhotonRec>& out,
                 Stats& st) {
    uint32_t seg = 0;
    while (it < C.budget) {
        // the haze: the leg's collision drawn as it starts, from the photon's own stream (haze.js:255-273 hazeDraw)
        const bool use_haze = C.haze.on;
        if (use_haze && r.tmax == T(0) && !walks(C, r)) {
            V3<T> A = r.pos - r.dir * (std::max(r.ltot - r.absLtot, T(0)) / std::max(r.n, T(1e-4)));
            Rng hr = path_rng(ps, id, SEED_SALT_HAZE + seg);
            r.tmax = C.haze.draw(A, r.dir, r.absLtot, r.n, T(C.d.env_radius), hr);
        }
        uint32_t evals = 0;
        const WalkIO wio{ps, id, (C.sppm && r.passed && r.bounces + 2 <= C.p.maxbounce) ? 1 : 0, &out};
        T dh = march(C, r, st, use_haze, evals, &wio);
        uint32_t chunks = std::max(1u, (evals + MARCH_CHUNK - 1) / MARCH_CHUNK);
        it = std::min(it + chunks - 1, C.budget - 1);
        bool last = it + 1 == C.budget;
        if (r.state == RAY_SCATTER) {
            // a collision in the air (haze.js:491-545, a photon's): the albedo, the connection once past a delta
            // event, its end
            r.bounces += 1;
            r.beta = r.beta * C.haze.albedo;
            if (C.lt && r.passed && r.bounces <= C.p.maxbounce)
                lt_connect_medium(C, r.pos, r.dir, r.rad * r.beta, ps, id, cell, st);
            break;
        }
        if (r.state != RAY_ACTIVE) break;
        V3<T> nn = hit_normal(C, r.pos, dh);
        bool inside = dh < T(0);
        V3<T> nrm = inside ? -nn : nn;
        T otol = T(10) * march_tol(r.pos, C.tol);
        if (dot(-r.dir, nrm) < T(0)) {                                             // leaving: moved on, no event
            move_by(r, r.dir * otol);
            if (last) break;
            it++;
            continue;
        }
        SceneHit<T> h = scene_eval(*C.s, r.pos);
        const st_material& m = C.s->materials[std::min(h.m, C.s->n_materials - 1)];
        if (std::max(std::max(m.emissive[0], m.emissive[1]), m.emissive[2]) > 0.f) break;
        // light tracing: connected first, once it has passed a delta event, in air, within the bounce cap
        if (C.lt && r.passed && std::fabs(r.n - T(1)) <= T(1e-3) && r.bounces + 1 <= C.p.maxbounce)
            lt_connect(C, m, r.pos, nrm, r.dir, r.rad * r.beta, r.lam, ps, id, cell, st);
        if (r.passed && sppm_evaluable(m, false)) {
            V3<T> pw = r.rad * r.beta;
            if (C.sppm && r.bounces + 2 <= C.p.maxbounce && luma(pw) > T(0)) {       // sppm.js sppmStores / sppmStore
                Rng rs = path_rng(ps, id, SPPM_STORE_SALT);
                float us[4]; rs.next4(us);
                uint32_t sub = std::min((uint32_t)(us[1] * (float)SPPM_SUBS), SPPM_SUBS - 1);
                PhotonRec rec;
                rec.pos[0] = (float)r.pos.x; rec.pos[1] = (float)r.pos.y; rec.pos[2] = (float)r.pos.z;
                rec.power[0] = (float)pw.x; rec.power[1] = (float)pw.y; rec.power[2] = (float)pw.z;
                float dv[3] = {(float)-r.dir.x, (float)-r.dir.y, (float)-r.dir.z};
                float nv[3] = {(float)nrm.x, (float)nrm.y, (float)nrm.z};
                rec.dir = sppm_oct(dv);
                rec.nrm = sppm_oct(nv);
                rec.flags = (r.bounces + 1) | (sub << SPPM_SUB_SHIFT);
                out.push_back(rec);
                if (!C.lt && cell < LT_N) {                                        // (light tracing's connections teach it)
#pragma omp atomic
                    C.lt_hit[cell]++;
                }
            }
            break;
        }
        r.bounces += 1;
        r.absLtot = r.ltot;                                                        // the ltot on arrival here
        r.tmax = T(0);                                                             // the next leg's collision: afresh
        Rng rng = path_rng(ps, id, 1 + seg);
        seg++;
        T n0 = r.n, n1d = std::max(T(m.ior), n0), v1 = T(0);
        uint32_t beyond = inside ? 0u : std::min(h.m, C.s->n_materials - 1);
        if (m.transmission > 0 && m.metallic < 1) {
            SceneHit<T> mb = scene_eval(*C.s, r.pos + (-nrm) * (otol * T(2)));
            beyond = std::min(mb.a, C.s->n_materials - 1);
            const st_material& mm = C.s->materials[beyond];
            n1d = T(mm.ior);
            v1 = T(mm.abbe);
        }
        const T lam0 = r.lam;
        const T n1 = lam0 > T(0) ? cauchy_n(n1d, v1, lam0) : n1d;
        const bool draw = v1 > T(0) && lam0 == T(0);
        T nT = n1, lamD = T(0);
        V3<T> specW(T(1), T(1), T(1));
        if (draw) {
            T ul[4]; rng.next4(ul);
            lamD = lambda_coded(spec_draw(ul[0], specW));
            nT = cauchy_n(n1d, v1, lamD);
        }
        T pG = refract_share<T>(m);
        T trans = T(m.transmission), specv = T(m.specular), hz = T(m.haze);
        bool diffFace = pG <= T(0) && m.transmission > 0.f;
        if (inside && pG > T(0) && pG < T(1)) {
            T k = mixT(T(2) * T(m.specular), T(1), pG);
            T u4[4]; rng.next4(u4);
            if (u4[0] < pG) { trans = T(1); hz = T(0); }
            else {
                trans = sat(sat(T(m.transmission)) * sat(T(m.haze)) / std::max(T(1) - pG, T(1e-6)));
                hz = T(1); specv = T(0.5) * k; diffFace = true;
            }
        }
        T etaFace = diffFace ? std::min(n0, n1) / std::max(n0, n1) : n0 / n1;
        Lobes<T> lb = make_lobes(nrm, -r.dir, m, etaFace, C.tb, trans, specv, hz, n0, inside, lam0);
        lb.etaT = n0 / nT;
        coat_pick(lb, r.beta);
        T ur[4]; rng.next4(ur);
        LobeSample<T> smp = lobes_sample(lb, ur);
        r.dir = smp.dir;
        r.beta *= smp.w;
        if (smp.transmitted) {
            r.n = nT;
            if (draw) { r.beta *= specW; r.lam = lamD; }
            r.medium = beyond;
        }
        move_by(r, r.dir * otol);
        bool alive = max3(smp.w) > T(0) && smp.ev == EV_DELTA && r.bounces <= C.p.maxbounce;
        if (alive && C.p.rr != 0 && r.bounces >= 3) {
            T p = clampT(max3(r.beta), T(0.1), T(0.95));
            T uu[4]; rng.next4(uu);
            if (uu[0] > p) alive = false;
            else r.beta = r.beta / p;
        }
        r.passed = true;
        if (!alive || last) break;
        it++;
    }
}

template <class T>
static int render_impl(const st_scene_desc* s, const st_params* p, const st_view* v, uint32_t sample0,
                       uint32_t nsamples, double* acc_rgb, double* mV, double* mS, uint32_t* acc_cnt,
                       uint64_t* counters, int threads, uint32_t path_first, uint32_t path_count, bool cull = false) {
    // the lights' faces, drawn as sheets appended to the primitives (the scene the rest of the oracle sees)
    std::vector<st_prim> prims_x(s->prims, s->prims + s->n_prims);
    std::vector<OFace> faces;
    st_scene_desc sx = *s;
    Ctx<T> C;
    {
        std::string why;
        if (!build_faces(*s, prims_x, faces, C.face_of, why)) return -1;
        sx.prims = prims_x.data();
        sx.n_prims = (uint32_t)prims_x.size();
        if (!faces.empty()) C.faces = &faces;
        s = &sx;
    }
    std::vector<CullBox> boxes;
    if (cull) { boxes = cull_boxes(*s); C.cull = &boxes; }
    C.s = s; C.p = *p; C.d = derive(*p, *s);
    C.env.init(*p, C.d);
    std::vector<float> preset_tex, preset_cache;    // a preset's map (the image's is its own) and texture
    if (C.env.mode != 0 && !C.env.img) {
        if (p->env_cache) {
            const uint32_t tw = (p->env_cache_size == 1024u || p->env_cache_size == 4096u) ? p->env_cache_size : 2048u;
            preset_cache = preset_texture(C.env, tw, tw / 2);
            C.env.cache = &preset_cache;
            C.env.cache_w = tw; C.env.cache_h = tw / 2;
        }
        preset_tex = preset_map(C.env);
        C.env.init(*p, C.d, &preset_tex);
        if (p->env_cache) {                          // init starts over: the texture back in
            const uint32_t tw = (p->env_cache_size == 1024u || p->env_cache_size == 4096u) ? p->env_cache_size : 2048u;
            C.env.cache = &preset_cache;
            C.env.cache_w = tw; C.env.cache_h = tw / 2;
        }
    }
    C.tb = tables<T>();
    C.tol = T(C.d.tol_setting);
    C.envR2 = T(C.d.env_radius * C.d.env_radius);
    C.stepscale = T(p->stepscale);
    // THE ITERATION BUDGET IS THE WORST CASE (raytrace_main.js:1795-1815): a segment per bounce, and room for a
    // path's steps-off-a-surface (a march chunk's worth each in the reference, ceil(maxiter / 32) of them)
    C.budget = p->budget ? p->budget : std::max(2u, p->maxbounce + 1 + (p->maxiter + 31) / 32);
    C.haze.init(*s);
    for (uint32_t k = 0; k < s->n_materials; k++)
        if (s->materials[k].scatter_distance > 0.f) C.scatter_on = true;
    const uint32_t W = p->width, H = p->height, P = W * H;
    uint32_t pend = std::min(P, path_first + (path_count ? path_count : P));
    Stats st;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    Frame<T> fr;
    fr.rgb.assign((size_t)P * 3, 0.0);
    fr.cnt.assign(P, 0);
    // the photon map runs while it is set and the sun shines (its photons are the sun's)
    const bool sppm_on = p->sppm != 0 && C.env.sun_on && p->env_uniform <= 0.f;
    // light tracing runs while it is set and there are photons (the sun's while it shines, the emitters' in a scene
    // with emissive materials), the same photons as the map's while it runs
    bool any_emit = false;
    for (uint32_t i = 0; i < s->n_materials; i++)
        if (std::max(s->materials[i].emissive[0], std::max(s->materials[i].emissive[1], s->materials[i].emissive[2])) > 0.f)
            any_emit = true;
    const bool sun_photons = C.env.sun_on && p->env_uniform <= 0.f;
    const bool lt_on = p->lt != 0 && (sun_photons || any_emit);
    const uint32_t NPH = sppm_on ? (p->sppm_photons ? p->sppm_photons : P) : (p->lt_photons ? p->lt_photons : P);
    SppmGrid grid;
    if (sppm_on) {
        C.sppm = true;
        C.grid = &grid;
        C.sp_budget = 512;
    }
    if (sppm_on || lt_on) C.sp_half = p->sppm_half > 0.f ? p->sppm_half : std::min(15.f, (float)C.d.env_radius);
    std::vector<double> splat;
    std::vector<uint32_t>& ltcount = g_lt_count;
    ltcount.assign(P, 0);
    if (lt_on) {
        C.lt = true;
        C.view = v;
        splat.assign((size_t)P * 3, 0.0);
        C.splat = &splat;
        C.ltcount = &ltcount;
    }
    std::vector<uint32_t> lt_emit(LT_N, 0), lt_hit(LT_N, 0);
    std::vector<float> lt_cdf(LT_N + LT_G);
    lt_uniform(lt_cdf.data());
    C.sp_learn = (sppm_on || lt_on) && p->sppm_learn != 0;
    C.lt_emit = lt_emit.data(); C.lt_hit = lt_hit.data(); C.lt_cdf = lt_cdf.data();
    // the emitter list, in a scene with an emissive material: a grid a thread, the merged grid, the list
    EmitList elist;
    std::vector<uint32_t> egrid(EMIT_CELLS * 8);
    std::vector<std::vector<uint32_t>> egrids(1);
#ifdef _OPENMP
    egrids.resize(omp_get_max_threads());
#endif
    for (uint32_t i = 0; i < s->n_materials; i++)
        if (std::max(s->materials[i].emissive[0], std::max(s->materials[i].emissive[1], s->materials[i].emissive[2])) > 0.f)
            C.em_on = true;
    if (C.em_on) {
        C.em_nee = p->emit_off == 0;
        C.em_share = p->emit_share > 0.f ? p->emit_share : 0.5f;
        const float set = p->emit_radius > 0.f ? p->emit_radius : 15.f;     // photometry.js:147-148 photonHalf
        C.em_half = std::max(std::min(std::max(set, 1e-3f), (float)C.d.env_radius), 1e-6f);
        emit_grid_init(egrid.data());
        for (auto& g : egrids) { g.resize(EMIT_CELLS * 8); emit_grid_init(g.data()); }
        C.em = &elist;
        C.em_grids = &egrids;
    }
    // light tracing's emitter probes (raytrace_main.js:1634-1635): their share of the photons, all of them with no sun
    if (lt_on && C.em_on) {
        const float set = p->lt_emit_share > 0.f ? p->lt_emit_share : 0.5f;
        const double share = sun_photons ? std::min(0.95, std::max(0.05, (double)set)) : 1.0;
        C.lt_emit_n = (uint32_t)std::llround(share * (double)NPH);
    }
    for (uint32_t si = 0; si < nsamples; si++) {
        U4 sseed = sample_seed(p->seed, sample0 + si);
        // the list rebuilt between samples, every EMIT_EPOCH (a wave a sample)
        if (C.em_on && sample0 + si >= elist.last + EMIT_EPOCH) {
            emit_build(egrid.data(), elist, C.em_half, (float)C.d.tol_setting);
            elist.last = sample0 + si;
        }
        std::fill(fr.rgb.begin(), fr.rgb.end(), 0.0);
        std::fill(fr.cnt.begin(), fr.cnt.end(), 0u);
        if (lt_on) std::fill(splat.begin(), splat.end(), 0.0);
        if (sppm_on || lt_on) {
            // THE SAMPLE'S PHOTONS FIRST: the radius r_k (k = the sample's number from 1), the photons traced and
            // stored, the grid of cell 2 r_k built
            // (light tracing alone: the photons and their connections, no records)
            const double r1 = p->sppm_r1 > 0.f ? p->sppm_r1 : 0.005, al = p->sppm_alpha > 0.f ? p->sppm_alpha : 2.0 / 3.0;
            const double rk = sppm_radius(r1, (int)(sample0 + si + 1), al);
            C.sp_r2 = (float)rk * (float)rk;
            C.sp_cell = (float)(2.0 * rk);
            C.sp_inv_area = 1.0 / (PI_D * rk * rk);
            const double r1v = p->sppm_r1_volume > 0.f ? p->sppm_r1_volume : 4.0 * (double)(float)r1;
            const double rv = sppm_radius_volume((double)(float)r1v, (int)(sample0 + si + 1), al);
            C.sp_vr2 = (float)rv * (float)rv;
            C.sp_vcell = (float)(2.0 * rv);
            C.sp_inv_vol = 3.0 / (4.0 * PI_D * rv * rv * rv);
            const U4 ps = sample_seed(p->seed ^ PHOTON_SEED_SALT, sample0 + si);
            const uint32_t kk = sample0 + si;
            if (C.sp_learn && kk > 0 && (kk & 3u) == 0) lt_build(lt_emit.data(), lt_hit.data(), lt_cdf.data());
            std::vector<std::vector<PhotonRec>> recs(1);
#ifdef _OPENMP
            recs.resize(omp_get_max_threads());
#endif
#pragma omp parallel for schedule(dynamic, 256)
            for (long i = 0; i < (long)NPH; i++) {
                int tid = 0;
#ifdef _OPENMP
                tid = omp_get_thread_num();
#endif
                trace_photon(C, ps, (uint32_t)i, NPH, recs[tid], st);
            }
            std::vector<float> pos, pw;
            std::vector<uint32_t> dirs, nrms, flags;
            for (auto& v : recs)
                for (auto& rr : v) {
                    for (int k = 0; k < 3; k++) { pos.push_back(rr.pos[k]); pw.push_back(rr.power[k]); }
                    dirs.push_back(rr.dir); nrms.push_back(rr.nrm); flags.push_back(rr.flags);
                }
            if (sppm_on) {
                sppm_build(grid, pos.data(), pw.data(), nrms.data(), flags.data(), (uint32_t)flags.size(), C.sp_cell,
                           C.sp_vcell);
                grid.dir = dirs;
            }
        }
#pragma omp parallel for schedule(dynamic, 64)
        for (long t = (long)path_first; t < (long)pend; t++) trace_path(C, sseed, (uint32_t)t, *v, W, H, fr, st);
        if (C.em_on)                                               // the threads' discoveries into the grid
            for (auto& g : egrids) {
                for (uint32_t i = 0; i < EMIT_CELLS * 8; i++) {
                    const uint32_t k = i & 7u;
                    if (k < 3) egrid[i] = std::min(egrid[i], g[i]);
                    else if (k < 7) egrid[i] = std::max(egrid[i], g[i]);
                    else egrid[i] += g[i];
                }
                emit_grid_init(g.data());
            }
        // resolve (wavefront.js:414-494, measure.js:36-51) in double precision
        for (uint32_t i = 0; i < P; i++) {
            uint32_t n = fr.cnt[i];
            if (n == 0) continue;
            double s3[3] = {fr.rgb[i * 3] / n, fr.rgb[i * 3 + 1] / n, fr.rgb[i * 3 + 2] / n};
            if (lt_on)                                 // light tracing's estimate, added as it is (wavefront.js:459-462)
                for (int c = 0; c < 3; c++) s3[c] += splat[i * 3 + c];
            double prevn = p->maxaverages ? std::min<double>(acc_cnt[i], p->maxaverages) : double(acc_cnt[i]);
            double cnt = prevn + 1;
            acc_cnt[i] = (uint32_t)cnt;
            double prev[3];
            for (int c = 0; c < 3; c++) prev[c] = std::min(std::max(acc_rgb[i * 3 + c], -1e20), 1e20);
            for (int c = 0; c < 3; c++) acc_rgb[i * 3 + c] = (prev[c] * prevn + s3[c]) / cnt;
            double y = s3[0] * LUMA_R + s3[1] * LUMA_G + s3[2] * LUMA_B;
            step_moments(prevn, y, prev[0] * LUMA_R + prev[1] * LUMA_G + prev[2] * LUMA_B, mV[i], mS[i]);
        }
    }
    if (counters) {
        counters[0] += st.paths; counters[1] += st.segments; counters[2] += st.march_steps;
        counters[3] += st.shadow_rays; counters[4] += st.shadow_steps; counters[5] += st.nonfinite;
        counters[6] += st.flushed; counters[7] += st.shadowcut;
    }
    if (C.sp_learn) { g_lt_emit = lt_emit; g_lt_hit = lt_hit; g_lt_cdf = lt_cdf; }
    return 0;
}

extern "C" {

// Render nsamples samples from sample0 on, folding each into the FP64 accumulation (caller-owned, continued across
// calls). fp64: 0 the reference-equivalent f32 arithmetic, 1 the accuracy oracle, 2 the f32 arithmetic with the
// reference's bounding-box culling at the root (the work its generated code does a step). path_first/path_count restrict the
// traced paths (a crop, for the CPU baseline's bounded sample); 0/0 = all.
// the environment image for every render that follows (envimage.js; envmap.js the map, baked here in double at the
// library's 2 x 2 points a texel and tabulated as the library tabulates it); rgb NULL: back to the sun and sky
int sto_set_env_image(const float* rgb, uint32_t w, uint32_t h, float luminance, float turn_deg) {
    EnvImage& im = env_image_state();
    if (!rgb) { im = EnvImage(); return 0; }
    if (w < 2 || h < 1) return -1;
    im.rgb.assign(rgb, rgb + (size_t)w * h * 3);
    for (float& c : im.rgb) if (!std::isfinite(c)) c = 0.f;
    im.w = w; im.h = h;
    im.lum = luminance > 0.f ? luminance : 179.0;
    im.turn = turn_deg;
    std::vector<double> lum((size_t)ENV_MW * ENV_MH);
    for (int i = 0; i < ENV_MW * ENV_MH; i++) {
        const int x = i % ENV_MW, y = i / ENV_MW;
        double acc[3] = {0, 0, 0};
        for (int sy = 0; sy < 2; sy++)
            for (int sx = 0; sx < 2; sx++) {
                const double ux = (x + (sx + 0.5) * 0.5) / ENV_MW, uy = (y + (sy + 0.5) * 0.5) / ENV_MH;
                const double z = 1 - 2 * uy, sz = std::sqrt(std::max(0.0, 1 - z * z)), ph = 2 * PI_D * ux;
                double c[3];
                env_image_at(im, sz * std::cos(ph), sz * std::sin(ph), z, c);
                for (int k = 0; k < 3; k++) acc[k] += c[k];
            }
        lum[i] = 0.25 * (0.2126 * acc[0] + 0.7152 * acc[1] + 0.0722 * acc[2]);
    }
    env_tables(lum, im.tex);
    return 0;
}
// the map's tables from given texel luminances (the library's st_env_map_tables, restated)
int sto_env_map_tables(const float* lum, float* tex) {
    std::vector<double> l(lum, lum + ENV_MW * ENV_MH);
    std::vector<float> t;
    env_tables(l, t);
    std::copy(t.begin(), t.end(), tex);
    return 0;
}
// the environment's radiance as the oracle has it, in n given directions (rgb out)
int sto_env_radiance(const st_params* p, const st_scene_desc* s, const double* dirs, uint32_t n, double* out) {
    Env<double> e;
    e.init(*p, derive(*p, *s));
    for (uint32_t i = 0; i < n; i++) {
        V3<double> c = e.radiance(V3<double>(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
        out[3 * i] = c.x; out[3 * i + 1] = c.y; out[3 * i + 2] = c.z;
    }
    return 0;
}
int sto_render(const st_scene_desc* s, const st_params* p, const st_view* v, uint32_t sample0, uint32_t nsamples,
               int fp64, double* acc_rgb, double* mV, double* mS, uint32_t* acc_cnt, uint64_t* counters, int threads,
               uint32_t path_first, uint32_t path_count) {
    if (!s || !p || !v || !acc_rgb || !mV || !mS || !acc_cnt) return -1;
    if (s->n_materials == 0 || s->n_prims == 0) return -1;
    if (fp64 == 1)
        return render_impl<double>(s, p, v, sample0, nsamples, acc_rgb, mV, mS, acc_cnt, counters, threads, path_first, path_count);
    return render_impl<float>(s, p, v, sample0, nsamples, acc_rgb, mV, mS, acc_cnt, counters, threads, path_first, path_count,
                              fp64 == 2);
}

int sto_mf_tables(int fp64, float* ec, float* ecavg, float* e1) {
    const MfTables* t = fp64 ? tables<double>() : tables<float>();
    std::memcpy(ec, t->ec.data(), t->ec.size() * 4);
    std::memcpy(ecavg, t->ecavg.data(), t->ecavg.size() * 4);
    std::memcpy(e1, t->e1.data(), t->e1.size() * 4);
    return 0;
}

int sto_scene_sdf(const st_scene_desc* s, const float* pts, uint32_t n, float* d, uint32_t* mat, uint32_t* med) {
    for (uint32_t i = 0; i < n; i++) {
        SceneHit<double> h = scene_eval(*s, V3<double>(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
        d[i] = (float)h.d;
        if (mat) mat[i] = h.m;
        if (med) med[i] = h.a;
    }
    return 0;
}

void sto_pcg4d(const uint32_t* in, uint32_t* out) {
    U4 v = {in[0], in[1], in[2], in[3]};
    v = pcg4d(v);
    out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
}

// n draws of PRNG() after SEED_uvec4(seed4) and SEED_u32 of each of the k words (tracebasics.js:335-380)
void sto_prng(const uint32_t* seed4, const uint32_t* words, int k, int n, float* out) {
    Rng r; r.h = {seed4[0], seed4[1], seed4[2], seed4[3]};
    for (int i = 0; i < k; i++) r.seed_u32(words[i]);
    for (int i = 0; i < n; i++) r.next4(out + 4 * i);
}

void sto_sample_seed(uint32_t base, uint32_t sample, uint32_t* out) {
    U4 s = sample_seed(base, sample);
    out[0] = s.x; out[1] = s.y; out[2] = s.z; out[3] = s.w;
}

void sto_derive(const st_params* p, const st_scene_desc* s, double* out) {
    Derived d = derive(*p, *s);
    out[0] = d.sun_half; out[1] = d.sun_omc; out[2] = d.sun_sin2; out[3] = d.sun_omega; out[4] = d.disc_lum;
    out[5] = d.sun_on; out[6] = d.nee_sun_pick; out[7] = d.tol_setting; out[8] = d.env_radius;
    out[9] = d.sun_tint[0]; out[10] = d.sun_tint[1]; out[11] = d.sun_tint[2];
}

double sto_fresnel_dielectric(double cosI, double eta) { return fresnel_dielectric<double>(cosI, eta); }

// lobesEval / lobesPdf of a material at normal (0,0,1) for view v and light l (double precision), for the tests
void sto_lobes(const st_material* m, const double* v, const double* l, double eta, double* f, double* pdf) {
    const MfTables* tb = tables<double>();
    Lobes<double> lb = make_lobes(V3<double>(0, 0, 1), V3<double>(v[0], v[1], v[2]), *m, eta, tb);
    V3<double> fv = lobes_eval(lb, V3<double>(l[0], l[1], l[2]), 0.0);
    f[0] = fv.x; f[1] = fv.y; f[2] = fv.z;
    *pdf = lobes_pdf(lb, V3<double>(l[0], l[1], l[2]));
}

// a coating's reflectance per channel (spectral.js edgeRGB) and at one wavelength (edgeAt1), for the tests
void sto_coat_rgb(double lo, double hi, double edge, double width, double* out) { coat_edge_rgb(lo, hi, edge, width, out); }
double sto_coat_at_lambda(double lo, double hi, double edge, double width, double lam) {
    return coat_edge_at_lambda(lo, hi, edge, width, lam);
}
// n draws of lobesSample for a coated material at normal (0,0,1), view v, seen from medium n0 (inside or not), a ray of
// wavelength lam (0 none) carrying beta (coatPick): directions (3n) and weights (3n)
void sto_lobes_sample_coat(const st_material* m, const double* v, double eta, double n0, int inside, double lam,
                           const double* beta, uint32_t seed, int n, double* dirs, double* w) {
    const MfTables* tb = tables<double>();
    Lobes<double> lb = make_lobes(V3<double>(0, 0, 1), V3<double>(v[0], v[1], v[2]), *m, eta, tb, -1.0, -1.0, -1.0, n0,
                                  inside != 0, lam);
    coat_pick(lb, V3<double>(beta[0], beta[1], beta[2]));
    Rng r; r.h = sample_seed(seed, 0);
    for (int i = 0; i < n; i++) {
        double u[4]; r.next4(u);
        LobeSample<double> s = lobes_sample(lb, u);
        dirs[3 * i] = s.dir.x; dirs[3 * i + 1] = s.dir.y; dirs[3 * i + 2] = s.dir.z;
        w[3 * i] = s.w.x; w[3 * i + 1] = s.w.y; w[3 * i + 2] = s.w.z;
    }
}

// n draws of lobesSample for a material at normal (0,0,1), view v: directions (3n) and weights (3n)
void sto_lobes_sample(const st_material* m, const double* v, double eta, uint32_t seed, int n, double* dirs, double* w) {
    const MfTables* tb = tables<double>();
    Lobes<double> lb = make_lobes(V3<double>(0, 0, 1), V3<double>(v[0], v[1], v[2]), *m, eta, tb);
    Rng r; r.h = sample_seed(seed, 0);
    for (int i = 0; i < n; i++) {
        double u[4]; r.next4(u);
        LobeSample<double> s = lobes_sample(lb, u);
        dirs[3 * i] = s.dir.x; dirs[3 * i + 1] = s.dir.y; dirs[3 * i + 2] = s.dir.z;
        w[3 * i] = s.w.x; w[3 * i + 1] = s.w.y; w[3 * i + 2] = s.w.z;
    }
}

// the last optics run's tallies by object and material, counts and detector hits, per instance (for the tests)
struct OptDetail { std::vector<double> tag, mat; uint64_t counts[4] = {0, 0, 0, 0}; std::vector<float> hits; };
static std::map<uint32_t, OptDetail>& opt_detail() {
    static std::map<uint32_t, OptDetail> d;
    return d;
}
int sto_optics_detail(uint32_t inst, double* tag, double* mat, uint64_t* counts, float* hits, uint32_t max_hits,
                      uint32_t* n_hits) {
    auto it = opt_detail().find(inst);
    if (it == opt_detail().end()) return -1;
    const OptDetail& d = it->second;
    if (tag) std::copy(d.tag.begin(), d.tag.end(), tag);
    if (mat) std::copy(d.mat.begin(), d.mat.end(), mat);
    if (counts) for (int k = 0; k < 4; k++) counts[k] = d.counts[k];
    const uint32_t n = (uint32_t)(d.hits.size() / 12);
    if (n_hits) *n_hits = n;
    if (hits) std::copy(d.hits.begin(), d.hits.begin() + (size_t)std::min(n, max_hits) * 12, hits);
    return 0;
}

// Trace an optics batch (config: the scene, its settings for the march; sources with their instance; per instance its
// ray count, far-field frame, lux plane). Tallies per instance into far (n_inst * nG * nC), lux (n_inst * cells^2),
// totals (n_inst * 6: emitted, escaped, lost, detected, absorbed, interactions).
// the ray table the ray sets of the runs that follow read (8 floats a ray); n 0 clears it
int sto_optics_set_rays(const float* rays, uint32_t n) {
    optics_rays().assign(rays, rays + (size_t)n * 8);
    return 0;
}
int sto_optics_run(const st_scene_desc* const* scenes, const st_params* p, const st_optics_source* src, uint32_t nsrc,
                   const uint32_t* ray_count, uint32_t n_inst, const float* frames, uint32_t nC, uint32_t nG,
                   uint32_t cells, float half, float height, uint32_t maxbounce, uint32_t seed, int fp64,
                   double* far, double* lux, double* totals, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    opt_detail().clear();
    for (uint32_t inst = 0; inst < n_inst; inst++) {
        std::vector<st_optics_source> mine;
        for (uint32_t i = 0; i < nsrc; i++) if (src[i].instance == inst) mine.push_back(src[i]);
        if (mine.empty() || !ray_count[inst]) continue;
        double tot = 0;
        for (auto& s : mine) tot += s.flux;
        std::vector<float> cdf(mine.size());
        double acc = 0;
        for (size_t i = 0; i < mine.size(); i++) { acc += mine[i].flux; cdf[i] = (float)(acc / tot); }
        cdf.back() = 1.f;
        OptFrame F;
        const float* fr = frames + inst * 12;
        for (int k = 0; k < 3; k++) { F.origin[k] = fr[k]; F.axis[k] = fr[3 + k]; F.c0[k] = fr[6 + k]; }
        F.c90[0] = F.axis[1] * F.c0[2] - F.axis[2] * F.c0[1];
        F.c90[1] = F.axis[2] * F.c0[0] - F.axis[0] * F.c0[2];
        F.c90[2] = F.axis[0] * F.c0[1] - F.axis[1] * F.c0[0];
        F.nC = nC; F.nG = nG; F.cells = cells; F.half = half; F.height = height;
        U4 bseed = sample_seed(seed, inst);
        auto run = [&](auto zero) {
            using T = decltype(zero);
            Ctx<T> C;
            st_params pp = *p;
            pp.maxbounce = maxbounce;
            C.s = scenes[inst]; C.p = pp; C.d = derive(pp, *scenes[inst]);
            C.env.init(pp, C.d);
            C.tb = tables<T>();
            C.tol = T(C.d.tol_setting);
            C.envR2 = T(C.d.env_radius * C.d.env_radius);
            C.stepscale = T(pp.stepscale);
            C.budget = 0;
            C.haze.init(*scenes[inst]);
            int nt = 1;
#ifdef _OPENMP
            nt = omp_get_max_threads();
#endif
            std::vector<OptTally> tls(nt);
            for (auto& t : tls) {
                t.far.assign((size_t)nC * nG, 0.0); t.lux.assign((size_t)cells * cells, 0.0);
                t.tag.assign((size_t)scenes[inst]->n_prims * 3, 0.0);
                t.mat.assign((size_t)scenes[inst]->n_materials * 3, 0.0);
            }
#pragma omp parallel for schedule(dynamic, 256)
            for (long id = 0; id < (long)ray_count[inst]; id++) {
                int tid = 0;
#ifdef _OPENMP
                tid = omp_get_thread_num();
#endif
                optics_ray(C, bseed, (uint32_t)id, mine.data(), cdf.data(), (uint32_t)mine.size(), F, maxbounce, tls[tid]);
            }
            double* fo = far + (size_t)inst * nC * nG;
            double* lo = lux + (size_t)inst * cells * cells;
            double* to = totals + (size_t)inst * 6;
            OptDetail& dt = opt_detail()[inst];
            dt = OptDetail{};
            dt.tag.assign((size_t)scenes[inst]->n_prims * 3, 0.0);
            dt.mat.assign((size_t)scenes[inst]->n_materials * 3, 0.0);
            for (auto& t : tls) {
                for (size_t i = 0; i < t.far.size(); i++) fo[i] += t.far[i];
                for (size_t i = 0; i < t.lux.size(); i++) lo[i] += t.lux[i];
                to[0] += t.emitted; to[1] += t.escaped; to[2] += t.lost; to[3] += t.detected; to[4] += t.absorbed;
                to[5] += (double)t.interactions;
                for (size_t i = 0; i < t.tag.size(); i++) dt.tag[i] += t.tag[i];
                for (size_t i = 0; i < t.mat.size(); i++) dt.mat[i] += t.mat[i];
                dt.counts[0] += t.n_escaped; dt.counts[1] += t.n_lost; dt.counts[2] += t.n_detected;
                dt.counts[3] += t.n_absorbed;
                dt.hits.insert(dt.hits.end(), t.hits.begin(), t.hits.end());
            }
        };
        if (fp64) run(0.0); else run(0.0f);
    }
    return 0;
}

// ---- the photon map (st_oracle_sppm.h) ----
static SppmGrid g_grid;
// state = {Y, V, S, cnt}; window: the EMA cap on the earlier samples' count (infinity: a true mean; 0: a reset)
void sto_step_moments(double* state, double x, double window) {
    double prevn = std::min(state[3], window);
    double prevY = state[0];
    state[0] = (prevY * prevn + x) / (prevn + 1);
    step_moments(prevn, x, prevY, state[1], state[2]);
    state[3] = prevn + 1;
}
// the photon pass of one sample alone (tests): the records' count, and their power summed over a box (lo, hi)
int sto_sppm_photons(const st_scene_desc* s, const st_params* p, uint32_t sample, const float* lo, const float* hi,
                     double* out) {
    Ctx<float> C;
    C.s = s; C.p = *p; C.d = derive(*p, *s);
    C.env.init(*p, C.d);
    C.tb = tables<float>();
    C.tol = float(C.d.tol_setting);
    C.envR2 = float(C.d.env_radius * C.d.env_radius);
    C.stepscale = p->stepscale;
    C.budget = p->budget ? p->budget : std::max(2u, p->maxbounce + 1 + (p->maxiter + 31) / 32);
    C.haze.init(*s);
    C.sppm = true;
    C.sp_half = p->sppm_half > 0.f ? p->sppm_half : std::min(15.f, (float)C.d.env_radius);
    const uint32_t N = p->sppm_photons ? p->sppm_photons : p->width * p->height;
    const U4 ps = sample_seed(p->seed ^ PHOTON_SEED_SALT, sample);
    Stats st;
    std::vector<PhotonRec> recs;
    for (uint32_t i = 0; i < N; i++) trace_photon(C, ps, i, N, recs, st);
    double sum[3] = {0, 0, 0};
    for (auto& r : recs) {
        bool in = true;
        for (int k = 0; k < 3; k++) in = in && r.pos[k] >= lo[k] && r.pos[k] <= hi[k];
        if (in) for (int k = 0; k < 3; k++) sum[k] += r.power[k];
    }
    out[0] = (double)recs.size(); out[1] = sum[0]; out[2] = sum[1]; out[3] = sum[2];
    return 0;
}
double sto_cauchy_n(double nd, double vd, double lam) { return cauchy_n<double>(nd, vd, lam); }
uint32_t sto_lambda_code(double l) { return lambda_code(l); }
double sto_lambda_of(uint32_t c) { return lambda_of(c); }
void sto_spec_table(float* cdf, float* col) {
    const SpecTable& t = spec_table();
    for (int i = 0; i < SPEC_N; i++) { cdf[i] = t.cdf[i]; for (int c = 0; c < 3; c++) col[3 * i + c] = t.col[i][c]; }
}
double sto_spec_draw(double u, double* w) {
    V3<double> v;
    double l = spec_draw<double>(u, v);
    w[0] = v.x; w[1] = v.y; w[2] = v.z;
    return l;
}
uint32_t sto_sppm_hash(int32_t i, int32_t j, int32_t k) { return sppm_hash(i, j, k); }
double sto_sppm_radius(double r1, int k, double alpha) { return sppm_radius(r1, k, alpha); }
// prog_lt_build on the given counts (halved in place) into cdf (LT_N + LT_G floats)
void sto_lt_build(uint32_t* emit, uint32_t* hit, float* cdf) { lt_build(emit, hit, cdf); }
// the last render's emission map (sent, stored: LT_N each; cdf LT_N + LT_G); 0, or -1 if none ran
// light tracing's connections that reached each pixel over the last render call (n pixels)
int sto_last_lt_counts(uint32_t* out, uint32_t n) {
    if (g_lt_count.size() != n) return -1;
    std::copy(g_lt_count.begin(), g_lt_count.end(), out);
    return 0;
}
int sto_last_lt(uint32_t* emit, uint32_t* hit, float* cdf) {
    if (g_lt_cdf.empty()) return -1;
    std::copy(g_lt_emit.begin(), g_lt_emit.end(), emit);
    std::copy(g_lt_hit.begin(), g_lt_hit.end(), hit);
    std::copy(g_lt_cdf.begin(), g_lt_cdf.end(), cdf);
    return 0;
}
double sto_sppm_keep(double capacity, double demand) { return sppm_keep(capacity, demand); }
uint32_t sto_sppm_subs_of(uint32_t count, uint32_t share) { return sppm_subs_of(count, share); }
uint32_t sto_sppm_oct(const float* v) { return sppm_oct(v); }
void sto_sppm_unoct(uint32_t w, float* out) { sppm_unoct(w, out); }
int sto_sppm_build(const float* pos, const float* power, const uint32_t* nrm, const uint32_t* flags, uint32_t n,
                   float cell, uint32_t* key, uint32_t* cell_count) {
    sppm_build(g_grid, pos, power, nrm, flags, n, cell);
    if (key) for (uint32_t i = 0; i < n; i++) key[i] = g_grid.key[i];
    if (cell_count) for (uint32_t h = 0; h < SPPM_HEADS; h++) cell_count[h] = (uint32_t)g_grid.lists[h].size();
    return 0;
}
int sto_sppm_gather(const float* qpos, const float* qnrm, const float* qalb, const uint32_t* qb, uint32_t m, float radius,
                    uint32_t maxbounce, uint32_t budget, uint32_t seed, double* out, uint32_t* visits, uint32_t* cuts) {
    U4 ss = sample_seed(seed, 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (long i = 0; i < (long)m; i++) {
        Rng r; r.h = ss; r.seed_u32((uint32_t)i); r.seed_u32(0x53505000u);
        uint32_t v = 0; bool cut = false;
        sppm_gather(g_grid, &qpos[3 * i], &qnrm[3 * i], &qalb[3 * i], qb[i], radius, maxbounce, budget, r, &out[3 * i], v, cut);
        if (visits) visits[i] = v;
        if (cuts) cuts[i] = cut ? 1 : 0;
    }
    return 0;
}

// ---- haze (st_oracle_extra.h) and the far field (st_oracle_optics.h), for the tests ----
void sto_haze_span(const st_scene_desc* s, const double* A, const double* d, double len, double R, double* t) {
    HazeBox<double> h; h.init(*s);
    h.span(V3<double>(A[0], A[1], A[2]), V3<double>(d[0], d[1], d[2]), len, R, t[0], t[1]);
}
double sto_hg_eval(double c, double g) { return hg_eval(c, g); }
void sto_hg_sample(double g, const double* d, uint32_t seed, int n, double* out) {
    Rng r; r.h = sample_seed(seed, 1);
    for (int i = 0; i < n; i++) {
        double u[4]; r.next4(u);
        V3<double> v = hg_sample(V3<double>(d[0], d[1], d[2]), g, u[0], u[1]);
        out[3 * i] = v.x; out[3 * i + 1] = v.y; out[3 * i + 2] = v.z;
    }
}
uint32_t sto_far_bin(const float* d, const float* ax, const float* c0, uint32_t nC, uint32_t nG) { return far_bin(d, ax, c0, nC, nG); }
void sto_far_geometry(uint32_t nC, uint32_t nG, double* omega) { far_geometry(nC, nG, omega); }
void sto_far_intensity(const double* flux, uint32_t nC, uint32_t nG, double* I) { far_intensity(flux, nC, nG, I); }

}  // extern "C"

// ---- the learned proposal (st_oracle_guide.h) ----
extern "C" {

void sto_guide_forward(const float* P, uint32_t n, const float* pos, const float* nrm, const float* lo, float inv_ext,
                       int bf, double* raw) {
    guide::Fwd f;
    for (uint32_t i = 0; i < n; i++) {
        if (bf) guide::forward<true>(P, pos + 3 * i, nrm + 3 * i, lo, inv_ext, f);
        else guide::forward<false>(P, pos + 3 * i, nrm + 3 * i, lo, inv_ext, f);
        for (int o = 0; o < guide::OUT; o++) raw[(size_t)i * guide::OUT + o] = f.y[o];
    }
}
void sto_guide_decode(const double* raw, uint32_t n, double* mix) {
    for (uint32_t i = 0; i < n; i++)
        guide::decode(raw + (size_t)i * guide::OUT, reinterpret_cast<double(*)[5]>(mix + (size_t)i * 40));
}
double sto_guide_grad(const float* P, uint32_t n, const float* pos, const float* nrm, const float* dir, const float* wt,
                      const float* lo, float inv_ext, int bf, double* G) {
    return bf ? guide::batch_grad<true>(P, (int)n, pos, nrm, dir, wt, lo, inv_ext, G)
              : guide::batch_grad<false>(P, (int)n, pos, nrm, dir, wt, lo, inv_ext, G);
}
double sto_guide_loss(const float* P, uint32_t n, const float* pos, const float* nrm, const float* dir, const float* wt,
                      const float* lo, float inv_ext) {
    std::vector<double> G(guide::NPARAM, 0.0);
    return guide::batch_grad<false>(P, (int)n, pos, nrm, dir, wt, lo, inv_ext, G.data());
}
double sto_guide_mix_pdf(const double* mix, const double* d) {
    return guide::mix_pdf(reinterpret_cast<const double(*)[5]>(mix), d);
}
void sto_guide_mix_sample(const double* mix, const double* u, uint32_t n, double* d) {
    for (uint32_t i = 0; i < n; i++)
        guide::mix_sample(reinterpret_cast<const double(*)[5]>(mix), u[3 * i], u[3 * i + 1], u[3 * i + 2], d + 3 * i);
}
float sto_bf16(float x) { return guide::bf16(x); }

}  // extern "C"
