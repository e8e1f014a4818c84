// st_capi.cu -- the C ABI of libshadytracer.so (include/shadytracer.h): the context, the scene / settings / camera,
// the wave's device buffers, and the per-sample launch chain.
//
// A SAMPLE, AS THE HOST RUNS IT (the reference's R.trace, core/raytrace_main.js:1574-2300): genrays, then `budget`
// wavefront iterations of march -> shade -> occlude, then resolve. Nothing is read back inside it; every kernel
// sizes itself from the device counters, so the chain is recorded once into a CUDA graph per (scene, settings,
// wave size) and replayed per wave -- the sample index the kernels seed from lives in device memory and resolve
// advances it. A WAVE holds several samples of a small picture at once (samples_per_wave), so a 256 x 256 image
// still puts two million paths in flight; a 1080p one runs one sample a wave.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "st_internal.h"
#include "st_ext.h"
#include "st_sky.h"
#include "st_spectral.h"

#define SPPM_WAVE_BUDGET 512u                 // records a gather walks before it subsamples (sppm.js SPPM_VISIT)

using namespace st;

namespace {
struct KTimeAcc { std::string name; uint32_t launches = 0; double ms = 0; };
struct PendingEvent { int idx; cudaEvent_t a, b; };
const double PI_D = 3.14159265358979323846;
}  // namespace

struct st_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sms = 1;
    std::string err;
    // the scene
    std::vector<st_prim> prims;
    std::vector<st_material> mats;
    st_scene_desc desc{};
    bool has_scene = false, has_params = false, has_view = false;
    DPrim* d_prims = nullptr;
    float4* d_faces = nullptr;            // the lights' faces (FACE_F4 float4s each), then the material -> face map
    uint32_t n_faces = 0;
    float* d_sc = nullptr;                // the step cache's cells, and the grid they were filled for
    size_t sc_cap = 0;
    bool sc_live = false;
    uint64_t sc_scene = 0, scene_gen = 0;
    float sc_lo[3] = {0, 0, 0}, sc_cs = 0.f, sc_cells = 0.f;
    uint32_t sc_dims[3] = {0, 0, 0};
    float4* d_envimg = nullptr;           // the environment image (rgb, 0) and its map's tables; null, none
    float4* d_envmap = nullptr;
    uint32_t env_w = 0, env_h = 0;
    float4* d_skytab = nullptr;           // the sun and sky's 16 bands (st_sky.h), once a context
    // many views in one wave (st_set_views): their cameras and the table the kernels read them from (VIEW_F4 float4s a
    // view; null with one); view 0 is `view`
    std::vector<st_view> views;
    uint32_t nv = 1;
    uint32_t acc_views = 0;               // the views the accumulation holds
    float4* d_views = nullptr;
    std::vector<float> env_key;           // what the preset's map was baked from (empty: no preset map)
    float4* d_envtex = nullptr;           // the preset in a texture (envCache), env_tw x env_th; null, none
    uint32_t env_tw = 0, env_th = 0;
    float env_lum = 0.f, env_turn = 0.f;
    st_material* d_mats = nullptr;
    st_params params{};
    st_view view{};
    // the albedo tables
    float *d_ec = nullptr, *d_ecavg = nullptr, *d_e1 = nullptr;
    float4* d_coat = nullptr;             // a coating's 10 nm bins (st_spectral.h coat_bin_table), COAT_BINS float4s
    float4* d_spec = nullptr;             // the camera's wavelength table (st_spectral.h), SPEC_CELLS float4s
    // the wave
    uint32_t W = 0, H = 0, P = 0, spw = 0, slot_cap = 0;
    PathBuf pb{};
    Queues q{};
    DevCtr* d_ctr = nullptr;
    float4* d_frame = nullptr;
    float4* d_splat = nullptr;            // light tracing's connections this sample, per pixel (rgb)
    uint32_t* d_ltcount = nullptr;        // ...and the connections that reached each pixel since the last invalidate
    Acc4* d_acc = nullptr;
    double2* d_mom = nullptr;
    uint32_t samples = 0;
    bool in_flight = false;
    // the launch chain as a graph, per wave size
    cudaGraphExec_t graph = nullptr;      // the wave chain of graph_w samples, captured
    uint32_t graph_w = 0;
    cudaGraphExec_t graph2 = nullptr;     // ...and a second size's (an emitter scene's first, short waves)
    uint32_t graph2_w = 0, graph2_launches = 0;
    bool graph_ok = true;
    uint32_t rec_launches = 0;            // kernels in the last recorded wave chain
    uint32_t graph_launches = 0;          // ...and in the graph's (its kernel nodes)
    uint64_t launches = 0;                // kernels run by the wave chains since the context was made
    uint32_t wait_limit = 0, wait_arm_only = 0;   // the device-side waits (st_set_wait_limit), kept across resets
    // per-kernel timing (core/kerneltime.js's role): CUDA events on this stream around each launch, when on
    bool timing = false;
    bool count_work = false;              // a counting pass: the march counts its fold's work
    bool grid_ok = false;                 // the bounded primitives' box, for the march queue's space order
    float grid_lo[3] = {0, 0, 0}, grid_hi[3] = {1, 1, 1};
    std::vector<KTimeAcc> ktimes;
    std::vector<PendingEvent> pending;
    std::vector<cudaEvent_t> event_pool;
    StExt ext;   // the photon map's and the optics bench's state (st_sppm.cu, st_optics.cu)
    SceneCode code;                       // the scene as compiled code (st_scene_rtc.cu), when it was given as code
    bool has_code = false;
    uint32_t tune_claim = 0, tune_chunk = 0;   // the autotuner's picks (st_autotune); 0, the defaults
};

static int fail(st_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}
static int cuda_fail(st_ctx* c, cudaError_t e, const char* what) {
    return fail(c, e == cudaErrorMemoryAllocation ? ST_ERR_OOM : ST_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call, what)                                         \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

// the device-side waits' settings into the counters, where the kernels read them (after any reset of the counters)
static cudaError_t push_wait(st_ctx* ctx) {
    const uint32_t w[2] = {ctx->wait_limit, ctx->wait_arm_only};
    cudaError_t e = cudaMemcpyAsync(&ctx->d_ctr->wait_limit, w, sizeof(w), cudaMemcpyHostToDevice, ctx->stream);
    return e == cudaSuccess ? cudaStreamSynchronize(ctx->stream) : e;
}

static void free_wave(st_ctx* ctx) {
    void* ptrs[] = {ctx->pb.pos, ctx->pb.dir, ctx->pb.beta, ctx->pb.rad, ctx->pb.meta, ctx->pb.lam, ctx->pb.lprev,
                    ctx->q.ray[0], ctx->q.ray[1],
                    ctx->q.hit, ctx->q.hitd, ctx->q.hsurf, ctx->q.sorted, ctx->q.skey, ctx->q.srank, ctx->q.bcnt,
                    ctx->q.boff, ctx->q.ssorted, ctx->q.sskey, ctx->q.ssrank, ctx->q.s_org[0], ctx->q.s_dir[0], ctx->q.s_rad[0], ctx->q.s_steps[0],
                    ctx->q.s_org[1], ctx->q.s_dir[1], ctx->q.s_rad[1], ctx->q.s_steps[1], ctx->d_frame,
                    ctx->d_acc, ctx->d_mom, ctx->d_splat, ctx->d_ltcount};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    ctx->pb = PathBuf{};
    ctx->q = Queues{};
    ctx->d_frame = nullptr;
    ctx->d_acc = nullptr;
    ctx->d_mom = nullptr;
    ctx->d_splat = nullptr;
    ctx->d_ltcount = nullptr;
    ctx->slot_cap = 0;
    if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; ctx->graph_w = 0; }
    if (ctx->graph2) { cudaGraphExecDestroy(ctx->graph2); ctx->graph2 = nullptr; ctx->graph2_w = 0; }
}

static int time_index(st_ctx* ctx, const char* name) {
    for (size_t i = 0; i < ctx->ktimes.size(); i++)
        if (ctx->ktimes[i].name == name) return (int)i;
    ctx->ktimes.push_back(KTimeAcc{name, 0, 0});
    return (int)ctx->ktimes.size() - 1;
}
static cudaEvent_t take_event(st_ctx* ctx) {
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
static void collect_times(st_ctx* ctx) {
    for (auto& p : ctx->pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            ctx->ktimes[p.idx].ms += ms;
            ctx->ktimes[p.idx].launches++;
        }
        ctx->event_pool.push_back(p.a);
        ctx->event_pool.push_back(p.b);
    }
    ctx->pending.clear();
}

// ------------------------------------------------------------------------------------------------------------
// the uniforms, derived on the host in double precision (core/photometry.js:55-73 sunCone / discLuminance,
// :182-237 derive), then rounded once
// ------------------------------------------------------------------------------------------------------------
// what depends only on the scene's description, the settings and the camera (the render that allocates nothing,
// st_noalloc.cu, takes its uniforms from here too); env_image: an environment image replaces the sun and sky
Uni make_uni_base(const st_scene_desc& s, const st_params& p, const st_view& v, uint32_t n_prims, uint32_t n_mats,
                  bool env_image) {
    Uni u{};
    u.W = p.width; u.H = p.height; u.P = p.width * p.height;
    const double N = double(u.W) * double(u.H);
    u.tilesX = std::max<uint32_t>(1, (uint32_t)std::llround(std::sqrt(N * (double(u.W) / std::max<double>(1, u.H)))));
    u.tilesY = std::max<uint32_t>(1, (uint32_t)std::ceil(N / u.tilesX));
    u.invTX = float(1.0 / u.tilesX);
    u.invTY = float(1.0 / u.tilesY);
    u.maxbounce = p.maxbounce; u.maxiter = p.maxiter; u.nee = p.nee; u.rr = p.rr;
    // THE ITERATION BUDGET IS THE WORST CASE (core/raytrace_main.js:1795-1815): maxbounce + 1 + ceil(maxiter / 32)
    u.budget = p.budget ? p.budget : std::max(2u, p.maxbounce + 1 + (p.maxiter + 31) / 32);
    u.stepscale = p.stepscale;
    double tol = p.eps > 0 ? p.eps : (s.tolerance > 0 ? s.tolerance : 1e-3);
    double R = s.env_radius > 0 ? s.env_radius : 400.0;
    u.tol = (float)tol;
    u.envR = (float)R;
    u.envR2 = (float)(R * R);
    u.cam = mk(v.cam_pos[0], v.cam_pos[1], v.cam_pos[2]);
    u.right = mk(v.right[0], v.right[1], v.right[2]);
    u.up = mk(v.up[0], v.up[1], v.up[2]);
    u.fwd = mk(v.fwd[0], v.fwd[1], v.fwd[2]);
    u.fx = v.fx; u.fy = v.fy; u.camtype = v.camtype;
    u.lens_r = v.lens_radius > 0.f ? v.lens_radius : 0.f;
    u.lens_f = v.focus_distance;
    double half = std::max((double)p.sun_diameter, 1e-3) * PI_D / 360.0;
    double sh = std::sin(half / 2);
    double omc = 2 * sh * sh;
    double sin2 = std::sin(half) * std::sin(half);
    double disc = (double)p.sun_illuminance / (PI_D * sin2);
    const double raw[3] = {1.0, 0.96, 0.9};
    double y = raw[0] * 0.2126 + raw[1] * 0.7152 + raw[2] * 0.0722;
    bool furnace = p.env_uniform > 0;
    // the presets (environment.js): the image or the furnace replace them; the studio has no sun to aim at
    const uint32_t env_mode = (furnace || env_image || p.env_mode > ST_ENV_STUDIO) ? 0u : p.env_mode;
    // an environment image is the whole environment, with no sun to aim at (envimage.js, the image preset)
    int sun_on = (p.sun_hint != 0 && p.sun_elevation * PI_D / 180.0 + half > 0 && !furnace && !env_image &&
                  env_mode != ST_ENV_STUDIO) ? 1 : 0;
    double e = p.sun_elevation * PI_D / 180.0, az = p.sun_azimuth * PI_D / 180.0;
    u.sun_dir = mk((float)(std::cos(e) * std::sin(az)), (float)(std::cos(e) * std::cos(az)), (float)std::sin(e));
    u.sun_sin2 = (float)sin2;
    u.sun_omc = (float)omc;
    u.sun_omega = (float)(2 * PI_D * omc);
    u.pick = (float)((sun_on && p.env_sun_gain > 0) ? p.nee_sun_pick : 0.0);
    u.sun_on = sun_on;
    u.disc = mk((float)(disc * raw[0] / y), (float)(disc * raw[1] / y), (float)(disc * raw[2] / y));
    u.sky = p.sky_luminance; u.ground = p.ground_luminance; u.uniform = p.env_uniform;
    u.sun_gain = std::max(0.f, p.env_sun_gain); u.sky_gain = std::max(0.f, p.env_sky_gain);
    u.env_mode = env_mode;
    u.sun_outside = p.sun_outside > 0.f ? p.sun_outside : 128000.f;              // environment.js: 128 klx
    u.aerosol = (float)(0.05 + 0.1 * std::max(0.0, (double)p.sky_turbidity));
    {
        const double top = std::min(std::max((double)p.studio_top, 0.0), 1.0);
        double c[3] = {std::max(0.0, (double)p.studio_color[0]), std::max(0.0, (double)p.studio_color[1]),
                       std::max(0.0, (double)p.studio_color[2])};
        const double y = std::max(c[0] * 0.2126 + c[1] * 0.7152 + c[2] * 0.0722, 1e-6);
        u.studio_l0 = (float)(std::max(0.0, (double)p.studio_illuminance) / (PI_D * (1.0 + 2.0 * top / 3.0)));
        u.studio_top = (float)top;
        u.studio_tint = mk((float)(c[0] / y), (float)(c[1] / y), (float)(c[2] / y));
    }
    u.haze_on = s.haze_sigma_t > 0 ? 1 : 0;
    u.hc = mk(s.haze_centre[0], s.haze_centre[1], s.haze_centre[2]);
    u.hu = mk(s.haze_axes[0], s.haze_axes[1], s.haze_axes[2]);
    u.hv = mk(s.haze_axes[3], s.haze_axes[4], s.haze_axes[5]);
    u.hw = mk(s.haze_axes[6], s.haze_axes[7], s.haze_axes[8]);
    u.hhu = s.haze_half[0]; u.hhv = s.haze_half[1]; u.hhw = s.haze_half[2];
    u.hsig = s.haze_sigma_t;
    auto sat01 = [](float x) { return std::min(std::max(x, 0.f), 1.f); };
    u.halb = mk(sat01(s.haze_albedo[0]), sat01(s.haze_albedo[1]), sat01(s.haze_albedo[2]));
    u.hg = std::min(std::max(s.haze_g, -0.95f), 0.95f);
    u.seed = p.seed; u.maxaverages = p.maxaverages;
    u.n_prims = n_prims;
    u.n_mats = n_mats;
    return u;
}

static Uni make_uni(const st_ctx* ctx) {
    const st_params& p = ctx->params;
    Uni u = make_uni_base(ctx->desc, p, ctx->view, (uint32_t)ctx->prims.size(), (uint32_t)ctx->mats.size(),
                          ctx->d_envimg != nullptr);
    u.claim = ctx->tune_claim;
    u.chunk = ctx->tune_chunk;
    for (const st_material& m : ctx->mats)                     // the march walks the materials that scatter inside
        if (m.scatter_distance > 0.f) u.scatter_on = 1u;
    // the worst case counted in chunks of at most 32 (the reference's dispatches): a tuned chunk below that gets the
    // iterations its longer marches need
    if (!p.budget && u.chunk && u.chunk < 32u)
        u.budget = std::max(2u, p.maxbounce + 1 + (p.maxiter + u.chunk - 1) / u.chunk);
    if (ctx->d_envimg) {
        u.env_img = ctx->d_envimg; u.env_w = ctx->env_w; u.env_h = ctx->env_h;
        u.env_lum = ctx->env_lum; u.env_turn = ctx->env_turn;
    }
    u.sky_tab = ctx->d_skytab;
    if (ctx->d_envtex && u.env_mode != ST_ENV_ANALYTIC && !ctx->env_key.empty()) {
        u.env_tex = ctx->d_envtex; u.env_tw = ctx->env_tw; u.env_th = ctx->env_th;
    }
    u.nv = ctx->nv;
    u.views = ctx->nv > 1 ? ctx->d_views : nullptr;
    // the map light sampling draws from: an image's, or a preset's (envmap.js bakes one for every environment)
    if (ctx->d_envimg || (u.env_mode != ST_ENV_ANALYTIC && !ctx->env_key.empty())) {
        u.env_map = ctx->d_envmap;
        u.env_mshare = ctx->d_envmap && !p.env_map_off ? 0.5f : 0.f;    // ENV_MAP_SHARE
    }
    if (ctx->sc_live && p.step_cache) {
        u.sc = ctx->d_sc;
        u.sc_lo = mk(ctx->sc_lo[0], ctx->sc_lo[1], ctx->sc_lo[2]);
        u.sc_cs = ctx->sc_cs;
        u.sc_dx = ctx->sc_dims[0]; u.sc_dy = ctx->sc_dims[1]; u.sc_dz = ctx->sc_dims[2];
        u.sc_looks = p.step_cache >= 2 ? 3u : 1u;
    }
    // the march queue's space order: a grid over the bounded primitives' spheres (none bounded: no sort)
    // the space order pays where a step is dear: a table of a few primitives marches fast in any order, and there the
    // sort's three launches an iteration cost more than the coherence saves (the SDF room, 27 primitives: 19 % faster
    // sorted; the photon map's caustic, 3: 2 % slower)
    u.sort_on = ctx->grid_ok && ctx->q.sorted && ctx->prims.size() >= SORT_MIN_PRIMS ? 1u : 0u;
    u.glo = mk(ctx->grid_lo[0], ctx->grid_lo[1], ctx->grid_lo[2]);
    u.ginv = mk(SORT_G / (ctx->grid_hi[0] - ctx->grid_lo[0]), SORT_G / (ctx->grid_hi[1] - ctx->grid_lo[1]),
                SORT_G / (ctx->grid_hi[2] - ctx->grid_lo[2]));
    return u;
}

// ------------------------------------------------------------------------------------------------------------
// A PRIMITIVE AS THE KERNELS READ IT (st_device.cuh DPrim): its fields in 16-byte words, the radius of a sphere
// about its centre that holds it -- inflated by 0.1 % + 10 um so the f32 test never passes a primitive whose own f32
// distance is nearer -- and a prism's edge constants (shapes.js:266-283), in double here. +inf where the distance is
// not an exact one (the aspheric lens's is a bound, shapes.js:621-640) or the shape is unbounded (the plane).
// ------------------------------------------------------------------------------------------------------------
// THE LIGHTS' FACES (builder/lights.js; codegen.js:861-912 emitLightFaces): each checked, its frame made orthonormal
// (u, v at right angles, n = u x v), drawn as a sheet of its material appended to the primitives (a rectangle a box
// of no thickness, a disc a cylinder of none) and packed for the device, with the map from its material to it
static bool light_faces(const st_scene_desc* d, std::vector<st_prim>& prims, std::vector<float4>& out,
                        std::string& why) {
    const uint32_t nl = d->lights ? d->n_lights : 0u;
    if (nl > ST_MAX_LIGHTS) { why = "n_lights out of range (0..64)"; return false; }
    if (prims.size() + nl > ST_MAX_PRIMS) { why = "n_prims + n_lights above 256"; return false; }
    uint8_t* of = reinterpret_cast<uint8_t*>(out.data() + ST_MAX_LIGHTS * FACE_F4);
    for (uint32_t i = 0; i < nl; i++) {
        const st_light& L = d->lights[i];
        const std::string at = "light " + std::to_string(i) + ": ";
        if (L.shape != ST_LIGHT_DISC && L.shape != ST_LIGHT_RECTANGLE) { why = at + "unknown shape"; return false; }
        if (L.material == 0 || L.material >= d->n_materials) { why = at + "material out of range (1..n_materials-1)"; return false; }
        if (of[L.material]) { why = at + "its material draws another light (one material a light)"; return false; }
        if (!(L.half_w > 0.f) || (L.shape == ST_LIGHT_RECTANGLE && !(L.half_h > 0.f))) { why = at + "no size"; return false; }
        if (!(L.beam_cos >= 0.f && L.beam_cos < 1.f) || !(L.n >= 0.f) || L.dist > ST_LIGHT_UNIFORM) {
            why = at + "beam out of range"; return false;
        }
        if (!(L.le[0] >= 0.f && L.le[1] >= 0.f && L.le[2] >= 0.f)) { why = at + "negative luminance"; return false; }
        double u[3] = {L.u[0], L.u[1], L.u[2]}, v[3] = {L.v[0], L.v[1], L.v[2]};
        const double lu = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        if (!(lu > 1e-12)) { why = at + "no u axis"; return false; }
        for (double& c : u) c /= lu;
        const double uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
        for (int k = 0; k < 3; k++) v[k] -= uv * u[k];
        const double lv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (!(lv > 1e-12)) { why = at + "v along u"; return false; }
        for (double& c : v) c /= lv;
        const double n[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
        const float hh = L.shape == ST_LIGHT_DISC ? L.half_w : L.half_h;
        float4* f = out.data() + (size_t)i * FACE_F4;
        f[0] = make_float4(L.centre[0], L.centre[1], L.centre[2], L.half_w);
        f[1] = make_float4((float)u[0], (float)u[1], (float)u[2], hh);
        f[2] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)L.shape);
        f[3] = make_float4((float)n[0], (float)n[1], (float)n[2], L.beam_cos);
        f[4] = make_float4(L.le[0], L.le[1], L.le[2], L.dist == ST_LIGHT_UNIFORM ? -1.f : L.n);
        of[L.material] = (uint8_t)(i + 1);
        st_prim p{};
        p.type = L.shape == ST_LIGHT_DISC ? ST_PRIM_CYLINDER : ST_PRIM_BOX;
        p.op = ST_OP_ITEM;
        p.material = L.material;
        for (int k = 0; k < 3; k++) {
            p.pos[k] = L.centre[k];
            p.rot[k] = (float)u[k]; p.rot[3 + k] = (float)v[k]; p.rot[6 + k] = (float)n[k];   // world -> local rows
        }
        if (L.shape == ST_LIGHT_DISC) { p.p[0] = 0.f; p.p[1] = L.half_w; }
        else { p.p[0] = L.half_w; p.p[1] = L.half_h; p.p[2] = 0.f; }
        prims.push_back(p);
    }
    return true;
}

DPrim pack_prim(const st_prim& p) {
    DPrim d{};
    const float* q = p.p;
    double R = INFINITY;
    switch (p.type) {
        case ST_PRIM_SPHERE: R = std::fabs(q[0]); break;
        case ST_PRIM_BOX: R = std::sqrt(double(q[0]) * q[0] + double(q[1]) * q[1] + double(q[2]) * q[2]); break;
        case ST_PRIM_ROUNDBOX:
            R = std::sqrt(double(q[0]) * q[0] + double(q[1]) * q[1] + double(q[2]) * q[2]) + std::fabs(q[3]);
            break;
        case ST_PRIM_TORUS: R = std::fabs(q[0]) + std::fabs(q[1]); break;
        case ST_PRIM_PRISM: R = std::sqrt(double(q[1]) * q[1] + 0.25 * double(q[2]) * q[2]) + std::fabs(q[3]); break;
        case ST_PRIM_CYLINDER: R = std::sqrt(double(q[0]) * q[0] + double(q[1]) * q[1]); break;
        default: R = INFINITY;
    }
    float Rf = std::isfinite(R) ? (float)(R * 1.001 + 1e-5) : INFINITY;
    d.a = make_float4(p.pos[0], p.pos[1], p.pos[2], Rf);
    d.r0 = make_float4(p.rot[0], p.rot[1], p.rot[2], p.k);
    d.r1 = make_float4(p.rot[3], p.rot[4], p.rot[5], q[0]);
    d.r2 = make_float4(p.rot[6], p.rot[7], p.rot[8], q[1]);
    d.e = make_float4(q[2], q[3], q[4], q[5]);
    d.f = make_float4(q[6], q[7], q[8], q[9]);
    if (p.type == ST_PRIM_PRISM) {
        double n = std::min(std::max(std::nearbyint((double)q[0]), 3.0), 64.0);
        double an = PI_D / n, Rp = std::max((double)q[1], 0.0);
        d.g = make_float4((float)(Rp * std::cos(an)), (float)(Rp * std::sin(an)), (float)(2 * an), (float)n);
    }
    d.h = make_uint4(p.type, p.op, p.material, p.flags);
    return d;
}

static bool sppm_runs(const st_ctx* ctx);
static bool photons_run(const st_ctx* ctx);
static uint32_t sppm_photons(const st_ctx* ctx);
static uint32_t samples_per_wave(const st_ctx* ctx) {
    // the photon map or light tracing: each sample its own photons (and the map's radius and grid)
    if (photons_run(ctx)) return 1;
    if (ctx->params.samples_per_wave) return ctx->params.samples_per_wave;
    const uint32_t target = 4u << 20;   // about four million paths a wave: twenty a lane of a full persistent grid
    const uint32_t per = ctx->P * ctx->nv;      // a sample of every view
    uint32_t s = (target + per - 1) / per;
    return std::max(1u, std::min(s, 64u));
}

// a scene with an emissive material: the emitter list's discovery and light sampling run
static bool has_emitters(const st_ctx* ctx) {
    for (const st_material& m : ctx->mats)
        if (std::max(m.emissive[0], std::max(m.emissive[1], m.emissive[2])) > 0.f) return true;
    return false;
}

static int ensure_wave(st_ctx* ctx) {
    if (photons_run(ctx)) {
        // the map's records (light tracing alone stores none) and the emission map's counts: a record a photon at
        // most on surfaces; in a scene that scatters inside a material, one at each collision too -- room for 32 a
        // photon, at most 64 M records, a sample's stores past its share thinned without bias (k_sppm_begin's keep)
        uint32_t need = sppm_runs(ctx) ? sppm_photons(ctx) : 1024u;
        if (sppm_runs(ctx) && make_uni(ctx).scatter_on) need = (uint32_t)std::min<uint64_t>((uint64_t)need * 32u, 64u << 20);
        int rc = sppm_ensure(ctx, need);
        if (rc) return rc;
        if (sppm_runs(ctx)) ctx_ext(ctx).sppm.wave = true;
    }
    if (ctx->params.guide) {
        const uint32_t spw_g = samples_per_wave(ctx);
        uint32_t cap_g = spw_g * ctx->nv * ctx->P;
        if (photons_run(ctx)) cap_g = std::max(cap_g, std::min(sppm_photons(ctx), 4u << 20));
        int rc = guide_ensure(ctx, cap_g, spw_g * ctx->nv * ctx->P, ctx->params.guide_seed);
        if (rc) return rc;
    }
    uint32_t spw = samples_per_wave(ctx);
    uint32_t cap = spw * ctx->nv * ctx->P;
    // the photons run in chunks of the wave's slots: give them room for up to four million at once
    if (photons_run(ctx)) cap = std::max(cap, std::min(sppm_photons(ctx), 4u << 20));
    if (has_emitters(ctx)) {                   // the list's per-slot weights and its hit queue (a shadow side's room)
        int rc = emit_ensure(ctx, cap, 2u * cap);
        if (rc) return rc;
    }
    bool pixels_changed = !ctx->d_acc || ctx->acc_views != ctx->nv;
    if (ctx->slot_cap == cap && ctx->spw == spw && !pixels_changed) return ST_OK;
    free_wave(ctx);
    ctx->spw = spw;
    size_t S = cap;
    CK(cudaMalloc(&ctx->pb.pos, S * sizeof(float4)), "cudaMalloc path state");
    CK(cudaMalloc(&ctx->pb.dir, S * sizeof(float4)), "cudaMalloc path state");
    CK(cudaMalloc(&ctx->pb.beta, S * sizeof(float4)), "cudaMalloc path state");
    CK(cudaMalloc(&ctx->pb.rad, S * sizeof(float4)), "cudaMalloc path state");
    CK(cudaMalloc(&ctx->pb.meta, S * sizeof(uint4)), "cudaMalloc path state");
    CK(cudaMalloc(&ctx->pb.lam, S * sizeof(float)), "cudaMalloc path state");
    CK(cudaMalloc(&ctx->pb.lprev, S * sizeof(float2)), "cudaMalloc path state");
    CK(cudaMalloc(&ctx->q.ray[0], S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.ray[1], S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.hit, S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.hitd, S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.hsurf, S * sizeof(float4)), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.sorted, S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.skey, S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.srank, S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.ssorted, 2 * S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.sskey, 2 * S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.ssrank, 2 * S * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.bcnt, SORT_BUCKETS * 4), "cudaMalloc queues");
    CK(cudaMalloc(&ctx->q.boff, SORT_BUCKETS * 4), "cudaMalloc queues");
    CK(cudaMemset(ctx->q.bcnt, 0, SORT_BUCKETS * 4), "memset queues");
    // each shadow side holds this iteration's new rays (at most one a path) and the last one's continuations
    size_t SS = 2 * S;
    for (int k = 0; k < 2; k++) {
        CK(cudaMalloc(&ctx->q.s_org[k], SS * sizeof(float4)), "cudaMalloc shadow queue");
        CK(cudaMalloc(&ctx->q.s_dir[k], SS * sizeof(float4)), "cudaMalloc shadow queue");
        CK(cudaMalloc(&ctx->q.s_rad[k], SS * sizeof(float4)), "cudaMalloc shadow queue");
        CK(cudaMalloc(&ctx->q.s_steps[k], SS * sizeof(uint32_t)), "cudaMalloc shadow queue");
    }
    ctx->q.scap = (uint32_t)SS;
    CK(cudaMalloc(&ctx->d_frame, S * sizeof(float4)), "cudaMalloc frame");
    CK(cudaMalloc(&ctx->d_acc, (size_t)ctx->nv * ctx->P * sizeof(Acc4)), "cudaMalloc accumulation");
    CK(cudaMalloc(&ctx->d_mom, (size_t)ctx->nv * ctx->P * sizeof(double2)), "cudaMalloc moments");
    ctx->acc_views = ctx->nv;
    CK(cudaMalloc(&ctx->d_splat, (size_t)ctx->P * sizeof(float4)), "cudaMalloc splat");
    CK(cudaMalloc(&ctx->d_ltcount, (size_t)ctx->P * sizeof(uint32_t)), "cudaMalloc splat");
    ctx->q.cap = cap;
    ctx->slot_cap = cap;
    CK(cudaMemsetAsync(ctx->d_frame, 0, S * sizeof(float4), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_acc, 0, (size_t)ctx->acc_views * ctx->P * sizeof(Acc4), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_mom, 0, (size_t)ctx->acc_views * ctx->P * sizeof(double2), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_splat, 0, (size_t)ctx->P * sizeof(float4), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_ltcount, 0, (size_t)ctx->P * sizeof(uint32_t), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_ctr, 0, sizeof(DevCtr), ctx->stream), "memset");
    if (ctx->wait_limit || ctx->wait_arm_only) CK(push_wait(ctx), "wait limit");
    ctx->samples = 0;
    return ST_OK;
}

// the photon map runs while it is set and the sun shines (its photons are the sun's)
static bool sppm_runs(const st_ctx* ctx) {
    if (!ctx->has_params || !ctx->params.sppm) return false;
    const Uni u = make_uni(ctx);
    return u.sun_on != 0 && ctx->params.env_uniform <= 0.f;
}
static bool has_emitters(const st_ctx* ctx);
// light tracing runs while it is set and there are photons: the sun's while it shines, the emitters' in a scene with
// emissive materials
static bool lt_runs(const st_ctx* ctx) {
    if (!ctx->has_params || !ctx->params.lt) return false;
    const Uni u = make_uni(ctx);
    return (u.sun_on != 0 && ctx->params.env_uniform <= 0.f) || has_emitters(ctx);
}
static bool photons_run(const st_ctx* ctx) { return sppm_runs(ctx) || lt_runs(ctx); }
// the sun's photons a sample: the map's count while it runs (they serve both), else light tracing's
static uint32_t sppm_photons(const st_ctx* ctx) {
    if (sppm_runs(ctx)) return ctx->params.sppm_photons ? ctx->params.sppm_photons : ctx->P;
    return ctx->params.lt_photons ? ctx->params.lt_photons : ctx->P;
}

static WaveArgs wave_args(st_ctx* ctx, uint32_t w) {
    WaveArgs a;
    a.u = make_uni(ctx);
    a.u.count_work = ctx->count_work ? 1u : 0u;
    a.prims = ctx->d_prims;
    a.mats = ctx->d_mats;
    a.tab = MfTab{ctx->d_ec, ctx->d_ecavg, ctx->d_e1, ctx->d_coat};
    a.spec = ctx->d_spec;
    a.pb = ctx->pb;
    a.q = ctx->q;
    a.ctr = ctx->d_ctr;
    a.frame = ctx->d_frame;
    a.splat = ctx->d_splat;
    a.ltcount = ctx->d_ltcount;
    a.acc = ctx->d_acc;
    a.mom = ctx->d_mom;
    a.spw = w;
    a.slots = w * ctx->nv * ctx->P;
    a.code = ctx->has_code ? &ctx->code : nullptr;
    if (photons_run(ctx)) {
        a.u.sppm_on = sppm_runs(ctx) ? 1u : 0u;
        a.u.lt_on = lt_runs(ctx) ? 1u : 0u;
        a.u.sppm_n = sppm_photons(ctx);
        a.u.sppm_budget = SPPM_WAVE_BUDGET;
        a.u.sppm_half = ctx->params.sppm_half > 0.f ? ctx->params.sppm_half : std::min(15.f, a.u.envR);
        a.u.sppm_r1 = ctx->params.sppm_r1 > 0.f ? ctx->params.sppm_r1 : 0.005f;
        a.u.sppm_alpha = ctx->params.sppm_alpha > 0.f ? ctx->params.sppm_alpha : (float)(2.0 / 3.0);
        a.u.sppm_r1v = ctx->params.sppm_r1_volume > 0.f ? ctx->params.sppm_r1_volume : 4.f * a.u.sppm_r1;
        a.u.sppm_learn = ctx->params.sppm_learn ? 1u : 0u;
        a.sp = sppm_bufs(ctx_ext(ctx).sppm);
    }
    if (ctx->params.guide)
        a.gd = guide_bufs(ctx, 1u, ctx->params.guide_train ? 1u : 0u,
                          ctx->params.guide_alpha > 0.f ? std::min(ctx->params.guide_alpha, 1.f) : 0.5f, a.slots);
    if (has_emitters(ctx) && ctx_ext(ctx).emit.grid) {
        // the grid's half-size as the reference derives emitHalf (photometry.js:147-148 photonHalf, :223)
        const float set = ctx->params.emit_radius > 0.f ? ctx->params.emit_radius : 15.f;
        const float half = std::max(std::min(std::max(set, 1e-3f), a.u.envR), 1e-6f);
        a.em = emit_bufs(ctx, (!ctx->params.emit_off && a.u.nee) ? 1u : 0u,
                         ctx->params.emit_share > 0.f ? ctx->params.emit_share : 0.5f, half);
    }
    // light tracing's emitter probes (raytrace_main.js:1634-1635): their share of the photons, all of them with no sun
    if (a.u.lt_on && a.em.dev) {
        const bool sun = a.u.sun_on != 0 && ctx->params.env_uniform <= 0.f;
        const float set = ctx->params.lt_emit_share > 0.f ? ctx->params.lt_emit_share : 0.5f;
        const double share = sun ? std::min(0.95, std::max(0.05, (double)set)) : 1.0;
        a.u.lt_emit_n = (uint32_t)std::llround(share * (double)a.u.sppm_n);
    }
    if (ctx->n_faces) {
        a.lf.face = ctx->d_faces;
        a.lf.of = reinterpret_cast<const uint8_t*>(ctx->d_faces + ST_MAX_LIGHTS * FACE_F4);
        a.lf.n = ctx->n_faces;
    }
    return a;
}

// one wave's launch chain, onto the stream (recorded into a graph, or run directly when timing)
static cudaError_t record_wave(st_ctx* ctx, const WaveArgs& a) {
    cudaStream_t s = ctx->stream;
    const bool T = ctx->timing;
    ctx->rec_launches = 0;
    auto timed = [&](const char* name, auto&& launch) -> cudaError_t {
        ctx->rec_launches++;
        if (!T) return launch();
        PendingEvent pe{time_index(ctx, name), take_event(ctx), take_event(ctx)};
        cudaEventRecord(pe.a, s);
        cudaError_t e = launch();
        cudaEventRecord(pe.b, s);
        ctx->pending.push_back(pe);
        return e;
    };
    cudaError_t e;
    // the emitter list, from what the camera paths discovered: rebuilt between samples, every EMIT_EPOCH -- before the
    // sample's photons, whose probes draw from the list the camera's paths then weigh against
    if (a.em.on && (e = timed("emit_build", [&] { return launch_emit_build(a, 0.f, s); }))) return e;
    if (a.u.sppm_on || a.u.lt_on) {
        // THE SAMPLE'S PHOTONS FIRST (photons.js planBatches's `first`): in chunks of the wave's slots, each through
        // the march, the surface kernel and the photon's shade (and, with light tracing, the occlusion pass of the
        // connections it made); then the map's grid
        ctx->rec_launches++;
        if (a.u.sppm_on && (e = launch_sppm_begin(a, s))) return e;
        if (a.u.sppm_learn && (e = timed("lt_build", [&] { return launch_lt_build(a, s); }))) return e;
        const uint32_t N = a.u.sppm_n, C = ctx->slot_cap;          // the slots the path state holds
        for (uint32_t first = 0; first < N; first += C) {
            WaveArgs pa = a;
            pa.slots = std::min(C, N - first);
            pa.u.photon_pass = 1u;               // photons: the haze's collisions drawn from their own streams; one ends
                                                 // a photon (with light tracing, after its connection)
            pa.u.sort_on = 0;                    // the sun's photons start in order already (parallel, on a square)
            ctx->rec_launches++;
            if ((e = launch_iter_begin(pa, 0, 1, 1, s))) return e;
            if ((e = timed("photons", [&] { return launch_genphotons(pa, first, pa.slots, ctx->sms, s); }))) return e;
            int pc = 0;
            for (uint32_t it = 0; it < pa.u.budget; it++) {
                int nxt = pc ^ 1, last = it + 1 == pa.u.budget;
                if (it > 0 && (++ctx->rec_launches, e = launch_iter_begin(pa, (int)it, nxt, 0, s))) return e;
                if (pa.u.sort_on) {
                    if ((e = timed("photon_sort", [&] { return launch_sort(pa, pc, ctx->sms, s); }))) return e;
                    ctx->rec_launches += 2;
                }
                if ((e = timed("photon_march", [&] { return launch_march(pa, pc, nxt, last, ctx->sms, s); }))) return e;
                if ((e = timed("photon_surface", [&] { return launch_surface(pa, ctx->sms, s); }))) return e;
                const int side = (int)(it & 1u);
                if ((e = timed("photon_shade", [&] { return launch_photon_shade(pa, nxt, last, side, ctx->sms, s); })))
                    return e;
                if (pa.u.lt_on && (e = timed("photon_occlude", [&] { return launch_occlude(pa, side, last, ctx->sms, s); })))
                    return e;
                pc = nxt;
            }
        }
        if (a.u.sppm_on) {
            if ((e = timed("grid", [&] { return sppm_grid_launch(ctx_ext(ctx).sppm, ctx->sms, s); }))) return e;
            ctx->rec_launches += 5;                                  // key, three scan phases, scatter
        }
    }
    ctx->rec_launches++;
    if (a.gd.train && (e = guide_wave_begin(ctx, a.slots, s))) return e;
    if (a.gd.on && (e = guide_stamps_clear(ctx, ctx->nv * ctx->P, s))) return e;
    if ((e = launch_iter_begin(a, 0, 1, 1, s))) return e;
    if ((e = timed("genrays", [&] { return launch_genrays(a, ctx->sms, s); }))) return e;
    int cur = 0;
    // the camera's rays march unsorted: they leave one point in pixel-tile order, already coherent, where the space
    // order would only split them by octant
    WaveArgs a_eye = a;
    a_eye.u.sort_on = 0;
    for (uint32_t it = 0; it < a.u.budget; it++) {
        int nxt = cur ^ 1;
        int last = it + 1 == a.u.budget;
        int side = (int)(it & 1u);
        if (it > 0 && (++ctx->rec_launches, e = launch_iter_begin(a, (int)it, nxt, 0, s))) return e;
        if (a.u.sort_on && it > 0) {
            if ((e = timed("sort", [&] { return launch_sort(a, cur, ctx->sms, s); }))) return e;
            ctx->rec_launches += 2;                                  // key, scan, scatter
        }
        const WaveArgs& am = it == 0 ? a_eye : a;
        if ((e = timed("march", [&] { return launch_march(am, cur, nxt, last, ctx->sms, s); }))) return e;
        if ((e = timed("surface", [&] { return launch_surface(a, ctx->sms, s); }))) return e;
        if (a.u.sppm_on && (e = timed("gather", [&] { return launch_gather(a, ctx->sms, s); }))) return e;
        if (a.gd.on && !last && (e = timed("guide", [&] { return launch_guide_infer(a, ctx->sms, s); }))) return e;
        if ((e = timed("shade", [&] { return launch_shade(a, nxt, side, last, ctx->sms, s); }))) return e;
        if (a.u.sort_on) {
            if ((e = timed("sort", [&] { return launch_sort_shadow(a, side, ctx->sms, s); }))) return e;
            ctx->rec_launches += 2;
        }
        if ((e = timed("occlude", [&] { return launch_occlude(a, side, last, ctx->sms, s); }))) return e;
        if (a.em.on && (e = timed("emit_resolve", [&] { return launch_emit_resolve(a, ctx->sms, s); }))) return e;
        cur = nxt;
    }
    if (a.gd.train) {   // the records into a batch, then the training steps
        if ((e = timed("guide_collect", [&] { return launch_guide_collect(a, ctx->sms, s); }))) return e;
        const float lr = ctx->params.guide_lr > 0.f ? ctx->params.guide_lr : 0.005f;
        int n = 0;
        if ((e = timed("guide_train", [&] { return guide_train_launch(ctx, lr, ctx->sms, s, &n); }))) return e;
        ctx->rec_launches += n - 1;
    }
    return timed("resolve", [&] { return launch_resolve(a, s); });
}

static int run_wave(st_ctx* ctx, uint32_t w) {
    WaveArgs a = wave_args(ctx, w);
    if (ctx->timing || !ctx->graph_ok) {
        CK(record_wave(ctx, a), "launch");
        ctx->launches += ctx->rec_launches;
    } else {
        if (ctx->graph2 && ctx->graph2_w == w) {                // the other size's graph: swap the two
            std::swap(ctx->graph, ctx->graph2);
            std::swap(ctx->graph_w, ctx->graph2_w);
            std::swap(ctx->graph_launches, ctx->graph2_launches);
        } else if (ctx->graph && ctx->graph_w != w) {           // keep this one as the other size's
            if (ctx->graph2) cudaGraphExecDestroy(ctx->graph2);
            ctx->graph2 = ctx->graph;
            ctx->graph2_w = ctx->graph_w;
            ctx->graph2_launches = ctx->graph_launches;
            ctx->graph = nullptr;
            ctx->graph_w = 0;
        }
        if (!ctx->graph || ctx->graph_w != w) {
            if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; }
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "capture");
            cudaError_t e = record_wave(ctx, a);
            cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &g);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                cudaGetLastError();
                ctx->graph_ok = false;                       // fall back to direct launches, still on the GPU
                CK(record_wave(ctx, a), "launch");
                ctx->launches += ctx->rec_launches;
                ctx->samples += w;
                return ST_OK;
            }
            CK(cudaGraphInstantiate(&ctx->graph, g, 0), "graph instantiate");
            cudaGraphDestroy(g);
            ctx->graph_w = w;
            ctx->graph_launches = ctx->rec_launches;
        }
        CK(cudaGraphLaunch(ctx->graph, ctx->stream), "graph launch");
        ctx->launches += ctx->graph_launches;
    }
    ctx->samples += w;
    return ST_OK;
}

static void invalidate_graph(st_ctx* ctx) {
    if (ctx->graph) { cudaGraphExecDestroy(ctx->graph); ctx->graph = nullptr; ctx->graph_w = 0; }
    if (ctx->graph2) { cudaGraphExecDestroy(ctx->graph2); ctx->graph2 = nullptr; ctx->graph2_w = 0; }
}

extern "C" {

int st_abi_version(void) { return ST_ABI_VERSION; }

const char* st_last_error(const st_ctx* ctx) {
    if (ctx) return ctx->err.c_str();
    const char* m = noalloc_last_error();         // the calls with no context: st_render_noalloc's refusals
    return *m ? m : "no context";
}

int st_create(int device, st_ctx** out) {
    if (!out) return ST_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return ST_ERR_CUDA;
    if (device < 0 || device >= n) return ST_ERR_ARG;
    st_ctx* ctx = new st_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete ctx; return ST_ERR_CUDA; }
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return ST_ERR_CUDA; }
    const size_t NEC = 16 * 32 * 32, NAVG = 16 * 32, NE1 = 32 * 32;
    if (cudaMalloc(&ctx->d_ec, NEC * 4) || cudaMalloc(&ctx->d_ecavg, NAVG * 4) || cudaMalloc(&ctx->d_e1, NE1 * 4) ||
        cudaMalloc(&ctx->d_ctr, sizeof(DevCtr)) || cudaMalloc(&ctx->d_spec, SPEC_CELLS * sizeof(float4)) ||
        cudaMalloc(&ctx->d_coat, COAT_BINS * sizeof(float4))) {
        st_destroy(ctx);
        return ST_ERR_OOM;
    }
    cudaMemsetAsync(ctx->d_ctr, 0, sizeof(DevCtr), ctx->stream);
    {
        const std::vector<double> t = spectral_table();
        std::vector<float4> f(SPEC_CELLS);
        for (int i = 0; i < SPEC_CELLS; i++)
            f[i] = make_float4((float)t[4 * i], (float)t[4 * i + 1], (float)t[4 * i + 2], (float)t[4 * i + 3]);
        const std::vector<double> c = coat_bin_table();
        float4 cb[COAT_BINS];
        for (int k = 0; k < COAT_BINS; k++) cb[k] = make_float4((float)c[3 * k], (float)c[3 * k + 1], (float)c[3 * k + 2], 0.f);
        if (cudaMemcpy(ctx->d_spec, f.data(), SPEC_CELLS * sizeof(float4), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(ctx->d_coat, cb, sizeof(cb), cudaMemcpyHostToDevice) != cudaSuccess) {
            st_destroy(ctx);
            return ST_ERR_CUDA;
        }
    }
    if (launch_mf_tables(ctx->d_ec, ctx->d_ecavg, ctx->d_e1, ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        st_destroy(ctx);
        return ST_ERR_CUDA;
    }
    *out = ctx;
    return ST_OK;
}

int st_destroy(st_ctx* ctx) {
    if (!ctx) return ST_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_wave(ctx);
    ext_free(ctx->ext);
    if (ctx->has_code) scene_code_free(ctx->code);
    for (void* p : {(void*)ctx->d_prims, (void*)ctx->d_faces, (void*)ctx->d_envimg, (void*)ctx->d_envmap, (void*)ctx->d_skytab, (void*)ctx->d_views, (void*)ctx->d_envtex, (void*)ctx->d_sc,
                    (void*)ctx->d_mats, (void*)ctx->d_ec, (void*)ctx->d_ecavg,
                    (void*)ctx->d_e1, (void*)ctx->d_ctr, (void*)ctx->d_spec, (void*)ctx->d_coat})
        if (p) cudaFree(p);
    for (auto& pe : ctx->pending) { cudaEventDestroy(pe.a); cudaEventDestroy(pe.b); }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return ST_OK;
}

int st_set_scene(st_ctx* ctx, const char* cuda_src, const st_scene_desc* d, char* errbuf, size_t errlen) {
    if (!ctx) return ST_ERR_ARG;
    auto refuse = [&](int code, const std::string& m) {
        if (errbuf && errlen) { std::snprintf(errbuf, errlen, "%s", m.c_str()); }
        return fail(ctx, code, m);
    };
    if (ctx->in_flight) return refuse(ST_ERR_BUSY, "a trace is in flight: st_sync first");
    // a scene as code: the table may be empty (its primitives, when given, still bound the space sort and the step
    // cache and are what the optics trace folds)
    const uint32_t min_prims = cuda_src ? 0u : 1u;
    if (!d || (!d->prims && d->n_prims) || !d->materials) return refuse(ST_ERR_ARG, "no scene table");
    if (d->n_prims < min_prims || d->n_prims > ST_MAX_PRIMS) return refuse(ST_ERR_ARG, "n_prims out of range (1..256)");
    if (d->n_materials == 0 || d->n_materials > ST_MAX_MATERIALS) return refuse(ST_ERR_ARG, "n_materials out of range (1..256)");
    if (d->n_prims && d->prims[0].op != ST_OP_ITEM) return refuse(ST_ERR_ARG, "the first primitive must start an item (ST_OP_ITEM)");
    for (uint32_t i = 0; i < d->n_prims; i++) {
        if (d->prims[i].type > ST_PRIM_CYLINDER) return refuse(ST_ERR_ARG, "primitive " + std::to_string(i) + ": unknown type");
        if (d->prims[i].op > ST_OP_SUB) return refuse(ST_ERR_ARG, "primitive " + std::to_string(i) + ": unknown op");
        if (d->prims[i].material >= d->n_materials)
            return refuse(ST_ERR_ARG, "primitive " + std::to_string(i) + ": material out of range");
    }
    if (!(d->env_radius >= 0) || !(d->tolerance >= 0)) return refuse(ST_ERR_ARG, "negative radius or tolerance");
    std::vector<st_prim> prims(d->prims, d->prims + d->n_prims);
    std::vector<st_material> mats(d->materials, d->materials + d->n_materials);
    // THE SCENE'S CODE first: a source that does not compile leaves everything as it was (README.md:216-218)
    SceneCode code;
    if (cuda_src) {
        cudaSetDevice(ctx->device);
        std::string why;
        if (!scene_code_build(cuda_src, code, why)) return refuse(ST_ERR_COMPILE, why);
    }
    std::vector<float4> faces(ST_MAX_LIGHTS * FACE_F4 + ST_MAX_MATERIALS / 16, make_float4(0.f, 0.f, 0.f, 0.f));
    {
        std::string why;
        if (!light_faces(d, prims, faces, why)) {
            if (cuda_src) scene_code_free(code);
            return refuse(ST_ERR_ARG, why);
        }
    }
    cudaSetDevice(ctx->device);
    if (prims.size() > ctx->prims.size() || !ctx->d_prims) {
        if (ctx->d_prims) cudaFree(ctx->d_prims);
        ctx->d_prims = nullptr;
        CK(cudaMalloc(&ctx->d_prims, ST_MAX_PRIMS * sizeof(DPrim)), "cudaMalloc scene");
    }
    if (!ctx->d_mats) CK(cudaMalloc(&ctx->d_mats, ST_MAX_MATERIALS * sizeof(st_material)), "cudaMalloc materials");
    if (!ctx->d_faces) CK(cudaMalloc(&ctx->d_faces, faces.size() * sizeof(float4)), "cudaMalloc light faces");
    std::vector<DPrim> packed(prims.size());
    for (size_t i = 0; i < prims.size(); i++) packed[i] = pack_prim(prims[i]);
    {
        double lo[3] = {1e30, 1e30, 1e30}, hi[3] = {-1e30, -1e30, -1e30};
        bool any = false;
        for (const DPrim& q : packed) {
            if (!(q.a.w < 1e30f)) continue;                   // unbounded (a plane) or a bound-only distance
            const double c[3] = {q.a.x, q.a.y, q.a.z};
            for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], c[k] - q.a.w); hi[k] = std::max(hi[k], c[k] + q.a.w); }
            any = true;
        }
        ctx->grid_ok = any;
        for (int k = 0; k < 3; k++) {
            double pad = 1e-3 * (hi[k] - lo[k]) + 1e-6;
            ctx->grid_lo[k] = any ? (float)(lo[k] - pad) : 0.f;
            ctx->grid_hi[k] = any ? (float)(hi[k] + pad) : 1.f;
        }
    }
    CK(cudaMemcpyAsync(ctx->d_prims, packed.data(), packed.size() * sizeof(DPrim), cudaMemcpyHostToDevice, ctx->stream), "scene upload");
    CK(cudaMemcpyAsync(ctx->d_mats, mats.data(), mats.size() * sizeof(st_material), cudaMemcpyHostToDevice, ctx->stream), "scene upload");
    CK(cudaMemcpyAsync(ctx->d_faces, faces.data(), faces.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream), "scene upload");
    ctx->n_faces = d->lights ? d->n_lights : 0u;
    CK(cudaStreamSynchronize(ctx->stream), "scene upload");
    ctx->prims = std::move(prims);
    ctx->mats = std::move(mats);
    if (ctx->has_code) scene_code_free(ctx->code);
    ctx->code = code;
    ctx->has_code = cuda_src != nullptr;
    ctx->desc = *d;
    ctx->desc.prims = nullptr;
    ctx->desc.materials = nullptr;
    ctx->desc.lights = nullptr;
    ctx->has_scene = true;
    ctx->scene_gen++;
    invalidate_graph(ctx);
    return st_invalidate(ctx);
}

static int env_preset_ensure(st_ctx* ctx);
int st_set_params(st_ctx* ctx, const st_params* p, uint64_t* unknown_mask) {
    if (!ctx || !p) return ST_ERR_ARG;
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    if (unknown_mask) *unknown_mask = 0;
    if (p->width == 0 || p->height == 0 || (uint64_t)p->width * p->height > (1u << 26))
        return fail(ctx, ST_ERR_ARG, "picture size out of range");
    if (p->maxbounce == 0 || p->maxbounce > 64) return fail(ctx, ST_ERR_ARG, "maxbounce out of range (1..64)");
    if (p->maxiter == 0 || p->maxiter > 65535) return fail(ctx, ST_ERR_ARG, "maxiter out of range (1..65535)");
    if (!(p->stepscale > 0 && p->stepscale <= 1)) return fail(ctx, ST_ERR_ARG, "stepscale out of range (0, 1]");
    if (p->budget > 256) return fail(ctx, ST_ERR_ARG, "budget out of range (0..256)");
    if (p->samples_per_wave > 1024) return fail(ctx, ST_ERR_ARG, "samples_per_wave out of range (0..1024)");
    if (p->lt > 1) return fail(ctx, ST_ERR_ARG, "lt is 0 or 1");
    if (p->env_mode > ST_ENV_STUDIO) return fail(ctx, ST_ERR_ARG, "env_mode out of range (ST_ENV_*)");
    cudaSetDevice(ctx->device);
    bool resize = p->width != ctx->params.width || p->height != ctx->params.height ||
                  p->samples_per_wave != ctx->params.samples_per_wave || !ctx->has_params;
    ctx->params = *p;
    ctx->has_params = true;
    ctx->W = p->width; ctx->H = p->height; ctx->P = p->width * p->height;
    invalidate_graph(ctx);
    {
        int rc = env_preset_ensure(ctx);
        if (rc) return rc;
    }
    if (resize) {
        free_wave(ctx);
        int rc = ensure_wave(ctx);
        if (rc) return rc;
    }
    return st_invalidate(ctx);
}

// envSampling (envmap.js:215-260): each texel's weight its luminance (non-finite or negative: 0) plus a floor of
// 1e-3 of the mean (1 in a black environment: a uniform map), then the CDFs along each row and down the rows, and
// each texel's density per steradian, its share of the total times the texels a steradian
int st_env_map_tables(const float* lum, float* tex) {
    if (!lum || !tex) return ST_ERR_ARG;
    const int W = ENV_MW, H = ENV_MH, N = W * H;
    auto ok = [](float x) { return (x > 0.f && std::isfinite(x)) ? (double)x : 0.0; };
    double sum = 0.0;
    for (int i = 0; i < N; i++) sum += ok(lum[i]);
    const double mean = sum / N;
    const double floor_w = mean > 0.0 ? 1e-3 * mean : 1.0;
    std::vector<double> w(N);
    double total = 0.0;
    for (int i = 0; i < N; i++) { w[i] = ok(lum[i]) + floor_w; total += w[i]; }
    const double density = N / (4.0 * PI_D);
    double below = 0.0;
    for (int row = 0; row < H; row++) {
        double rowSum = 0.0;
        for (int x = 0; x < W; x++) rowSum += w[row * W + x];
        const double rowCdf = row == H - 1 ? 1.0 : (below + rowSum) / total;
        double along = 0.0;
        for (int x = 0; x < W; x++) {
            const int i = row * W + x;
            along += w[i];
            tex[4 * i] = x == W - 1 ? 1.f : (float)(along / rowSum);
            tex[4 * i + 1] = (float)(w[i] / total * density);
            tex[4 * i + 2] = (float)rowCdf;
            tex[4 * i + 3] = 0.f;
        }
        below += rowSum;
    }
    return ST_OK;
}

// THE MAP, baked on the GPU from the environment as it returns it (the image, or a preset), tabulated here
static int env_map_bake(st_ctx* ctx) {
    if (ctx->d_envmap) { cudaFree(ctx->d_envmap); ctx->d_envmap = nullptr; }
    Uni u = make_uni(ctx);
    float* d_lum = nullptr;
    CK(cudaMalloc(&d_lum, (size_t)ENV_MW * ENV_MH * sizeof(float)), "cudaMalloc environment bake");
    std::vector<float> lum((size_t)ENV_MW * ENV_MH);
    cudaError_t e = launch_env_bake(u, d_lum, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(lum.data(), d_lum, lum.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_lum);
    if (e != cudaSuccess) return fail(ctx, ST_ERR_CUDA, std::string("environment bake: ") + cudaGetErrorString(e));
    std::vector<float> tex(lum.size() * 4);
    st_env_map_tables(lum.data(), tex.data());
    CK(cudaMalloc(&ctx->d_envmap, tex.size() * sizeof(float)), "cudaMalloc environment map");
    CK(cudaMemcpyAsync(ctx->d_envmap, tex.data(), tex.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
       "environment map upload");
    CK(cudaStreamSynchronize(ctx->stream), "environment map upload");
    return ST_OK;
}
// a preset's map, made again when what it is baked from changes (no image: an image's map is its own)
static int env_preset_ensure(st_ctx* ctx) {
    const st_params& p = ctx->params;
    if (ctx->d_envimg) return ST_OK;
    if (p.env_mode == ST_ENV_ANALYTIC || p.env_mode > ST_ENV_STUDIO || p.env_uniform > 0.f) {
        if (!ctx->env_key.empty()) {
            if (ctx->d_envmap) { cudaFree(ctx->d_envmap); ctx->d_envmap = nullptr; }
            if (ctx->d_envtex) { cudaFree(ctx->d_envtex); ctx->d_envtex = nullptr; }
            ctx->env_key.clear();
        }
        return ST_OK;
    }
    if (!ctx->d_skytab) {
        const std::vector<double> t = sky_band_table();
        std::vector<float> f(t.begin(), t.end());
        CK(cudaMalloc(&ctx->d_skytab, f.size() * sizeof(float)), "cudaMalloc sky table");
        CK(cudaMemcpy(ctx->d_skytab, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice), "sky table upload");
    }
    const uint32_t tw = p.env_cache ? (p.env_cache_size == 1024u || p.env_cache_size == 4096u ? p.env_cache_size : 2048u)
                                    : 0u;
    const std::vector<float> key = {(float)p.env_mode, p.sun_elevation, p.sun_azimuth, p.sun_diameter, p.sun_outside,
                                    p.sky_turbidity, p.studio_illuminance, p.studio_top, p.studio_color[0],
                                    p.studio_color[1], p.studio_color[2], (float)p.sun_hint, (float)tw};
    if (key == ctx->env_key && ctx->d_envmap) return ST_OK;
    // the texture (envmap.js THE ENVIRONMENT IN A TEXTURE), baked from the preset itself, then the map from either
    if (ctx->d_envtex) { cudaFree(ctx->d_envtex); ctx->d_envtex = nullptr; }
    ctx->env_key.clear();
    if (tw) {
        const uint32_t th = tw / 2;
        CK(cudaMalloc(&ctx->d_envtex, (size_t)tw * th * sizeof(float4)), "cudaMalloc environment texture");
        Uni u = make_uni(ctx);                                   // no texture yet: the preset itself
        CK(launch_env_cache(u, ctx->d_envtex, tw, th, ctx->stream), "environment texture");
        ctx->env_tw = tw; ctx->env_th = th;
    }
    ctx->env_key = key;
    return env_map_bake(ctx);
}

int st_set_env_image(st_ctx* ctx, const float* rgb, uint32_t w, uint32_t h, float luminance, float turn_deg) {
    if (!ctx) return ST_ERR_ARG;
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    cudaSetDevice(ctx->device);
    if (!rgb) {                                           // back to the sun and sky (or the preset)
        if (ctx->d_envimg) cudaFree(ctx->d_envimg);
        if (ctx->d_envmap) cudaFree(ctx->d_envmap);
        ctx->d_envimg = ctx->d_envmap = nullptr;
        ctx->env_w = ctx->env_h = 0;
        ctx->env_key.clear();
        invalidate_graph(ctx);
        if (!ctx->has_params) return ST_OK;
        int rc = env_preset_ensure(ctx);
        return rc ? rc : st_invalidate(ctx);
    }
    if (w < 2 || h < 1 || w > 16384 || h > 8192) return fail(ctx, ST_ERR_ARG, "environment image size out of range");
    if (!(luminance >= 0.f) || !std::isfinite(turn_deg)) return fail(ctx, ST_ERR_ARG, "bad luminance or turn");
    std::vector<float4> px((size_t)w * h);
    for (size_t i = 0; i < px.size(); i++) {
        float c[3];
        for (int k = 0; k < 3; k++) c[k] = std::isfinite(rgb[3 * i + k]) ? rgb[3 * i + k] : 0.f;
        px[i] = make_float4(c[0], c[1], c[2], 0.f);
    }
    if (ctx->d_envimg && (size_t)ctx->env_w * ctx->env_h < px.size()) { cudaFree(ctx->d_envimg); ctx->d_envimg = nullptr; }
    if (!ctx->d_envimg) CK(cudaMalloc(&ctx->d_envimg, px.size() * sizeof(float4)), "cudaMalloc environment image");
    CK(cudaMemcpyAsync(ctx->d_envimg, px.data(), px.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream),
       "environment image upload");
    ctx->env_w = w; ctx->env_h = h;
    ctx->env_lum = luminance > 0.f ? luminance : 179.f;
    ctx->env_turn = turn_deg;
    ctx->env_key.clear();
    int rc = env_map_bake(ctx);
    if (rc) return rc;
    invalidate_graph(ctx);
    return ctx->has_params ? st_invalidate(ctx) : ST_OK;
}

int st_set_view(st_ctx* ctx, const st_view* v) { return st_set_views(ctx, v, 1); }

// the views rendered together (include/shadytracer.h st_set_views): the table the kernels read, the accumulation of
// each, the waves sized for all of them
int st_set_views(st_ctx* ctx, const st_view* views, uint32_t n) {
    if (!ctx || !views || n == 0 || n > ST_MAX_VIEWS) return ST_ERR_ARG;
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    cudaSetDevice(ctx->device);
    ctx->views.assign(views, views + n);
    ctx->view = views[0];
    ctx->has_view = true;
    if (n > 1) {
        std::vector<float4> t((size_t)n * VIEW_F4);
        for (uint32_t i = 0; i < n; i++) {
            const st_view& v = views[i];
            float camtype;                                        // its bits, as the kernels read them back
            std::memcpy(&camtype, &v.camtype, sizeof(float));
            t[i * VIEW_F4 + 0] = make_float4(v.cam_pos[0], v.cam_pos[1], v.cam_pos[2], camtype);
            t[i * VIEW_F4 + 1] = make_float4(v.right[0], v.right[1], v.right[2], v.fx);
            t[i * VIEW_F4 + 2] = make_float4(v.up[0], v.up[1], v.up[2], v.fy);
            t[i * VIEW_F4 + 3] = make_float4(v.fwd[0], v.fwd[1], v.fwd[2], v.lens_radius > 0.f ? v.lens_radius : 0.f);
            t[i * VIEW_F4 + 4] = make_float4(v.focus_distance, 0.f, 0.f, 0.f);
        }
        if (!ctx->d_views) CK(cudaMalloc(&ctx->d_views, (size_t)ST_MAX_VIEWS * VIEW_F4 * sizeof(float4)), "cudaMalloc views");
        CK(cudaMemcpy(ctx->d_views, t.data(), t.size() * sizeof(float4), cudaMemcpyHostToDevice), "views upload");
    }
    if (n != ctx->nv) {
        ctx->nv = n;
        if (ctx->has_params) {
            free_wave(ctx);
            int rc = ensure_wave(ctx);
            if (rc) return rc;
        }
    }
    invalidate_graph(ctx);
    return st_invalidate(ctx);
}

int st_invalidate(st_ctx* ctx) {
    if (!ctx) return ST_ERR_ARG;
    if (!ctx->d_acc) return ST_OK;
    cudaSetDevice(ctx->device);
    // stream-ordered: it takes effect after whatever is queued, so it needs no st_sync (RT.invalidate may be called
    // between queued samples); the sample index restarts, the statistics keep accumulating
    CK(cudaMemsetAsync(ctx->d_acc, 0, (size_t)ctx->acc_views * ctx->P * sizeof(Acc4), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_mom, 0, (size_t)ctx->acc_views * ctx->P * sizeof(double2), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_frame, 0, (size_t)ctx->slot_cap * sizeof(float4), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_splat, 0, (size_t)ctx->P * sizeof(float4), ctx->stream), "memset");
    CK(cudaMemsetAsync(ctx->d_ltcount, 0, (size_t)ctx->P * sizeof(uint32_t), ctx->stream), "memset");
    CK(cudaMemsetAsync(&ctx->d_ctr->sample, 0, sizeof(uint32_t), ctx->stream), "memset");
    CK(sppm_lt_reset(ctx_ext(ctx).sppm, ctx->stream), "memset");     // the emission map starts over uniform
    CK(emit_reset(ctx), "emitter list reset");                         // and the emitters' discovery
    ctx->samples = 0;
    return ST_OK;
}

// THE STEP CACHE'S GRID (raytrace_main.js:984-1004 setStepCacheBox, :1049-1080 the fill): the bounded primitives'
// box cut into about step_cache_cells million cubes, filled on the stream when the scene or the cells change
static int sc_ensure(st_ctx* ctx) {
    const st_params& p = ctx->params;
    if (!p.step_cache || !ctx->grid_ok) {
        if (ctx->sc_live) { ctx->sc_live = false; invalidate_graph(ctx); }
        return ST_OK;
    }
    const float cells = std::min(16.f, std::max(0.25f, p.step_cache_cells > 0.f ? p.step_cache_cells : 4.f)) * 1e6f;
    if (ctx->sc_live && ctx->sc_scene == ctx->scene_gen && ctx->sc_cells == cells) return ST_OK;
    double size[3], vol = 1.0;
    for (int k = 0; k < 3; k++) { size[k] = std::max((double)ctx->grid_hi[k] - ctx->grid_lo[k], 1e-6); vol *= size[k]; }
    const double cs = std::cbrt(vol / cells);
    size_t n = 1;
    for (int k = 0; k < 3; k++) {
        ctx->sc_dims[k] = (uint32_t)std::max(1.0, std::ceil(size[k] / cs));
        n *= ctx->sc_dims[k];
        ctx->sc_lo[k] = ctx->grid_lo[k];
    }
    ctx->sc_cs = (float)cs;
    if (n > ctx->sc_cap) {
        if (ctx->d_sc) cudaFree(ctx->d_sc);
        ctx->d_sc = nullptr;
        ctx->sc_cap = 0;
        CK(cudaMalloc(&ctx->d_sc, n * sizeof(float)), "cudaMalloc step cache");
        ctx->sc_cap = n;
    }
    CK(launch_sc_fill(ctx->d_prims, (uint32_t)ctx->prims.size(), mk(ctx->sc_lo[0], ctx->sc_lo[1], ctx->sc_lo[2]),
                      ctx->sc_cs, ctx->sc_dims[0], ctx->sc_dims[1], ctx->sc_dims[2], ctx->d_sc, ctx->sms, ctx->stream,
                      ctx->has_code ? &ctx->code : nullptr),
       "step cache fill");
    ctx->sc_live = true;
    ctx->sc_scene = ctx->scene_gen;
    ctx->sc_cells = cells;
    invalidate_graph(ctx);
    return ST_OK;
}

int st_step_async(st_ctx* ctx, int n) {
    if (!ctx || n < 0) return ST_ERR_ARG;
    if (!ctx->has_scene || !ctx->has_params || !ctx->has_view)
        return fail(ctx, ST_ERR_STATE, "set a scene, the settings and the view first");
    if (ctx->nv > 1 && ctx->params.lt)
        return fail(ctx, ST_ERR_ARG, "light tracing connects to one camera: one view with st_params.lt");
    cudaSetDevice(ctx->device);
    int rc = ensure_wave(ctx);
    if (rc) return rc;
    rc = sc_ensure(ctx);
    if (rc) return rc;
    uint32_t left = (uint32_t)n;
    const bool emitters = has_emitters(ctx);
    while (left > 0) {
        uint32_t w = std::min(left, ctx->spw);
        // an emitter scene's first two waves are EMIT_EPOCH samples each: the list is built between waves (samples
        // in a wave run together), so it is found after the first and aimed at from the second on
        if (emitters && ctx->samples < 2 * EMIT_EPOCH) w = std::min(w, EMIT_EPOCH);
        rc = run_wave(ctx, w);
        if (rc) return rc;
        left -= w;
    }
    ctx->in_flight = n > 0;
    return ST_OK;
}

int st_sync(st_ctx* ctx, int timeout_ms) {
    if (!ctx) return ST_ERR_ARG;
    cudaSetDevice(ctx->device);
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(ctx->stream);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) { ctx->in_flight = false; return cuda_fail(ctx, e, "trace"); }
        if (timeout_ms >= 0) {
            double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            if (ms > timeout_ms) return fail(ctx, ST_ERR_TIMEOUT, "the trace did not finish in time");
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    ctx->in_flight = false;
    if (ctx->timing) collect_times(ctx);
    DevCtr c;
    CK(cudaMemcpy(&c, ctx->d_ctr, sizeof(DevCtr), cudaMemcpyDeviceToHost), "counters");
    if (c.errflag) {
        // reported once: the flag is cleared, so the next trace that finishes its waits reports success
        CK(cudaMemsetAsync(&ctx->d_ctr->errflag, 0, sizeof(uint32_t), ctx->stream), "counters");
        CK(cudaStreamSynchronize(ctx->stream), "counters");
        return fail(ctx, ST_ERR_TIMEOUT, "a kernel's wait for its scene table ran out of iterations");
    }
    return ST_OK;
}

// THE DEVICE-SIDE WAITS' LIMIT: every kernel that stages a table into shared memory waits for its copy at most this
// many times (0: the default, 2^24) before it flags ST_ERR_TIMEOUT and returns; arm_only 1 arms the waits and issues
// no copy, so each runs out at its limit with nothing in flight -- the failure path, exercised without a fault
int st_set_wait_limit(st_ctx* ctx, uint32_t iterations, int arm_only) {
    if (!ctx) return ST_ERR_ARG;
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    cudaSetDevice(ctx->device);
    ctx->wait_limit = iterations;
    ctx->wait_arm_only = arm_only ? 1u : 0u;
    CK(push_wait(ctx), "wait limit");
    return ST_OK;
}

int st_step(st_ctx* ctx, int n) {
    int rc = st_step_async(ctx, n);
    if (rc) return rc;
    return st_sync(ctx, -1);
}

// THE CHECKPOINT: a header (magic, version, width, height, views, samples), then the accumulation, the moments, the
// splat buffer and the connection counts as the device holds them
struct CkHeader { uint32_t magic, version, W, H, nv, samples, pad0, pad1; };
static constexpr uint32_t CK_MAGIC = 0x4B435453u;             // "STCK"
static size_t ck_bytes(const st_ctx* ctx) {
    return sizeof(CkHeader) + (size_t)ctx->acc_views * ctx->P * (sizeof(Acc4) + sizeof(double2)) +
           (size_t)ctx->P * (sizeof(float4) + sizeof(uint32_t));
}
int st_checkpoint_size(st_ctx* ctx, size_t* bytes) {
    if (!ctx || !bytes) return ST_ERR_ARG;
    if (!ctx->d_acc) return fail(ctx, ST_ERR_STATE, "nothing rendered yet");
    *bytes = ck_bytes(ctx);
    return ST_OK;
}
int st_checkpoint_save(st_ctx* ctx, void* out, size_t bytes) {
    if (!ctx || !out) return ST_ERR_ARG;
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    if (!ctx->d_acc) return fail(ctx, ST_ERR_STATE, "nothing rendered yet");
    if (bytes < ck_bytes(ctx)) return fail(ctx, ST_ERR_ARG, "the checkpoint's buffer is too small");
    cudaSetDevice(ctx->device);
    unsigned char* o = static_cast<unsigned char*>(out);
    const CkHeader h{CK_MAGIC, 1u, ctx->W, ctx->H, ctx->acc_views, (uint32_t)ctx->samples, 0u, 0u};
    std::memcpy(o, &h, sizeof(h));
    o += sizeof(h);
    const size_t na = (size_t)ctx->acc_views * ctx->P;
    CK(cudaMemcpyAsync(o, ctx->d_acc, na * sizeof(Acc4), cudaMemcpyDeviceToHost, ctx->stream), "checkpoint");
    o += na * sizeof(Acc4);
    CK(cudaMemcpyAsync(o, ctx->d_mom, na * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream), "checkpoint");
    o += na * sizeof(double2);
    CK(cudaMemcpyAsync(o, ctx->d_splat, (size_t)ctx->P * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream), "checkpoint");
    o += (size_t)ctx->P * sizeof(float4);
    CK(cudaMemcpyAsync(o, ctx->d_ltcount, (size_t)ctx->P * 4, cudaMemcpyDeviceToHost, ctx->stream), "checkpoint");
    CK(cudaStreamSynchronize(ctx->stream), "checkpoint");
    return ST_OK;
}
int st_checkpoint_load(st_ctx* ctx, const void* in, size_t bytes) {
    if (!ctx || !in || bytes < sizeof(CkHeader)) return ST_ERR_ARG;
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    if (!ctx->has_scene || !ctx->has_params) return fail(ctx, ST_ERR_STATE, "set the scene and the settings first");
    CkHeader h;
    std::memcpy(&h, in, sizeof(h));
    if (h.magic != CK_MAGIC || h.version != 1u) return fail(ctx, ST_ERR_ARG, "not a checkpoint");
    if (h.W != ctx->W || h.H != ctx->H || h.nv != std::max(ctx->nv, 1u))
        return fail(ctx, ST_ERR_ARG, "the checkpoint is of another picture (its width, height or views)");
    cudaSetDevice(ctx->device);
    int rc = ensure_wave(ctx);
    if (rc) return rc;
    if (bytes < ck_bytes(ctx)) return fail(ctx, ST_ERR_ARG, "the checkpoint is short");
    const unsigned char* p = static_cast<const unsigned char*>(in) + sizeof(h);
    const size_t na = (size_t)ctx->acc_views * ctx->P;
    CK(cudaMemcpyAsync(ctx->d_acc, p, na * sizeof(Acc4), cudaMemcpyHostToDevice, ctx->stream), "resume");
    p += na * sizeof(Acc4);
    CK(cudaMemcpyAsync(ctx->d_mom, p, na * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream), "resume");
    p += na * sizeof(double2);
    CK(cudaMemcpyAsync(ctx->d_splat, p, (size_t)ctx->P * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream), "resume");
    p += (size_t)ctx->P * sizeof(float4);
    CK(cudaMemcpyAsync(ctx->d_ltcount, p, (size_t)ctx->P * 4, cudaMemcpyHostToDevice, ctx->stream), "resume");
    CK(cudaMemcpyAsync(&ctx->d_ctr->sample, &h.samples, sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream), "resume");
    CK(cudaStreamSynchronize(ctx->stream), "resume");
    ctx->samples = h.samples;
    return ST_OK;
}

int st_read_accum(st_ctx* ctx, double* rgb, double* V, double* S, uint32_t* count) {
    return st_read_accum_view(ctx, 0, rgb, V, S, count);
}
int st_read_accum_view(st_ctx* ctx, uint32_t view, double* rgb, double* V, double* S, uint32_t* count) {
    if (!ctx) return ST_ERR_ARG;
    if (!ctx->d_acc) return fail(ctx, ST_ERR_STATE, "nothing rendered yet");
    if (view >= ctx->acc_views) return fail(ctx, ST_ERR_ARG, "no such view");
    if (ctx->in_flight) { int rc = st_sync(ctx, -1); if (rc) return rc; }
    cudaSetDevice(ctx->device);
    std::vector<Acc4> acc(ctx->P);
    std::vector<double2> mom(ctx->P);
    const size_t off = (size_t)view * ctx->P;
    CK(cudaMemcpyAsync(acc.data(), ctx->d_acc + off, acc.size() * sizeof(Acc4), cudaMemcpyDeviceToHost, ctx->stream),
       "readback");
    CK(cudaMemcpyAsync(mom.data(), ctx->d_mom + off, mom.size() * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream),
       "readback");
    CK(cudaStreamSynchronize(ctx->stream), "readback");
    for (uint32_t i = 0; i < ctx->P; i++) {
        if (rgb) { rgb[3 * i] = acc[i].x; rgb[3 * i + 1] = acc[i].y; rgb[3 * i + 2] = acc[i].z; }
        if (count) count[i] = (uint32_t)acc[i].w;
        if (V) V[i] = mom[i].x;
        if (S) S[i] = mom[i].y;
    }
    return ST_OK;
}

// light tracing's connections per pixel since the last invalidate (include/shadytracer.h st_lt_counts)
int st_lt_counts(st_ctx* ctx, uint32_t* counts) {
    if (!ctx || !counts) return ST_ERR_ARG;
    if (!ctx->d_ltcount) return fail(ctx, ST_ERR_STATE, "nothing rendered yet");
    if (ctx->in_flight) { int rc = st_sync(ctx, -1); if (rc) return rc; }
    cudaSetDevice(ctx->device);
    CK(cudaMemcpyAsync(counts, ctx->d_ltcount, (size_t)ctx->P * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream),
       "readback");
    CK(cudaStreamSynchronize(ctx->stream), "readback");
    return ST_OK;
}

int st_image_stats(st_ctx* ctx, st_image_stats_t* out) {
    if (!ctx || !out) return ST_ERR_ARG;
    std::vector<double> rgb(3 * (size_t)ctx->P), V(ctx->P), S(ctx->P);
    std::vector<uint32_t> cnt(ctx->P);
    int rc = st_read_accum(ctx, rgb.data(), V.data(), S.data(), cnt.data());
    if (rc) return rc;
    std::vector<double> L;
    double sum = 0, rel = 0;
    uint32_t nrel = 0;
    for (uint32_t i = 0; i < ctx->P; i++) {
        if (!cnt[i]) continue;
        double y = rgb[3 * i] * 0.2126 + rgb[3 * i + 1] * 0.7152 + rgb[3 * i + 2] * 0.0722;
        L.push_back(y);
        sum += y;
        if (y > 0 && S[i] > 0 && S[i] < 1) { rel += std::sqrt(S[i] * V[i] / (1 - S[i])) / y; nrel++; }
    }
    *out = st_image_stats_t{};
    out->sampled = (uint32_t)L.size();
    out->samples = ctx->samples;
    if (L.empty()) return ST_OK;
    out->mean_luma = sum / L.size();
    std::sort(L.begin(), L.end());
    out->median_luma = L[L.size() / 2];
    size_t cut = L.size() / 100, a = cut, b = L.size() - cut;
    double ts = 0;
    for (size_t i = a; i < b; i++) ts += L[i];
    out->trimmed_mean_luma = b > a ? ts / (b - a) : out->mean_luma;
    out->mean_rel_se = nrel ? rel / nrel : 0;
    return ST_OK;
}

int st_read_counters(st_ctx* ctx, st_counters_t* out) {
    if (!ctx || !out) return ST_ERR_ARG;
    if (ctx->in_flight) { int rc = st_sync(ctx, -1); if (rc) return rc; }
    cudaSetDevice(ctx->device);
    DevCtr c;
    CK(cudaMemcpy(&c, ctx->d_ctr, sizeof(DevCtr), cudaMemcpyDeviceToHost), "counters");
    out->paths = c.paths; out->segments = c.segments; out->march_steps = c.march_steps;
    out->shadow_rays = c.shadow_rays; out->shadow_steps = c.shadow_steps;
    out->nonfinite = c.nonfinite; out->flushed = c.flushed; out->shadowcut = c.shadowcut;
    out->samples = ctx->samples;
    out->launches = ctx->launches;
    for (int k = 0; k < 8; k++) { out->prim_evals[k] = c.work[WC_EVAL + k]; out->prim_warp_evals[k] = c.work[WC_WEVAL + k]; }
    out->bound_tests = c.work[WC_TEST];
    out->bound_warp_tests = c.work[WC_WTEST];
    for (int k = 0; k < 4; k++) out->op_evals[k] = c.work[WC_OP + k];
    return ST_OK;
}

int st_eval_sdf(st_ctx* ctx, const float* pts, uint32_t n, float* out) {
    if (!ctx || (n && (!pts || !out))) return ST_ERR_ARG;
    if (!ctx->has_scene) return fail(ctx, ST_ERR_STATE, "set a scene first");
    if (ctx->in_flight) { int rc = st_sync(ctx, -1); if (rc) return rc; }
    if (n == 0) return ST_OK;
    cudaSetDevice(ctx->device);
    float* dp = nullptr;
    CK(cudaMalloc(&dp, (size_t)n * 16), "cudaMalloc points");
    cudaError_t e = cudaMemcpyAsync(dp, pts, (size_t)n * 12, cudaMemcpyHostToDevice, ctx->stream);
    if (!e) e = launch_eval_sdf(ctx->d_prims, (uint32_t)ctx->prims.size(), dp, n, dp + 3 * (size_t)n, ctx->stream,
                                ctx->has_code ? &ctx->code : nullptr);
    if (!e) e = cudaMemcpyAsync(out, dp + 3 * (size_t)n, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (!e) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dp);
    CK(e, "scene distance");
    return ST_OK;
}

int st_enable_kernel_times(st_ctx* ctx, int on) {
    if (!ctx) return ST_ERR_ARG;
    ctx->timing = on != 0;
    ctx->count_work = (on & 2) != 0;
    return ST_OK;
}

int st_kernel_times(st_ctx* ctx, st_kernel_time* out, int max, int* n_out) {
    if (!ctx || (!out && max > 0)) return ST_ERR_ARG;
    if (ctx->in_flight) { int rc = st_sync(ctx, -1); if (rc) return rc; }
    collect_times(ctx);
    int n = std::min<int>(max, (int)ctx->ktimes.size());
    for (int i = 0; i < n; i++) {
        std::memset(out[i].name, 0, sizeof(out[i].name));
        std::snprintf(out[i].name, sizeof(out[i].name), "%s", ctx->ktimes[i].name.c_str());
        out[i].launches = ctx->ktimes[i].launches;
        out[i].ms = ctx->ktimes[i].ms;
    }
    if (n_out) *n_out = (int)ctx->ktimes.size();
    return ST_OK;
}

int st_reset_kernel_times(st_ctx* ctx) {
    if (!ctx) return ST_ERR_ARG;
    if (ctx->in_flight) { int rc = st_sync(ctx, -1); if (rc) return rc; }
    collect_times(ctx);
    ctx->ktimes.clear();
    return ST_OK;
}

int st_mf_tables(st_ctx* ctx, float* ec, float* ecavg, float* e1) {
    if (!ctx || !ec || !ecavg || !e1) return ST_ERR_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaMemcpy(ec, ctx->d_ec, 16 * 32 * 32 * 4, cudaMemcpyDeviceToHost), "tables");
    CK(cudaMemcpy(ecavg, ctx->d_ecavg, 16 * 32 * 4, cudaMemcpyDeviceToHost), "tables");
    CK(cudaMemcpy(e1, ctx->d_e1, 32 * 32 * 4, cudaMemcpyDeviceToHost), "tables");
    return ST_OK;
}

// the struct sizes this library was built with, for the host's bindings to check theirs against
// THE AUTOTUNER: each (queue tile, march chunk) pair of the candidates timed over `samples` samples of the scene, view
// and settings in force (CUDA events on the context's stream, each after one untimed sample that records its graph),
// the fastest kept for the renders that follow; the accumulation is cleared after
int st_autotune(st_ctx* ctx, int samples, st_tune* out) {
    if (!ctx || samples <= 0) return ST_ERR_ARG;
    if (!ctx->has_scene || !ctx->has_params || !ctx->has_view)
        return fail(ctx, ST_ERR_STATE, "set a scene, the settings and the view first");
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    static const uint32_t claims[] = {32u, 64u, 128u};
    static const uint32_t chunks[] = {24u, 32u, 48u, 64u, 96u, 160u};
    cudaSetDevice(ctx->device);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "event");
    CK(cudaEventCreate(&e1), "event");
    float best = 1e30f, base = 0.f;
    uint32_t bc = CLAIM, bk = MARCH_CHUNK;
    int rc = ST_OK;
    // one candidate's time for `samples` samples, its graph recorded and caches warm first
    auto time_it = [&](uint32_t cl, uint32_t ch, float& ms) -> int {
        ctx->tune_claim = cl;
        ctx->tune_chunk = ch;
        invalidate_graph(ctx);
        int r = st_step(ctx, 1);
        if (r) return r;
        cudaEventRecord(e0, ctx->stream);
        if ((r = st_step_async(ctx, samples))) return r;
        cudaEventRecord(e1, ctx->stream);
        if ((r = st_sync(ctx, -1))) return r;
        cudaEventElapsedTime(&ms, e0, e1);
        return ST_OK;
    };
    struct Cand { uint32_t cl, ch; float ms; };
    std::vector<Cand> cands;
    for (uint32_t cl : claims) {
        for (uint32_t ch : chunks) {
            float ms = 0.f;
            if ((rc = time_it(cl, ch, ms))) break;
            cands.push_back({cl, ch, ms});
            if (cl == CLAIM && ch == MARCH_CHUNK) base = ms;
        }
        if (rc) break;
    }
    // the three fastest and the defaults timed twice more, interleaved, each kept at its best: one pass's noise (a few
    // per cent at a sample or two of a large picture) picks no candidate on its own
    if (!rc) {
        std::sort(cands.begin(), cands.end(), [](const Cand& x, const Cand& y) { return x.ms < y.ms; });
        std::vector<Cand> top(cands.begin(), cands.begin() + std::min<size_t>(3, cands.size()));
        bool has_default = false;
        for (const Cand& c : top) has_default = has_default || (c.cl == CLAIM && c.ch == MARCH_CHUNK);
        if (!has_default) top.push_back({CLAIM, MARCH_CHUNK, base});
        for (int pass = 0; pass < 2 && !rc; pass++)
            for (Cand& c : top) {
                float ms = 0.f;
                if ((rc = time_it(c.cl, c.ch, ms))) break;
                c.ms = std::min(c.ms, ms);
            }
        for (const Cand& c : top) {
            if (c.cl == CLAIM && c.ch == MARCH_CHUNK) base = c.ms;
            if (c.ms < best) { best = c.ms; bc = c.cl; bk = c.ch; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->tune_claim = rc ? 0u : bc;
    ctx->tune_chunk = rc ? 0u : bk;
    invalidate_graph(ctx);
    if (rc) return rc;
    if (out) { out->claim = bc; out->chunk = bk; out->ms = best; out->ms_default = base; }
    return st_invalidate(ctx);
}

int st_set_tune(st_ctx* ctx, const st_tune* t) {
    if (!ctx || !t) return ST_ERR_ARG;
    if (ctx->in_flight) return fail(ctx, ST_ERR_BUSY, "a trace is in flight: st_sync first");
    if (t->claim > 1024u || (t->chunk && t->chunk < 4u) || t->chunk > 4096u)
        return fail(ctx, ST_ERR_ARG, "tune out of range (claim <= 1024, chunk 4..4096, 0 the defaults)");
    ctx->tune_claim = t->claim;
    ctx->tune_chunk = t->chunk;
    invalidate_graph(ctx);
    return ST_OK;
}

int st_scene_code_info(st_ctx* ctx, int* is_code, double* compile_ms, uint64_t* cubin_bytes) {
    if (!ctx) return ST_ERR_ARG;
    if (is_code) *is_code = ctx->has_code ? 1 : 0;
    if (compile_ms) *compile_ms = ctx->has_code ? ctx->code.compile_ms : 0.0;
    if (cubin_bytes) *cubin_bytes = ctx->has_code ? (uint64_t)ctx->code.cubin_bytes : 0u;
    return ST_OK;
}

int st_struct_sizes(uint32_t* out, int max) {
    const uint32_t s[] = {(uint32_t)sizeof(st_prim), (uint32_t)sizeof(st_material), (uint32_t)sizeof(st_scene_desc),
                          (uint32_t)sizeof(st_params), (uint32_t)sizeof(st_view), (uint32_t)sizeof(st_counters_t),
                          (uint32_t)sizeof(st_image_stats_t), (uint32_t)sizeof(st_kernel_time),
                          (uint32_t)sizeof(st_sppm_stats), (uint32_t)sizeof(st_optics_source),
                          (uint32_t)sizeof(st_optics_far), (uint32_t)sizeof(st_optics_batch),
                          (uint32_t)sizeof(st_optics_totals), (uint32_t)sizeof(st_mlp_stats),
                          (uint32_t)sizeof(st_light), (uint32_t)sizeof(st_optics_detail), (uint32_t)sizeof(st_tune)};
    int n = (int)(sizeof(s) / sizeof(s[0]));
    for (int i = 0; i < n && i < max; i++) out[i] = s[i];
    return n;
}

// the context's stream, for a host that times or orders its own work against the library's (cudaStream_t)
void* st_stream(st_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

}  // extern "C"

// the extension units' access to the context (st_ext.h)
StExt& ctx_ext(st_ctx* ctx) { return ctx->ext; }
// the learned proposal's hash-grid box: the primitives' bounds as the space sort has them, a cube of their longest
// side from their low corner; a scene of unbounded primitives only, a 50 m cube about the origin
void guide_box(st_ctx* ctx, f3& lo, float& inv_ext) {
    if (!ctx->grid_ok) { lo = mk(-25.f); inv_ext = 1.f / 50.f; return; }
    lo = mk(ctx->grid_lo[0], ctx->grid_lo[1], ctx->grid_lo[2]);
    const float ext = std::max(ctx->grid_hi[0] - ctx->grid_lo[0],
                               std::max(ctx->grid_hi[1] - ctx->grid_lo[1], ctx->grid_hi[2] - ctx->grid_lo[2]));
    inv_ext = 1.f / std::max(ext, 1e-6f);
}
cudaStream_t ctx_stream(st_ctx* ctx) { return ctx->stream; }
int ctx_device(st_ctx* ctx) { return ctx->device; }
int ctx_sms(st_ctx* ctx) { return ctx->sms; }
void ctx_set_error(st_ctx* ctx, const std::string& m) { ctx->err = m; }
const DPrim* ctx_d_prims(st_ctx* ctx) { return ctx->d_prims; }
const st_material* ctx_d_mats(st_ctx* ctx) { return ctx->d_mats; }
uint32_t ctx_n_prims(st_ctx* ctx) { return (uint32_t)ctx->prims.size(); }
uint32_t ctx_n_mats(st_ctx* ctx) { return (uint32_t)ctx->mats.size(); }
const st_scene_desc& ctx_desc(st_ctx* ctx) { return ctx->desc; }
bool ctx_has_scene(st_ctx* ctx) { return ctx->has_scene; }
uint64_t ctx_scene_gen(st_ctx* ctx) { return ctx->scene_gen; }
DevCtr* ctx_counters(st_ctx* ctx) { return ctx->d_ctr; }
MfTab ctx_tab(st_ctx* ctx) { return MfTab{ctx->d_ec, ctx->d_ecavg, ctx->d_e1, ctx->d_coat}; }
const float4* ctx_spec(st_ctx* ctx) { return ctx->d_spec; }
