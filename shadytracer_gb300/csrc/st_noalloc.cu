// st_noalloc.cu -- st_render_noalloc: a small render that allocates no device memory.
//
// WHO NEEDS IT. A host that may not call cudaMalloc at the moment it wants a picture: one running under a device
// memory budget fixed when it started (a plugin inside an application that owns the GPU's memory), one on a
// real-time thread where an allocation's unbounded latency is not allowed, or one whose allocations would be
// caught up in a stream capture it does not control. The regular path (st_create, st_step) allocates the wave's
// buffers when the picture's size is set; this one takes every scratch buffer from a single array compiled into the
// library, so it allocates nothing, ever: no cudaMalloc, no cudaFree, no allocating library call.
//
// WHAT IT COSTS AND ITS LIMIT. The array is ST_NOALLOC_SCRATCH_BYTES (8 MiB) of device memory on every GPU that loads
// the library, held until the process exits. It holds one sample's wave for a picture of at most
// ST_NOALLOC_MAX_PIXELS (128 x 128) pixels, the scene's tables (at most 256 primitives and 256 materials) and the
// microfacet albedo tables; a larger request is refused with ST_ERR_ARG and a message, never truncated.
//
// SHARED STATE. Every call uses the same array; it keeps the last call's contents, and each call clears what must
// start at zero (the accumulation, the moments, the frame, the counters) before it renders. Calls that overlap on
// the GPU -- from two host threads at once, for one device -- race on the array and give wrong pictures; a caller
// serialises them. The kernels are the regular path's own (st_render.cu), launched on the device's legacy default
// stream, so the picture equals st_step's for the same scene, settings, camera and samples.
//
// SET-UP. The first call on a device, with that device current, takes the array's device address with
// cudaGetSymbolAddress and builds the albedo tables in it; make that first call before any stream capture.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "st_spectral.h"
#include "st_internal.h"

using namespace st;

#define ST_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[ST_NOALLOC_SCRATCH_BYTES];

namespace {
const double PI_D = 3.14159265358979323846;

struct Layout {
    size_t pos, dir, beta, rad, meta, ray0, ray1, hit, hitd, hsurf, so[2], sd[2], sr[2], ss[2], frame, acc, mom, cnt, ctr,
        ec, ecavg, e1, spec, lam, prims, mats, end;
};
// the array carved for P paths a wave (one sample), each buffer 256-byte aligned: first what does not depend on the
// picture's size (the albedo tables, built once, the scene's tables, the counters), then the wave's buffers
Layout layout(size_t P) {
    Layout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o += (bytes + 255) & ~size_t(255); return at; };
    L.ec = take(16 * 32 * 32 * 4); L.ecavg = take(16 * 32 * 4); L.e1 = take(32 * 32 * 4);
    L.spec = take(SPEC_CELLS * sizeof(float4));
    L.prims = take(ST_MAX_PRIMS * sizeof(DPrim)); L.mats = take(ST_MAX_MATERIALS * sizeof(st_material));
    L.ctr = take(sizeof(DevCtr));
    const size_t SS = 2 * P;                                   // a shadow side: new rays and continuations
    L.pos = take(P * 16); L.dir = take(P * 16); L.beta = take(P * 16); L.rad = take(P * 16); L.meta = take(P * 16);
    L.lam = take(P * 4);
    L.ray0 = take(P * 4); L.ray1 = take(P * 4); L.hit = take(P * 4); L.hitd = take(P * 4);
    L.hsurf = take(P * 16);
    for (int k = 0; k < 2; k++) {
        L.so[k] = take(SS * 16); L.sd[k] = take(SS * 16); L.sr[k] = take(SS * 16); L.ss[k] = take(SS * 4);
    }
    L.frame = take(P * 16); L.acc = take(P * sizeof(Acc4)); L.mom = take(P * 16); L.cnt = take(P * 4);
    L.end = o;
    return L;
}

std::mutex g_setup_mutex;
unsigned char* g_base[ST_NOALLOC_MAX_DEVICES] = {};

// the counts as the caller reads them: the FP64 accumulation's sample count word, as u32
__global__ void k_counts(const Acc4* acc, uint32_t* cnt, uint32_t P) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < P) cnt[i] = (uint32_t)acc[i].w;
}

// a primitive as the kernels read it: st_capi.cu's packing, restated here so this file changes nothing there
DPrim pack(const st_prim& p) {
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

// the uniforms, derived on the host in double precision as st_capi.cu's make_uni does
Uni uniforms(const st_scene_desc& s, const st_params& p, const st_view& v, uint32_t n_prims, uint32_t n_mats) {
    Uni u{};
    u.W = p.width; u.H = p.height; u.P = p.width * p.height;
    const double N = double(u.W) * double(u.H);
    u.tilesX = std::max<uint32_t>(1, (uint32_t)std::llround(std::sqrt(N * (double(u.W) / std::max<double>(1, u.H)))));
    u.tilesY = std::max<uint32_t>(1, (uint32_t)std::ceil(N / u.tilesX));
    u.invTX = float(1.0 / u.tilesX);
    u.invTY = float(1.0 / u.tilesY);
    u.maxbounce = p.maxbounce; u.maxiter = p.maxiter; u.nee = p.nee; u.rr = p.rr;
    u.budget = p.budget ? p.budget : std::max(2u, p.maxbounce + 1 + (p.maxiter + 31) / 32);
    u.stepscale = p.stepscale;
    double tol = p.eps > 0 ? p.eps : (s.tolerance > 0 ? s.tolerance : 1e-3);
    double R = s.env_radius > 0 ? s.env_radius : 400.0;
    u.tol = (float)tol; u.envR = (float)R; u.envR2 = (float)(R * R);
    u.cam = mk(v.cam_pos[0], v.cam_pos[1], v.cam_pos[2]);
    u.right = mk(v.right[0], v.right[1], v.right[2]);
    u.up = mk(v.up[0], v.up[1], v.up[2]);
    u.fwd = mk(v.fwd[0], v.fwd[1], v.fwd[2]);
    u.fx = v.fx; u.fy = v.fy; u.camtype = v.camtype;
    u.lens_r = v.lens_radius > 0.f ? v.lens_radius : 0.f;
    u.lens_f = v.focus_distance;
    double half = std::max((double)p.sun_diameter, 1e-3) * PI_D / 360.0;
    double sh = std::sin(half / 2), omc = 2 * sh * sh, sin2 = std::sin(half) * std::sin(half);
    double disc = (double)p.sun_illuminance / (PI_D * sin2);
    const double raw[3] = {1.0, 0.96, 0.9};
    double y = raw[0] * 0.2126 + raw[1] * 0.7152 + raw[2] * 0.0722;
    int sun_on = (p.sun_hint != 0 && p.sun_elevation * PI_D / 180.0 + half > 0 && !(p.env_uniform > 0)) ? 1 : 0;
    double e = p.sun_elevation * PI_D / 180.0, az = p.sun_azimuth * PI_D / 180.0;
    u.sun_dir = mk((float)(std::cos(e) * std::sin(az)), (float)(std::cos(e) * std::cos(az)), (float)std::sin(e));
    u.sun_sin2 = (float)sin2; u.sun_omc = (float)omc; u.sun_omega = (float)(2 * PI_D * omc);
    u.pick = (float)((sun_on && p.env_sun_gain > 0) ? p.nee_sun_pick : 0.0);
    u.sun_on = sun_on;
    u.disc = mk((float)(disc * raw[0] / y), (float)(disc * raw[1] / y), (float)(disc * raw[2] / y));
    u.sky = p.sky_luminance; u.ground = p.ground_luminance; u.uniform = p.env_uniform;
    u.sun_gain = std::max(0.f, p.env_sun_gain); u.sky_gain = std::max(0.f, p.env_sky_gain);
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
    u.n_prims = n_prims; u.n_mats = n_mats;
    return u;
}
}  // namespace

extern "C" int st_render_noalloc(int device, const st_scene_desc* desc, const st_params* p, const st_view* v,
                                 int nsamples, double* rgb, double* V, double* S, uint32_t* count) {
    if (!desc || !p || !v || nsamples < 0 || !desc->prims || !desc->materials) return ST_ERR_ARG;
    if (device < 0 || device >= ST_NOALLOC_MAX_DEVICES) return ST_ERR_ARG;
    const size_t P = (size_t)p->width * p->height;
    if (p->width == 0 || p->height == 0 || P > ST_NOALLOC_MAX_PIXELS) {
        std::fprintf(stderr, "st_render_noalloc: %ux%u pixels is over its limit of %u pixels (128 x 128)\n",
                     p->width, p->height, ST_NOALLOC_MAX_PIXELS);
        return ST_ERR_ARG;
    }
    if (desc->lights && desc->n_lights) {
        std::fprintf(stderr, "st_render_noalloc: a scene with light faces takes the context path (st_set_scene)\n");
        return ST_ERR_ARG;
    }
    if (desc->n_prims == 0 || desc->n_prims > ST_MAX_PRIMS || desc->n_materials == 0 ||
        desc->n_materials > ST_MAX_MATERIALS || desc->prims[0].op != ST_OP_ITEM)
        return ST_ERR_ARG;
    for (uint32_t i = 0; i < desc->n_prims; i++)
        if (desc->prims[i].type > ST_PRIM_CYLINDER || desc->prims[i].op > ST_OP_SUB ||
            desc->prims[i].material >= desc->n_materials)
            return ST_ERR_ARG;
    if (p->maxbounce == 0 || p->maxbounce > 64 || p->maxiter == 0 || p->maxiter > 65535 || !(p->stepscale > 0) ||
        p->stepscale > 1 || p->budget > 256)
        return ST_ERR_ARG;
    const Layout L = layout(P);
    if (L.end > ST_NOALLOC_SCRATCH_BYTES) return ST_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return ST_ERR_CUDA;
    cudaStream_t s = 0;

    // set-up, once per device, with the device current: the array's address, and the albedo tables built in it
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_base[device]) {
            void* ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return ST_ERR_CUDA;
            unsigned char* b = static_cast<unsigned char*>(ptr);
            if (launch_mf_tables((float*)(b + L.ec), (float*)(b + L.ecavg), (float*)(b + L.e1), s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                return ST_ERR_CUDA;
            const std::vector<double> t = spectral_table();             // the camera's wavelength table
            float4 f[SPEC_CELLS];
            for (int i = 0; i < SPEC_CELLS; i++)
                f[i] = make_float4((float)t[4 * i], (float)t[4 * i + 1], (float)t[4 * i + 2], (float)t[4 * i + 3]);
            if (cudaMemcpy(b + L.spec, f, sizeof(f), cudaMemcpyHostToDevice) != cudaSuccess) return ST_ERR_CUDA;
            g_base[device] = b;
        }
        base = g_base[device];
    }
    // the scene's tables
    DPrim packed[ST_MAX_PRIMS];
    for (uint32_t i = 0; i < desc->n_prims; i++) packed[i] = pack(desc->prims[i]);
    if (cudaMemcpyAsync(base + L.prims, packed, desc->n_prims * sizeof(DPrim), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(base + L.mats, desc->materials, desc->n_materials * sizeof(st_material), cudaMemcpyHostToDevice,
                        s) != cudaSuccess)
        return ST_ERR_CUDA;
    // what must start at zero: the accumulation, the moments, the frame, the counters
    if (cudaMemsetAsync(base + L.acc, 0, P * sizeof(Acc4), s) != cudaSuccess ||
        cudaMemsetAsync(base + L.mom, 0, P * 16, s) != cudaSuccess ||
        cudaMemsetAsync(base + L.frame, 0, P * 16, s) != cudaSuccess ||
        cudaMemsetAsync(base + L.ctr, 0, sizeof(DevCtr), s) != cudaSuccess)
        return ST_ERR_CUDA;

    WaveArgs a{};
    a.u = uniforms(*desc, *p, *v, desc->n_prims, desc->n_materials);
    a.prims = reinterpret_cast<const DPrim*>(base + L.prims);
    a.mats = reinterpret_cast<const st_material*>(base + L.mats);
    a.tab = MfTab{(const float*)(base + L.ec), (const float*)(base + L.ecavg), (const float*)(base + L.e1)};
    a.spec = (const float4*)(base + L.spec);
    a.pb = PathBuf{(float4*)(base + L.pos), (float4*)(base + L.dir), (float4*)(base + L.beta), (float4*)(base + L.rad),
                   (uint4*)(base + L.meta)};
    a.pb.lam = (float*)(base + L.lam);
    a.q.ray[0] = (uint32_t*)(base + L.ray0);
    a.q.ray[1] = (uint32_t*)(base + L.ray1);
    a.q.hit = (uint32_t*)(base + L.hit);
    a.q.hitd = (float*)(base + L.hitd);
    a.q.hsurf = (float4*)(base + L.hsurf);
    for (int k = 0; k < 2; k++) {
        a.q.s_org[k] = (float4*)(base + L.so[k]);
        a.q.s_dir[k] = (float4*)(base + L.sd[k]);
        a.q.s_rad[k] = (float4*)(base + L.sr[k]);
        a.q.s_steps[k] = (uint32_t*)(base + L.ss[k]);
    }
    a.q.cap = (uint32_t)P;
    a.q.scap = (uint32_t)(2 * P);
    a.ctr = (DevCtr*)(base + L.ctr);
    a.frame = (float4*)(base + L.frame);
    a.acc = (Acc4*)(base + L.acc);
    a.mom = (double2*)(base + L.mom);
    a.spw = 1;
    a.slots = (uint32_t)P;
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);

    // the regular path's launch chain, one sample a wave (st_capi.cu record_wave)
    for (int smp = 0; smp < nsamples; smp++) {
        if (launch_iter_begin(a, 0, 1, 1, s) != cudaSuccess || launch_genrays(a, sms, s) != cudaSuccess)
            return ST_ERR_CUDA;
        int cur = 0;
        for (uint32_t it = 0; it < a.u.budget; it++) {
            int nxt = cur ^ 1, last = it + 1 == a.u.budget, side = (int)(it & 1u);
            if (it > 0 && launch_iter_begin(a, (int)it, nxt, 0, s) != cudaSuccess) return ST_ERR_CUDA;
            if (launch_march(a, cur, nxt, last, sms, s) != cudaSuccess ||
                launch_surface(a, sms, s) != cudaSuccess ||
                launch_shade(a, nxt, side, last, sms, s) != cudaSuccess ||
                launch_occlude(a, side, last, sms, s) != cudaSuccess)
                return ST_ERR_CUDA;
            cur = nxt;
        }
        if (launch_resolve(a, s) != cudaSuccess) return ST_ERR_CUDA;
    }
    // the picture into the caller's buffers: strided copies, no staging buffer
    k_counts<<<(unsigned)((P + 255) / 256), 256, 0, s>>>(a.acc, (uint32_t*)(base + L.cnt), (uint32_t)P);
    if (cudaGetLastError() != cudaSuccess) return ST_ERR_CUDA;
    if (rgb && cudaMemcpy2DAsync(rgb, 3 * sizeof(double), base + L.acc, sizeof(Acc4), 3 * sizeof(double), P,
                                 cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return ST_ERR_CUDA;
    if (V && cudaMemcpy2DAsync(V, sizeof(double), base + L.mom, 16, sizeof(double), P, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return ST_ERR_CUDA;
    if (S && cudaMemcpy2DAsync(S, sizeof(double), base + L.mom + 8, 16, sizeof(double), P, cudaMemcpyDeviceToHost, s) !=
                 cudaSuccess)
        return ST_ERR_CUDA;
    if (count && cudaMemcpyAsync(count, base + L.cnt, P * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return ST_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return ST_ERR_CUDA;
    DevCtr c;
    if (cudaMemcpy(&c, base + L.ctr, sizeof(DevCtr), cudaMemcpyDeviceToHost) != cudaSuccess) return ST_ERR_CUDA;
    if (c.errflag) return ST_ERR_TIMEOUT;
    return ST_OK;
}
