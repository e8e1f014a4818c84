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
// stream, with the uniforms and the packed table from the same host functions (st_capi.cu make_uni_base,
// pack_prim), so the picture equals st_step's for the same scene, settings, camera and samples. What this render
// does not carry -- light faces, the photon map, the learned proposal, the step cache, light sampling of emissive
// materials -- is refused with ST_ERR_ARG and a message (st_last_error(NULL)), never silently left out.
//
// THE CALLER'S DEVICE. The call makes its device current while it runs and puts the caller's back before it returns.
//
// SET-UP. The first call on a device, with that device current, takes the array's device address with
// cudaGetSymbolAddress and builds the albedo tables in it; make that first call before any stream capture.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "st_spectral.h"
#include "st_internal.h"

using namespace st;

#define ST_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[ST_NOALLOC_SCRATCH_BYTES];

namespace {
struct Layout {
    size_t pos, dir, beta, rad, meta, ray0, ray1, hit, hitd, hsurf, so[2], sd[2], sr[2], ss[2], frame, acc, mom, cnt, ctr,
        ec, ecavg, e1, spec, coat, lam, prims, mats, end;
};
// the array carved for P paths a wave (one sample), each buffer 256-byte aligned: first what does not depend on the
// picture's size (the albedo tables, built once, the scene's tables, the counters), then the wave's buffers
Layout layout(size_t P) {
    Layout L{};
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o += (bytes + 255) & ~size_t(255); return at; };
    L.ec = take(16 * 32 * 32 * 4); L.ecavg = take(16 * 32 * 4); L.e1 = take(32 * 32 * 4);
    L.spec = take(SPEC_CELLS * sizeof(float4));
    L.coat = take(COAT_BINS * sizeof(float4));
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

thread_local std::string g_err;         // why the last call on this thread was refused (st_last_error(NULL))

// the calling thread's current device, put back on every way out: a host that counts on its device staying put
// finds it as it was
struct DeviceGuard {
    int prev = -1;
    DeviceGuard() { if (cudaGetDevice(&prev) != cudaSuccess) prev = -1; }
    ~DeviceGuard() { if (prev >= 0) cudaSetDevice(prev); }
};

int refuse(const char* fmt, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = std::string("st_render_noalloc: ") + buf;
    std::fprintf(stderr, "%s\n", g_err.c_str());
    return ST_ERR_ARG;
}
}  // namespace

const char* noalloc_last_error() { return g_err.c_str(); }

extern "C" int st_render_noalloc(int device, const st_scene_desc* desc, const st_params* p, const st_view* v,
                                 int nsamples, double* rgb, double* V, double* S, uint32_t* count) {
    g_err.clear();
    if (!desc || !p || !v || nsamples < 0 || !desc->prims || !desc->materials)
        return refuse("a null scene, settings or camera, or a negative sample count");
    if (device < 0 || device >= ST_NOALLOC_MAX_DEVICES) return refuse("device %d out of range", device);
    const size_t P = (size_t)p->width * p->height;
    if (p->width == 0 || p->height == 0 || P > ST_NOALLOC_MAX_PIXELS)
        return refuse("%ux%u pixels is over its limit of %u pixels (128 x 128)", p->width, p->height,
                      ST_NOALLOC_MAX_PIXELS);
    // what this render does not do, refused rather than left out: its picture would differ from st_step's
    if (desc->lights && desc->n_lights) return refuse("a scene with light faces takes the context path (st_set_scene)");
    if (p->sppm) return refuse("the photon map (st_params.sppm) takes the context path");
    if (p->guide) return refuse("the learned proposal (st_params.guide) takes the context path");
    if (p->lt) return refuse("light tracing (st_params.lt) takes the context path");
    if (p->env_mode != ST_ENV_ANALYTIC && p->env_uniform <= 0.f)
        return refuse("the environment's presets (st_params.env_mode: their tables and map) take the context path");
    if (p->step_cache) return refuse("the step cache (st_params.step_cache) takes the context path");
    for (uint32_t i = 0; i < desc->n_materials && !p->emit_off; i++) {
        const float* e = desc->materials[i].emissive;
        if (e[0] > 0.f || e[1] > 0.f || e[2] > 0.f)
            return refuse("material %u is emissive: its light sampling (the emitter list) takes the context path; "
                          "set st_params.emit_off to render it by the BSDF's hits alone", i);
    }
    if (desc->n_prims == 0 || desc->n_prims > ST_MAX_PRIMS || desc->n_materials == 0 ||
        desc->n_materials > ST_MAX_MATERIALS || desc->prims[0].op != ST_OP_ITEM)
        return refuse("the table's size is out of range (1..256 primitives and materials) or it starts with no item");
    for (uint32_t i = 0; i < desc->n_materials; i++)
        if (desc->materials[i].scatter_distance > 0.f)
            return refuse("material %u scatters inside (st_material.scatter_distance): its walk takes the context path", i);
    for (uint32_t i = 0; i < desc->n_prims; i++)
        if (desc->prims[i].type > ST_PRIM_CYLINDER || desc->prims[i].op > ST_OP_SUB ||
            desc->prims[i].material >= desc->n_materials)
            return refuse("primitive %u: unknown type or op, or material out of range", i);
    if (p->maxbounce == 0 || p->maxbounce > 64 || p->maxiter == 0 || p->maxiter > 65535 || !(p->stepscale > 0) ||
        p->stepscale > 1 || p->budget > 256)
        return refuse("maxbounce, maxiter, stepscale or budget out of range");
    const Layout L = layout(P);
    if (L.end > ST_NOALLOC_SCRATCH_BYTES) return refuse("the picture's buffers do not fit the scratch array");
    DeviceGuard keep_device;
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
            const std::vector<double> c = coat_bin_table();                 // a coating's 10 nm bins
            float4 cb[COAT_BINS];
            for (int k = 0; k < COAT_BINS; k++)
                cb[k] = make_float4((float)c[3 * k], (float)c[3 * k + 1], (float)c[3 * k + 2], 0.f);
            if (cudaMemcpy(b + L.spec, f, sizeof(f), cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(b + L.coat, cb, sizeof(cb), cudaMemcpyHostToDevice) != cudaSuccess)
                return ST_ERR_CUDA;
            g_base[device] = b;
        }
        base = g_base[device];
    }
    // the scene's tables
    DPrim packed[ST_MAX_PRIMS];
    for (uint32_t i = 0; i < desc->n_prims; i++) packed[i] = pack_prim(desc->prims[i]);
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
    a.u = make_uni_base(*desc, *p, *v, desc->n_prims, desc->n_materials, false);
    a.prims = reinterpret_cast<const DPrim*>(base + L.prims);
    a.mats = reinterpret_cast<const st_material*>(base + L.mats);
    a.tab = MfTab{(const float*)(base + L.ec), (const float*)(base + L.ecavg), (const float*)(base + L.e1),
                  (const float4*)(base + L.coat)};
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
