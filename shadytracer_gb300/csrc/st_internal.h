// st_internal.h -- what the host side of libshadytracer (st_capi.cu) and the kernels (st_render.cu, st_sppm.cu,
// st_optics.cu) share: the device buffers of a wave, the device counters, and the launch wrappers.
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#include <cuda_runtime.h>
#endif
#include "st_device.cuh"

namespace st {

// Ray states (core/tracebasics.js:101-111; haze.js RAY_SCATTER)
#define RAY_ACTIVE 0u
#define RAY_ABSORBED 1u
#define RAY_ESCAPED 2u
#define RAY_MAXITER 4u
#define RAY_SOURCE 5u
#define RAY_TERMINATED 8u
#define RAY_SCATTER 9u
#define RAY_GATHER 10u                    // a camera ray's collision in a scattering material the map gathers at

// A MARCH CHUNK: the most SDF evaluations a ray takes in one launch of the march or the occlusion pass before it is
// handed to the next iteration (the reference's MARCH_STEPS, wavefront.js:870, is 32); the last iteration's launches
// march to the end. It bounds the tail a persistent launch spends on its longest rays.
// meta.y's upper byte: the photon map's classes (materials_pbr.js lensField / TAG_PASSED)
#define META_PASSED (1u << 24)            // a photon that has passed a delta event
#define META_LENS_SHIFT 25u               // a camera path's lens field (2 bits): 1 delta events only since the eye,
                                          // 2 at its D, 3 delta events since its D (the map owns the sun it reaches)
#define META_TRAIN (1u << 27)             // a camera path that holds a training record for the learned proposal
#define META_CAND (1u << 28)              // light tracing's class (tracebasics.js:195-196 CLS_CAND, CLS_SPEC): a camera
#define META_SPEC (1u << 29)              // path whose first vertex drew an evaluable lobe; ...and delta events since
#define META_PROBE (1u << 30)             // an emitter photon's probe (TAG_PROBE): looking for where its photon starts
#define META_LOW 0x00ffffffu
// meta.z: the march steps over the path (bits 0-23) and the medium it is in (bits 24-31): the material whose volume
// holds it, 0 none -- what a scattering material's walk reads (materials.js:134-148 the medium a ray carries)
#define META_STEPS 0x00ffffffu
#define MEDIUM_SHIFT 24u
#define SURF_NONE 0xffffu                 // hsurf: no medium asked (n1 is the material's own index of refraction)
#define SURF_LEAVING 0xffffffffu          // hsurf: the surface seen from behind, the ray moved on
#define SORT_G 16u                        // the march queue's space order: SORT_G^3 cells ...
#define SORT_BUCKETS (SORT_G * SORT_G * SORT_G * 8u)   // ... x 8 direction octants
#define SORT_MIN_PRIMS 8u                 // scenes of fewer primitives march their queues unsorted
#define MARCH_CHUNK 48u
#define CLAIM 64u                         // queue entries a warp of the march or the occlusion pass claims at a time

// meta.y: the bounces (bits 0-7), the path's segment -- its shades so far, which its random numbers are seeded by
// (bits 8-15) -- and the state (bits 16-23)
__host__ __device__ __forceinline__ uint32_t meta_y(uint32_t bounces, uint32_t seg, uint32_t state) {
    return (bounces & 0xffu) | ((seg & 0xffu) << 8) | (state << 16);
}

// THE WAVE'S PATH STATE, structure of arrays indexed by the path's slot (slot = sample-in-wave * P + tile): the
// reference's 112-byte Ray (tracebasics.js:400-460) cut to what the hot path carries, as four float4 and one uint4
// so every access is one 128-bit load or store.
struct PathBuf {
    float4* pos;    // xyz position, w ltot (optical length travelled)
    float4* dir;    // xyz direction, w n (index of the medium it is in)
    float4* beta;   // xyz throughput, w sunmis (the environment's MIS weight on escape)
    float4* rad;    // xyz radiance collected, w tmax (the haze's collision, as ltot)
    uint4* meta;    // x pix, y bounces | segment << 8 | state << 16, z march steps over the path, w absLtot (f32)
    float* lam = nullptr;   // the wavelength a dispersive refraction gave the path (nm, as coded), 0 none
    float2* lprev = nullptr;  // x: the last vertex's density for the direction it sent the path on, the light
                              // faces' share folded in (< 0: no weight against them); y: ltot at that vertex
};
// THE QUEUES: indices into the path state, appended with one atomic per warp (ballot + popc)
struct Queues {
    uint32_t* ray[2];    // the march's input, ping-pong: new segments and march continuations
    uint32_t* hit;       // the shade queue: slot
    float* hitd;         // ...and the signed distance at the hit
    uint32_t* sorted;    // the march queue of this iteration in space order (cell, octant), when sort_on
    uint32_t* skey;      // ...each entry's bucket and its rank in it
    uint32_t* srank;
    uint32_t* ssorted;   // the shadow queue of this iteration in space order: positions into its side's arrays
    uint32_t* sskey;     // ...each entry's bucket and its rank in it
    uint32_t* ssrank;
    uint32_t* bcnt;      // SORT_BUCKETS counts (zero between sorts) and their exclusive offsets
    uint32_t* boff;
    float4* hsurf;       // ...and what k_surface found there: the outward normal (xyz, before facing) and, as bits in
                         // w, the material | the medium beyond << 16 (SURF_NONE: none asked; SURF_LEAVING in both:
                         // seen from behind)
    // shadow rays, ping-pong (side it & 1 read by the occlusion pass of iteration it, continuations to the other)
    float4* s_org[2];    // xyz where it is, w ltot
    float4* s_dir[2];    // xyz direction, w pix in the wave's frames (u32 bits)
    float4* s_rad[2];    // xyz what it deposits if it reaches, w n
    uint32_t* s_steps[2];
    uint32_t cap;        // slots in a wave: the path queues hold at most this many
    uint32_t scap;       // each shadow side's room; appends past it are dropped and counted
};
// THE COUNTERS (wavefront.js:150 Counters), on the device. The statistics accumulate from the context's creation.
struct DevCtr {
    uint32_t rayCount[2], hitCount, shadowCount[2];
    uint32_t marchHead, occHead, errflag;
    uint32_t nonfinite, flushed, shadowcut, sample;   // sample: the first sample of the wave in flight
    uint32_t shadowdrop, emitHits;                    // emitHits: this iteration's shadow rays that met something
                                                      // while aiming at an emitter
    uint32_t wait_limit, wait_arm_only;               // the device-side waits' limit (0: WAIT_LIMIT) and the test of
                                                      // their failure path (st_set_wait_limit)
    unsigned long long paths, segments, march_steps, shadow_rays, shadow_steps;
    unsigned long long work[WC_N];     // the march's fold, counted in a counting pass (WC_* in st_device.cuh)
};

// THE PHOTON MAP ON THE DEVICE (st_sppm.cu builds its grid, st_photons.cu stores and gathers): the sample's radius
// and the records' count, then the records as stored and in cell order
struct SppmDev {
    uint32_t count, cap, dropped, gathers;   // records stored (may pass cap: the rest are dropped), capacity
    float r, cell, inv_area, r2;              // this sample's radius, the grid's cell (2r), 1 / (pi r^2), r^2
    unsigned long long visits, stores;
    // in the volume (sppm.js sppmRadiusVolume): the radius, its records' cell (2R), 3 / (4 pi R^3), R^2
    float vr, vcell, inv_vol, vr2;
    uint32_t vstores, vgathers;
    // ...and its thinning (sppm.js:150-158 sppmKeep): the share of a sample's collisions kept as records, each then
    // carrying its power over the share -- from the last sample's demand, so the records fit half the capacity
    float vkeep;
    uint32_t vdemand;
};
struct SppmBufs {
    SppmDev* dev = nullptr;
    uint32_t cap = 0;                         // the records' capacity
    float4 *pos = nullptr, *power = nullptr;  // as stored: point, power
    uint32_t *dir_oct = nullptr, *nrm_oct = nullptr, *flags = nullptr;
    const uint32_t* start = nullptr;          // per (cell hash, sub-list) bucket: its first record in cell order
    const uint32_t* heads = nullptr;          // per cell hash: its first record (start at the hash's sub-list 0)
    const float4 *spos = nullptr, *spow = nullptr;
    const uint32_t *sdir = nullptr, *snrm = nullptr, *sflags = nullptr;
    // the learned emission map (wavefront.js:628-711): per cell of the LT_GRID^2 square the photons sent and those
    // stored, and the CDF the sun's photons are drawn from (LT_CELLS conditional row entries, then LT_GRID rows)
    uint32_t *lt_emit = nullptr, *lt_hit = nullptr;
    float* lt_cdf = nullptr;
};
#define LT_GRID 128u
#define LT_CELLS (LT_GRID * LT_GRID)
#define LT_FLOOR 0.2f

struct __align__(32) Acc4 { double x, y, z, w; };   // FP64 mean rgb + the sample count

// THE LEARNED PROPOSAL (st_guide.cu, st_guide.cuh): per hit-queue entry the mixture its vertex samples from; per path
// (its pixel in the wave's frames) the training record of its first guided vertex and the light found after it; the
// batch those records make at the wave's end; the weights the kernels read.
struct GuideRec { float4 a, b; };         // a: position, pdf of the direction; b: normal, direction (oct16 bits),
                                          // throughput luminance reaching the vertex, radiance luminance before it
struct GuideSample { float4 a, b, c; };   // a: position, weight (f cos L_in / pdf); b: normal; c: direction
struct GuideDev {
    uint32_t count, step, inferred, pad1; // samples in the batch; Adam steps taken; vertices the network ran at
    float wsum, loss, loss_n, pad2;       // the batch's summed weight; the last step's summed loss and samples
};
struct GuideBufs {
    uint32_t on = 0, train = 0;           // guided sampling; records and training
    float alpha = 0.5f;                   // the guide's share of one-sample MIS
    f3 lo = {0.f, 0.f, 0.f};              // the hash grid's box: its low corner and 1 / its longest side
    float inv_ext = 1.f;
    const float2* table = nullptr;        // hash-grid features, FP32
    const uint16_t* wbf = nullptr;        // the network's weights, BF16 bits, [out][in] row-major, W1 W2 W3 W4
    uint2* mix = nullptr;                 // 8 packed lobes a pixel of the wave's views (view * P + pixel)
    uint32_t* stamp = nullptr;            // ...and whether a path of the pixel has had it inferred this wave
    GuideRec* rec = nullptr;              // a path's record (by its pixel in the wave's frames)
    float* acc = nullptr;                 // ...and the luminance found after its vertex
    GuideSample* samp = nullptr;          // the training batch
    GuideDev* dev = nullptr;
    uint32_t cap = 0;                     // the batch's room
    uint32_t keep = 0;                    // a record joins the batch when its hash is below this (of 2^32)
};

// THE EMITTER LIST (core/tracebasics.js:1140-1210 EMIT_LIST; wavefront.js:715-815 prog_emit_collect / publish;
// materials_pbr.js:887-905 emitDeposit): what the camera paths that hit emissive surfaces found, in a grid of
// EMIT_G^3 voxels over +-half, turned every EMIT_EPOCH samples into at most EMIT_MAX bounding spheres that light
// sampling aims at (st_emit.cu, st_emit.cuh)
#define EMIT_G 16u
#define EMIT_CELLS (EMIT_G * EMIT_G * EMIT_G)
#define EMIT_MAX 64u
#define EMIT_EPOCH 2u
#define SHADOW_EMIT 0x80000000u           // a shadow side's steps word: the ray aims at an emitter (TAG_EMIT)
#define SHADOW_FACE 0x40000000u           // ...at a point of a light's face (TAG_FNEE): it arrives when ltot,
                                          // started at minus the way there, reaches 0
#define SHADOW_CONN 0x20000000u           // ...a photon's connection to the camera (TAG_CONN), a face's ray in its
                                          // length; what arrives goes to the splat buffer
#define SHADOW_FLAGS (SHADOW_EMIT | SHADOW_FACE | SHADOW_CONN)
#define SC_BURST 4u                       // step-cache balls a lane may cross in a row before it asks the scene
// THE LIGHTS' FACES (st_light.cuh): FACE_F4 float4s a face, then a byte a material (its face + 1, 0 none)
#define FACE_F4 5
struct LightBufs {
    const float4* face = nullptr;         // centre|half_w, u|half_h, v|shape, n|beam_cos, le|(n, or -1 even)
    const uint8_t* of = nullptr;          // ST_MAX_MATERIALS: the face a material draws, plus 1
    uint32_t n = 0;                       // faces; 0, none (the light samples go as they always went)
};
struct EmitDev {
    uint32_t count, last, pad0, pad1;     // boxes listed; the sample the list was last built before
    float4 box[EMIT_MAX];                 // centre, radius: each box's bounding sphere
    float4 pc[EMIT_MAX];                  // its probability, the cumulative probability, 0, 0
};
struct EmitBufs {
    uint32_t on = 0;                      // the scene has emissive materials: discovery, the list, the MIS weights
    uint32_t nee = 0;                     // light sampling aims at the list's boxes
    float share = 0.5f;                   // ...with this share of the light samples once anything is listed
    float half = 15.f;                    // the grid's half-size, metres
    uint32_t* grid = nullptr;             // EMIT_CELLS x 8 words: min q xyz, max q xyz, brightness code, hits
    EmitDev* dev = nullptr;
    float* w = nullptr;                   // per slot: an emitter hit's MIS weight against the last vertex's light sample
    float4 *hpos = nullptr, *hdir = nullptr, *hrad = nullptr;   // shadow rays that met something: where, dir | pixel,
                                                                // contribution | n (resolved by k_emit_resolve)
};

// A SCENE AS CODE, compiled (st_scene_rtc.cu): the scene-calling kernels of st_scene_kernels.cuh built by NVRTC for
// sm_103a with the scene's own functions, loaded as a library; each kernel a cudaKernel_t (as the runtime's launch
// calls take it), and the persistent kernels' occupancies, found once. Host-side only; the kernels never read it.
struct SceneCode {
    void* lib = nullptr;                          // cudaLibrary_t
    const void* march[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};   // [media][counting pass]
    const void* surface = nullptr;
    const void* occlude[2] = {nullptr, nullptr};  // by the shadow side read
    const void* emit_resolve = nullptr;
    const void* sc_fill = nullptr;
    const void* eval_sdf = nullptr;
    mutable int occ_march[2][2] = {{0, 0}, {0, 0}};   // found at the first launch
    mutable int occ_surface = 0, occ_occlude = 0;
    double compile_ms = 0.0;                      // NVRTC's time for it (0: taken from the cache)
    size_t cubin_bytes = 0;
};

struct WaveArgs {
    Uni u;
    const DPrim* prims;
    const st_material* mats;
    MfTab tab;
    PathBuf pb;
    Queues q;
    DevCtr* ctr;
    float4* frame;      // spw * P: this wave's deposits, rgb + count
    float4* splat = nullptr;     // P: light tracing's connections this sample, rgb (wavefront.js splat_u32)
    uint32_t* ltcount = nullptr; // P: the connections that reached each pixel since the last invalidate
    Acc4* acc;         // P: FP64 mean rgb + count
    double2* mom;       // P: FP64 V, S (the error bar's moments)
    uint32_t spw;       // samples in this wave
    uint32_t slots;     // spw * P
    const float4* spec = nullptr;         // the camera's wavelength table (SPEC_NCELLS cells: CDF, colour rgb)
    SppmBufs sp;                          // the photon map, while it runs
    const uint2* inst_range = nullptr;   // a batch of instances (the optics bench): each one's [first, count) of the
                                         // table, the instance in meta.w; null for a picture
    GuideBufs gd;                         // the learned proposal, while it runs
    EmitBufs em;                          // the emitter list, in a scene with emitters
    LightBufs lf;                         // the lights' faces
    const SceneCode* code = nullptr;      // the scene as compiled code (host-side: which kernels to launch); null, the table
};

#ifndef __CUDACC_RTC__                 // host-side: the launch wrappers and the host helpers
// launch wrappers (st_render.cu)
cudaError_t launch_mf_tables(float* ec, float* ecavg, float* e1, cudaStream_t s);
cudaError_t launch_genrays(const WaveArgs& a, int sms, cudaStream_t s);
cudaError_t launch_iter_begin(const WaveArgs& a, int it, int nxt, int first, cudaStream_t s);
cudaError_t launch_surface(const WaveArgs& a, int sms, cudaStream_t s);
cudaError_t launch_sort(const WaveArgs& a, int cur, int sms, cudaStream_t s);
// the photon map in the wavefront (st_photons.cu)
cudaError_t launch_sppm_begin(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_lt_build(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_genphotons(const WaveArgs& a, uint32_t first, uint32_t n, int sms, cudaStream_t s);
cudaError_t launch_photon_shade(const WaveArgs& a, int nxt, int last, int side, int sms, cudaStream_t s);
cudaError_t launch_gather(const WaveArgs& a, int sms, cudaStream_t s);
cudaError_t launch_eval_sdf(const DPrim* prims, uint32_t n_prims, const float* pts, uint32_t n, float* out,
                            cudaStream_t s, const SceneCode* code = nullptr);
cudaError_t launch_sort_shadow(const WaveArgs& a, int side, int sms, cudaStream_t s);
cudaError_t launch_march(const WaveArgs& a, int cur, int nxt, int last, int sms, cudaStream_t s);
cudaError_t launch_shade(const WaveArgs& a, int nxt, int side, int last, int sms, cudaStream_t s);
cudaError_t launch_occlude(const WaveArgs& a, int side, int last, int sms, cudaStream_t s);
cudaError_t launch_resolve(const WaveArgs& a, cudaStream_t s);
cudaError_t launch_env_bake(const Uni& u, float* out, cudaStream_t s);
cudaError_t launch_env_cache(const Uni& u, float4* out, uint32_t w, uint32_t h, cudaStream_t s);
cudaError_t launch_sc_fill(const DPrim* prims, uint32_t n_prims, f3 lo, float cs, uint32_t dx, uint32_t dy, uint32_t dz,
                           float* out, int sms, cudaStream_t s, const SceneCode* code = nullptr);
// the emitter list (st_emit.cu)
cudaError_t launch_emit_build(const WaveArgs& a, float margin, cudaStream_t s);
cudaError_t launch_emit_resolve(const WaveArgs& a, int sms, cudaStream_t s);
cudaError_t launch_emit_reset(const EmitBufs& em, cudaStream_t s);
// the learned proposal (st_guide.cu)
cudaError_t launch_guide_infer(const WaveArgs& a, int sms, cudaStream_t s);
cudaError_t launch_guide_collect(const WaveArgs& a, int sms, cudaStream_t s);
cudaError_t launch_guide_eval_tc(const GuideSample* samp, uint32_t n, f3 lo, float inv_ext, const float2* table,
                                 const uint16_t* wbf, float* raw, uint2* mix, uint32_t* err, int sms, cudaStream_t s);
#endif  // __CUDACC_RTC__

}  // namespace st

#ifndef __CUDACC_RTC__
// HOST HELPERS (st_capi.cu) that the context path and the render that allocates nothing (st_noalloc.cu) share, so
// the two derive the same uniforms and pack the same table: the uniforms that depend only on the scene's
// description, the settings and the camera (env_image: an environment image replaces the sun and sky), and a
// primitive as the kernels read it
st::Uni make_uni_base(const st_scene_desc& s, const st_params& p, const st_view& v, uint32_t n_prims, uint32_t n_mats,
                      bool env_image);
st::DPrim pack_prim(const st_prim& p);
// why st_render_noalloc last refused a call on this thread ("" if it did not)
const char* noalloc_last_error();
#include <string>
namespace st {
// a scene given as code (st_scene_rtc.cu): compiled by NVRTC with the scene-calling kernels and loaded; on failure err
// says why (with the scene's line) and nothing is kept
bool scene_code_build(const char* user_src, SceneCode& out, std::string& err);
bool scene_code_compile(const char* user_src, double& ms, std::string& err);
void scene_code_free(SceneCode& c);
}  // namespace st

#endif  // __CUDACC_RTC__
