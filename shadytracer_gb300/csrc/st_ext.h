// st_ext.h -- the photon map's and the optics bench's state inside a context, and the context accessors their
// translation units (st_sppm.cu, st_optics.cu) use.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "st_device.cuh"
#include "st_internal.h"

struct st_ctx;

struct SppmState {
    uint32_t n = 0, cap = 0;
    float cell = 0;
    // records, structure of arrays (core/sppm.js:350-423: point, power, incoming direction, normal, flags)
    float4* pos = nullptr;       // xyz point, w unused
    float4* power = nullptr;     // xyz power, w unused
    uint32_t* dir_oct = nullptr;
    uint32_t* nrm_oct = nullptr;
    uint32_t* flags = nullptr;   // bounce (low 16) | sub-list << 16 | SPPM_ALL / SPPM_VOL bits
    uint32_t* key = nullptr;     // each record's cell hash
    uint32_t* order = nullptr;   // the records in cell order (the counting sort's output)
    uint32_t* cell_count = nullptr;   // 2^20
    uint32_t* cell_start = nullptr;   // per (hash, sub-list) bucket: its first record, 2^25 (+1)
    uint32_t* heads = nullptr;        // per hash: its first record, 2^20 (+1) -- the gathers' cell ranges, 4 MB
    uint32_t* scan_part = nullptr;    // the scan's block partials
    float4* spos = nullptr;      // the records' point and power, permuted into cell order
    float4* spow = nullptr;
    uint32_t* sdir = nullptr;
    uint32_t* snrm = nullptr;
    uint32_t* sflags = nullptr;
    uint32_t* stats = nullptr;   // gathers, cut, visits_max, visits lo, visits hi
    uint32_t* bucket = nullptr;  // the sort's scratch: each record's bucket and rank in it
    uint32_t* rank = nullptr;
    st::SppmDev* dev = nullptr;  // the count, the capacity, the radius and cell on the device
    bool wave = false;           // the wavefront's map ran last (st_sppm_stats_read reads its device state)
    uint32_t* lt_emit = nullptr; // the learned emission map: photons sent, photons stored, the CDF
    uint32_t* lt_hit = nullptr;
    float* lt_cdf = nullptr;
    std::vector<float> lt_uniform;   // the uniform CDF the map starts from (and returns to at an invalidate)
};
int sppm_ensure(st_ctx* ctx, uint32_t n);
cudaError_t sppm_lt_reset(SppmState& s, cudaStream_t st);
cudaError_t sppm_grid_launch(SppmState& s, int sms, cudaStream_t st);
st::SppmBufs sppm_bufs(const SppmState& s);

struct OpticsState {
    std::vector<st_optics_source> sources;
    float4* rays = nullptr;      // the ray table: two float4s a ray (position | weight, direction | wavelength)
    uint32_t n_rays = 0;
    st_optics_far far{};
    bool has_far = false;
    st_optics_detail detail{};   // what a run keeps beyond its tallies (hits, paths)
    uint64_t sources_gen = 0;    // the sources' and the ray table's changes (a batch's graph is recorded with them)
    uint64_t launches = 0;       // kernels the batches' graphs ran
    uint32_t tune_claim = 0, tune_chunk = 0;   // the optics autotuner's picks (st_optics_autotune); 0, the defaults
    std::vector<float> spectra;  // st_optics_set_spectra's rows, ST_SPECTRUM_NODES values each
    void* scratch = nullptr;     // the run's device buffers (st_optics.cu OptBuf), grown as needed
};

// THE LEARNED PROPOSAL (st_guide.cu): FP32 weights and features with their gradients and Adam moments, the BF16
// copy the kernels read, the batch and a mini-batch's activations, the per-queue mixtures and per-path records
struct GuideState {
    float* param = nullptr;          // GUIDE_NPARAM: W1 W2 W3 W4 (GUIDE_NW), then the hash grid's features
    float* grad = nullptr;
    float* m1 = nullptr;
    float* m2 = nullptr;
    uint16_t* wbf = nullptr;
    st::GuideDev* dev = nullptr;
    st::GuideSample* samp = nullptr;
    uint16_t* act = nullptr;
    uint2* mix = nullptr;
    uint32_t* stamp = nullptr;       // per pixel of the wave's views: its mixture inferred this wave (1) or not (0)
    uint32_t mix_cap = 0;
    st::GuideRec* rec = nullptr;
    float* acc = nullptr;
    uint32_t rec_cap = 0;
    uint32_t seed = 0;               // the seed the weights were drawn from
};
int guide_ensure(st_ctx* ctx, uint32_t queue_cap, uint32_t slots, uint32_t seed);
int guide_upload(st_ctx* ctx, const float* h);
st::GuideBufs guide_bufs(st_ctx* ctx, uint32_t on, uint32_t train, float alpha, uint32_t slots);
cudaError_t guide_wave_begin(st_ctx* ctx, uint32_t slots, cudaStream_t st);
cudaError_t guide_stamps_clear(st_ctx* ctx, uint32_t pixels, cudaStream_t st);
cudaError_t guide_train_launch(st_ctx* ctx, float lr, int sms, cudaStream_t st, int* launches);
cudaError_t guide_eval_launch(st_ctx* ctx, uint32_t n, float* d_raw, uint2* d_mix, cudaStream_t st);
int guide_eval(st_ctx* ctx, const float* pos, const float* nrm, uint32_t n, float* raw, float* mix);
int guide_grad(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight, uint32_t n,
               float* grad, float* loss);
void guide_unpack_host(uint2 v, float* out);
int guide_train_samples(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight,
                        uint32_t n, uint32_t steps, float lr);
void guide_box(st_ctx* ctx, st::f3& lo, float& inv_ext);     // the hash grid's box (st_capi.cu)

// THE EMITTER LIST (st_emit.cu): the discovery grid and the list, the per-slot MIS weights, the hit queue
struct EmitState {
    uint32_t* grid = nullptr;
    st::EmitDev* dev = nullptr;
    float* w = nullptr;
    uint32_t w_cap = 0;
    float4 *hpos = nullptr, *hdir = nullptr, *hrad = nullptr;
    uint32_t h_cap = 0;
};
int emit_ensure(st_ctx* ctx, uint32_t slots, uint32_t scap);
st::EmitBufs emit_bufs(st_ctx* ctx, uint32_t nee, float share, float half);
cudaError_t emit_reset(st_ctx* ctx);

struct StExt {
    SppmState sppm;
    OpticsState optics;
    GuideState guide;
    EmitState emit;
};

void ext_free(StExt& e);
void optics_free(OpticsState& os);

StExt& ctx_ext(st_ctx* ctx);
cudaStream_t ctx_stream(st_ctx* ctx);
int ctx_device(st_ctx* ctx);
int ctx_sms(st_ctx* ctx);
void ctx_set_error(st_ctx* ctx, const std::string& m);
const st::DPrim* ctx_d_prims(st_ctx* ctx);
const st_material* ctx_d_mats(st_ctx* ctx);
uint32_t ctx_n_prims(st_ctx* ctx);
uint32_t ctx_n_mats(st_ctx* ctx);
const st_scene_desc& ctx_desc(st_ctx* ctx);
bool ctx_has_scene(st_ctx* ctx);
uint64_t ctx_scene_gen(st_ctx* ctx);
st::DevCtr* ctx_counters(st_ctx* ctx);     // a count of the scenes set (a graph recorded with one is stale after)
st::MfTab ctx_tab(st_ctx* ctx);
const float4* ctx_spec(st_ctx* ctx);
