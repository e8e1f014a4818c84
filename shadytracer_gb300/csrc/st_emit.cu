// st_emit.cu -- EMISSIVE SURFACES: the list light sampling aims at, built from what the camera paths discovered
// (core/wavefront.js:715-815 prog_emit_collect / prog_emit_publish), and the shadow rays aimed at it resolved
// (:1694-1749 prog_occlude_emit), with the C ABI's st_emit_list.
//
//   k_emit_reset    the discovery grid emptied (bounds at their extremes), the list emptied (an invalidate)
//   k_emit_build    between samples, every EMIT_EPOCH: each voxel with hits a box -- the bounding sphere of its
//                   hits' bounds, with a margin -- scored by its brightest emission times its size squared; the
//                   hits and the brightness fade by a tenth; at most EMIT_MAX boxes, in voxel order; probabilities
//                   by score and their running sum
//   k_emit_resolve  after each occlusion pass: a shadow ray aimed at an emitter that met something asks the scene's
//                   material there and deposits the emission it carries times that material's emission
//
// The reference lists the boxes in the order its atomics ran; here one block lists them in voxel order, so the list
// is a function of the grid alone and a second run, or the oracle, finds the same one.
#include <algorithm>
#include <vector>

#include "../../include/shadytracer.h"
#include "st_emit.cuh"
#include "st_ext.h"
#include "st_kernels.cuh"
#include "st_scene_kernels.cuh"

namespace st {

__global__ void k_emit_reset(uint32_t* __restrict__ grid, EmitDev* __restrict__ dev) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < EMIT_CELLS * 8u; i += gridDim.x * blockDim.x)
        grid[i] = (i & 7u) < 3u ? 0xFFFFFFFFu : 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) { dev->count = 0u; dev->last = 0u; }
}

#define EMIT_BUILD_THREADS 1024u
#define EMIT_PER (EMIT_CELLS / EMIT_BUILD_THREADS)
__global__ void __launch_bounds__(EMIT_BUILD_THREADS) k_emit_build(uint32_t* __restrict__ grid, EmitDev* __restrict__ dev,
                                                                 const DevCtr* __restrict__ ctr, float half, float tol,
                                                                 float margin) {
    __shared__ uint32_t wsum[32];
    __shared__ float sscore[EMIT_MAX];
    const uint32_t sample = ctr->sample;
    // between samples, every EMIT_EPOCH: the wave starting at `sample` takes the list built before it
    if (sample < dev->last + EMIT_EPOCH) return;
    const float R = half;
    float4 box[EMIT_PER];
    float score[EMIT_PER];
    uint32_t mine = 0;
#pragma unroll
    for (uint32_t k = 0; k < EMIT_PER; k++) {
        const uint32_t cell = threadIdx.x * EMIT_PER + k;
        uint32_t* g = grid + (size_t)cell * 8u;
        box[k] = make_float4(0.f, 0.f, 0.f, -1.f);
        score[k] = 0.f;
        const uint32_t w = g[6], n = g[7];
        if (n == 0u) continue;
        const uint32_t n2 = n - n / 10u;
        const uint32_t w2 = max(w, EMIT_LUM_DECAY + 1u) - EMIT_LUM_DECAY;   // never below 1, "seen"
        g[6] = w2;
        g[7] = n2;
        if (n2 == 0u) {                                                  // faded out: its bounds forgotten too
            g[0] = g[1] = g[2] = 0xFFFFFFFFu;
            g[3] = g[4] = g[5] = 0u;
            continue;
        }
        const f3 mn = mk((float)g[0] / EMIT_Q * (2.f * R) - R, (float)g[1] / EMIT_Q * (2.f * R) - R,
                         (float)g[2] / EMIT_Q * (2.f * R) - R);
        const f3 mx = mk((float)g[3] / EMIT_Q * (2.f * R) - R, (float)g[4] / EMIT_Q * (2.f * R) - R,
                         (float)g[5] / EMIT_Q * (2.f * R) - R);
        const f3 c = (mn + mx) * 0.5f;
        // the margin: the quantisation step, a hit's distance from the surface (an offset tolerance), a little of
        // the size
        const float pad = margin > 0.f ? margin : 10.f * march_tol(c, tol);
        const float r = length(mx - mn) * 0.5f * 1.05f + pad + 4.f * (2.f * R) / EMIT_Q;
        box[k] = make_float4(c.x, c.y, c.z, r);
        score[k] = emit_lum_decode(w2) * r * r;                         // brightest emission x size^2 ~ power
        mine++;
    }
    // the boxes' places in voxel order: the block's exclusive scan of the threads' counts
    const uint32_t lane = threadIdx.x & 31u, wp = threadIdx.x >> 5;
    uint32_t incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    if (lane == 31u) wsum[wp] = incl;
    __syncthreads();
    if (wp == 0u) {
        const uint32_t x = wsum[lane];
        uint32_t xi = x;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(FULL_MASK, xi, o);
            if (lane >= (uint32_t)o) xi += v;
        }
        wsum[lane] = xi - x;
    }
    __syncthreads();
    uint32_t at = wsum[wp] + incl - mine;
    const uint32_t total = wsum[31] + __shfl_sync(FULL_MASK, incl, 31);   // valid in warp 31 only
#pragma unroll
    for (uint32_t k = 0; k < EMIT_PER; k++) {
        if (box[k].w < 0.f) continue;
        if (at < EMIT_MAX) {                                             // past EMIT_MAX a voxel is simply not listed
            dev->box[at] = box[k];
            sscore[at] = score[k];
        }
        at++;
    }
    __shared__ uint32_t s_total;
    if (threadIdx.x == EMIT_BUILD_THREADS - 1u) s_total = total;
    __syncthreads();
    if (threadIdx.x == 0u) {
        const uint32_t K = min(s_total, EMIT_MAX);
        float tot = 0.f;
        for (uint32_t b = 0; b < K; b++) tot += sscore[b];
        float acc = 0.f;
        for (uint32_t b = 0; b < K; b++) {
            const float P = tot > 0.f ? sscore[b] / tot : 1.f / (float)K;
            acc += P;
            dev->pc[b] = make_float4(P, b + 1u == K ? 1.f : acc, 0.f, 0.f);
        }
        dev->count = K;
        dev->last = sample;
    }
}

cudaError_t launch_emit_reset(const EmitBufs& em, cudaStream_t s) {
    k_emit_reset<<<32, 256, 0, s>>>(em.grid, em.dev);
    return cudaGetLastError();
}
cudaError_t launch_emit_build(const WaveArgs& a, float margin, cudaStream_t s) {
    k_emit_build<<<1, EMIT_BUILD_THREADS, 0, s>>>(a.em.grid, a.em.dev, a.ctr, a.em.half, a.u.tol, margin);
    return cudaGetLastError();
}
cudaError_t launch_emit_resolve(const WaveArgs& a, int sms, cudaStream_t s) {
    if (a.code) {
        if (!a.code->emit_resolve) return cudaErrorInvalidDeviceFunction;
        void* args[] = {(void*)&a};
        return cudaLaunchKernel(a.code->emit_resolve, dim3((unsigned)sms * 2u), dim3(256), args, 0, s);
    }
    k_emit_resolve<TableScene><<<sms * 2, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace st

using namespace st;

// the list's buffers in a context: the grid and list once, the per-slot weights and the hit queue with the wave
int emit_ensure(st_ctx* ctx, uint32_t slots, uint32_t scap) {
    EmitState& e = ctx_ext(ctx).emit;
    auto fail = [&](const char* what) { ctx_set_error(ctx, what); return ST_ERR_OOM; };
    if (!e.grid) {
        if (cudaMalloc(&e.grid, (size_t)EMIT_CELLS * 8 * 4) || cudaMalloc(&e.dev, sizeof(EmitDev)))
            return fail("cudaMalloc emitter list");
        if (launch_emit_reset(EmitBufs{0, 0, 0.5f, 15.f, e.grid, e.dev}, ctx_stream(ctx)) ||
            cudaStreamSynchronize(ctx_stream(ctx)))
            return fail("emitter list reset");
    }
    if (slots > e.w_cap) {
        if (e.w) cudaFree(e.w);
        e.w = nullptr;
        e.w_cap = 0;
        if (cudaMalloc(&e.w, (size_t)slots * 4)) return fail("cudaMalloc emitter weights");
        e.w_cap = slots;
    }
    if (scap > e.h_cap) {
        for (float4* p : {e.hpos, e.hdir, e.hrad}) if (p) cudaFree(p);
        e.hpos = e.hdir = e.hrad = nullptr;
        e.h_cap = 0;
        if (cudaMalloc(&e.hpos, (size_t)scap * 16) || cudaMalloc(&e.hdir, (size_t)scap * 16) ||
            cudaMalloc(&e.hrad, (size_t)scap * 16))
            return fail("cudaMalloc emitter hits");
        e.h_cap = scap;
    }
    return ST_OK;
}
EmitBufs emit_bufs(st_ctx* ctx, uint32_t nee, float share, float half) {
    EmitState& e = ctx_ext(ctx).emit;
    EmitBufs b;
    b.on = 1u;
    b.nee = nee;
    b.share = share;
    b.half = half;
    b.grid = e.grid;
    b.dev = e.dev;
    b.w = e.w;
    b.hpos = e.hpos;
    b.hdir = e.hdir;
    b.hrad = e.hrad;
    return b;
}
// an invalidate: the discovery starts over, as the reference's learnInit does (raytrace_main.js:347)
cudaError_t emit_reset(st_ctx* ctx) {
    EmitState& e = ctx_ext(ctx).emit;
    if (!e.grid) return cudaSuccess;
    EmitBufs b;
    b.grid = e.grid;
    b.dev = e.dev;
    return launch_emit_reset(b, ctx_stream(ctx));
}

extern "C" int st_emit_list(st_ctx* ctx, float* out, uint32_t max_n, uint32_t* n) {
    if (!ctx || !n || (max_n && !out)) return ST_ERR_ARG;
    cudaSetDevice(ctx_device(ctx));
    *n = 0;
    EmitState& e = ctx_ext(ctx).emit;
    if (!e.dev) return ST_OK;
    EmitDev d;
    if (cudaStreamSynchronize(ctx_stream(ctx)) || cudaMemcpy(&d, e.dev, sizeof(d), cudaMemcpyDeviceToHost))
        return ST_ERR_CUDA;
    const uint32_t K = std::min(std::min(d.count, EMIT_MAX), max_n);
    for (uint32_t b = 0; b < K; b++) {
        float* o = out + 6 * (size_t)b;
        o[0] = d.box[b].x; o[1] = d.box[b].y; o[2] = d.box[b].z; o[3] = d.box[b].w;
        o[4] = d.pc[b].x; o[5] = d.pc[b].y;
    }
    *n = std::min(d.count, EMIT_MAX);
    return ST_OK;
}
