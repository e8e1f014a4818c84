// st_guide_tc.cu -- the learned proposal's network on the 5th-generation tensor cores (tcgen05): its inference at a
// wave's guided vertices (k_guide_infer_tc) and at given points (k_guide_eval_tc, st_mlp_eval).
//
// A CTA of 128 threads takes the vertices 128 at a time, a row a thread: the thread works out its row's 48 inputs
// (the hash grid's 16 levels x 2 features, trilinear over 8 corners, and the normal's 16 harmonics) and writes them,
// BF16, into the A tile in shared memory; one thread issues each layer's MMAs (M = 128 rows, N = 64 outputs, or 48 for
// the last -- 40 and 8 zero rows of weights --, K = 16 a step) into 64 columns of tensor memory and commits them to an
// mbarrier; every thread reads its row's 64 accumulators back (tcgen05.ld, 32 lanes a warp), and between layers
// writes the ReLU'd BF16 activations back as the next A. The four weight matrices sit in shared memory for the CTA's
// life, in the operand layout (st_tc.cuh). The arithmetic is the mma.sync path's: BF16 operands, FP32 accumulation,
// each hidden layer rounded to BF16 after its ReLU.
#include "st_guide.cuh"
#include "st_tc.cuh"
#include "st_kernels.cuh"
#include "st_ext.h"

namespace st {

// the shared-memory layout: W1 (64 x 48), W2, W3 (64 x 64), W4 (48 x 64: 40 rows and 8 of zeros), then A (128 x 64)
#define TC_W1 0u
#define TC_W2 (TC_W1 + 64u * 48u * 2u)
#define TC_W3 (TC_W2 + 64u * 64u * 2u)
#define TC_W4 (TC_W3 + 64u * 64u * 2u)
#define TC_A (TC_W4 + 48u * 64u * 2u)
#define TC_BYTES (TC_A + 128u * 64u * 2u)        // 45 056
#define TC_COLS 64u                              // tensor-memory columns: one layer's 64 FP32 outputs a row

// the weights ([out][in] BF16 row-major in global memory) into their operand layout, the padding rows zero
__device__ void tc_stage_weights(const uint16_t* __restrict__ wbf, unsigned char* s) {
    for (uint32_t i = threadIdx.x; i < GUIDE_NW + 8u * 64u; i += blockDim.x) {
        uint32_t layer, o, in, K, base;
        uint16_t v = 0;
        if (i < GUIDE_W2) { layer = 0; o = i / GUIDE_IN; in = i % GUIDE_IN; K = GUIDE_IN; base = TC_W1; }
        else if (i < GUIDE_W3) { layer = 1; o = (i - GUIDE_W2) / GUIDE_H; in = (i - GUIDE_W2) % GUIDE_H; K = 64; base = TC_W2; }
        else if (i < GUIDE_W4) { layer = 2; o = (i - GUIDE_W3) / GUIDE_H; in = (i - GUIDE_W3) % GUIDE_H; K = 64; base = TC_W3; }
        else if (i < GUIDE_NW) { layer = 3; o = (i - GUIDE_W4) / GUIDE_H; in = (i - GUIDE_W4) % GUIDE_H; K = 64; base = TC_W4; }
        else { layer = 3; o = GUIDE_OUT + (i - GUIDE_NW) / 64u; in = (i - GUIDE_NW) % 64u; K = 64; base = TC_W4; }
        if (i < GUIDE_NW) v = wbf[i];
        (void)layer;
        *reinterpret_cast<uint16_t*>(s + base + tc_off(o, in, K)) = v;
    }
}

// a row's 48 inputs: per level the trilinear blend of its 8 corners' two features, then the normal's harmonics
__device__ __forceinline__ void tc_row_input(const float2* __restrict__ table, f3 u, f3 n, float* x) {
#pragma unroll 4
    for (uint32_t l = 0; l < GUIDE_LEVELS; l++) {
        const GuideCorners c = guide_corners(u, l);
        float fx = 0.f, fy = 0.f;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const float2 e = __ldg(&table[c.idx[k]]);
            fx += c.w[k] * e.x;
            fy += c.w[k] * e.y;
        }
        x[2 * l] = fx;
        x[2 * l + 1] = fy;
    }
    guide_sh(n.x, n.y, n.z, x + 32);
}
// eight values, BF16, into the 16 bytes of row r, columns k0..k0+7 of the A tile
__device__ __forceinline__ void tc_put8(unsigned char* sA, uint32_t r, uint32_t k0, const float* x) {
    uint4 w;
    w.x = pack_bf16(x[0], x[1]);
    w.y = pack_bf16(x[2], x[3]);
    w.z = pack_bf16(x[4], x[5]);
    w.w = pack_bf16(x[6], x[7]);
    *reinterpret_cast<uint4*>(sA + tc_off(r, k0, 64u)) = w;
}

// THE NETWORK ON THE TILE: A holds every row's inputs; each thread gets its row's 40 outputs. All 128 threads call
// it. False if a layer's MMAs did not signal completion within the wait's limit (the error is the caller's to flag).
__device__ bool tc_network(unsigned char* s, uint32_t tmem, uint64_t* mbar, uint32_t& phase, uint32_t wait_limit,
                           float* y) {
    const uint32_t sbase = tc_smem(s);
    const uint32_t warp = threadIdx.x >> 5, row = threadIdx.x;
    const uint32_t wofs[4] = {TC_W1, TC_W2, TC_W3, TC_W4};
    const uint32_t Ks[4] = {GUIDE_IN, 64u, 64u, 64u};
    const uint32_t Ns[4] = {64u, 64u, 64u, 48u};
    uint32_t v[64];
#pragma unroll 1
    for (uint32_t layer = 0; layer < 4; layer++) {
        tc_fence_smem();                                // this thread's A rows, for the tensor cores to read
        tc_fence_before();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
            const uint32_t idesc = tc_idesc_bf16(128u, Ns[layer]);
            for (uint32_t k = 0; k < Ks[layer] / 16u; k++) {
                const uint64_t ad = tc_desc(sbase + TC_A + k * 256u, 128u, 64u * 16u);
                const uint64_t bd = tc_desc(sbase + wofs[layer] + k * 256u, 128u, Ks[layer] * 16u);
                tc_mma(tmem, ad, bd, idesc, k > 0 ? 1u : 0u);
            }
            tc_commit(mbar);
        }
        const bool ok = mbar_wait(mbar, phase, wait_limit);
        if (__syncthreads_or(!ok)) return false;
        phase ^= 1u;
        tc_fence_after();
        tc_ld64(tmem + ((warp * 32u) << 16), v);
        if (layer < 3u) {
#pragma unroll
            for (uint32_t j = 0; j < 64u; j += 8u) {
                float x[8];
#pragma unroll
                for (int q = 0; q < 8; q++) x[q] = fmaxf(__uint_as_float(v[j + q]), 0.f);
                tc_put8(s + TC_A, row, j, x);
            }
        } else {
#pragma unroll
            for (uint32_t j = 0; j < GUIDE_OUT; j++) y[j] = __uint_as_float(v[j]);
        }
        tc_fence_before();
    }
    return true;
}

// the CTA's set-up (tensor memory, the barrier, the weights) and its end (the memory freed); on a wait that ran out,
// the MMAs it gave up on waited for once more, bounded, before the memory goes
struct TcCta { uint32_t tmem, phase; };
__device__ __forceinline__ TcCta tc_begin(unsigned char* s, const uint16_t* wbf, uint32_t* tmem_slot, uint64_t* mbar) {
    tc_stage_weights(wbf, s);
    if (threadIdx.x < 32u) tc_alloc(tmem_slot, TC_COLS);
    if (threadIdx.x == 0) mbar_init(mbar, 1u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    return TcCta{*tmem_slot, 0u};
}
__device__ __forceinline__ void tc_end(TcCta& c, uint64_t* mbar, bool failed, DevCtr* ctr) {
    if (failed) {
        if (threadIdx.x == 0 && ctr) atomicExch(&ctr->errflag, 1u);
        mbar_wait(mbar, c.phase, WAIT_LIMIT);
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32u) {
        tc_fence_after();
        tc_dealloc(c.tmem, TC_COLS);
    }
}

// INFERENCE OVER THE HIT QUEUE: per round the block's 128 entries whose vertex is guided, compacted, one tile. ONE A
// PIXEL A WAVE: a pixel's paths meet their first vertices within its footprint, and the first of them to reach the
// network claims the pixel (its stamp) and has its mixture inferred there; the pixel's other paths sample from that
// mixture -- a density fixed before they draw, so the one-sample MIS estimator stays unbiased whichever vertex made it
// A CTA stages the weights and takes its tensor memory only at its first round with a vertex to infer: past the
// wave's first iterations most rounds find none (a pixel's mixture is made once), and such a CTA only scans.
__global__ void __launch_bounds__(128) k_guide_infer_tc(WaveArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ uint32_t list[128];
    __shared__ uint32_t wcnt[4];
    const Uni& u = a.u;
    unsigned char* s = smem;
    TcCta c{0u, 0u};
    bool begun = false;
    const uint32_t wl = a.ctr->wait_limit ? a.ctr->wait_limit : WAIT_LIMIT;
    const uint32_t count = a.ctr->hitCount;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    bool failed = false;
    for (uint32_t base = blockIdx.x * 128u; base < count; base += gridDim.x * 128u) {
        const uint32_t q = base + threadIdx.x;
        bool want = false;
        if (q < count) {
            const uint32_t slot = a.q.hit[q];
            const uint32_t my = a.pb.meta[slot].y;
            const uint32_t ids = __float_as_uint(a.q.hsurf[q].w);
            if (((my >> 16) & 0xffu) == RAY_ACTIVE && (my & 0xffu) == 0u && ids != SURF_LEAVING && a.q.hitd[q] >= 0.f &&
                guide_vertex(a.mats[min(ids & 0xffffu, u.n_mats - 1u)]))
                want = atomicExch(&a.gd.stamp[guide_pixel(u, slot, a.pb.meta[slot].x)], 1u) == 0u;
        }
        const uint32_t m = __ballot_sync(FULL_MASK, want);
        if (lane == 0u) wcnt[warp] = __popc(m);
        __syncthreads();
        uint32_t off = 0, n = 0;
        for (uint32_t w = 0; w < 4u; w++) { if (w < warp) off += wcnt[w]; n += wcnt[w]; }
        if (want) list[off + __popc(m & lanemask_lt())] = q;
        if (threadIdx.x == 0u && n) atomicAdd(&a.gd.dev->inferred, n);
        __syncthreads();
        if (n == 0u) continue;                                      // the whole block agrees
        if (!begun) {
            c = tc_begin(s, a.gd.wbf, &tmem_slot, &mbar);
            begun = true;
        }
        float x[GUIDE_IN];
        if (threadIdx.x < n) {
            const uint32_t qq = list[threadIdx.x];
            tc_row_input(a.gd.table, guide_unit(xyz(a.pb.pos[a.q.hit[qq]]), a.gd.lo, a.gd.inv_ext),
                         xyz(a.q.hsurf[qq]), x);
        } else {
            for (uint32_t j = 0; j < GUIDE_IN; j++) x[j] = 0.f;
        }
#pragma unroll
        for (uint32_t j = 0; j < GUIDE_IN; j += 8u) tc_put8(s + TC_A, threadIdx.x, j, x + j);
        float y[GUIDE_OUT];
        if (!tc_network(s, c.tmem, &mbar, c.phase, wl, y)) { failed = true; break; }
        if (threadIdx.x < n) {
            uint2 out[GUIDE_LOBES];
            guide_decode(y, out);
            const uint32_t sl = a.q.hit[list[threadIdx.x]];
            uint2* dst = a.gd.mix + (size_t)guide_pixel(u, sl, a.pb.meta[sl].x) * GUIDE_LOBES;
#pragma unroll
            for (uint32_t k = 0; k < GUIDE_LOBES; k++) dst[k] = out[k];
        }
    }
    if (begun) tc_end(c, &mbar, failed, a.ctr);
}

// THE NETWORK AT GIVEN POINTS (st_mlp_eval): the samples' positions and normals in, the 40 outputs and the mixture out
__global__ void __launch_bounds__(128) k_guide_eval_tc(const GuideSample* __restrict__ samp, uint32_t n, f3 lo,
                                                       float inv_ext, const float2* __restrict__ table,
                                                       const uint16_t* __restrict__ wbf, float* __restrict__ raw,
                                                       uint2* __restrict__ mix, uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    unsigned char* s = smem;
    TcCta c = tc_begin(s, wbf, &tmem_slot, &mbar);
    bool failed = false;
    for (uint32_t base = blockIdx.x * 128u; base < n; base += gridDim.x * 128u) {
        const uint32_t r = base + threadIdx.x;
        float x[GUIDE_IN];
        if (r < n) tc_row_input(table, guide_unit(xyz(samp[r].a), lo, inv_ext), xyz(samp[r].b), x);
        else for (uint32_t j = 0; j < GUIDE_IN; j++) x[j] = 0.f;
#pragma unroll
        for (uint32_t j = 0; j < GUIDE_IN; j += 8u) tc_put8(s + TC_A, threadIdx.x, j, x + j);
        float y[GUIDE_OUT];
        if (!tc_network(s, c.tmem, &mbar, c.phase, WAIT_LIMIT, y)) { failed = true; break; }
        if (r < n) {
            for (uint32_t k = 0; k < GUIDE_OUT; k++) raw[(size_t)r * GUIDE_OUT + k] = y[k];
            uint2 out[GUIDE_LOBES];
            guide_decode(y, out);
            for (uint32_t k = 0; k < GUIDE_LOBES; k++) mix[(size_t)r * GUIDE_LOBES + k] = out[k];
        }
    }
    if (failed && threadIdx.x == 0) atomicExch(err, 1u);
    tc_end(c, &mbar, failed, nullptr);
}

static size_t tc_infer_smem(uint32_t) { return TC_BYTES; }

cudaError_t launch_guide_infer(const WaveArgs& a, int sms, cudaStream_t s) {
    const size_t smem = tc_infer_smem(a.u.n_mats);
    cudaFuncSetAttribute(k_guide_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_guide_infer_tc, 128, smem);
    // at least what the registers (128 threads x 128) and the shared memory allow, 4 CTAs an SM with a small table of
    // materials; at most 512 / TC_COLS CTAs an SM hold tensor memory at once (an allocation beyond that would wait).
    // A CTA's rounds are its own (by blockIdx), so a CTA that has to wait for room only starts later
    nb = std::max(nb, std::min(4, (int)((228u << 10) / (smem + 1024u))));
    nb = std::min(std::max(nb, 1), (int)(512u / TC_COLS));
    k_guide_infer_tc<<<sms * nb, 128, smem, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_guide_eval_tc(const GuideSample* samp, uint32_t n, f3 lo, float inv_ext, const float2* table,
                                 const uint16_t* wbf, float* raw, uint2* mix, uint32_t* err, int sms, cudaStream_t s) {
    cudaFuncSetAttribute(k_guide_eval_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_BYTES);
    const uint32_t blocks = std::max(1u, std::min((n + 127u) / 128u, (uint32_t)sms * 2u));
    k_guide_eval_tc<<<blocks, 128, TC_BYTES, s>>>(samp, n, lo, inv_ext, table, wbf, raw, mix, err);
    return cudaGetLastError();
}

}  // namespace st
