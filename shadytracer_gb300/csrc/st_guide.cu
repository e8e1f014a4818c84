// st_guide.cu -- THE LEARNED PROPOSAL: the network's inference over a wavefront iteration's hit queue, the training
// batch made from the camera paths' records at a wave's end, and the training step (forward and backward on the
// tensor cores, the weight gradients as one GEMM over the batch, Adam), with the C ABI's st_mlp_* entry points.
//
//   k_guide_infer     after the surface kernel: one mixture (8 packed vMF lobes) a pixel a wave, at its first guided vertex
//   k_guide_collect   a wave's end: each path's record -> (position, normal, direction, f cos L_in / pdf)
//   k_guide_train     a mini-batch: forward, the loss's gradient at the 40 outputs, backward to the 48 inputs; the
//                     activations and their gradients (BF16) for the weight GEMM; the hash grid's gradient by atomics
//   k_guide_dw        dW_l = dZ_l^T A_l over the mini-batch (K = samples), split over the blocks, FP32 atomics
//   k_guide_adam      Adam on the FP32 weights and features; the BF16 copy the kernels read
//
// THE LOSS. A record at vertex x, direction w drawn with density p, and the luminance the path collected after the
// bounce over the throughput that reached x -- which is f(w) cos(w) L_in(w) / p(w), the integrand over the density
// -- is one Monte-Carlo sample of the light the vertex reflects from w; the network's mixture q is fitted to that
// integrand by minimising E[-(f cos L_in / p) log q(w)], the cross entropy of q against the normalised integrand
// (the KL divergence up to a constant: the density that would make the vertex's estimate noise-free), each weight
// over the batch's mean and capped at GUIDE_WCAP.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/shadytracer.h"
#include "st_ext.h"
#include "st_guide.cuh"
#include "st_internal.h"
#include "st_kernels.cuh"

namespace st {

#define GUIDE_MB 16384u                 // samples a training step
#define GUIDE_STEPS 8u                  // training steps a wave
#define GUIDE_CAP (GUIDE_MB * GUIDE_STEPS)
#define GUIDE_WCAP 1000.f
#define GUIDE_ACT 8u                    // activation arrays of a mini-batch: X H1 H2 H3 dY dH3 dH2 dH1
#define GUIDE_ACT_LD 64u
// the weights in shared memory: forward W1 [64][56], W2 [64][72], W3 [64][72], W4 [40][72]; the training kernel
// adds the transposes W1T [48][72], W2T [64][72], W3T [64][72], W4T [64][56] (W4T's columns 40-47 zero)
#define SW1 0u
#define SW2 (SW1 + GUIDE_H * GUIDE_LD_IN)
#define SW3 (SW2 + GUIDE_H * GUIDE_LD_H)
#define SW4 (SW3 + GUIDE_H * GUIDE_LD_H)
#define SW_FWD (SW4 + GUIDE_OUT * GUIDE_LD_H)
#define SW1T SW_FWD
#define SW2T (SW1T + GUIDE_IN * GUIDE_LD_H)
#define SW3T (SW2T + GUIDE_H * GUIDE_LD_H)
#define SW4T (SW3T + GUIDE_H * GUIDE_LD_H)
#define SW_ALL (SW4T + GUIDE_H * GUIDE_LD_IN)

// the weights from their BF16 copy in global memory into padded rows (and, for training, the transposes)
__device__ void guide_stage_weights(const uint16_t* __restrict__ wbf, uint16_t* sw, bool transposes) {
    for (uint32_t i = threadIdx.x; i < GUIDE_NW; i += blockDim.x) {
        const uint16_t v = wbf[i];
        uint32_t layer, o, in, n_in;
        if (i < GUIDE_W2) { layer = 0; o = i / GUIDE_IN; in = i % GUIDE_IN; n_in = GUIDE_IN; }
        else if (i < GUIDE_W3) { layer = 1; o = (i - GUIDE_W2) / GUIDE_H; in = (i - GUIDE_W2) % GUIDE_H; n_in = GUIDE_H; }
        else if (i < GUIDE_W4) { layer = 2; o = (i - GUIDE_W3) / GUIDE_H; in = (i - GUIDE_W3) % GUIDE_H; n_in = GUIDE_H; }
        else { layer = 3; o = (i - GUIDE_W4) / GUIDE_H; in = (i - GUIDE_W4) % GUIDE_H; n_in = GUIDE_H; }
        const uint32_t ld = n_in == GUIDE_IN ? GUIDE_LD_IN : GUIDE_LD_H;
        const uint32_t base = layer == 0 ? SW1 : layer == 1 ? SW2 : layer == 2 ? SW3 : SW4;
        sw[base + o * ld + in] = v;
        if (transposes) {
            // W^T [in][out]: W1T, W2T, W3T with rows of GUIDE_LD_H; W4T with rows of GUIDE_LD_IN (48 + 8)
            const uint32_t tb = layer == 0 ? SW1T : layer == 1 ? SW2T : layer == 2 ? SW3T : SW4T;
            const uint32_t tld = layer == 3 ? GUIDE_LD_IN : GUIDE_LD_H;
            sw[tb + in * tld + o] = v;
        }
    }
    if (transposes)   // W4T's columns 40-47: zero (dY is padded to 48 columns)
        for (uint32_t i = threadIdx.x; i < GUIDE_H * 8u; i += blockDim.x)
            sw[SW4T + (i / 8u) * GUIDE_LD_IN + GUIDE_OUT + (i % 8u)] = 0;
}

// the forward pass of a warp's 16 rows from their input fragments to the 40 outputs (C tiles), keeping the hidden
// layers' A fragments for the backward pass
struct GuideFwd { uint32_t h1[4][4], h2[4][4], h3[4][4]; float o[5][4]; };
__device__ __forceinline__ void guide_forward(const uint32_t (*a_in)[4], const __nv_bfloat16* sw, uint32_t g,
                                              uint32_t t, GuideFwd& f) {
    float c[8][4];
    guide_layer<8, 3>(a_in, sw + SW1, GUIDE_LD_IN, g, t, c);
    relu_to_a<4>(c, f.h1);
    guide_layer<8, 4>(f.h1, sw + SW2, GUIDE_LD_H, g, t, c);
    relu_to_a<4>(c, f.h2);
    guide_layer<8, 4>(f.h2, sw + SW3, GUIDE_LD_H, g, t, c);
    relu_to_a<4>(c, f.h3);
    guide_layer<5, 4>(f.h3, sw + SW4, GUIDE_LD_H, g, t, f.o);
}
// C tiles of 16 x 40 into a row-major [16][40] FP32 scratch
__device__ __forceinline__ void store_out(const float (*o)[4], float* ws, uint32_t g, uint32_t t) {
#pragma unroll
    for (int j = 0; j < 5; j++) {
        ws[g * GUIDE_OUT + 8 * j + 2 * t] = o[j][0];
        ws[g * GUIDE_OUT + 8 * j + 2 * t + 1] = o[j][1];
        ws[(g + 8) * GUIDE_OUT + 8 * j + 2 * t] = o[j][2];
        ws[(g + 8) * GUIDE_OUT + 8 * j + 2 * t + 1] = o[j][3];
    }
}

// ---------------------------------------------------------------------------------------------------------------
// THE BATCH: a wave's records, a hashed subsample of about GUIDE_CAP of them, each with the luminance found after it
// ---------------------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_guide_collect(WaveArgs a) {
    const uint32_t sample = a.ctr->sample;
    float wsum = 0.f;
    for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < a.slots; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + (threadIdx.x & 31u);
        bool take = false;
        GuideRec r;
        if (i < a.slots) {
            r = a.gd.rec[i];
            uint32_t h = i * 0x9E3779B1u ^ (sample * 0x85EBCA77u + 0x165667B1u);
            h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
            take = r.a.w > 0.f && h < a.gd.keep;
        }
        const uint32_t at = warp_append(&a.gd.dev->count, take);
        if (take && at < a.gd.cap) {
            const float W = fmaxf(a.gd.acc[i], 0.f) / fmaxf(r.b.z, 1e-30f);    // f cos L_in / p
            GuideSample s;
            s.a = make_float4(r.a.x, r.a.y, r.a.z, W);
            const f3 nn = guide_unoct16(__float_as_uint(r.b.x)), d = guide_unoct16(__float_as_uint(r.b.y));
            s.b = make_float4(nn.x, nn.y, nn.z, 0.f);
            s.c = make_float4(d.x, d.y, d.z, 0.f);
            a.gd.samp[at] = s;
            wsum += W;
        }
    }
    for (int o = 16; o > 0; o >>= 1) wsum += __shfl_down_sync(FULL_MASK, wsum, o);
    if ((threadIdx.x & 31u) == 0u && wsum > 0.f) atomicAdd(&a.gd.dev->wsum, wsum);
}

// ---------------------------------------------------------------------------------------------------------------
// TRAINING
// ---------------------------------------------------------------------------------------------------------------
struct GuideTrain {
    const GuideSample* samp;
    GuideDev* dev;
    uint32_t first;          // the mini-batch's first sample
    f3 lo; float inv_ext;
    const float2* table;
    float2* gtable;          // the features' gradient
    const uint16_t* wbf;
    uint16_t* act;           // [GUIDE_ACT][GUIDE_MB][GUIDE_ACT_LD] BF16
    float* gw;               // the weights' gradient (GUIDE_NW)
};
__device__ __forceinline__ uint32_t guide_batch_n(const GuideDev* dev, uint32_t first) {
    const uint32_t c = min(dev->count, GUIDE_CAP);
    return c > first ? min(c - first, GUIDE_MB) : 0u;
}
// an A fragment's four words into rows r0 (g) and r0 + 8 of an activation array
__device__ __forceinline__ void store_frag(uint16_t* arr, uint32_t row, uint32_t col, const uint32_t* a) {
    uint32_t* p0 = reinterpret_cast<uint32_t*>(arr + (size_t)row * GUIDE_ACT_LD + col);
    uint32_t* p1 = reinterpret_cast<uint32_t*>(arr + (size_t)(row + 8u) * GUIDE_ACT_LD + col);
    p0[0] = a[0];
    p1[0] = a[1];
    p0[4] = a[2];            // col + 8
    p1[4] = a[3];
}
// the gradient's C tiles masked by the layer's ReLU (its A fragments) into A fragments
template <int KT>
__device__ __forceinline__ void masked_to_a(const float (*c)[4], const uint32_t (*h)[4], uint32_t (*d)[4]) {
#pragma unroll
    for (int kt = 0; kt < KT; kt++) {
#pragma unroll
        for (int hi = 0; hi < 2; hi++) {
            const float* cc = c[2 * kt + hi];
            const uint32_t r0 = h[kt][2 * hi], r1 = h[kt][2 * hi + 1];
            d[kt][2 * hi] = pack_bf16(bf16_lo(r0) > 0.f ? cc[0] : 0.f, bf16_hi(r0) > 0.f ? cc[1] : 0.f);
            d[kt][2 * hi + 1] = pack_bf16(bf16_lo(r1) > 0.f ? cc[2] : 0.f, bf16_hi(r1) > 0.f ? cc[3] : 0.f);
        }
    }
}

// the loss's gradient at one sample's 40 outputs (in place), returning its loss
__device__ float guide_loss_grad(float* y, f3 d, float w) {
    float mx = -1e30f;
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) mx = fmaxf(mx, y[5 * k + 4]);
    float pi[GUIDE_LOBES], lv[GUIDE_LOBES], kap[GUIDE_LOBES], cs[GUIDE_LOBES], len[GUIDE_LOBES], s = 0.f;
    f3 mu[GUIDE_LOBES];
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) { pi[k] = expf(y[5 * k + 4] - mx); s += pi[k]; }
    float lmax = -1e30f;
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) {
        pi[k] /= s;
        const f3 m = mk(y[5 * k], y[5 * k + 1], y[5 * k + 2]);
        len[k] = fmaxf(sqrtf(m.x * m.x + m.y * m.y + m.z * m.z), 1e-12f);
        mu[k] = m / len[k];
        kap[k] = expf(fminf(fmaxf(y[5 * k + 3], GUIDE_KLO), GUIDE_KHI));
        cs[k] = dot(mu[k], d);
        // log of the vMF density: log kappa - log 2pi - log(1 - e^-2kappa) + kappa (cos - 1)
        lv[k] = logf(kap[k]) - logf(2.f * ST_PI) - log1pf(-expf(-2.f * kap[k])) + kap[k] * (cs[k] - 1.f) + logf(pi[k]);
        lmax = fmaxf(lmax, lv[k]);
    }
    float acc = 0.f;
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) acc += expf(lv[k] - lmax);
    const float lq = lmax + logf(acc);
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) {
        const float r = expf(lv[k] - lq);                               // the lobe's responsibility
        const float e2 = expf(-2.f * kap[k]);
        const float dk = 1.f / kap[k] - 2.f * e2 / (1.f - e2) + (cs[k] - 1.f);
        const float kr = y[5 * k + 3];
        const float inr = (kr > GUIDE_KLO && kr < GUIDE_KHI) ? 1.f : 0.f;
        const float gm = -w * r * kap[k] / len[k];
        y[5 * k] = gm * (d.x - mu[k].x * cs[k]);
        y[5 * k + 1] = gm * (d.y - mu[k].y * cs[k]);
        y[5 * k + 2] = gm * (d.z - mu[k].z * cs[k]);
        y[5 * k + 3] = -w * r * dk * kap[k] * inr;
        y[5 * k + 4] = -w * (r - pi[k]);
    }
    return -w * lq;
}

__global__ void __launch_bounds__(256) k_guide_train(GuideTrain tr) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ float ws_all[8][16 * GUIDE_OUT];
    uint16_t* sw = reinterpret_cast<uint16_t*>(smem);
    const uint32_t n = guide_batch_n(tr.dev, tr.first);
    if (n == 0u) return;
    guide_stage_weights(tr.wbf, sw, true);
    __syncthreads();
    const __nv_bfloat16* swb = reinterpret_cast<const __nv_bfloat16*>(sw);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3u;
    float* ws = ws_all[warp];
    const float mean = tr.dev->wsum / (float)max(min(tr.dev->count, GUIDE_CAP), 1u);
    const float inv_mean = mean > 0.f ? 1.f / mean : 0.f;
    const uint32_t tiles = (n + 15u) / 16u;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    float loss = 0.f, nl = 0.f;
    for (uint32_t tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile < tiles; tile += nwarps) {
        const uint32_t r0 = tile * 16u + g, r1 = r0 + 8u;           // rows of the mini-batch
        f3 u0 = mk(0.5f), u1 = mk(0.5f), n0 = mk(0.f, 0.f, 1.f), n1 = mk(0.f, 0.f, 1.f);
        if (r0 < n) {
            const GuideSample s = tr.samp[tr.first + r0];
            u0 = guide_unit(xyz(s.a), tr.lo, tr.inv_ext);
            n0 = xyz(s.b);
        }
        if (r1 < n) {
            const GuideSample s = tr.samp[tr.first + r1];
            u1 = guide_unit(xyz(s.a), tr.lo, tr.inv_ext);
            n1 = xyz(s.b);
        }
        uint32_t a_in[3][4];
        guide_input(tr.table, u0, n0, u1, n1, t, a_in);
        GuideFwd f;
        guide_forward(a_in, swb, g, t, f);
        store_out(f.o, ws, g, t);
        __syncwarp();
        if (lane < 16u) {
            const uint32_t r = tile * 16u + lane;
            float* y = ws + lane * GUIDE_OUT;
            if (r < n) {
                const GuideSample s = tr.samp[tr.first + r];
                const float w = fminf(s.a.w * inv_mean, GUIDE_WCAP);
                loss += guide_loss_grad(y, xyz(s.c), w);
                nl += 1.f;
            } else {
                for (uint32_t k = 0; k < GUIDE_OUT; k++) y[k] = 0.f;
            }
        }
        __syncwarp();
        // dY as A fragments (48 columns, 40-47 zero)
        uint32_t a_dy[3][4];
#pragma unroll
        for (uint32_t kt = 0; kt < 3; kt++) {
            const uint32_t c0 = 16u * kt + 2u * t, c1 = c0 + 8u;
            a_dy[kt][0] = c0 < GUIDE_OUT ? pack_bf16(ws[g * GUIDE_OUT + c0], ws[g * GUIDE_OUT + c0 + 1]) : 0u;
            a_dy[kt][1] = c0 < GUIDE_OUT ? pack_bf16(ws[(g + 8) * GUIDE_OUT + c0], ws[(g + 8) * GUIDE_OUT + c0 + 1]) : 0u;
            a_dy[kt][2] = c1 < GUIDE_OUT ? pack_bf16(ws[g * GUIDE_OUT + c1], ws[g * GUIDE_OUT + c1 + 1]) : 0u;
            a_dy[kt][3] = c1 < GUIDE_OUT ? pack_bf16(ws[(g + 8) * GUIDE_OUT + c1], ws[(g + 8) * GUIDE_OUT + c1 + 1]) : 0u;
        }
        __syncwarp();
        // backward: dH3 = dY W4, dH2 = dH3 W3, dH1 = dH2 W2 (each masked by its ReLU), dX = dH1 W1
        float c[8][4];
        uint32_t d3[4][4], d2[4][4], d1[4][4];
        guide_layer<8, 3>(a_dy, swb + SW4T, GUIDE_LD_IN, g, t, c);
        masked_to_a<4>(c, f.h3, d3);
        guide_layer<8, 4>(d3, swb + SW3T, GUIDE_LD_H, g, t, c);
        masked_to_a<4>(c, f.h2, d2);
        guide_layer<8, 4>(d2, swb + SW2T, GUIDE_LD_H, g, t, c);
        masked_to_a<4>(c, f.h1, d1);
        float dx[6][4];
        guide_layer<6, 4>(d1, swb + SW1T, GUIDE_LD_H, g, t, dx);
        // the activations and their gradients for the weight GEMM (rows past n: their dZ is zero)
        const uint32_t row = tile * 16u + g;
        const size_t A = (size_t)GUIDE_MB * GUIDE_ACT_LD;
#pragma unroll
        for (uint32_t kt = 0; kt < 4; kt++) {
            if (kt < 3) store_frag(tr.act + 0 * A, row, 16u * kt + 2u * t, a_in[kt]);
            store_frag(tr.act + 1 * A, row, 16u * kt + 2u * t, f.h1[kt]);
            store_frag(tr.act + 2 * A, row, 16u * kt + 2u * t, f.h2[kt]);
            store_frag(tr.act + 3 * A, row, 16u * kt + 2u * t, f.h3[kt]);
            if (kt < 3) store_frag(tr.act + 4 * A, row, 16u * kt + 2u * t, a_dy[kt]);
            store_frag(tr.act + 5 * A, row, 16u * kt + 2u * t, d3[kt]);
            store_frag(tr.act + 6 * A, row, 16u * kt + 2u * t, d2[kt]);
            store_frag(tr.act + 7 * A, row, 16u * kt + 2u * t, d1[kt]);
        }
        // the hash grid's gradient: this lane's levels 4j + t (features 8j + 2t, +1) of rows g and g+8
#pragma unroll
        for (uint32_t j = 0; j < 4; j++) {
#pragma unroll
            for (uint32_t half = 0; half < 2; half++) {
                const uint32_t r = half ? r1 : r0;
                if (r >= n) continue;
                const float gx = dx[j][2 * half], gy = dx[j][2 * half + 1];
                if (gx == 0.f && gy == 0.f) continue;
                const GuideCorners cc = guide_corners(half ? u1 : u0, 4u * j + t);
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    atomicAdd(&tr.gtable[cc.idx[k]].x, cc.w[k] * gx);
                    atomicAdd(&tr.gtable[cc.idx[k]].y, cc.w[k] * gy);
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        loss += __shfl_down_sync(FULL_MASK, loss, o);
        nl += __shfl_down_sync(FULL_MASK, nl, o);
    }
    if (lane == 0u && nl > 0.f) {
        atomicAdd(&tr.dev->loss, loss);
        atomicAdd(&tr.dev->loss_n, nl);
    }
}

// THE WEIGHT GRADIENTS: the 112 16 x 8 tiles of dW1 (64 x 48), dW2, dW3 (64 x 64) and dW4 (40 x 64, as 48 rows),
// 14 a warp; K the mini-batch's rows, 16 a step, staged in shared memory
#define DW_FRAGS 112u
__global__ void __launch_bounds__(256) k_guide_dw(const GuideDev* __restrict__ dev, uint32_t first,
                                                  const uint16_t* __restrict__ act, float* __restrict__ gw) {
    __shared__ __align__(16) uint16_t tile[GUIDE_ACT][16][GUIDE_ACT_LD];
    const uint32_t n = guide_batch_n(dev, first);
    if (n == 0u) return;
    const uint32_t tiles = (n + 15u) / 16u;
    const uint32_t t0 = (uint32_t)(((unsigned long long)tiles * blockIdx.x) / gridDim.x);
    const uint32_t t1 = (uint32_t)(((unsigned long long)tiles * (blockIdx.x + 1u)) / gridDim.x);
    if (t0 == t1) return;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3u;
    float c[14][4];
#pragma unroll
    for (int f = 0; f < 14; f++) c[f][0] = c[f][1] = c[f][2] = c[f][3] = 0.f;
    const size_t A = (size_t)GUIDE_MB * GUIDE_ACT_LD;
    for (uint32_t tl = t0; tl < t1; tl++) {
        // stage the 8 arrays' 16 rows: 8 x 16 x 128 B, 16 bytes a thread-load
        for (uint32_t i = threadIdx.x; i < GUIDE_ACT * 16u * (GUIDE_ACT_LD / 8u); i += blockDim.x) {
            const uint32_t arr = i / (16u * (GUIDE_ACT_LD / 8u)), rem = i % (16u * (GUIDE_ACT_LD / 8u));
            const uint32_t r = rem / (GUIDE_ACT_LD / 8u), c8 = rem % (GUIDE_ACT_LD / 8u);
            reinterpret_cast<uint4*>(&tile[arr][r][0])[c8] =
                reinterpret_cast<const uint4*>(act + arr * A + (size_t)(tl * 16u + r) * GUIDE_ACT_LD)[c8];
        }
        __syncthreads();
#pragma unroll
        for (uint32_t fi = 0; fi < 14; fi++) {
            const uint32_t fr = warp * 14u + fi;
            uint32_t dz, aa, mt, nt;
            if (fr < 24u) { dz = 7; aa = 0; mt = fr / 6u; nt = fr % 6u; }
            else if (fr < 56u) { dz = 6; aa = 1; mt = (fr - 24u) / 8u; nt = (fr - 24u) % 8u; }
            else if (fr < 88u) { dz = 5; aa = 2; mt = (fr - 56u) / 8u; nt = (fr - 56u) % 8u; }
            else { dz = 4; aa = 3; mt = (fr - 88u) / 8u; nt = (fr - 88u) % 8u; }
            const uint16_t(*Z)[GUIDE_ACT_LD] = tile[dz];
            const uint16_t(*X)[GUIDE_ACT_LD] = tile[aa];
            const uint32_t o0 = 16u * mt, i0 = 8u * nt;
            uint32_t af[4];
            af[0] = (uint32_t)Z[2 * t][o0 + g] | ((uint32_t)Z[2 * t + 1][o0 + g] << 16);
            af[1] = (uint32_t)Z[2 * t][o0 + g + 8] | ((uint32_t)Z[2 * t + 1][o0 + g + 8] << 16);
            af[2] = (uint32_t)Z[2 * t + 8][o0 + g] | ((uint32_t)Z[2 * t + 9][o0 + g] << 16);
            af[3] = (uint32_t)Z[2 * t + 8][o0 + g + 8] | ((uint32_t)Z[2 * t + 9][o0 + g + 8] << 16);
            const uint32_t b0 = (uint32_t)X[2 * t][i0 + g] | ((uint32_t)X[2 * t + 1][i0 + g] << 16);
            const uint32_t b1 = (uint32_t)X[2 * t + 8][i0 + g] | ((uint32_t)X[2 * t + 9][i0 + g] << 16);
            mma_bf16(c[fi], af, b0, b1);
        }
        __syncthreads();
    }
#pragma unroll
    for (uint32_t fi = 0; fi < 14; fi++) {
        const uint32_t fr = warp * 14u + fi;
        uint32_t off, ins, outs, mt, nt;
        if (fr < 24u) { off = GUIDE_W1; ins = GUIDE_IN; outs = GUIDE_H; mt = fr / 6u; nt = fr % 6u; }
        else if (fr < 56u) { off = GUIDE_W2; ins = GUIDE_H; outs = GUIDE_H; mt = (fr - 24u) / 8u; nt = (fr - 24u) % 8u; }
        else if (fr < 88u) { off = GUIDE_W3; ins = GUIDE_H; outs = GUIDE_H; mt = (fr - 56u) / 8u; nt = (fr - 56u) % 8u; }
        else { off = GUIDE_W4; ins = GUIDE_H; outs = GUIDE_OUT; mt = (fr - 88u) / 8u; nt = (fr - 88u) % 8u; }
        const uint32_t oa = 16u * mt + g, ob = oa + 8u, i = 8u * nt + 2u * t;
        if (oa < outs) { atomicAdd(&gw[off + oa * ins + i], c[fi][0]); atomicAdd(&gw[off + oa * ins + i + 1], c[fi][1]); }
        if (ob < outs) { atomicAdd(&gw[off + ob * ins + i], c[fi][2]); atomicAdd(&gw[off + ob * ins + i + 1], c[fi][3]); }
    }
}

// one Adam step: the mini-batch's mean gradient; the BF16 copy of the weights rewritten; the gradients cleared
__global__ void k_guide_step(GuideDev* dev, uint32_t first) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && guide_batch_n(dev, first) > 0u) dev->step += 1u;
}
__global__ void __launch_bounds__(256) k_guide_adam(const GuideDev* __restrict__ dev, uint32_t first, float lr,
                                                    float* __restrict__ param, float* __restrict__ grad,
                                                    float* __restrict__ m1, float* __restrict__ m2,
                                                    uint16_t* __restrict__ wbf) {
    const uint32_t n = guide_batch_n(dev, first);
    if (n == 0u) return;
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-10f;
    const float tt = (float)dev->step;
    const float c1 = 1.f - powf(b1, tt), c2 = 1.f - powf(b2, tt);
    const float inv_n = 1.f / (float)n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < GUIDE_NPARAM; i += gridDim.x * blockDim.x) {
        const float gr = grad[i] * inv_n;
        grad[i] = 0.f;
        const float a = b1 * m1[i] + (1.f - b1) * gr, b = b2 * m2[i] + (1.f - b2) * gr * gr;
        m1[i] = a;
        m2[i] = b;
        const float p = param[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        param[i] = p;
        if (i < GUIDE_NW) {
            const __nv_bfloat16 h = __float2bfloat16_rn(p);
            wbf[i] = *reinterpret_cast<const uint16_t*>(&h);
        }
    }
}
// the BF16 copy from the FP32 weights (after an upload)
__global__ void k_guide_cast(const float* __restrict__ param, uint16_t* __restrict__ wbf) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < GUIDE_NW; i += gridDim.x * blockDim.x) {
        const __nv_bfloat16 h = __float2bfloat16_rn(param[i]);
        wbf[i] = *reinterpret_cast<const uint16_t*>(&h);
    }
}

cudaError_t launch_guide_collect(const WaveArgs& a, int sms, cudaStream_t s) {
    k_guide_collect<<<sms * 8, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace st

using namespace st;

// ---------------------------------------------------------------------------------------------------------------
// HOST: the proposal's buffers in a context, its initialisation, the training chain, the C ABI
// ---------------------------------------------------------------------------------------------------------------
static uint32_t pcg_next(uint64_t& s) {
    const uint64_t old = s;
    s = old * 6364136223846793005ull + 1442695040888963407ull;
    const uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u), r = (uint32_t)(old >> 59u);
    return (x >> r) | (x << ((32u - r) & 31u));
}
// the initial weights: each matrix uniform in +-sqrt(6 / (fan_in + fan_out)) (the last a tenth of that, so the first
// mixture is broad and even), the features uniform in +-1e-4; a PCG32 stream from the seed
void guide_init_weights(uint32_t seed, float* p) {
    uint64_t s = 0x853c49e6748fea9bull ^ ((uint64_t)seed << 1);
    auto uni = [&](float a) { return a * (2.f * (float)(pcg_next(s) >> 8) * (1.f / 16777216.f) - 1.f); };
    const struct { uint32_t off, in, out; float k; } L[4] = {{GUIDE_W1, GUIDE_IN, GUIDE_H, 1.f}, {GUIDE_W2, GUIDE_H, GUIDE_H, 1.f},
                                                              {GUIDE_W3, GUIDE_H, GUIDE_H, 1.f}, {GUIDE_W4, GUIDE_H, GUIDE_OUT, 0.1f}};
    for (const auto& l : L) {
        const float a = l.k * std::sqrt(6.f / (float)(l.in + l.out));
        for (uint32_t i = 0; i < l.in * l.out; i++) p[l.off + i] = uni(a);
    }
    for (uint32_t i = 0; i < GUIDE_NHASH; i++) p[GUIDE_NW + i] = uni(1e-4f);
}

int guide_ensure(st_ctx* ctx, uint32_t queue_cap, uint32_t slots, uint32_t seed) {
    GuideState& g = ctx_ext(ctx).guide;
    auto fail = [&](const char* what) { ctx_set_error(ctx, what); return ST_ERR_OOM; };
    cudaStream_t st = ctx_stream(ctx);
    if (!g.param) {
        if (cudaMalloc(&g.param, (size_t)GUIDE_NPARAM * 4) || cudaMalloc(&g.grad, (size_t)GUIDE_NPARAM * 4) ||
            cudaMalloc(&g.m1, (size_t)GUIDE_NPARAM * 4) || cudaMalloc(&g.m2, (size_t)GUIDE_NPARAM * 4) ||
            cudaMalloc(&g.wbf, (size_t)GUIDE_NW * 2) || cudaMalloc(&g.dev, sizeof(GuideDev)) ||
            cudaMalloc(&g.samp, (size_t)GUIDE_CAP * sizeof(GuideSample)) ||
            cudaMalloc(&g.act, (size_t)GUIDE_ACT * GUIDE_MB * GUIDE_ACT_LD * 2))
            return fail("cudaMalloc learned proposal");
        g.seed = seed + 1u;   // differs from any seed, so the weights are drawn below
    }
    if (g.seed != seed) {
        std::vector<float> h(GUIDE_NPARAM);
        guide_init_weights(seed, h.data());
        if (guide_upload(ctx, h.data())) return ST_ERR_CUDA;
        g.seed = seed;
    }
    if (queue_cap > g.mix_cap) {
        if (g.mix) cudaFree(g.mix);
        if (g.stamp) cudaFree(g.stamp);
        g.mix = nullptr;
        g.stamp = nullptr;
        g.mix_cap = 0;
        if (cudaMalloc(&g.mix, (size_t)queue_cap * GUIDE_LOBES * sizeof(uint2)) ||
            cudaMalloc(&g.stamp, (size_t)queue_cap * 4) ||
            cudaMemset(g.mix, 0, (size_t)queue_cap * GUIDE_LOBES * sizeof(uint2)) ||
            cudaMemset(g.stamp, 0, (size_t)queue_cap * 4))
            return fail("cudaMalloc learned proposal");
        g.mix_cap = queue_cap;
    }
    if (slots > g.rec_cap) {
        if (g.rec) cudaFree(g.rec);
        if (g.acc) cudaFree(g.acc);
        g.rec = nullptr; g.acc = nullptr; g.rec_cap = 0;
        if (cudaMalloc(&g.rec, (size_t)slots * sizeof(GuideRec)) || cudaMalloc(&g.acc, (size_t)slots * 4))
            return fail("cudaMalloc learned proposal");
        g.rec_cap = slots;
    }
    (void)st;
    return ST_OK;
}
// the FP32 weights and features from the host, the moments and gradients cleared, the BF16 copy made
int guide_upload(st_ctx* ctx, const float* h) {
    GuideState& g = ctx_ext(ctx).guide;
    cudaStream_t st = ctx_stream(ctx);
    cudaError_t e = cudaMemcpyAsync(g.param, h, (size_t)GUIDE_NPARAM * 4, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemsetAsync(g.grad, 0, (size_t)GUIDE_NPARAM * 4, st);
    if (!e) e = cudaMemsetAsync(g.m1, 0, (size_t)GUIDE_NPARAM * 4, st);
    if (!e) e = cudaMemsetAsync(g.m2, 0, (size_t)GUIDE_NPARAM * 4, st);
    if (!e) e = cudaMemsetAsync(g.dev, 0, sizeof(GuideDev), st);
    if (!e) { k_guide_cast<<<64, 256, 0, st>>>(g.param, g.wbf); e = cudaGetLastError(); }
    if (!e) e = cudaStreamSynchronize(st);
    if (e) { ctx_set_error(ctx, std::string("learned proposal upload: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
    return ST_OK;
}
GuideBufs guide_bufs(st_ctx* ctx, uint32_t on, uint32_t train, float alpha, uint32_t slots) {
    GuideState& g = ctx_ext(ctx).guide;
    GuideBufs b;
    b.on = on;
    b.train = train;
    b.alpha = alpha;
    guide_box(ctx, b.lo, b.inv_ext);
    b.table = reinterpret_cast<const float2*>(g.param + GUIDE_NW);
    b.wbf = g.wbf;
    b.mix = g.mix;
    b.stamp = g.stamp;
    b.rec = g.rec;
    b.acc = g.acc;
    b.samp = g.samp;
    b.dev = g.dev;
    b.cap = GUIDE_CAP;
    const double f = std::min(1.0, (double)GUIDE_CAP / std::max(slots, 1u));
    b.keep = f >= 1.0 ? 0xffffffffu : (uint32_t)(f * 4294967296.0);
    return b;
}
// a wave's start with guiding on: no pixel's mixture inferred yet
cudaError_t guide_stamps_clear(st_ctx* ctx, uint32_t pixels, cudaStream_t st) {
    GuideState& g = ctx_ext(ctx).guide;
    return cudaMemsetAsync(g.stamp, 0, (size_t)std::min(pixels, g.mix_cap) * 4, st);
}
// a wave's start: the records cleared, the batch emptied
cudaError_t guide_wave_begin(st_ctx* ctx, uint32_t slots, cudaStream_t st) {
    GuideState& g = ctx_ext(ctx).guide;
    cudaError_t e = cudaMemsetAsync(g.rec, 0, (size_t)slots * sizeof(GuideRec), st);
    if (!e) e = cudaMemsetAsync(g.acc, 0, (size_t)slots * 4, st);
    if (!e) e = cudaMemsetAsync(g.dev, 0, 4, st);                         // count
    if (!e) e = cudaMemsetAsync(reinterpret_cast<char*>(g.dev) + 8, 0, 4, st);     // inferred
    if (!e) e = cudaMemsetAsync(reinterpret_cast<char*>(g.dev) + 16, 0, 16, st);   // wsum, loss, loss_n
    return e;
}
// the training chain of a wave: GUIDE_STEPS mini-batches, each forward/backward, the weight GEMM, Adam
cudaError_t guide_train_launch(st_ctx* ctx, float lr, int sms, cudaStream_t st, int* launches) {
    GuideState& g = ctx_ext(ctx).guide;
    GuideTrain tr;
    tr.samp = g.samp;
    tr.dev = g.dev;
    guide_box(ctx, tr.lo, tr.inv_ext);
    tr.table = reinterpret_cast<const float2*>(g.param + GUIDE_NW);
    tr.gtable = reinterpret_cast<float2*>(g.grad + GUIDE_NW);
    tr.wbf = g.wbf;
    tr.act = g.act;
    tr.gw = g.grad;
    const size_t smem = (size_t)SW_ALL * 2;
    cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    for (uint32_t k = 0; k < GUIDE_STEPS; k++) {
        tr.first = k * GUIDE_MB;
        k_guide_train<<<sms * 2, 256, smem, st>>>(tr);
        k_guide_dw<<<sms * 2, 256, 0, st>>>(g.dev, tr.first, g.act, g.grad);
        k_guide_step<<<1, 32, 0, st>>>(g.dev, tr.first);
        k_guide_adam<<<sms * 4, 256, 0, st>>>(g.dev, tr.first, lr, g.param, g.grad, g.m1, g.m2, g.wbf);
        if (launches) *launches += 4;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------------------------
// THE C ABI
// ---------------------------------------------------------------------------------------------------------------
extern "C" {

int st_mlp_get_weights(st_ctx* ctx, float* out, size_t n) {
    if (!ctx || !out || n < GUIDE_NPARAM) return ST_ERR_ARG;
    cudaSetDevice(ctx_device(ctx));
    GuideState& g = ctx_ext(ctx).guide;
    if (!g.param) { ctx_set_error(ctx, "the learned proposal has not run"); return ST_ERR_STATE; }
    cudaStream_t st = ctx_stream(ctx);
    if (cudaMemcpyAsync(out, g.param, (size_t)GUIDE_NPARAM * 4, cudaMemcpyDeviceToHost, st) || cudaStreamSynchronize(st))
        return ST_ERR_CUDA;
    return ST_OK;
}

int st_mlp_set_weights(st_ctx* ctx, const float* in, size_t n) {
    if (!ctx || !in || n < GUIDE_NPARAM) return ST_ERR_ARG;
    cudaSetDevice(ctx_device(ctx));
    int rc = guide_ensure(ctx, 0, 0, ctx_ext(ctx).guide.param ? ctx_ext(ctx).guide.seed : 0u);
    if (rc) return rc;
    return guide_upload(ctx, in);
}

// the network at n points: its 40 outputs a point (raw) and the decoded mixture (8 lobes x mean xyz, kappa, weight)
int st_mlp_eval(st_ctx* ctx, const float* pos, const float* nrm, uint32_t n, float* raw, float* mix) {
    if (!ctx || !pos || !nrm || (!raw && !mix)) return ST_ERR_ARG;
    if (n == 0) return ST_OK;
    cudaSetDevice(ctx_device(ctx));
    GuideState& g = ctx_ext(ctx).guide;
    if (!g.param) { ctx_set_error(ctx, "the learned proposal has no weights"); return ST_ERR_STATE; }
    return guide_eval(ctx, pos, nrm, n, raw, mix);
}

// the gradient of the batch's loss (the weights as the training step normalises them) with respect to every weight
// and feature, without a step; the summed loss
int st_mlp_grad(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight, uint32_t n,
                float* grad, float* loss) {
    if (!ctx || !pos || !nrm || !dir || !weight || !grad) return ST_ERR_ARG;
    if (n == 0 || n > GUIDE_MB) { ctx_set_error(ctx, "st_mlp_grad: 1 to 16384 samples"); return ST_ERR_ARG; }
    cudaSetDevice(ctx_device(ctx));
    GuideState& g = ctx_ext(ctx).guide;
    if (!g.param) { ctx_set_error(ctx, "the learned proposal has no weights"); return ST_ERR_STATE; }
    return guide_grad(ctx, pos, nrm, dir, weight, n, grad, loss);
}

// training steps on a given batch (up to GUIDE_CAP samples, mini-batches of GUIDE_MB in turn): the step a wave takes,
// on samples the caller chose
int st_mlp_train(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight, uint32_t n,
                 uint32_t steps, float lr) {
    if (!ctx || !pos || !nrm || !dir || !weight) return ST_ERR_ARG;
    if (n == 0 || n > GUIDE_CAP) { ctx_set_error(ctx, "st_mlp_train: 1 to 131072 samples"); return ST_ERR_ARG; }
    cudaSetDevice(ctx_device(ctx));
    GuideState& g = ctx_ext(ctx).guide;
    if (!g.param) { ctx_set_error(ctx, "the learned proposal has no weights"); return ST_ERR_STATE; }
    return guide_train_samples(ctx, pos, nrm, dir, weight, n, steps, lr > 0.f ? lr : 0.005f);
}

// the last wave's training batch: per sample position, normal, direction, weight (10 floats); returns how many
int st_mlp_read_batch(st_ctx* ctx, float* out, uint32_t max_n, uint32_t* n) {
    if (!ctx || !out || !n) return ST_ERR_ARG;
    cudaSetDevice(ctx_device(ctx));
    GuideState& g = ctx_ext(ctx).guide;
    *n = 0;
    if (!g.dev) return ST_OK;
    GuideDev d;
    cudaStream_t st = ctx_stream(ctx);
    if (cudaStreamSynchronize(st) || cudaMemcpy(&d, g.dev, sizeof(d), cudaMemcpyDeviceToHost)) return ST_ERR_CUDA;
    const uint32_t m = std::min(std::min(d.count, GUIDE_CAP), max_n);
    std::vector<GuideSample> hs(m);
    if (m && cudaMemcpy(hs.data(), g.samp, m * sizeof(GuideSample), cudaMemcpyDeviceToHost)) return ST_ERR_CUDA;
    for (uint32_t i = 0; i < m; i++) {
        float* o = out + 10 * (size_t)i;
        o[0] = hs[i].a.x; o[1] = hs[i].a.y; o[2] = hs[i].a.z;
        o[3] = hs[i].b.x; o[4] = hs[i].b.y; o[5] = hs[i].b.z;
        o[6] = hs[i].c.x; o[7] = hs[i].c.y; o[8] = hs[i].c.z;
        o[9] = hs[i].a.w;
    }
    *n = m;
    return ST_OK;
}

int st_mlp_stats_read(st_ctx* ctx, st_mlp_stats* out) {
    if (!ctx || !out) return ST_ERR_ARG;
    cudaSetDevice(ctx_device(ctx));
    *out = st_mlp_stats{};
    f3 lo;
    guide_box(ctx, lo, out->box_inv_ext);
    out->box_lo[0] = lo.x; out->box_lo[1] = lo.y; out->box_lo[2] = lo.z;
    GuideState& g = ctx_ext(ctx).guide;
    if (!g.dev) return ST_OK;
    GuideDev d;
    if (cudaStreamSynchronize(ctx_stream(ctx)) || cudaMemcpy(&d, g.dev, sizeof(d), cudaMemcpyDeviceToHost))
        return ST_ERR_CUDA;
    out->steps = d.step;
    out->samples = std::min(d.count, GUIDE_CAP);
    out->loss = d.loss_n > 0.f ? d.loss / d.loss_n : 0.f;
    out->mean_weight = d.count ? d.wsum / (float)std::min(d.count, GUIDE_CAP) : 0.f;
    out->inferred = d.inferred;
    return ST_OK;
}

}  // extern "C"

// the eval and gradient entries' device work: the samples uploaded into the batch's buffers, a kernel each
int guide_eval(st_ctx* ctx, const float* pos, const float* nrm, uint32_t n, float* raw, float* mix) {
    GuideState& g = ctx_ext(ctx).guide;
    cudaStream_t st = ctx_stream(ctx);
    for (uint32_t b0 = 0; b0 < n; b0 += GUIDE_CAP) {
        const uint32_t m = std::min(GUIDE_CAP, n - b0);
        std::vector<GuideSample> hs(m);
        for (uint32_t i = 0; i < m; i++) {
            const float* p = pos + 3 * (size_t)(b0 + i);
            const float* q = nrm + 3 * (size_t)(b0 + i);
            hs[i].a = make_float4(p[0], p[1], p[2], 0.f);
            hs[i].b = make_float4(q[0], q[1], q[2], 0.f);
            hs[i].c = make_float4(0.f, 0.f, 1.f, 0.f);
        }
        float* d_raw = nullptr;
        uint2* d_mix = nullptr;
        cudaError_t e = cudaMemcpyAsync(g.samp, hs.data(), m * sizeof(GuideSample), cudaMemcpyHostToDevice, st);
        if (!e) e = cudaMalloc(&d_raw, (size_t)m * GUIDE_OUT * 4);
        if (!e) e = cudaMalloc(&d_mix, (size_t)m * GUIDE_LOBES * sizeof(uint2));
        if (!e) e = guide_eval_launch(ctx, m, d_raw, d_mix, st);
        std::vector<uint2> hm;
        if (!e && raw) e = cudaMemcpyAsync(raw + (size_t)b0 * GUIDE_OUT, d_raw, (size_t)m * GUIDE_OUT * 4, cudaMemcpyDeviceToHost, st);
        if (!e && mix) { hm.resize((size_t)m * GUIDE_LOBES); e = cudaMemcpyAsync(hm.data(), d_mix, hm.size() * sizeof(uint2), cudaMemcpyDeviceToHost, st); }
        if (!e) e = cudaStreamSynchronize(st);
        if (d_raw) cudaFree(d_raw);
        if (d_mix) cudaFree(d_mix);
        if (e) { ctx_set_error(ctx, std::string("st_mlp_eval: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
        if (mix)
            for (size_t i = 0; i < hm.size(); i++) guide_unpack_host(hm[i], mix + ((size_t)b0 * GUIDE_LOBES + i) * 5);
    }
    return ST_OK;
}

cudaError_t guide_eval_launch(st_ctx* ctx, uint32_t n, float* d_raw, uint2* d_mix, cudaStream_t st) {
    GuideState& g = ctx_ext(ctx).guide;
    f3 lo;
    float inv_ext;
    guide_box(ctx, lo, inv_ext);
    // the tensor cores' network (st_guide_tc.cu); the error word is the context's counters' (a wait that ran out)
    return launch_guide_eval_tc(g.samp, n, lo, inv_ext, reinterpret_cast<const float2*>(g.param + GUIDE_NW), g.wbf,
                                d_raw, d_mix, &ctx_counters(ctx)->errflag, ctx_sms(ctx), st);
}

int guide_grad(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight, uint32_t n,
               float* grad, float* loss) {
    GuideState& g = ctx_ext(ctx).guide;
    cudaStream_t st = ctx_stream(ctx);
    std::vector<GuideSample> hs(n);
    double wsum = 0.0;
    for (uint32_t i = 0; i < n; i++) {
        hs[i].a = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], weight[i]);
        hs[i].b = make_float4(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2], 0.f);
        hs[i].c = make_float4(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2], 0.f);
        wsum += weight[i];
    }
    GuideDev d{};
    d.count = n;
    d.wsum = (float)wsum;
    GuideTrain tr;
    tr.samp = g.samp;
    tr.dev = g.dev;
    tr.first = 0;
    guide_box(ctx, tr.lo, tr.inv_ext);
    tr.table = reinterpret_cast<const float2*>(g.param + GUIDE_NW);
    tr.gtable = reinterpret_cast<float2*>(g.grad + GUIDE_NW);
    tr.wbf = g.wbf;
    tr.act = g.act;
    tr.gw = g.grad;
    const size_t smem = (size_t)SW_ALL * 2;
    cudaError_t e = cudaMemcpyAsync(g.samp, hs.data(), n * sizeof(GuideSample), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(g.dev, &d, sizeof(d), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemsetAsync(g.grad, 0, (size_t)GUIDE_NPARAM * 4, st);
    if (!e) e = cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (!e) {
        k_guide_train<<<ctx_sms(ctx) * 2, 256, smem, st>>>(tr);
        k_guide_dw<<<ctx_sms(ctx) * 2, 256, 0, st>>>(g.dev, 0, g.act, g.grad);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(grad, g.grad, (size_t)GUIDE_NPARAM * 4, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(&d, g.dev, sizeof(d), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemsetAsync(g.grad, 0, (size_t)GUIDE_NPARAM * 4, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) { ctx_set_error(ctx, std::string("st_mlp_grad: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
    if (loss) *loss = d.loss;
    return ST_OK;
}

// a packed lobe on the host: mean direction, kappa, weight (the device's guide_unpack, restated)
static float half_to_float(uint16_t h) {
    const uint32_t sgn = (uint32_t)(h >> 15) << 31, ex = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    uint32_t bits;
    if (ex == 0) {
        if (man == 0) bits = sgn;
        else {                                          // subnormal: normalise
            int e = -1;
            uint32_t m = man;
            do { e++; m <<= 1; } while (!(m & 0x400u));
            bits = sgn | ((uint32_t)(127 - 15 - e) << 23) | ((m & 0x3ffu) << 13);
        }
    } else if (ex == 31) bits = sgn | 0x7f800000u | (man << 13);
    else bits = sgn | ((ex - 15 + 127) << 23) | (man << 13);
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}
void guide_unpack_host(uint2 v, float* out) {
    float x = (float)(int16_t)(v.x & 0xffffu) / 32767.f, y = (float)(int16_t)(v.x >> 16) / 32767.f;
    const float z = 1.f - std::fabs(x) - std::fabs(y);
    if (z < 0.f) {
        const float ox = (1.f - std::fabs(y)) * (x >= 0.f ? 1.f : -1.f), oy = (1.f - std::fabs(x)) * (y >= 0.f ? 1.f : -1.f);
        x = ox; y = oy;
    }
    const float l = std::sqrt(x * x + y * y + z * z);
    out[0] = x / l; out[1] = y / l; out[2] = z / l;
    out[3] = half_to_float((uint16_t)(v.y & 0xffffu));
    out[4] = half_to_float((uint16_t)(v.y >> 16));
}

int guide_train_samples(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight,
                        uint32_t n, uint32_t steps, float lr) {
    GuideState& g = ctx_ext(ctx).guide;
    cudaStream_t st = ctx_stream(ctx);
    std::vector<GuideSample> hs(n);
    double wsum = 0.0;
    for (uint32_t i = 0; i < n; i++) {
        hs[i].a = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], weight[i]);
        hs[i].b = make_float4(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2], 0.f);
        hs[i].c = make_float4(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2], 0.f);
        wsum += weight[i];
    }
    GuideDev d;
    cudaError_t e = cudaMemcpyAsync(g.samp, hs.data(), n * sizeof(GuideSample), cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(&d, g.dev, sizeof(d), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) { ctx_set_error(ctx, std::string("st_mlp_train: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
    d.count = n;
    d.wsum = (float)wsum;
    d.loss = 0.f;
    d.loss_n = 0.f;
    e = cudaMemcpyAsync(g.dev, &d, sizeof(d), cudaMemcpyHostToDevice, st);
    GuideTrain tr;
    tr.samp = g.samp;
    tr.dev = g.dev;
    guide_box(ctx, tr.lo, tr.inv_ext);
    tr.table = reinterpret_cast<const float2*>(g.param + GUIDE_NW);
    tr.gtable = reinterpret_cast<float2*>(g.grad + GUIDE_NW);
    tr.wbf = g.wbf;
    tr.act = g.act;
    tr.gw = g.grad;
    const size_t smem = (size_t)SW_ALL * 2;
    if (!e) e = cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const uint32_t nmb = (n + GUIDE_MB - 1) / GUIDE_MB;
    const int sms = ctx_sms(ctx);
    for (uint32_t s = 0; s < steps && !e; s++) {
        tr.first = (s % nmb) * GUIDE_MB;
        k_guide_train<<<sms * 2, 256, smem, st>>>(tr);
        k_guide_dw<<<sms * 2, 256, 0, st>>>(g.dev, tr.first, g.act, g.grad);
        k_guide_step<<<1, 32, 0, st>>>(g.dev, tr.first);
        k_guide_adam<<<sms * 4, 256, 0, st>>>(g.dev, tr.first, lr, g.param, g.grad, g.m1, g.m2, g.wbf);
        e = cudaGetLastError();
    }
    if (!e) e = cudaStreamSynchronize(st);
    if (e) { ctx_set_error(ctx, std::string("st_mlp_train: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
    return ST_OK;
}
