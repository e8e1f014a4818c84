// st_guide.cuh -- THE LEARNED PROPOSAL's device half: a small network that maps a surface point (its position through
// a multi-resolution hash grid, its normal through real spherical harmonics) to a mixture of eight von Mises-Fisher
// lobes over the sphere of directions, the density BSDF sampling is mixed with under one-sample MIS at a camera path's
// evaluable opaque vertices (st_render.cu shade_surface). The network is trained online on the incident radiance the
// paths themselves find (st_guide.cu). No counterpart in the reference, which removed its path guiding; the mixture's
// density and sampling, and what the estimator weighs a guided direction by, are standard (one-sample MIS, Veach 1997
// section 9.2.4; vMF sampling after Jakob, "Numerically stable sampling of the von Mises-Fisher distribution on S^2",
// 2012).
//
// THE NETWORK. Input 48: 16 hash-grid levels x 2 features (a trilinear blend of the 8 corners' entries; level l's
// resolution 2 * 16^(l/15) cells across the scene's bounding box, floored) and the 16 real
// spherical harmonics of degree <= 3 of the normal. Three hidden layers of 64, ReLU, no biases (the constant harmonic
// is one); output 40 = 8 lobes x (mean direction m, 3, unnormalised; log kappa; mixture logit). BF16 operands, FP32
// accumulation (mma.sync m16n8k16), weights [out][in] row-major.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include "st_device.cuh"

namespace st {

#define GUIDE_LEVELS 16u
#define GUIDE_T (1u << 12)                       // hash-table entries a level
#define GUIDE_IN 48u
#define GUIDE_H 64u
#define GUIDE_OUT 40u
#define GUIDE_LOBES 8u
#define GUIDE_W1 0u                               // offsets of the four weight matrices in the packed parameters
#define GUIDE_W2 (GUIDE_W1 + GUIDE_H * GUIDE_IN)
#define GUIDE_W3 (GUIDE_W2 + GUIDE_H * GUIDE_H)
#define GUIDE_W4 (GUIDE_W3 + GUIDE_H * GUIDE_H)
#define GUIDE_NW (GUIDE_W4 + GUIDE_OUT * GUIDE_H)               // 13 824 network weights
#define GUIDE_NHASH (GUIDE_LEVELS * GUIDE_T * 2u)                // 131 072 hash-grid features
#define GUIDE_NPARAM (GUIDE_NW + GUIDE_NHASH)
#define GUIDE_KLO (-1.f)                          // log kappa's clamp: kappa in [e^-1, e^6]
#define GUIDE_KHI 6.f
// shared-memory rows of the weights, padded by 8 BF16 so the fragment loads of 8 rows meet 8 different bank groups
#define GUIDE_LD_IN (GUIDE_IN + 8u)
#define GUIDE_LD_H (GUIDE_H + 8u)

// the resolution of level l (cells across the box's longest side): floor(2 * 16^(l/15)), 2 to 32, as integers so
// every side of the build (and the oracle) agrees on them exactly. The finest cell is the box over 32 (25 cm in a
// room) and a level holds 4096 entries: the light a point receives changes slowly, and a finer or larger grid only
// memorises the noise of single paths (held-out cross entropy on a wave's records: 1.52 here, 2.9 with 6 mm cells
// and 32 768 entries a level, 1.66 for the cosine lobe alone).
static __constant__ float c_guide_res[GUIDE_LEVELS] = {2, 2, 2, 3, 4, 5, 6, 7, 8, 10, 12, 15, 18, 22, 26, 32};
static const float h_guide_res[GUIDE_LEVELS] = {2, 2, 2, 3, 4, 5, 6, 7, 8, 10, 12, 15, 18, 22, 26, 32};
__host__ __device__ __forceinline__ float guide_res(uint32_t l) {
#ifdef __CUDA_ARCH__
    return c_guide_res[l];
#else
    return h_guide_res[l];
#endif
}
// a corner's entry: the spatial hash of instant neural graphics primitives (Mueller et al. 2022), per level
__host__ __device__ __forceinline__ uint32_t guide_hash(uint32_t x, uint32_t y, uint32_t z) {
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (GUIDE_T - 1u);
}
// the 16 real spherical harmonics of degree <= 3 at unit n (the constants are the normalisations of the real
// harmonics, sqrt((2l+1)/4pi (l-m)!/(l+m)!) times the associated Legendre factors)
__host__ __device__ __forceinline__ void guide_sh(float x, float y, float z, float* o) {
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.94617469575755997f * zz - 0.31539156525251999f;
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = 0.59004358992664352f * y * (3.f * xx - yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = 0.45704579946446572f * y * (5.f * zz - 1.f);
    o[12] = 0.3731763325901154f * z * (5.f * zz - 3.f);
    o[13] = 0.45704579946446572f * x * (5.f * zz - 1.f);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = 0.59004358992664352f * x * (xx - 3.f * yy);
}
// one level's corners and trilinear weights at the point u in [0,1]^3 of the box
struct GuideCorners { uint32_t idx[8]; float w[8]; };
__host__ __device__ __forceinline__ GuideCorners guide_corners(f3 u, uint32_t l) {
    const float r = guide_res(l);
    const float px = u.x * r, py = u.y * r, pz = u.z * r;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const float tx = px - fx, ty = py - fy, tz = pz - fz;
    const uint32_t cx = (uint32_t)(int32_t)fx, cy = (uint32_t)(int32_t)fy, cz = (uint32_t)(int32_t)fz;
    GuideCorners c;
    for (uint32_t k = 0; k < 8; k++) {
        const uint32_t ox = k & 1u, oy = (k >> 1) & 1u, oz = (k >> 2) & 1u;
        c.idx[k] = l * GUIDE_T + guide_hash(cx + ox, cy + oy, cz + oz);
        c.w[k] = (ox ? tx : 1.f - tx) * (oy ? ty : 1.f - ty) * (oz ? tz : 1.f - tz);
    }
    return c;
}
// the point in the box's unit cube (clamped: the grid's cells outside the box alias those inside, as any hash does)
__host__ __device__ __forceinline__ f3 guide_unit(f3 p, f3 lo, float inv_ext) {
    return mk(fminf(fmaxf((p.x - lo.x) * inv_ext, 0.f), 1.f), fminf(fmaxf((p.y - lo.y) * inv_ext, 0.f), 1.f),
              fminf(fmaxf((p.z - lo.z) * inv_ext, 0.f), 1.f));
}

// the vertex a camera path's shade guides (met from outside): an opaque, mostly dielectric surface rough enough that
// what it reflects hardly depends on the direction it is seen from (the network does not see that direction: at a
// glossy vertex its one mixture for every view would fit none), not emitting
#define GUIDE_MIN_ROUGHNESS 0.5f
__device__ __forceinline__ bool guide_vertex(const st_material& m) {
    return m.transmission <= 0.f && m.metallic < 0.5f && m.roughness >= GUIDE_MIN_ROUGHNESS &&
           fmaxf(fmaxf(m.emissive[0], m.emissive[1]), m.emissive[2]) <= 0.f;
}
// the guide's share of the one-sample MIS: ramped in over its first GUIDE_RAMP training steps (a network not yet
// trained would only take samples from the BSDF); fixed within a wave, where the weights are
#define GUIDE_RAMP 64.f
__device__ __forceinline__ float guide_share(float alpha, const uint32_t* step, uint32_t train) {
    return train ? alpha * fminf(1.f, (float)*step / GUIDE_RAMP) : alpha;
}
// a path's pixel among the wave's views (its slot's frame, its pixel): the one mixture its first vertex samples from
__device__ __forceinline__ uint32_t guide_pixel(const Uni& u, uint32_t slot, uint32_t pix) {
    return slot_view(u, slot) * u.P + pix;
}

// ---------------------------------------------------------------------------------------------------------------
// THE MIXTURE, as the sampler reads it: per lobe the mean direction (octahedral, two 16-bit snorms) and kappa and
// the mixture weight (two halves). Sampling and density read the same quantised numbers, so they agree exactly.
// ---------------------------------------------------------------------------------------------------------------
struct GuideLobe { f3 mu; float kappa, pi; };
__device__ __forceinline__ uint32_t guide_oct16(f3 n) {
    const float s = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
    float x = n.x / s, y = n.y / s;
    if (n.z < 0.f) {
        const float ox = (1.f - fabsf(y)) * (x >= 0.f ? 1.f : -1.f), oy = (1.f - fabsf(x)) * (y >= 0.f ? 1.f : -1.f);
        x = ox; y = oy;
    }
    const int32_t qx = __float2int_rn(fminf(fmaxf(x, -1.f), 1.f) * 32767.f);
    const int32_t qy = __float2int_rn(fminf(fmaxf(y, -1.f), 1.f) * 32767.f);
    return ((uint32_t)qx & 0xffffu) | ((uint32_t)qy << 16);
}
__device__ __forceinline__ f3 guide_unoct16(uint32_t w) {
    float x = (float)(int16_t)(w & 0xffffu) / 32767.f, y = (float)(int16_t)(w >> 16) / 32767.f;
    const float z = 1.f - fabsf(x) - fabsf(y);
    if (z < 0.f) {
        const float ox = (1.f - fabsf(y)) * (x >= 0.f ? 1.f : -1.f), oy = (1.f - fabsf(x)) * (y >= 0.f ? 1.f : -1.f);
        x = ox; y = oy;
    }
    return normalize(mk(x, y, z));
}
__device__ __forceinline__ uint2 guide_pack(f3 mu, float kappa, float pi) {
    const __half2 h = __floats2half2_rn(kappa, pi);
    return make_uint2(guide_oct16(mu), *reinterpret_cast<const uint32_t*>(&h));
}
__device__ __forceinline__ GuideLobe guide_unpack(uint2 v) {
    GuideLobe g;
    g.mu = guide_unoct16(v.x);
    const __half2 h = *reinterpret_cast<const __half2*>(&v.y);
    g.kappa = __low2float(h);
    g.pi = __high2float(h);
    return g;
}
// the vMF density at cos = mu . w: kappa / (2 pi (1 - e^-2kappa)) e^(kappa (cos - 1))
__device__ __forceinline__ float vmf_pdf(float kappa, float c) {
    return kappa / (2.f * ST_PI * (1.f - __expf(-2.f * kappa))) * __expf(kappa * (c - 1.f));
}
// the mixture's density at w, from the packed lobes: the weights as quantised, over their sum (so that the draw below,
// which picks a lobe by the same quantised weights, has exactly this density)
__device__ __forceinline__ float guide_pdf(const uint2* __restrict__ mix, f3 w) {
    float p = 0.f, tot = 0.f;
#pragma unroll
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) {
        const GuideLobe g = guide_unpack(mix[k]);
        p += g.pi * vmf_pdf(g.kappa, dot(g.mu, w));
        tot += g.pi;
    }
    return tot > 0.f ? p / tot : 0.f;
}
// a direction from the mixture: the lobe by its weight (u0), then the vMF draw (u1, u2)
__device__ __forceinline__ f3 guide_sample(const uint2* __restrict__ mix, float u0, float u1, float u2) {
    float tot = 0.f;
#pragma unroll
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) tot += guide_unpack(mix[k]).pi;
    const float x = u0 * tot;
    GuideLobe g = guide_unpack(mix[GUIDE_LOBES - 1u]);
    float acc = 0.f;
#pragma unroll
    for (uint32_t k = 0; k + 1u < GUIDE_LOBES; k++) {
        const GuideLobe h = guide_unpack(mix[k]);
        acc += h.pi;
        if (x < acc) { g = h; break; }
    }
    const float e = __expf(-2.f * g.kappa);
    const float c = fminf(fmaxf(1.f + __logf(u1 + (1.f - u1) * e) / g.kappa, -1.f), 1.f);
    const float s = sqrtf(fmaxf(0.f, 1.f - c * c));
    float sp, cp;
    sincosf(2.f * ST_PI * u2, &sp, &cp);
    const f3 t1 = fabsf(g.mu.z) < 0.999f ? normalize(cross(g.mu, mk(0.f, 0.f, 1.f))) : normalize(cross(g.mu, mk(0.f, 1.f, 0.f)));
    const f3 t2 = cross(g.mu, t1);
    return normalize(g.mu * c + t1 * (s * cp) + t2 * (s * sp));
}

// ---------------------------------------------------------------------------------------------------------------
// TENSOR-CORE FRAGMENTS (mma.sync.m16n8k16, BF16 in, FP32 accumulate). For a warp with g = lane / 4, t = lane % 4:
// A (16 x 16): a0 = (row g, cols 2t, 2t+1), a1 = (row g+8, same cols), a2 = (row g, cols 2t+8, 2t+9), a3 = (row g+8,
// cols 2t+8, 2t+9); B (16 x 8): b0 = (rows 2t, 2t+1, col g), b1 = (rows 2t+8, 2t+9, col g); C (16 x 8): c0, c1 =
// (row g, cols 2t, 2t+1), c2, c3 = (row g+8, cols 2t, 2t+1). Each 32-bit register holds two BF16, the lower index in
// the low half. So two adjacent C tiles of one layer are, converted, the A fragment of the next layer's 16 columns.
// ---------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }
// the B fragment of W (row-major [n][k], leading dimension ld in BF16) for columns n0.. and rows k0..
__device__ __forceinline__ void frag_b(const __nv_bfloat16* w, uint32_t ld, uint32_t n0, uint32_t k0, uint32_t g,
                                       uint32_t t, uint32_t& b0, uint32_t& b1) {
    const __nv_bfloat16* r = w + (size_t)(n0 + g) * ld + k0 + 2u * t;
    b0 = *reinterpret_cast<const uint32_t*>(r);
    b1 = *reinterpret_cast<const uint32_t*>(r + 8);
}
// one layer: C[16 x 8*NT] = A[16 x 16*KT] . W^T, W [8*NT][16*KT] in shared memory with leading dimension ld
template <int NT, int KT>
__device__ __forceinline__ void guide_layer(const uint32_t (*a)[4], const __nv_bfloat16* w, uint32_t ld, uint32_t g,
                                            uint32_t t, float (*c)[4]) {
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < KT; kt++) {
            uint32_t b0, b1;
            frag_b(w, ld, 8u * nt, 16u * kt, g, t, b0, b1);
            mma_bf16(c[nt], a[kt], b0, b1);
        }
    }
}
// ReLU'd C tiles (8*2*KT columns) into the next layer's A fragments
template <int KT>
__device__ __forceinline__ void relu_to_a(const float (*c)[4], uint32_t (*a)[4]) {
#pragma unroll
    for (int kt = 0; kt < KT; kt++) {
        a[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
        a[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
        a[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
        a[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
    }
}

// the input fragments of two queries (rows g and g+8 of the tile): this lane's levels t, t+4, t+8, t+12 and
// harmonics 2t, 2t+1, 2t+8, 2t+9 of each; u in the box's unit cube, n unit
__device__ __forceinline__ void guide_input(const float2* __restrict__ table, f3 u0, f3 n0, f3 u1, f3 n1, uint32_t t,
                                            uint32_t (*a)[4]) {
    float f[2][4][2];                             // [query][level slot][feature]
#pragma unroll
    for (int qi = 0; qi < 2; qi++) {
        const f3 u = qi ? u1 : u0;
#pragma unroll
        for (int s = 0; s < 4; s++) {
            const GuideCorners c = guide_corners(u, t + 4u * s);
            float fx = 0.f, fy = 0.f;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const float2 e = __ldg(&table[c.idx[k]]);
                fx += c.w[k] * e.x;
                fy += c.w[k] * e.y;
            }
            f[qi][s][0] = fx;
            f[qi][s][1] = fy;
        }
    }
    // k-tile 0: levels 0-7 (cols 2t, 2t+1 = level t; 2t+8, 2t+9 = level t+4); k-tile 1: levels 8-15
    a[0][0] = pack_bf16(f[0][0][0], f[0][0][1]);
    a[0][1] = pack_bf16(f[1][0][0], f[1][0][1]);
    a[0][2] = pack_bf16(f[0][1][0], f[0][1][1]);
    a[0][3] = pack_bf16(f[1][1][0], f[1][1][1]);
    a[1][0] = pack_bf16(f[0][2][0], f[0][2][1]);
    a[1][1] = pack_bf16(f[1][2][0], f[1][2][1]);
    a[1][2] = pack_bf16(f[0][3][0], f[0][3][1]);
    a[1][3] = pack_bf16(f[1][3][0], f[1][3][1]);
    float h0[16], h1[16];
    guide_sh(n0.x, n0.y, n0.z, h0);
    guide_sh(n1.x, n1.y, n1.z, h1);
    // k-tile 2: the harmonics (the 16 values are registers only through the unrolled select below)
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, r0 = 0.f, r1 = 0.f, r2 = 0.f, r3 = 0.f;
#pragma unroll
    for (uint32_t k = 0; k < 4; k++)
        if (t == k) {
            s0 = h0[2 * k]; s1 = h0[2 * k + 1]; s2 = h0[2 * k + 8]; s3 = h0[2 * k + 9];
            r0 = h1[2 * k]; r1 = h1[2 * k + 1]; r2 = h1[2 * k + 8]; r3 = h1[2 * k + 9];
        }
    a[2][0] = pack_bf16(s0, s1);
    a[2][1] = pack_bf16(r0, r1);
    a[2][2] = pack_bf16(s2, s3);
    a[2][3] = pack_bf16(r2, r3);
}

// a query's 40 outputs into its packed mixture: mean directions normalised, kappa = e^clamp(y, KLO, KHI), the
// weights a softmax of the logits
__device__ __forceinline__ void guide_decode(const float* y, uint2* out) {
    float mx = -1e30f;
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) mx = fmaxf(mx, y[5 * k + 4]);
    float e[GUIDE_LOBES], s = 0.f;
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) { e[k] = __expf(y[5 * k + 4] - mx); s += e[k]; }
    for (uint32_t k = 0; k < GUIDE_LOBES; k++) {
        f3 m = mk(y[5 * k], y[5 * k + 1], y[5 * k + 2]);
        const float len = length(m);
        m = len > 1e-12f ? m / len : mk(0.f, 0.f, 1.f);
        const float kappa = __expf(fminf(fmaxf(y[5 * k + 3], GUIDE_KLO), GUIDE_KHI));
        out[k] = guide_pack(m, kappa, e[k] / s);
    }
}

}  // namespace st
