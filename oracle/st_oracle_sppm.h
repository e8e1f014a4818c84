// TEST INFRASTRUCTURE ONLY -- the oracle's photon map (core/sppm.js): the cell and its hash, the grid as the
// reference's lists hold it, the radius schedule, the keep, the sub-lists, and the gather. Restated from the
// reference's JS mirror (PhotonMap, sppm.js:211-301) and its WGSL (sppmWalk, sppmPut, sppm.js:305-423); never part of
// the product.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>
#include "st_oracle_core.h"

namespace sto {

const uint32_t SPPM_HEADS = 1u << 20;     // sppm.js:82
const uint32_t SPPM_SUBS = 32;            // sppm.js:105
const uint32_t SPPM_VISIT = 512;          // sppm.js:110
const uint32_t SPPM_VISIT_HARD = 8;       // sppm.js:114
const float SPPM_NORMAL_DOT = 0.9f;       // sppm.js:135
const double SPPM_FILL = 0.85;            // sppm.js:124
const uint32_t SPPM_B_MASK = 0xFFFFu, SPPM_SUB_SHIFT = 16;
const uint32_t SPPM_VOL = 0x40000000u;      // a record where a photon collided inside a medium (sppm.js:93-95)

// the cell a point is in, in f32 as the kernel computes it: floor(pos / cell) (sppm.js:381, WGSL vec3<i32>(floor(...)))
inline void sppm_cell(const float* p, float c, int32_t out[3]) {
    for (int a = 0; a < 3; a++) out[a] = (int32_t)std::floor(p[a] / c);
}
// the cell's list: 32-bit wrapping multiplies (sppm.js:197-198 hashCell, :383-386 sppmHash)
inline uint32_t sppm_hash(int32_t i, int32_t j, int32_t k, uint32_t heads = SPPM_HEADS) {
    return (((uint32_t)i * 73856093u) ^ ((uint32_t)j * 19349663u) ^ ((uint32_t)k * 83492791u)) & (heads - 1);
}
// r_k (sppm.js:177-181)
inline double sppm_radius(double r1, int k, double alpha) {
    double s = 1;
    for (int i = 1; i < std::max(1, k); i++) s *= (i + alpha) / (i + 1);
    return r1 * std::sqrt(s);
}
// ...and in a volume (sppm.js:182-191 sppmRadiusVolume): R^3 shrinks by the factor r^2 does
inline double sppm_radius_volume(double r1, int k, double alpha) {
    double s = 1;
    for (int i = 1; i < std::max(1, k); i++) s *= (i + alpha) / (i + 1);
    return r1 * std::cbrt(s);
}
// the keep (sppm.js:156-157)
inline double sppm_keep(double capacity, double demand) {
    if (!(demand > 0) || !(capacity > 0)) return 1;
    return std::min(1.0, SPPM_FILL * capacity / demand);
}
// sub-lists a gather walks in a cell (sppm.js:159-160)
inline uint32_t sppm_subs_of(uint32_t count, uint32_t share) {
    return count <= share ? SPPM_SUBS : std::max(1u, (uint32_t)std::floor((double)SPPM_SUBS * share / count));
}
// a direction in 32 bits, octahedral, two 16-bit snorms (sppm.js:366-379 sppmOct / sppmUnoct); pack2x16snorm
// rounds clamp(v, -1, 1) * 32767 to the nearest integer
inline uint32_t snorm16(float v) {
    float c = std::min(std::max(v, -1.f), 1.f);
    int32_t q = (int32_t)std::nearbyint(c * 32767.f);
    return (uint32_t)(uint16_t)(int16_t)q;
}
inline float unsnorm16(uint32_t w) {
    int16_t q = (int16_t)(uint16_t)(w & 0xFFFF);
    return std::max((float)q / 32767.f, -1.f);
}
inline uint32_t sppm_oct(const float* v) {
    float s = std::fabs(v[0]) + std::fabs(v[1]) + std::fabs(v[2]);
    float ax = v[0] / s, ay = v[1] / s, az = v[2] / s;
    float ex = ax, ey = ay;
    if (az < 0.f) {
        ex = (1.f - std::fabs(ay)) * (ax >= 0.f ? 1.f : -1.f);
        ey = (1.f - std::fabs(ax)) * (ay >= 0.f ? 1.f : -1.f);
    }
    return snorm16(ex) | (snorm16(ey) << 16);
}
inline void sppm_unoct(uint32_t w, float* out) {
    float ex = unsnorm16(w), ey = unsnorm16(w >> 16);
    float vx = ex, vy = ey, vz = 1.f - std::fabs(ex) - std::fabs(ey);
    if (vz < 0.f) {
        float nx = (1.f - std::fabs(vy)) * (vx >= 0.f ? 1.f : -1.f);
        float ny = (1.f - std::fabs(vx)) * (vy >= 0.f ? 1.f : -1.f);
        vx = nx; vy = ny;
    }
    float l = std::sqrt(vx * vx + vy * vy + vz * vz);
    out[0] = vx / l; out[1] = vy / l; out[2] = vz / l;
}

// THE GRID, as the reference's lists define it: for every record its cell's hash, per hash its records (the
// list's membership; the list's order is the atomics' and not part of the answer)
struct SppmGrid {
    float cell, vcell = 0;                       // the surface records' cell, the volume records' (sppm.js sppmPut)
    std::vector<float> pos, power;
    std::vector<uint32_t> nrm, flags, key, dir;
    std::vector<std::vector<uint32_t>> lists;   // per hash: record indices, ascending
};
inline void sppm_build(SppmGrid& g, const float* pos, const float* power, const uint32_t* nrm, const uint32_t* flags,
                       uint32_t n, float cell, float vcell = 0) {
    g.cell = cell;
    g.vcell = vcell > 0 ? vcell : cell;
    g.pos.assign(pos, pos + 3 * (size_t)n);
    g.power.assign(power, power + 3 * (size_t)n);
    g.nrm.assign(nrm, nrm + n);
    g.flags.assign(flags, flags + n);
    g.key.resize(n);
    g.lists.assign(SPPM_HEADS, {});
    for (uint32_t i = 0; i < n; i++) {
        int32_t c[3];
        sppm_cell(&pos[3 * i], (flags[i] & SPPM_VOL) ? g.vcell : cell, c);
        uint32_t h = sppm_hash(c[0], c[1], c[2]);
        g.key[i] = h;
        g.lists[h].push_back(i);
    }
}

// THE GATHER at x on a surface facing n (sppm.js:305-346 sppmWalk, :475-494 sppmGather), a Lambertian of albedo
// a there (f = a / pi). The eight cells -- its own, and on each axis the neighbour on the side of the cell's middle
// x is; in each, the whole list while its count is within its share of the budget, else m sub-lists from a drawn
// start, each record found weighing SUBS / m. Records of another cell with the same hash, past the radius, facing
// away, or past the bounce cap are passed by. Returns sum f * power (FP64), and the records looked at and whether
// the hard cap stopped it.
inline void sppm_gather(const SppmGrid& g, const float* x, const float* n, const float* albedo, uint32_t bounce,
                        float radius, uint32_t maxbounce, uint32_t budget, Rng& rng, double out[3],
                        uint32_t& visits, bool& cut) {
    out[0] = out[1] = out[2] = 0;
    visits = 0;
    cut = false;
    const float csz = g.cell;
    float gx[3] = {x[0] / csz, x[1] / csz, x[2] / csz};
    int32_t c0[3], side[3];
    for (int a = 0; a < 3; a++) {
        c0[a] = (int32_t)std::floor(gx[a]);
        side[a] = (gx[a] - std::floor(gx[a]) >= 0.5f) ? 1 : -1;
    }
    const uint32_t bc = bounce + 1;
    const bool unlimited = budget == 0;
    const uint32_t share = unlimited ? 0xFFFFFFFFu : std::max(1u, budget / 8);
    const uint64_t hard = unlimited ? UINT64_MAX : (uint64_t)SPPM_VISIT_HARD * budget;
    const float r2 = radius * radius;                       // f32, each product and sum rounded (no fused ops)
    for (uint32_t k = 0; k < 8; k++) {
        int32_t cell[3] = {c0[0] + ((k & 1) ? side[0] : 0), c0[1] + ((k & 2) ? side[1] : 0),
                           c0[2] + ((k & 4) ? side[2] : 0)};
        uint32_t h = sppm_hash(cell[0], cell[1], cell[2]);
        const std::vector<uint32_t>& L = g.lists[h];
        uint32_t count = (uint32_t)L.size();
        bool whole = count <= share;
        uint32_t subs = whole ? 1 : std::max(1u, (SPPM_SUBS * share) / std::max(count, 1u));
        double w = whole ? 1.0 : (double)SPPM_SUBS / subs;
        float u4[4];
        rng.next4(u4);
        uint32_t start = std::min((uint32_t)(u4[0] * (float)SPPM_SUBS), SPPM_SUBS - 1);
        for (uint32_t j = 0; j < subs; j++) {
            uint32_t s = (start + j) % SPPM_SUBS;
            for (uint32_t idx : L) {
                uint32_t b = g.flags[idx];
                if (!whole && ((b >> SPPM_SUB_SHIFT) & (SPPM_SUBS - 1)) != s) continue;   // another sub-list's
                if (visits >= hard) { cut = true; break; }
                visits++;
                const float* p = &g.pos[3 * idx];
                int32_t pc[3];
                sppm_cell(p, csz, pc);
                float d[3] = {p[0] - x[0], p[1] - x[1], p[2] - x[2]};
                if (pc[0] != cell[0] || pc[1] != cell[1] || pc[2] != cell[2]) continue;
                float dd = d[0] * d[0] + d[1] * d[1];
                dd = dd + d[2] * d[2];
                if (dd > r2) continue;
                if ((b & SPPM_VOL) || bc + (b & SPPM_B_MASK) > maxbounce + 1) continue;
                float pn[3];
                sppm_unoct(g.nrm[idx], pn);
                float nd = pn[0] * n[0] + pn[1] * n[1];
                nd = nd + pn[2] * n[2];
                if (nd < SPPM_NORMAL_DOT) continue;
                for (int c = 0; c < 3; c++) out[c] += w * ((double)albedo[c] / PI_D) * (double)g.power[3 * idx + c];
            }
            if (cut) break;
        }
        if (cut) break;
    }
}

}  // namespace sto
