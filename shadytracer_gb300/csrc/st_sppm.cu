// st_sppm.cu -- the photon map's grid and gather (core/sppm.js:305-511) for sm_103a.
//
// THE REFERENCE builds linked lists: each stored record is pushed on its cell's list (atomicExchange of the head)
// and on one of 32 sub-lists drawn at random, and a gather walks the lists of eight cells, all of a cell's records
// while their count is within the cell's share of the budget, else m of its sub-lists (each record then weighing
// 32 / m). Lists are pointer chasing: one dependent global load per record.
//
// HERE the records are sorted into buckets by a COUNTING SORT on (cell hash, sub-list) -- 2^20 hashes x 32 sub-lists
// -- so a cell's records are one contiguous range, each of its sub-lists a contiguous sub-range, and a gather reads
// them as streams. The build is four kernels: the key and each record's rank in its bucket (one atomicAdd, whose
// return value is the rank), an exclusive scan of the bucket counts (three phases: block sums, a scan of the sums,
// the block scans), and the scatter of the records into bucket order (structure of arrays: point, power, normal,
// flags). The membership of every cell and every sub-list is exactly the reference's lists'; the order within a
// bucket is the order the atomics ran in, as the reference's lists' order is. The gather sums in FP64.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "st_ext.h"
#include "st_internal.h"
#include "st_sppm_dev.cuh"

using namespace st;

#define SCAN_THREADS 256u
#define SCAN_ITEMS 16u
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)
#define SCAN_BLOCKS ((SPPM_BUCKETS + SCAN_TILE - 1) / SCAN_TILE)
#define SPPM_SALT 0x53505000u

namespace {

// THE KEYS: each record's cell hash, its bucket (hash, sub-list), its rank in the bucket
// (the count and the cell are the device's: the wavefront's photons stored them there, or st_sppm_build)
__global__ void __launch_bounds__(256) k_sppm_key(const float4* __restrict__ pos, const uint32_t* __restrict__ flags,
                                                  const SppmDev* __restrict__ d, uint32_t* __restrict__ key,
                                                  uint32_t* __restrict__ bucket, uint32_t* __restrict__ rank,
                                                  uint32_t* __restrict__ counts) {
    const uint32_t n = min(d->count, d->cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = pos[i];
        const float cell = (flags[i] & SPPM_VOL) ? d->vcell : d->cell;   // a volume's records on their own cells
        uint32_t h = sppm_hash(cell_of(p.x, cell), cell_of(p.y, cell), cell_of(p.z, cell));
        uint32_t b = h * SPPM_SUBS + ((flags[i] >> SPPM_SUB_SHIFT) & (SPPM_SUBS - 1));
        key[i] = h;
        bucket[i] = b;
        rank[i] = atomicAdd(&counts[b], 1u);
    }
}

// THE SCAN, exclusive, of the bucket counts into the buckets' starts, in place: block sums, the sums scanned, the
// blocks scanned with their offsets. starts[SPPM_BUCKETS] is the total.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(const uint32_t* __restrict__ c, uint32_t* __restrict__ part) {
    __shared__ uint32_t red[SCAN_THREADS / 32];
    const uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t s = 0;
    const uint4* c4 = reinterpret_cast<const uint4*>(c + base);
#pragma unroll
    for (uint32_t k = 0; k < SCAN_ITEMS / 4; k++) {
        uint4 v = c4[k];
        s += v.x + v.y + v.z + v.w;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < SCAN_THREADS / 32; w++) t += red[w];
        part[blockIdx.x] = t;
    }
}
__global__ void __launch_bounds__(1024) k_scan_partials(uint32_t* part, uint32_t nblocks, uint32_t* total,
                                                        uint32_t* total2) {
    __shared__ uint32_t sh[1024];
    const uint32_t per = (nblocks + 1023) / 1024;
    uint32_t lo = threadIdx.x * per, hi = min(lo + per, nblocks), s = 0;
    for (uint32_t i = lo; i < hi; i++) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {                  // inclusive Hillis-Steele over the thread sums
        uint32_t v = threadIdx.x >= off ? sh[threadIdx.x - off] : 0u;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? sh[threadIdx.x - 1] : 0u;
    for (uint32_t i = lo; i < hi; i++) { uint32_t v = part[i]; part[i] = run; run += v; }
    if (threadIdx.x == 1023) { *total = sh[1023]; *total2 = sh[1023]; }
}
// Each hash's first record (its sub-list 0's start) is also written to heads, so that a gather reads its eight cells'
// ranges from 4 MB rather than from the 128 MB of buckets.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(uint32_t* __restrict__ c, const uint32_t* __restrict__ part,
                                                            uint32_t* __restrict__ heads) {
    __shared__ uint32_t wsum[SCAN_THREADS / 32];
    const uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS];
    uint4* c4 = reinterpret_cast<uint4*>(c + base);
#pragma unroll
    for (uint32_t k = 0; k < SCAN_ITEMS / 4; k++) {
        uint4 q = c4[k];
        v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
    }
    uint32_t s = 0;
#pragma unroll
    for (uint32_t k = 0; k < SCAN_ITEMS; k++) s += v[k];
    // the thread's exclusive offset within the block: a warp scan, then the warps'
    uint32_t incl = s;
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[threadIdx.x >> 5] = incl;
    __syncthreads();
    uint32_t woff = 0;
    for (uint32_t w = 0; w < (threadIdx.x >> 5); w++) woff += wsum[w];
    uint32_t run = part[blockIdx.x] + woff + incl - s;
#pragma unroll
    for (uint32_t k = 0; k < SCAN_ITEMS; k++) { uint32_t t = v[k]; v[k] = run; run += t; }
#pragma unroll
    for (uint32_t k = 0; k < SCAN_ITEMS / 4; k++) c4[k] = make_uint4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    static_assert(SPPM_SUBS % SCAN_ITEMS == 0, "a hash's buckets start on a thread's first item");
    if (base % SPPM_SUBS == 0u) heads[base / SPPM_SUBS] = v[0];
}

// THE SCATTER: each record into its bucket's range at its rank, the records themselves permuted with it
__global__ void __launch_bounds__(256) k_sppm_scatter(const uint32_t* __restrict__ bucket, const uint32_t* __restrict__ rank,
                                                      const uint32_t* __restrict__ start, const SppmDev* __restrict__ d,
                                                      const float4* __restrict__ pos, const float4* __restrict__ pow,
                                                      const uint32_t* __restrict__ dir, const uint32_t* __restrict__ nrm,
                                                      const uint32_t* __restrict__ flags, uint32_t* __restrict__ order,
                                                      float4* __restrict__ spos, float4* __restrict__ spow,
                                                      uint32_t* __restrict__ sdir, uint32_t* __restrict__ snrm,
                                                      uint32_t* __restrict__ sflags) {
    const uint32_t n = min(d->count, d->cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t at = start[bucket[i]] + rank[i];
        order[at] = i;
        spos[at] = pos[i];
        spow[at] = pow[i];
        sdir[at] = dir[i];
        snrm[at] = nrm[i];
        sflags[at] = flags[i];
    }
}

// a hash's count and start, for the host's reading of the grid (the reference's per-cell counts, sppm.js:415)
__global__ void k_sppm_cells(const uint32_t* __restrict__ heads, uint32_t* __restrict__ cnt, uint32_t* __restrict__ cst) {
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < SPPM_HEADS; h += gridDim.x * blockDim.x) {
        uint32_t a = heads[h], b = heads[h + 1];
        cnt[h] = b - a;
        cst[h] = a;
    }
}

// THE GATHER (sppm.js:305-346 sppmWalk, :475-494 sppmGather) at each query point, a Lambertian surface of the given
// albedo there (f = albedo / pi): the eight cells, the whole cell's range while its count is within its share of
// the budget, else m sub-lists' ranges from a drawn start, each record found weighing 32 / m; records of another
// cell with the same hash, past the radius (f32, unfused, as the reference's), facing away (n . n_p < 0.9), or past
// the bounce cap passed by. FP64 sums.
__global__ void __launch_bounds__(128) k_sppm_gather(const float* __restrict__ qpos, const float* __restrict__ qnrm,
                                                     const float* __restrict__ qalb, const uint32_t* __restrict__ qb,
                                                     uint32_t m, float radius, float cell, uint32_t maxbounce,
                                                     uint32_t budget, uint4 sseed, const uint32_t* __restrict__ start,
                                                     const uint32_t* __restrict__ heads, const float4* __restrict__ spos, const float4* __restrict__ spow,
                                                     const uint32_t* __restrict__ snrm,
                                                     const uint32_t* __restrict__ sflags, double* __restrict__ out,
                                                     uint32_t* __restrict__ stats) {
    const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= m) return;
    const f3 x = mk(qpos[3 * qi], qpos[3 * qi + 1], qpos[3 * qi + 2]);
    const f3 nq = mk(qnrm[3 * qi], qnrm[3 * qi + 1], qnrm[3 * qi + 2]);
    const double ar = (double)qalb[3 * qi] / 3.14159265358979323846, ag = (double)qalb[3 * qi + 1] / 3.14159265358979323846,
                 ab = (double)qalb[3 * qi + 2] / 3.14159265358979323846;
    Rng rng = path_rng(sseed, qi, SPPM_SALT);
    const float gx[3] = {__fdiv_rn(x.x, cell), __fdiv_rn(x.y, cell), __fdiv_rn(x.z, cell)};
    int32_t c0[3], side[3];
    for (int a = 0; a < 3; a++) {
        c0[a] = (int32_t)floorf(gx[a]);
        side[a] = (__fsub_rn(gx[a], floorf(gx[a])) >= 0.5f) ? 1 : -1;
    }
    const uint32_t bc = qb[qi] + 1;
    const bool unlimited = budget == 0;
    const uint32_t share = unlimited ? 0xFFFFFFFFu : max(1u, budget / 8);
    const unsigned long long hard = unlimited ? ~0ull : (unsigned long long)SPPM_VISIT_HARD * budget;
    const float r2 = __fmul_rn(radius, radius);
    double sr = 0, sg = 0, sb = 0;
    unsigned long long visits = 0;
    bool cut = false;
    for (uint32_t k = 0; k < 8 && !cut; k++) {
        const int32_t cx = c0[0] + ((k & 1) ? side[0] : 0), cy = c0[1] + ((k & 2) ? side[1] : 0),
                      cz = c0[2] + ((k & 4) ? side[2] : 0);
        const uint32_t h = sppm_hash(cx, cy, cz);
        const uint32_t a0 = heads[h], a1 = heads[h + 1];
        const uint32_t count = a1 - a0;
        const bool whole = count <= share;
        const uint32_t subs = whole ? 1u : max(1u, (SPPM_SUBS * share) / max(count, 1u));
        const double w = whole ? 1.0 : (double)SPPM_SUBS / subs;
        float4 r4 = rng.next();
        const uint32_t st0 = min((uint32_t)(r4.x * (float)SPPM_SUBS), SPPM_SUBS - 1);
        for (uint32_t j = 0; j < subs && !cut; j++) {
            uint32_t lo, hi;
            if (whole) { lo = a0; hi = a1; }
            else { uint32_t s = (st0 + j) % SPPM_SUBS; lo = start[h * SPPM_SUBS + s]; hi = start[h * SPPM_SUBS + s + 1]; }
            for (uint32_t q = lo; q < hi; q++) {
                if (visits >= hard) { cut = true; break; }
                visits++;
                const float4 p = spos[q];
                if (cell_of(p.x, cell) != cx || cell_of(p.y, cell) != cy || cell_of(p.z, cell) != cz) continue;
                float dx = __fsub_rn(p.x, x.x), dy = __fsub_rn(p.y, x.y), dz = __fsub_rn(p.z, x.z);
                float dd = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                if (dd > r2) continue;
                const uint32_t b = sflags[q];
                if ((b & SPPM_VOL) || bc + (b & SPPM_B_MASK) > maxbounce + 1) continue;
                f3 pn = unoct(snrm[q]);
                float nd = __fadd_rn(__fadd_rn(__fmul_rn(pn.x, nq.x), __fmul_rn(pn.y, nq.y)), __fmul_rn(pn.z, nq.z));
                if (nd < 0.9f) continue;
                const float4 pw = spow[q];
                sr += w * (ar * (double)pw.x);
                sg += w * (ag * (double)pw.y);
                sb += w * (ab * (double)pw.z);
            }
        }
    }
    out[3 * qi] = sr; out[3 * qi + 1] = sg; out[3 * qi + 2] = sb;
    atomicAdd(&stats[0], 1u);
    if (cut) atomicAdd(&stats[1], 1u);
    atomicMax(&stats[2], (uint32_t)min(visits, 0xffffffffull));
    atomicAdd(reinterpret_cast<unsigned long long*>(&stats[4]), visits);
}

}  // namespace

// the map's buffers for n records (kept, grown as needed)
int sppm_ensure(st_ctx* ctx, uint32_t n) {
    SppmState& s = ctx_ext(ctx).sppm;
    auto fail = [&](const char* what) { ctx_set_error(ctx, what); return ST_ERR_OOM; };
    if (!s.cell_start) {
        if (cudaMalloc(&s.dev, sizeof(SppmDev)) != cudaSuccess) return fail("cudaMalloc photon grid");
        if (cudaMemset(s.dev, 0, sizeof(SppmDev)) != cudaSuccess) return fail("memset photon grid");
        if (cudaMalloc(&s.cell_start, (size_t)(SPPM_BUCKETS + SCAN_TILE) * 4) != cudaSuccess) return fail("cudaMalloc photon grid");
        if (cudaMalloc(&s.scan_part, (size_t)(SCAN_BLOCKS + 8) * 4) != cudaSuccess) return fail("cudaMalloc photon grid");
        if (cudaMalloc(&s.heads, (size_t)(SPPM_HEADS + 32) * 4) != cudaSuccess) return fail("cudaMalloc photon grid");
        if (cudaMalloc(&s.cell_count, (size_t)SPPM_HEADS * 4 * 2) != cudaSuccess) return fail("cudaMalloc photon grid");
        if (cudaMalloc(&s.stats, 8 * 4) != cudaSuccess) return fail("cudaMalloc photon grid");
        if (cudaMalloc(&s.lt_emit, LT_CELLS * 4) != cudaSuccess || cudaMalloc(&s.lt_hit, LT_CELLS * 4) != cudaSuccess ||
            cudaMalloc(&s.lt_cdf, (LT_CELLS + LT_GRID) * 4) != cudaSuccess)
            return fail("cudaMalloc emission map");
        // the uniform map: each row's conditional CDF (c + 1) / G, the rows' CDF likewise
        s.lt_uniform.assign(LT_CELLS + LT_GRID, 0.f);
        for (uint32_t r = 0; r < LT_GRID; r++)
            for (uint32_t c = 0; c < LT_GRID; c++) s.lt_uniform[r * LT_GRID + c] = c + 1 == LT_GRID ? 1.f : (float)(c + 1) / LT_GRID;
        for (uint32_t r = 0; r < LT_GRID; r++) s.lt_uniform[LT_CELLS + r] = r + 1 == LT_GRID ? 1.f : (float)(r + 1) / LT_GRID;
        if (sppm_lt_reset(s, ctx_stream(ctx)) != cudaSuccess || cudaStreamSynchronize(ctx_stream(ctx)) != cudaSuccess)
            return fail("emission map reset");
    }
    if (n > s.cap) {
        void* ps[] = {s.pos, s.power, s.dir_oct, s.nrm_oct, s.flags, s.key, s.order, s.spos, s.spow, s.sdir,
                      s.snrm, s.sflags, s.bucket, s.rank};
        for (void* p : ps) if (p) cudaFree(p);
        uint32_t cap = std::max(n, 1024u);
        bool ok = cudaMalloc(&s.pos, (size_t)cap * 16) == cudaSuccess && cudaMalloc(&s.power, (size_t)cap * 16) == cudaSuccess &&
                  cudaMalloc(&s.dir_oct, (size_t)cap * 4) == cudaSuccess && cudaMalloc(&s.nrm_oct, (size_t)cap * 4) == cudaSuccess &&
                  cudaMalloc(&s.flags, (size_t)cap * 4) == cudaSuccess && cudaMalloc(&s.key, (size_t)cap * 4) == cudaSuccess &&
                  cudaMalloc(&s.order, (size_t)cap * 4) == cudaSuccess && cudaMalloc(&s.spos, (size_t)cap * 16) == cudaSuccess &&
                  cudaMalloc(&s.spow, (size_t)cap * 16) == cudaSuccess && cudaMalloc(&s.sdir, (size_t)cap * 4) == cudaSuccess &&
                  cudaMalloc(&s.snrm, (size_t)cap * 4) == cudaSuccess && cudaMalloc(&s.sflags, (size_t)cap * 4) == cudaSuccess &&
                  cudaMalloc(&s.bucket, (size_t)cap * 4) == cudaSuccess && cudaMalloc(&s.rank, (size_t)cap * 4) == cudaSuccess;
        if (!ok) { s.cap = 0; return fail("cudaMalloc photon records"); }
        s.cap = cap;
    }
    return ST_OK;
}

// THE GRID'S BUILD from the records the device holds (count and cell in s.dev): the buckets zeroed, the keys and
// ranks, the three-phase scan, the scatter into cell order -- a fixed launch shape, so a graph can hold it
cudaError_t sppm_grid_launch(SppmState& s, int sms, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(s.cell_start, 0, (size_t)(SPPM_BUCKETS + SCAN_TILE) * 4, st);
    if (e) return e;
    k_sppm_key<<<(uint32_t)sms * 16u, 256, 0, st>>>(s.pos, s.flags, s.dev, s.key, s.bucket, s.rank, s.cell_start);
    k_scan_sums<<<SCAN_BLOCKS, SCAN_THREADS, 0, st>>>(s.cell_start, s.scan_part);
    k_scan_partials<<<1, 1024, 0, st>>>(s.scan_part, SCAN_BLOCKS, s.cell_start + SPPM_BUCKETS, s.heads + SPPM_HEADS);
    k_scan_apply<<<SCAN_BLOCKS, SCAN_THREADS, 0, st>>>(s.cell_start, s.scan_part, s.heads);
    // the sentinel: the total, past the last bucket (k_scan_apply's last tile covers [SPPM_BUCKETS - SCAN_TILE, SPPM_BUCKETS))
    k_sppm_scatter<<<(uint32_t)sms * 16u, 256, 0, st>>>(s.bucket, s.rank, s.cell_start, s.dev, s.pos, s.power, s.dir_oct,
                                                       s.nrm_oct, s.flags, s.order, s.spos, s.spow, s.sdir, s.snrm,
                                                       s.sflags);
    return cudaGetLastError();
}
// the emission map back to uniform, its counts cleared (raytrace_main.js:347, a reset)
cudaError_t sppm_lt_reset(SppmState& s, cudaStream_t st) {
    if (!s.lt_cdf) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(s.lt_emit, 0, LT_CELLS * 4, st);
    if (!e) e = cudaMemsetAsync(s.lt_hit, 0, LT_CELLS * 4, st);
    if (!e) e = cudaMemcpyAsync(s.lt_cdf, s.lt_uniform.data(), (LT_CELLS + LT_GRID) * 4, cudaMemcpyHostToDevice, st);
    return e;
}
SppmBufs sppm_bufs(const SppmState& s) {
    SppmBufs b;
    b.dev = s.dev;
    b.cap = s.cap;
    b.pos = s.pos; b.power = s.power; b.dir_oct = s.dir_oct; b.nrm_oct = s.nrm_oct; b.flags = s.flags;
    b.lt_emit = s.lt_emit; b.lt_hit = s.lt_hit; b.lt_cdf = s.lt_cdf;
    b.start = s.cell_start; b.heads = s.heads; b.spos = s.spos; b.spow = s.spow; b.sdir = s.sdir; b.snrm = s.snrm; b.sflags = s.sflags;
    return b;
}

extern "C" {

int st_sppm_build(st_ctx* ctx, const float* pos, const float* power, const uint32_t* dir_oct, const uint32_t* nrm_oct,
                  const uint32_t* flags, uint32_t n, float cell) {
    if (!ctx || (n && (!pos || !power || !nrm_oct || !flags)) || !(cell > 0)) return ST_ERR_ARG;
    if (n > (1u << 28)) { ctx_set_error(ctx, "more than 2^28 photon records"); return ST_ERR_ARG; }
    cudaSetDevice(ctx_device(ctx));
    int rc = sppm_ensure(ctx, n);
    if (rc) return rc;
    SppmState& s = ctx_ext(ctx).sppm;
    cudaStream_t st = ctx_stream(ctx);
    auto ck = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess) { ctx_set_error(ctx, std::string(what) + ": " + cudaGetErrorString(e)); return false; }
        return true;
    };
    // the records, host -> device, as float4 points and powers (16-byte loads in every kernel after)
    std::vector<float4> p4(n), w4(n);
    for (uint32_t i = 0; i < n; i++) {
        p4[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.f);
        w4[i] = make_float4(power[3 * i], power[3 * i + 1], power[3 * i + 2], 0.f);
    }
    s.wave = false;
    SppmDev hd{};
    hd.count = n; hd.cap = s.cap; hd.cell = cell; hd.vcell = cell;   // (records given here are a surface's)
    if (!ck(cudaMemcpyAsync(s.dev, &hd, sizeof(hd), cudaMemcpyHostToDevice, st), "photon upload") || !ck(cudaMemcpyAsync(s.pos, p4.data(), (size_t)n * 16, cudaMemcpyHostToDevice, st), "photon upload") ||
        !ck(cudaMemcpyAsync(s.power, w4.data(), (size_t)n * 16, cudaMemcpyHostToDevice, st), "photon upload") ||
        !ck(cudaMemcpyAsync(s.nrm_oct, nrm_oct, (size_t)n * 4, cudaMemcpyHostToDevice, st), "photon upload") ||
        !ck(cudaMemcpyAsync(s.flags, flags, (size_t)n * 4, cudaMemcpyHostToDevice, st), "photon upload") ||
        !ck(cudaMemsetAsync(s.stats, 0, 8 * 4, st), "memset"))
        return ST_ERR_CUDA;
    if (!ck(dir_oct ? cudaMemcpyAsync(s.dir_oct, dir_oct, (size_t)n * 4, cudaMemcpyHostToDevice, st)
                    : cudaMemsetAsync(s.dir_oct, 0, (size_t)n * 4, st), "photon upload"))
        return ST_ERR_CUDA;
    if (!ck(sppm_grid_launch(s, ctx_sms(ctx), st), "photon grid launch") || !ck(cudaStreamSynchronize(st), "photon grid"))
        return ST_ERR_CUDA;
    s.n = n;
    s.cell = cell;
    return ST_OK;
}

int st_sppm_read_grid(st_ctx* ctx, uint32_t* key, uint32_t* cell_count, uint32_t* cell_start, uint32_t* order) {
    if (!ctx) return ST_ERR_ARG;
    SppmState& s = ctx_ext(ctx).sppm;
    if (!s.cell_start) { ctx_set_error(ctx, "no photon grid built"); return ST_ERR_STATE; }
    cudaSetDevice(ctx_device(ctx));
    cudaStream_t st = ctx_stream(ctx);
    uint32_t* cnt = s.cell_count;
    uint32_t* cst = s.cell_count + SPPM_HEADS;
    k_sppm_cells<<<1024, 256, 0, st>>>(s.heads, cnt, cst);
    cudaError_t e = cudaGetLastError();
    if (!e && key && s.n) e = cudaMemcpyAsync(key, s.key, (size_t)s.n * 4, cudaMemcpyDeviceToHost, st);
    if (!e && order && s.n) e = cudaMemcpyAsync(order, s.order, (size_t)s.n * 4, cudaMemcpyDeviceToHost, st);
    if (!e && cell_count) e = cudaMemcpyAsync(cell_count, cnt, (size_t)SPPM_HEADS * 4, cudaMemcpyDeviceToHost, st);
    if (!e && cell_start) e = cudaMemcpyAsync(cell_start, cst, (size_t)SPPM_HEADS * 4, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) { ctx_set_error(ctx, std::string("photon grid readback: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
    return ST_OK;
}

int st_sppm_gather(st_ctx* ctx, const float* qpos, const float* qnrm, const float* qalbedo, const uint32_t* qbounce,
                   uint32_t m, float radius, uint32_t maxbounce, uint32_t budget, uint32_t seed, double* out) {
    if (!ctx || (m && (!qpos || !qnrm || !qalbedo || !qbounce || !out)) || !(radius > 0)) return ST_ERR_ARG;
    SppmState& s = ctx_ext(ctx).sppm;
    if (!s.cell_start) { ctx_set_error(ctx, "no photon grid built"); return ST_ERR_STATE; }
    if (!(2 * radius <= s.cell * 1.0001f)) {
        ctx_set_error(ctx, "the gather radius must be at most half the cell (sppm.js neighbourCells)");
        return ST_ERR_ARG;
    }
    if (m == 0) return ST_OK;
    cudaSetDevice(ctx_device(ctx));
    cudaStream_t st = ctx_stream(ctx);
    float *dq = nullptr;
    uint32_t* db = nullptr;
    double* dout = nullptr;
    cudaError_t e = cudaMalloc(&dq, (size_t)m * 9 * 4);
    if (!e) e = cudaMalloc(&db, (size_t)m * 4);
    if (!e) e = cudaMalloc(&dout, (size_t)m * 3 * 8);
    if (!e) e = cudaMemcpyAsync(dq, qpos, (size_t)m * 12, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(dq + 3 * (size_t)m, qnrm, (size_t)m * 12, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(dq + 6 * (size_t)m, qalbedo, (size_t)m * 12, cudaMemcpyHostToDevice, st);
    if (!e) e = cudaMemcpyAsync(db, qbounce, (size_t)m * 4, cudaMemcpyHostToDevice, st);
    if (!e) {
        k_sppm_gather<<<(m + 127) / 128, 128, 0, st>>>(dq, dq + 3 * (size_t)m, dq + 6 * (size_t)m, db, m, radius,
                                                      s.cell, maxbounce, budget, sample_seed(seed, 0), s.cell_start,
                                                      s.heads, s.spos, s.spow, s.snrm, s.sflags, dout, s.stats);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(out, dout, (size_t)m * 24, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (dq) cudaFree(dq);
    if (db) cudaFree(db);
    if (dout) cudaFree(dout);
    if (e) { ctx_set_error(ctx, std::string("photon gather: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
    return ST_OK;
}

int st_sppm_emission_map(st_ctx* ctx, uint32_t* sent, uint32_t* stored, float* cdf) {
    if (!ctx) return ST_ERR_ARG;
    SppmState& s = ctx_ext(ctx).sppm;
    if (!s.lt_cdf) { ctx_set_error(ctx, "no photon map has run"); return ST_ERR_STATE; }
    cudaSetDevice(ctx_device(ctx));
    cudaStream_t st = ctx_stream(ctx);
    cudaError_t e = cudaStreamSynchronize(st);
    if (!e && sent) e = cudaMemcpyAsync(sent, s.lt_emit, LT_CELLS * 4, cudaMemcpyDeviceToHost, st);
    if (!e && stored) e = cudaMemcpyAsync(stored, s.lt_hit, LT_CELLS * 4, cudaMemcpyDeviceToHost, st);
    if (!e && cdf) e = cudaMemcpyAsync(cdf, s.lt_cdf, (LT_CELLS + LT_GRID) * 4, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) { ctx_set_error(ctx, std::string("emission map readback: ") + cudaGetErrorString(e)); return ST_ERR_CUDA; }
    return ST_OK;
}

int st_sppm_stats_read(st_ctx* ctx, st_sppm_stats* out) {
    if (!ctx || !out) return ST_ERR_ARG;
    SppmState& s = ctx_ext(ctx).sppm;
    if (!s.stats) { *out = st_sppm_stats{}; return ST_OK; }
    cudaSetDevice(ctx_device(ctx));
    if (s.wave) {                              // the wavefront's map: its last sample's records, gathers and walks
        SppmDev d;
        if (cudaStreamSynchronize(ctx_stream(ctx)) != cudaSuccess ||
            cudaMemcpy(&d, s.dev, sizeof(d), cudaMemcpyDeviceToHost) != cudaSuccess)
            return ST_ERR_CUDA;
        *out = st_sppm_stats{};
        out->stored = std::min(d.count, d.cap);
        out->cut = d.dropped;
        out->gathers = d.gathers;
        out->visits = d.visits;
        return ST_OK;
    }
    uint32_t h[8];
    if (cudaMemcpy(h, s.stats, 32, cudaMemcpyDeviceToHost) != cudaSuccess) return ST_ERR_CUDA;
    out->stored = s.n;
    out->gathers = h[0];
    out->cut = h[1];
    out->visits_max = h[2];
    uint64_t v;
    std::memcpy(&v, &h[4], 8);
    out->visits = v;
    return ST_OK;
}

}  // extern "C"
