// st_kernels.cuh -- device helpers the wavefront kernels share (st_render.cu, st_optics.cu): the lane mask, the
// shared-memory table stage by a bulk copy with its bounded wait, the warp-aggregated queue append, the deposit.
#pragma once
#include "st_internal.h"

namespace st {

#define FULL_MASK 0xffffffffu
#define INVALID_SLOT 0xffffffffu
#define WAIT_LIMIT (1u << 24)

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------------------------------------------------------------------
// A TABLE INTO SHARED MEMORY BY ONE BULK COPY: thread 0 arms an mbarrier with the byte count and issues
// cp.async.bulk; every thread waits on the barrier's phase, a bounded number of times. bytes is a multiple of 16,
// both addresses 16-byte aligned (DPrim is 128 bytes, st_material 64, cudaMalloc 256-aligned). Returns false
// (and flags the counters) if the copy did not land within the limit.
//
// THE LIMIT is the counters' wait_limit (0: WAIT_LIMIT), so a host can make it short; with wait_arm_only set the
// barrier is armed but no copy is issued -- a test of this failure path: the wait runs out at its limit with nothing
// in flight, the CTA flags the error and returns, and the context stays usable. Where a real copy was issued and the
// wait ran out, the CTA waits once more (bounded again) for that copy to land in its shared memory before it leaves.
// The reference's own guards against a GPU that never finishes are host-side (core/wavefront.js:298-303 clamps the
// indirect dispatch, core/raytrace_main.js:67 cuts a frame's submissions); a wait on the device has none there.
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t mbar_try(uint32_t mb) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(mb) : "memory");
    return done;
}
__device__ __forceinline__ bool stage_table(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* mbar,
                                            DevCtr* ctr) {
    uint32_t mb = (uint32_t)__cvta_generic_to_shared(mbar);
    uint32_t dst = (uint32_t)__cvta_generic_to_shared(sdst);
    const uint32_t wl = ctr->wait_limit;
    const uint32_t limit = wl ? wl : WAIT_LIMIT;
    const bool issue = ctr->wait_arm_only == 0u;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
        if (issue)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         ::"r"(dst), "l"(gsrc), "r"(bytes), "r"(mb) : "memory");
    }
    uint32_t done = 0;
    for (uint32_t k = 0; k < limit && !done; k++) done = mbar_try(mb);
    // one decision for the whole CTA, so no thread leaves while another still waits at a barrier
    if (__syncthreads_or(!done)) {
        if (threadIdx.x == 0) atomicExch(&ctr->errflag, 1u);
        if (issue)                                   // the copy in flight: let it land before the CTA is gone
            for (uint32_t k = 0; k < WAIT_LIMIT && !done; k++) done = mbar_try(mb);
        __syncthreads();
        return false;
    }
    return true;
}

// warp-aggregated append: one atomic per warp for every lane with want set; returns this lane's position
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want) {
    uint32_t m = __ballot_sync(FULL_MASK, want);
    uint32_t base = 0;
    int lane = threadIdx.x & 31;
    int leader = m ? __ffs(m) - 1 : 0;
    if (m && lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(FULL_MASK, base, leader);
    return base + __popc(m & lanemask_lt());
}

// ------------------------------------------------------------------------------------------------------------
// THE DEPOSIT (wavefront.js:162-245): refused if a channel is NaN or inf or the luminance negative
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ bool bad_deposit(f3 c) {
    return !isfinite(c.x) || !isfinite(c.y) || !isfinite(c.z) || luma(c) < 0.f;
}
__device__ __forceinline__ void deposit(float4* frame, uint32_t pix, f3 c, DevCtr* ctr) {
    if (bad_deposit(c)) { atomicAdd(&ctr->nonfinite, 1u); return; }
    float* f = reinterpret_cast<float*>(frame + pix);
    if (c.x != 0.f) atomicAdd(f + 0, c.x);
    if (c.y != 0.f) atomicAdd(f + 1, c.y);
    if (c.z != 0.f) atomicAdd(f + 2, c.z);
}

}  // namespace st
