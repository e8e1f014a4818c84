// st_tc.cuh -- the 5th-generation tensor cores of sm_103a (tcgen05) for the learned proposal's network: the tensor
// memory (TMEM) that holds an MMA's accumulator, the shared-memory operand descriptors, the MMA itself issued by one
// thread, its completion signalled to an mbarrier, and the accumulator read back to registers.
//
// OPERANDS IN SHARED MEMORY, K-MAJOR, NO SWIZZLE (the canonical layout of core matrices): a core matrix is 8 rows x 16
// bytes (8 BF16 along K), its rows consecutive (128 bytes). For a matrix of R rows and K columns the core matrix of
// rows 8i.. and columns 8j.. sits at i * SBO + j * 128: LBO = 128 (the next core matrix along K), SBO = K / 8 * 128
// (the next 8 rows). One MMA takes K = 16 (two core matrices along K); the k-th starts 256 bytes on.
//
// THE INSTRUCTION DESCRIPTOR (kind::f16): D format F32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both
// K-major (bits 15, 16 = 0), N / 8 at bits 17-22, M / 16 at bits 24-28.
#pragma once
#include "st_internal.h"

namespace st {

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// a shared-memory matrix descriptor: start address, LBO, SBO (bytes), version 1 (bits 46-47), no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}
__host__ __device__ constexpr uint32_t tc_idesc_bf16(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}
// the byte offset of element (row r, column k) of a K-major no-swizzle BF16 matrix of K columns
__host__ __device__ __forceinline__ uint32_t tc_off(uint32_t r, uint32_t k, uint32_t K) {
    return (r >> 3) * (K * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// TMEM: allocated and freed by one whole warp; the address lands in shared memory
__device__ __forceinline__ void tc_alloc(uint32_t* dst_smem, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(dst_smem)),
                 "r"(cols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy writes to shared memory made visible to the tensor cores' (async proxy) reads
__device__ __forceinline__ void tc_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D (TMEM) = A . B^T (+ D when accumulate): one thread issues it
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate) : "memory");
}
// the issuing thread's MMAs so far signal the mbarrier when they are done
__device__ __forceinline__ void tc_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(mbar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// the barrier's phase `parity` completed, polled at most `limit` times; false if it never did
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
    const uint32_t mb = tc_smem(mbar);
    for (uint32_t k = 0; k < limit; k++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(mb), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// 64 columns of this warp's 32 TMEM lanes, one lane a thread: v[j] = column col + j of the thread's lane
#define TC_R8(i) "=r"(v[i]), "=r"(v[i + 1]), "=r"(v[i + 2]), "=r"(v[i + 3]), "=r"(v[i + 4]), "=r"(v[i + 5]), \
                 "=r"(v[i + 6]), "=r"(v[i + 7])
__device__ __forceinline__ void tc_ld64(uint32_t taddr, uint32_t (&v)[64]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,"
        "%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,"
        "%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
        : TC_R8(0), TC_R8(8), TC_R8(16), TC_R8(24), TC_R8(32), TC_R8(40), TC_R8(48), TC_R8(56)
        : "r"(taddr) : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
#undef TC_R8

}  // namespace st
