/* tc.cuh - fifth-generation tensor core (tcgen05) building blocks for sm_100 / sm_103, as inline PTX.
 *
 * One CTA (cta_group::1) computes D[M x N] (+)= A[M x K] * B[N x K]^T with A and B in shared memory (bf16, K-major)
 * and D in tensor memory (fp32). One elected thread issues the MMAs; tcgen05.commit arrives on an mbarrier when
 * they (and their shared-memory reads) are complete; the warps then read D with tcgen05.ld, warp w owning TMEM
 * lanes [32 (w % 4), 32 (w % 4) + 32), one row of D per lane for M = 128.
 *
 * Operand layout ("no swizzle", K-major): a tile of R rows and K bf16 columns is a grid of core matrices of
 * 8 rows x 8 columns (8 x 16 bytes, 128 contiguous bytes, row r of the core matrix at byte 16 r). Core matrix
 * (r / 8, k / 8) lives at byte ((r / 8) * (K / 8) + k / 8) * 128: neighbours along K are 128 bytes apart (the
 * descriptor's leading byte offset), neighbours along R are K * 16 bytes apart (its stride byte offset).
 *
 * Waits on mbarriers are bounded: a wait that runs out sets an error flag and gives up, so a kernel can never
 * spin forever.
 */
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace lh2g {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

/* byte offset of element (r, k) in a no-swizzle K-major tile with K columns */
__host__ __device__ __forceinline__ uint32_t kmajor_offset(uint32_t r, uint32_t k, uint32_t K) {
    return ((r >> 3) * (K >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

/* shared memory matrix descriptor: start address, leading (K) and stride (R) byte offsets, version 1 (sm_100),
 * no swizzle */
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

/* instruction descriptor of kind::f16: bf16 A and B (K-major), fp32 D, shape M x N */
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

/* ---- tensor memory allocation (one full warp) ---- */
__device__ __forceinline__ void tmem_alloc(uint32_t* dstSmem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dstSmem)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

/* ---- ordering between thread-synchronised code and tcgen05 operations ---- */
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
/* generic-proxy shared-memory writes become visible to the tensor core's (async proxy) reads */
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* ---- MMA: D[tmem] (+)= A * B^T, issued by one thread ---- */
__device__ __forceinline__ void mma_bf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dTmem),
        "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
/* the mbarrier receives one arrival when every MMA issued before by this thread has completed */
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

/* ---- mbarrier ---- */
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
/* waits for the phase with the given parity to complete; false after `limit` polls (the caller records an error) */
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

/* ---- tensor memory -> registers: 32 lanes x 16 consecutive 32-bit columns, one lane per thread. The wait is in
 * the same asm statement, so the registers are never read before the load has completed. ---- */
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
          "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace lh2g
