/*
 * tma.cuh - the bulk-copy (TMA) and mbarrier operations the calling kernels
 * use to stage read data in shared memory, as inline PTX for sm_103a.
 *
 *   bulk_copy_g2s   cp.async.bulk of `bytes` from global to shared memory,
 *                   completing on an mbarrier.  Both addresses 16-byte
 *                   aligned, bytes a multiple of 16.
 *   mbar_*          one shared-memory mbarrier per staging buffer, one
 *                   arrival (with the expected byte count) per phase.
 *   mbar_wait_bounded  waits for a phase with a time limit (globaltimer): a
 *                   phase that does not complete within the limit returns
 *                   false instead of spinning on, so that the kernel can
 *                   report an error and return.
 */
#ifndef GSNP_TMA_CUH
#define GSNP_TMA_CUH

#include <stdint.h>

namespace gsnp {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
    /* make the initialised barrier visible to the async (bulk-copy) proxy */
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* Wait, every lane of the warp together, until the barrier's phase of the
 * given parity has completed; false (warp-uniform) when limit_ns passes
 * first. */
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        const bool ok = mbar_test_wait(bar, parity);
        if (__all_sync(0xffffffffu, ok)) return true;
        bool late = globaltimer_ns() - t0 > limit_ns;
        late = __shfl_sync(0xffffffffu, late, 0);
        if (late) return false;
        __nanosleep(64);
    }
}

/* order this thread's earlier generic accesses of shared memory before
 * later bulk copies into it */
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

/* prefetch `bytes` of global memory into L2 with the bulk-copy unit (16-byte
 * aligned address, bytes a multiple of 16) */
__device__ __forceinline__ void bulk_prefetch_l2(const void* src_gmem, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src_gmem), "r"(bytes) : "memory");
}

}  // namespace gsnp

#endif
