/*
 * Bulk asynchronous copies between global and shared memory (the TMA engine's non-tensor form,
 * cp.async.bulk, sm_90 and later) with an mbarrier for completion, as inline PTX.
 *
 * Used to stage path-state records: every lane of a warp starts the copy of its own record with one
 * instruction, so a warp waits for one round trip to memory instead of one per record.
 *   global -> shared: cp.async.bulk ... mbarrier::complete_tx::bytes, completion on a per-warp
 *                     mbarrier whose expected byte count is the sum of the warp's copies;
 *   shared -> global: cp.async.bulk ... bulk_group, per-thread commit and wait.
 * Sizes and both addresses must be multiples of 16 bytes.  Every wait is bounded: a wait that runs
 * out sets an error bit for the host instead of spinning forever.
 */
#pragma once
#include <stdint.h>

namespace lg {

/* device error word bits (DeviceScene::err), read and cleared by the host after a render */
enum : int { LG_ERR_STACK = 1, LG_ERR_STAGE_TIMEOUT = 2 };

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(arrivals) : "memory");
}
/* make barrier initialisation visible to the asynchronous (copy engine) proxy */
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
/* order this thread's earlier ordinary shared-memory accesses before later asynchronous-proxy ones */
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
/* bounded wait for the phase of the given parity; false when the bound ran out */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (int i = 0; i < (1 << 22); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_load(void *dst_smem, const void *src_gmem, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst_smem)),
                 "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst_gmem, const void *src_smem, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_gmem), "r"(smem_addr(src_smem)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
/* the source of every committed store has been read (the shared memory may be reused) */
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
/* every committed store has completed */
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace lg
