// bulk_copy.cuh — copy-engine (TMA) tile loads into shared memory with mbarrier
// completion, and bounded waits on them.
//
// A tensor copy is described by a 128-byte tensor map built on the host
// (cuTensorMapEncodeTiled) and passed as a __grid_constant__ kernel parameter.
// One thread arms the slot's mbarrier with the byte count and issues the copy;
// every thread that reads the slot waits on the barrier's phase parity. Waits
// give up after about one second of global time, so a copy that never lands
// is reported (the caller sets a status word the host reads) instead of
// hanging the GPU.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace wfs {

// Host-built tensor map, carried as plain bytes (the driver's CUtensorMap is 128 bytes, 64-aligned).
struct alignas(64) TensorMapImage {
    unsigned long long opaque[16];
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
// Makes initialised barriers visible to the copy engine.
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
// Arrives on the barrier and adds `bytes` to the transaction count its phase waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}
// Default limit of a bounded wait: about one second of global time.
constexpr uint64_t kWaitLimitNs = 1000000000ull;
// Waits for the phase with the given parity to complete, for at most limit_ns of global
// time. A limit of 1 ns or less gives up at once without polling, which is how the
// engine's test hook (wfs_set_copy_wait_limit) makes the expiry path run.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
    if (limit_ns <= 1) return false;
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}
// Orders this thread's earlier generic-proxy accesses of shared memory before later
// copy-engine writes to it (a slot that threads read is about to be refilled).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// 3D tiled tensor copy global -> shared, completing on the barrier.
__device__ __forceinline__ void tensor_load_3d(uint32_t dst, const TensorMapImage* map, int x, int y, int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

}  // namespace wfs
