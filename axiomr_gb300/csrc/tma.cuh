// Tensor-memory-accelerator (TMA) copies of 16x16 framebuffer tiles and the shared-memory
// barrier that tracks their arrival, as inline PTX (PTX ISA: cp.async.bulk.tensor,
// mbarrier). The tensor maps describe one plane of a framebuffer (uint32 colour or float
// depth, [height][width], 16x16 boxes, no swizzle); a box that reaches past the plane's edge
// is clipped by the hardware on stores and filled with zeros on loads. A copy's x
// coordinate is a multiple of 16 pixels (64 bytes), so every copy starts 16-byte aligned.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch_types.h"

namespace axr {
namespace {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// This thread's shared-memory writes -> visible to the TMA unit (before a tensor store).
__device__ __forceinline__ void tma_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tma_store_tile(const TensorMap128* map, const void* smem, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
                 :
                 : "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_addr(smem)), "r"(x), "r"(y)
                 : "memory");
}

__device__ __forceinline__ void tma_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Wait until at most one committed store group is still reading shared memory.
__device__ __forceinline__ void tma_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }

// Wait until no committed store group is still reading shared memory.
__device__ __forceinline__ void tma_wait_read_0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

__device__ __forceinline__ void tma_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---- shared-memory barrier of tile loads (one thread arrives and announces the bytes; the
// loads complete the transaction)
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// The initialised barrier -> visible to the TMA unit.
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_tile(const TensorMap128* map, void* smem, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        :
        : "r"(smem_addr(smem)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return done != 0;
}

// Bounded wait for phase `phase` of the barrier: gives up after about `limit` polls (each
// try_wait suspends the thread for a while when the phase is incomplete) and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t limit = 1u << 20) {
    for (uint32_t i = 0; i < limit; ++i) {
        if (mbar_try_wait(bar, phase)) return true;
        if (i > 64) __nanosleep(128);
    }
    return false;
}

}  // namespace
}  // namespace axr
