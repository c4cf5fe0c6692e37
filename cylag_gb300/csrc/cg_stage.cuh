// cg_stage.cuh -- bulk-copy staging of particle-state tiles in shared memory.
//
// The mixed LSM1 step streams the particle state once per step (element
// index, position, PCG32 state, tag).  Each warp works through 32-particle
// tiles of the (element-sorted) state; while it steps one tile, the
// Blackwell bulk-copy engine brings the next into shared memory
// (cp.async.bulk global -> shared, completion counted on an mbarrier), so
// the HBM latency of the state leaves the per-particle dependency chain.
// Every wait is bounded: on a time-out the kernel records
// ERR_ASYNC_TIMEOUT, waits (bounded again) for its own copies and returns.
#pragma once

#include <cstdint>

namespace cg {

constexpr uint32_t ERR_ASYNC_TIMEOUT = 32;
constexpr uint32_t MBAR_POLL_LIMIT = 1u << 22;

// one warp's tile: 32 particles, 1024 bytes
struct alignas(128) WarpTile {
    float4 pos[32];      // split FP32 pairs, or the bits of FP64 pairs
    uint64_t rng[32];
    int tri[32];
    int tag[32];
};
constexpr uint32_t TILE_BYTES = sizeof(float4) * 32 + 8 * 32 + 4 * 32 + 4 * 32;
static_assert(TILE_BYTES == 1024, "tile layout");

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

// orders this thread's generic-proxy shared-memory accesses before later
// async-proxy ones (bulk copies into a buffer that was just read)
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
        "r"(bytes)
        : "memory");
}

// bytes (multiple of 16) from global src (16-byte aligned) to shared dst
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the phase with the given parity to complete
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t k = 0; k < MBAR_POLL_LIMIT; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// lane 0: the tile `tile` of the state arrays into `t` (all four copies
// complete one phase of `bar`)
__device__ __forceinline__ void stage_tile(WarpTile& t, uint64_t* bar, const void* pos,
                                           const uint64_t* rng, const int* tri, const int* tag,
                                           int tile) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(bar, TILE_BYTES);
    bulk_copy_g2s(t.pos, (const char*)pos + (size_t)tile * 512, 512, bar);
    bulk_copy_g2s(t.rng, rng + (size_t)tile * 32, 256, bar);
    bulk_copy_g2s(t.tri, tri + (size_t)tile * 32, 128, bar);
    bulk_copy_g2s(t.tag, tag + (size_t)tile * 32, 128, bar);
}

// ---------------------------------------------------------------------------
// per-thread asynchronous copies (cp.async): each thread prefetches its next
// particle's state into its own shared-memory slot one iteration ahead; the
// slot is private, so the thread's own wait_group is the only
// synchronization
// ---------------------------------------------------------------------------
struct ThreadSlot {
    float4 pos;
    uint64_t rng;
    int tri;
    int tag;
};

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
// all but the most recent `N` groups of this thread are complete
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// particle i's state into slot t (one group)
__device__ __forceinline__ void prefetch_slot(ThreadSlot& t, const void* pos, const uint64_t* rng,
                                              const int* tri, const int* tag, int i) {
    cp_async16(&t.pos, (const char*)pos + (size_t)i * 16);
    cp_async8(&t.rng, rng + i);
    cp_async4(&t.tri, tri + i);
    cp_async4(&t.tag, tag + i);
}

}  // namespace cg
