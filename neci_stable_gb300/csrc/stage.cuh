// stage.cuh -- tile staging for the row-stream kernels (k_sweep,
// k_merge_stats): 1-D TMA bulk copies (cp.async.bulk, global -> shared)
// completed on an mbarrier, double-buffered so that the copy of a block's
// next tile of CurrentDets rows runs while the current tile is processed.
//
// The rows of a tile are contiguous (NECI's CurrentDets layout), so a tile
// is one bulk copy however the rows are laid out; the kernels then read their
// row words from shared memory instead of issuing R strided 8-byte loads.
// Copies start 16-byte aligned and move a multiple of 16 bytes: a tile is
// kStageTile slots, the last partial tile is rounded up to a multiple of 4
// slots, and the arrays copied this way are allocated kStagePad slots longer.
#pragma once

#include <cstdint>

namespace neci {

constexpr int kStageTile = 256;  // slots per tile (= threads per block)
constexpr int kStagePad = 4;     // extra slots allocated behind the staged arrays

__device__ inline uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ inline void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ inline void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's earlier generic-proxy accesses of shared memory (made
// visible to it by a __syncthreads) before async-proxy writes it issues next.
__device__ inline void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ inline void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ inline void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ inline bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for a phase of the barrier (every try_wait may suspend the
// thread for a hardware-chosen time): false if it did not complete.
__device__ inline bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Slots of a tile to copy: the tile's slots below n, rounded up to a multiple
// of 4 (so that 8-byte and 4-byte arrays move multiples of 16 bytes).
__device__ inline int stage_rows(long long tile, long long n) {
    const long long first = tile * kStageTile;
    if (first >= n) return 0;
    const long long rows = n - first < kStageTile ? n - first : kStageTile;
    return (int)((rows + 3) & ~3ll);
}

}  // namespace neci
