// radix.cuh -- stable LSD radix sort of (key, value) pairs on the device.
//
// 8-bit digits, one reduce-then-scan round per digit:
//   k_radix_count    each block counts the digits of its contiguous chunk of
//                    elements (shared-memory histogram) and stores the 256
//                    counts digit-major, counts[digit * blocks + block];
//   k_radix_scan     one block per digit turns the digit's block counts into
//                    exclusive offsets and its total;
//   k_radix_scatter  each block adds the prefix of the digit totals, then
//                    walks its chunk in order, 1024 elements (4 per thread)
//                    per round, and ranks them stably: lanes with the same
//                    digit find each other with a warp match mask, items and
//                    warps are ordered through per-warp digit counts in shared
//                    memory, and the block's running offset of each digit
//                    advances by the round's total.
// The element count is read from device memory and the grids are fixed, so a
// sort is capturable in a CUDA graph whose element count changes per replay.
// Keys are unsigned (uint32_t or unsigned long long), values uint32_t, and
// counts are 32-bit: n < 2^31.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace neci {

constexpr int kRadixBits = 8;
constexpr int kRadixBins = 1 << kRadixBits;
constexpr int kRadixThreads = 256;

__device__ inline long long radix_n(const unsigned long long *n_ptr, long long cap) {
    const unsigned long long n = *n_ptr;
    return (long long)(n < (unsigned long long)cap ? n : (unsigned long long)cap);
}

// Elements [lo, hi) of block b of G: contiguous chunks whose length is a
// multiple of the block size (count and scatter use the same chunks).
__device__ inline void radix_chunk(long long n, int G, int b, long long &lo, long long &hi) {
    long long chunk = (n + G - 1) / G;
    chunk = (chunk + 4 * kRadixThreads - 1) / (4 * kRadixThreads) * (4 * kRadixThreads);
    lo = (long long)b * chunk;
    hi = lo + chunk;
    if (lo > n) lo = n;
    if (hi > n) hi = n;
}

template <typename K>
__device__ inline uint32_t radix_digit(K key, int shift) {
    return (uint32_t)(key >> shift) & (uint32_t)(kRadixBins - 1);
}

template <typename K>
__global__ void __launch_bounds__(kRadixThreads) k_radix_count(const K *keys, const unsigned long long *n_ptr,
                                                              long long cap, int shift, uint32_t *counts) {
    __shared__ uint32_t hist[kRadixBins];
    const int G = gridDim.x;
    for (int d = threadIdx.x; d < kRadixBins; d += blockDim.x) hist[d] = 0u;
    __syncthreads();
    const long long n = radix_n(n_ptr, cap);
    long long lo, hi;
    radix_chunk(n, G, blockIdx.x, lo, hi);
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) atomicAdd(&hist[radix_digit(keys[i], shift)], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixBins; d += blockDim.x) counts[(size_t)d * G + blockIdx.x] = hist[d];
}

// Exclusive scan of the block counts of each digit in place, one block per
// digit (blockIdx.x = digit): counts[d * G + b] becomes the number of digit-d
// elements in blocks before b, and totals[d] the number of digit-d elements.
// The scatter adds the prefix of the totals over the digits.
__global__ void __launch_bounds__(kRadixThreads) k_radix_scan(uint32_t *counts, uint32_t *totals, int G) {
    __shared__ uint32_t wsum[kRadixThreads / 32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t *c = counts + (size_t)blockIdx.x * G;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (int base = 0; base < G; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < G ? c[i] : 0u;
        uint32_t x = v;  // inclusive scan in the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[wid] = x;
        __syncthreads();
        uint32_t before = carry;
        for (int w = 0; w < wid; ++w) before += wsum[w];
        before += x - v;
        if (i < G) c[i] = before;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

constexpr int kRadixItems = 4;  // elements per thread in a round of the scatter

template <typename K>
__global__ void __launch_bounds__(kRadixThreads) k_radix_scatter(const K *kin, const uint32_t *vin, K *kout,
                                                                uint32_t *vout, const unsigned long long *n_ptr,
                                                                long long cap, int shift, const uint32_t *offsets,
                                                                const uint32_t *totals) {
    constexpr int NW = kRadixThreads / 32;
    __shared__ uint32_t run[kRadixBins];
    // per item slot of the round, warp and digit: the warp's count
    __shared__ uint32_t wcnt[kRadixItems][NW][kRadixBins];
    const int G = gridDim.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    {
        // the digit's first position: the digits below it (a block scan of
        // the totals, one digit per thread), then the blocks before this one
        static_assert(kRadixThreads == kRadixBins, "one thread per digit");
        const int d = threadIdx.x;
        const uint32_t t = totals[d];
        uint32_t x = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wcnt[0][0][wid] = x;
        __syncthreads();
        uint32_t below = x - t;
        for (int w = 0; w < wid; ++w) below += wcnt[0][0][w];
        __syncthreads();
        run[d] = below + offsets[(size_t)d * G + blockIdx.x];
#pragma unroll
        for (int k = 0; k < kRadixItems; ++k)
#pragma unroll
            for (int w = 0; w < NW; ++w) wcnt[k][w][d] = 0u;
    }
    __syncthreads();
    const long long n = radix_n(n_ptr, cap);
    long long lo, hi;
    radix_chunk(n, G, blockIdx.x, lo, hi);
    const unsigned int lt = (1u << lane) - 1u;
    constexpr int kRound = kRadixThreads * kRadixItems;
    for (long long base = lo; base < hi; base += kRound) {  // the same rounds in the whole block
        // item k of thread t is element base + k * 256 + t: element order is
        // item-major, then warp, then lane
        K key[kRadixItems];
        uint32_t val[kRadixItems], dig[kRadixItems], rank[kRadixItems];
#pragma unroll
        for (int k = 0; k < kRadixItems; ++k) {
            const long long i = base + (long long)k * kRadixThreads + threadIdx.x;
            const bool valid = i < hi;
            key[k] = valid ? kin[i] : (K)0;
            val[k] = valid ? vin[i] : 0u;
            dig[k] = valid ? radix_digit(key[k], shift) : (uint32_t)kRadixBins;  // matches no valid digit
        }
#pragma unroll
        for (int k = 0; k < kRadixItems; ++k) {
            const unsigned int peers = __match_any_sync(0xffffffffu, dig[k]);
            rank[k] = __popc(peers & lt);
            if (dig[k] < (uint32_t)kRadixBins && rank[k] == 0) wcnt[k][wid][dig[k]] = __popc(peers);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kRadixItems; ++k) {
            if (dig[k] >= (uint32_t)kRadixBins) continue;
            const uint32_t d = dig[k];
            uint32_t off = run[d] + rank[k];
            for (int k2 = 0; k2 < k; ++k2)
#pragma unroll
                for (int w = 0; w < NW; ++w) off += wcnt[k2][w][d];
            for (int w = 0; w < wid; ++w) off += wcnt[k][w][d];
            kout[off] = key[k];
            vout[off] = val[k];
        }
        __syncthreads();
        {
            const int d = threadIdx.x;  // one digit per thread
            uint32_t t = 0;
#pragma unroll
            for (int k = 0; k < kRadixItems; ++k)
#pragma unroll
                for (int w = 0; w < NW; ++w) {
                    t += wcnt[k][w][d];
                    wcnt[k][w][d] = 0u;
                }
            run[d] += t;
        }
        __syncthreads();
    }
}

// Sorts the first *n_ptr (at most cap) pairs of key[0]/val[0] by the low
// `bits` bits of the key (bits a multiple of 8), ping-ponging through
// key[1]/val[1]; returns the index of the buffers that hold the result.
// counts holds 256 * (blocks + 1) words (the block counts, then the totals).
template <typename K>
inline int radix_sort_pairs(cudaStream_t s, K *const key[2], uint32_t *const val[2], const unsigned long long *n_ptr,
                            long long cap, int bits, uint32_t *counts, int blocks) {
    uint32_t *const totals = counts + (size_t)kRadixBins * blocks;
    int cur = 0;
    for (int shift = 0; shift < bits; shift += kRadixBits) {
        k_radix_count<K><<<blocks, kRadixThreads, 0, s>>>(key[cur], n_ptr, cap, shift, counts);
        k_radix_scan<<<kRadixBins, kRadixThreads, 0, s>>>(counts, totals, blocks);
        k_radix_scatter<K><<<blocks, kRadixThreads, 0, s>>>(key[cur], val[cur], key[cur ^ 1], val[cur ^ 1], n_ptr,
                                                            cap, shift, counts, totals);
        cur ^= 1;
    }
    return cur;
}

}  // namespace neci
