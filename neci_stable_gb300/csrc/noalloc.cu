// noalloc.cu -- CompressSpawnedList for callers that cannot allocate memory.
//
// Some hosts cannot call cudaMalloc: code running inside another program's
// allocator or memory pool, a caller that must not grow its footprint after
// start-up, or one that only owns the buffers it was handed.  For them
// neci_gpu_compress_spawns_noalloc merges a spawn list that is already in
// device memory without any allocation: the open-addressing table and the
// per-determinant accumulators live in the file-scope device arrays below,
// whose size is fixed at build time (kNoAllocMaxSpawns records) and which
// every GPU that loads the library holds until the process exits.
#include <cstdio>
#include <mutex>

#include "engine.cuh"
#include "internal.h"

namespace neci {
namespace {

constexpr long long kNoAllocMaxSpawns = 1 << 18;              // records per call
constexpr unsigned long long kNoAllocBuckets = 1ull << 19;   // power of two >= 2 * max
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocCounters {
    unsigned long long n_reps;
    unsigned long long n_out;
    unsigned long long abs_q[2];
    unsigned long long abs_s[2];
    int err;
    int pad;
};

// Scratch shared by every call on a device (calls that overlap on the GPU race).
static __device__ __align__(256) uint32_t g_na_table[kNoAllocBuckets];        // record index + 1
static __device__ __align__(256) uint32_t g_na_reps[kNoAllocMaxSpawns];       // owner records
static __device__ __align__(256) long long g_na_q[kNoAllocMaxSpawns * 2];     // fixed-point sums
static __device__ __align__(256) uint32_t g_na_cnt[kNoAllocMaxSpawns * 3];    // per run counts | init, records
static __device__ __align__(256) NoAllocCounters g_na_ctr;

struct NoAllocScratch {
    uint32_t *table, *reps, *cnt;
    long long *q;
    NoAllocCounters *ctr;
};

__device__ inline long long na_fixed(long long word, int *ovf) { return to_fixed(word_to_double(word), ovf); }

__device__ inline unsigned long long na_hash(const long long *rec, int W) {
    unsigned long long h = 0x243F6A8885A308D3ull;
    for (int w = 0; w < W; ++w) h = splitmix64(h ^ (unsigned long long)rec[w]);
    return h;
}

// Sum of |q| per run over a block's threads, added with one atomic per warp
// (an atomic per record on these two addresses would serialise the pass).
__device__ inline void na_add_abs(unsigned long long (&a)[2], unsigned long long *dst, int L) {
    for (int k = 0; k < L; ++k) {
        unsigned long long v = a[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&dst[k], v);
    }
}

// Position of this lane's item among the warp's items (want: this lane has
// one), from one atomic per warp on `counter`.  Every lane of the warp calls it.
__device__ inline unsigned long long na_append(unsigned long long *counter, bool want) {
    const unsigned int lane = threadIdx.x & 31;
    const unsigned int m = __ballot_sync(0xffffffffu, want);
    unsigned long long base = 0;
    if (lane == 0 && m) base = atomicAdd(counter, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + __popc(m & ((1u << lane) - 1u));
}

// Pass 1: every record finds (or claims) the table bucket of its
// determinant and adds its amplitude to the owner's accumulators.  The loop
// runs the same number of rounds in every lane (the appends are warp-wide).
__global__ void k_na_merge(const long long *spawned, long long n, int W, int L, NoAllocScratch sc) {
    const int R = W + L + 1;
    int ovf = 0;
    unsigned long long aq[2] = {0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((n + stride - 1) / stride) * stride;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nround; i += stride) {
        bool claimed = false;
        if (i < n) {
            const long long *rec = spawned + i * R;
            unsigned long long b = na_hash(rec, W) & (kNoAllocBuckets - 1);
            long long owner = -1;
            for (unsigned long long p = 0; p < kNoAllocBuckets; ++p) {
                const uint32_t e = atomicCAS(&sc.table[b], 0u, (uint32_t)(i + 1));
                if (e == 0u) {
                    owner = i;
                    claimed = true;
                    break;
                }
                const long long o = (long long)e - 1;
                bool same = true;
                for (int w = 0; w < W; ++w) same = same && spawned[o * R + w] == rec[w];
                if (same) { owner = o; break; }
                b = (b + 1) & (kNoAllocBuckets - 1);
            }
            if (owner < 0) {
                atomicCAS(&sc.ctr->err, 0, NECI_GPU_ERR_HASH_FULL);
            } else {
                const long long fl = rec[W + L];
                atomicAdd(&sc.cnt[owner * 3 + 2], 1u);
                for (int k = 0; k < L; ++k) {
                    // a record's initiator bit of a run counts whatever its
                    // amplitude there (FindResidualParticle)
                    if (test_bit(fl, init_flag_bit(k))) atomicOr(&sc.cnt[owner * 3 + k], 0x80000000u);
                    const long long q = na_fixed(rec[W + k], &ovf);
                    if (q == 0) continue;
                    atomicAdd((unsigned long long *)&sc.q[owner * 2 + k], (unsigned long long)q);
                    aq[k] += (unsigned long long)(q < 0 ? -q : q);
                    atomicAdd(&sc.cnt[owner * 3 + k], 1u);
                }
            }
        }
        // the records that claimed a bucket are the determinants' owners
        const unsigned long long pos = na_append(&sc.ctr->n_reps, claimed);
        if (claimed) sc.reps[pos] = (uint32_t)i;
    }
    na_add_abs(aq, sc.ctr->abs_q, L);
    if (ovf) atomicCAS(&sc.ctr->err, 0, NECI_GPU_ERR_OVERFLOW);
}

// Pass 2: one output row per determinant whose summed amplitude is not zero
// (the flag rules of FindResidualParticle, Annihilation.F90:551-634).
__global__ void k_na_out(const long long *spawned, int W, int L, int trunc_init, int coherent, long long *out,
                         NoAllocScratch sc) {
    const int R = W + L + 1;
    const long long n = (long long)sc.ctr->n_reps;
    unsigned long long as[2] = {0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((n + stride - 1) / stride) * stride;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < nround; r += stride) {
        bool emit = false;
        long long i = 0, flags = 0;
        long long q[2] = {0, 0};
        if (r < n) {
            i = sc.reps[r];
            q[0] = sc.q[i * 2];
            q[1] = sc.q[i * 2 + 1];
            for (int k = 0; k < L; ++k) {
                if (q[k] != 0) emit = true;
                as[k] += (unsigned long long)(q[k] < 0 ? -q[k] : q[k]);
            }
            if (sc.cnt[i * 3 + 2] == 1u) {
                flags = spawned[i * R + W + L];
            } else if (trunc_init) {
                for (int k = 0; k < L; ++k) {
                    const uint32_t c = sc.cnt[i * 3 + k];
                    if ((coherent && (c & 0x7FFFFFFFu) >= 2u) || (c & 0x80000000u)) flags |= 1ll << init_flag_bit(k);
                }
            }
        }
        const unsigned long long pos = na_append(&sc.ctr->n_out, emit);
        if (!emit) continue;
        const long long *rec = spawned + i * R;
        long long *o = out + pos * R;
        for (int w = 0; w < W; ++w) o[w] = rec[w];
        for (int k = 0; k < L; ++k) o[W + k] = double_to_word(from_fixed(q[k]));
        o[W + L] = flags;
    }
    na_add_abs(as, sc.ctr->abs_s, L);
}

std::mutex g_na_mutex;
NoAllocScratch g_na_scratch[kNoAllocMaxDevices];
bool g_na_ready[kNoAllocMaxDevices] = {};

}  // namespace
}  // namespace neci

using namespace neci;

// Message into the caller's buffer (snprintf into caller memory: nothing is allocated).
static int na_fail(char *errbuf, int32_t errlen, int code, const char *msg, long long a = 0, long long b = 0) {
    if (errbuf && errlen > 0) std::snprintf(errbuf, (size_t)errlen, msg, a, b);
    return code;
}

extern "C" int32_t neci_gpu_compress_spawns_noalloc(const int64_t *d_spawned, int64_t n, int32_t nifd,
                                                    int32_t lenof_sign, int32_t t_trunc_initiator,
                                                    int32_t t_init_coherent_rule, int64_t *d_out, int64_t *n_out,
                                                    double *nannihil, void *stream, char *errbuf,
                                                    int32_t errbuf_len) {
    if (errbuf && errbuf_len > 0) errbuf[0] = 0;
    if (n < 0 || n > kNoAllocMaxSpawns)
        return na_fail(errbuf, errbuf_len, NECI_GPU_ERR_INVALID,
                       "neci_gpu_compress_spawns_noalloc: %lld spawn records given, at most %lld per call",
                       (long long)n, kNoAllocMaxSpawns);
    if (nifd < 0 || nifd + 1 > kMaxWords || (lenof_sign != 1 && lenof_sign != 2) || !n_out ||
        (n > 0 && (!d_spawned || !d_out)))
        return na_fail(errbuf, errbuf_len, NECI_GPU_ERR_INVALID, "neci_gpu_compress_spawns_noalloc: bad argument");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
        return na_fail(errbuf, errbuf_len, NECI_GPU_ERR_CUDA, "neci_gpu_compress_spawns_noalloc: no usable current device");
    NoAllocScratch sc;
    {
        // once per device, with that device current: device addresses of the
        // scratch arrays (their host-side names are not device addresses)
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ready[dev]) {
            NoAllocScratch t;
            cudaError_t e1 = cudaGetSymbolAddress((void **)&t.table, g_na_table);
            cudaError_t e2 = cudaGetSymbolAddress((void **)&t.reps, g_na_reps);
            cudaError_t e3 = cudaGetSymbolAddress((void **)&t.q, g_na_q);
            cudaError_t e4 = cudaGetSymbolAddress((void **)&t.cnt, g_na_cnt);
            cudaError_t e5 = cudaGetSymbolAddress((void **)&t.ctr, g_na_ctr);
            if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess || e5 != cudaSuccess)
                return na_fail(errbuf, errbuf_len, NECI_GPU_ERR_CUDA,
                               "neci_gpu_compress_spawns_noalloc: cudaGetSymbolAddress failed");
            g_na_scratch[dev] = t;
            g_na_ready[dev] = true;
        }
        sc = g_na_scratch[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int W = nifd + 1, L = lenof_sign;
    // the scratch keeps the previous call's contents: clear what must start at zero
    cudaError_t ce = cudaMemsetAsync(sc.table, 0, kNoAllocBuckets * sizeof(uint32_t), s);
    if (ce == cudaSuccess && n > 0) ce = cudaMemsetAsync(sc.q, 0, (size_t)n * 2 * sizeof(long long), s);
    if (ce == cudaSuccess && n > 0) ce = cudaMemsetAsync(sc.cnt, 0, (size_t)n * 3 * sizeof(uint32_t), s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(sc.ctr, 0, sizeof(NoAllocCounters), s);
    if (ce != cudaSuccess)
        return na_fail(errbuf, errbuf_len, NECI_GPU_ERR_CUDA, "neci_gpu_compress_spawns_noalloc: cudaMemsetAsync failed");
    if (n > 0) {
        k_na_merge<<<512, 256, 0, s>>>((const long long *)d_spawned, n, W, L, sc);
        k_na_out<<<512, 256, 0, s>>>((const long long *)d_spawned, W, L, t_trunc_initiator, t_init_coherent_rule,
                                     (long long *)d_out, sc);
    }
    NoAllocCounters h;
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&h, sc.ctr, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess)
        return na_fail(errbuf, errbuf_len, NECI_GPU_ERR_CUDA, "neci_gpu_compress_spawns_noalloc: CUDA error %lld",
                       (long long)ce);
    if (h.err) return na_fail(errbuf, errbuf_len, h.err, "neci_gpu_compress_spawns_noalloc: device error %lld", h.err);
    *n_out = (int64_t)h.n_out;
    if (nannihil)
        for (int k = 0; k < L; ++k) nannihil[k] = (double)(long long)(h.abs_q[k] - h.abs_s[k]) * 0x1.0p-32;
    return NECI_GPU_OK;
}
