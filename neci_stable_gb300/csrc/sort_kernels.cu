// sort_kernels.cu -- the sort form of the annihilation and the device
// selection of the semistochastic core space, both built on the radix sort
// of radix.cuh.
//
// Sort form of CompressSpawnedList + AnnihilateSpawnedParts
// (Annihilation.F90:249-515, 965-1352).  NECI sorts the spawn list by ilut_lt
// (:273) and then reduces each block of equal determinants
// (FindResidualParticle, :551-634).  Here the records are sorted by a 32-bit
// key cut from the 64-bit FindWalkerHash value (the walker-hash bucket in the
// high bits), so that runs of equal keys come out contiguous and in
// walker-hash bucket order:
//   k_sk_keys    per record: the hash, the key, the record index (and the
//                sum of |amplitude| that the compression count needs)
//   radix passes 3 stable 8-bit passes over (24-bit key, index)
//   k_sk_group   one thread per run of at most kShortRun equal keys: the run
//                is split into groups of equal determinants (two different
//                determinants can share a key), each group is summed in
//                fixed point -- the sums do not depend on the order -- and
//                looked up once in the walker hash: a found determinant gets
//                its sums, counts and initiator bits in acc/meta (the found
//                branch, merged by k_merge_stats), an absent one becomes a
//                new unique determinant for k_ann_decide
//   k_sk_long    the same for longer runs, one block per run
// The result is the hash form's, bit for bit: the same sums, the same flag
// rules (FindResidualParticle's coherent rule and initiator bits, from the
// per-run counts) and the same statistics.
#include "common.cuh"
#include "internal.h"
#include "radix.cuh"

namespace neci {

constexpr int kShortRun = 32;       // runs up to this long are grouped by one thread

// The sort key of a record, kSortKeyBits wide: the walker-hash bucket of its
// determinant (the low hb bits of abs(FindWalkerHash)) in the high bits, the
// next bits of the hash below them, cut to the top kSortKeyBits of 32.
// Different determinants that share a key are rare (at 5e5 unique
// determinants about 8e3 pairs per step) and are told apart by their words.
constexpr int kSortKeyBits = 24;  // three 8-bit radix passes
__device__ inline uint32_t sort_key(unsigned long long h, int hb) {
    const long long hs = (long long)h;
    const unsigned long long mag = hs < 0 ? (0ull - (unsigned long long)hs) : (unsigned long long)hs;
    uint32_t k32;
    if (hb >= 32) {
        k32 = (uint32_t)(mag & 0xFFFFFFFFull);
    } else {
        const unsigned long long bucket = mag & ((1ull << hb) - 1ull);
        const unsigned long long below = (mag >> hb) & ((1ull << (32 - hb)) - 1ull);
        k32 = (uint32_t)((bucket << (32 - hb)) | below);
    }
    return k32 >> (32 - kSortKeyBits);
}

__device__ inline long long spawn_count(const DevState &st) {
    return (long long)min(st.ctl->n_spawned, (unsigned long long)st.max_spawned);
}

// ---------------------------------------------------------------------------
// k_sk_keys
// ---------------------------------------------------------------------------
template <int LR>
__global__ void __launch_bounds__(256) k_sk_keys(DevSys s, DevState st) {
    if (halted(st)) return;
    extern __shared__ int32_t sh_rh2[];
    load_rh2(s, sh_rh2);
    Control *c = st.ctl;
    const long long n = spawn_count(st);
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    unsigned long long aq[2] = {0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long *rec = st.spawn + i * R;
        unsigned long long d[kMaxWords];
        NECI_FOR_WORDS(w, W) d[w] = (unsigned long long)rec[w];
        NECI_FOR_RUNS(k, L) {
            const long long q = rec[W + k];
            aq[k] += (unsigned long long)(q < 0 ? -q : q);
        }
        const unsigned long long h = neci_hash(d, W, sh_rh2);
        st.sk_h[i] = h;
        st.sk_key[0][i] = sort_key(h, st.sk_hb);
        st.sk_val[0][i] = (uint32_t)i;
    }
    unsigned long long *const dst[2] = {&c->abs_q[0], &c->abs_q[1]};
    block_add_u<2>(aq, dst);
}

// The sums of one group of equal determinants, in the layout of the hash
// form: per run the fixed-point sum and the count of records with a non-zero
// amplitude for that run | the OR of their initiator bits << 31, and the
// number of records.
struct Group {
    long long q[2];
    uint32_t cnt[2];
    uint32_t nrec;
};

__device__ inline void group_add(Group &g, const long long *rec, int W, int L) {
    ++g.nrec;
    const long long fl = rec[W + L];
    NECI_FOR_RUNS(k, L) {
        // a record's initiator bit of a run counts whatever its amplitude
        // there (FindResidualParticle)
        if (test_bit(fl, init_flag_bit(k))) g.cnt[k] |= 0x80000000u;
        const long long q = rec[W + k];
        if (q == 0) continue;
        g.q[k] = (long long)((unsigned long long)g.q[k] + (unsigned long long)q);  // two's-complement wrap, as the atomics
        g.cnt[k] += 1u;
    }
}

// A group's determinant in the walker list: its sums go to the found branch
// (acc/meta, read by k_merge_stats).  Each determinant is one group, so its
// slot is written by one thread only.
__device__ inline void group_found(const DevState &st, long long slot, const Group &g, int L) {
    NECI_FOR_RUNS(k, L) {
        st.acc[slot * L + k] = g.q[k];
        st.meta[slot * L + k] = g.cnt[k];
    }
}

// A group whose determinant is absent: unique determinant number pos for
// k_ann_decide (candidate pos = record `lead`, its sums in rep_q/rep_cnt).
__device__ inline void group_absent(const DevState &st, unsigned long long pos, long long lead, const Group &g, int L) {
    if (pos >= (unsigned long long)st.max_spawned) {
        set_err(st.ctl, NECI_GPU_ERR_SPAWN_FULL);
        return;
    }
    st.cand[pos] = (uint32_t)lead;
    st.cand_h[pos] = st.sk_h[lead];
    NECI_FOR_RUNS(k, L) {
        st.rep_q[pos * L + k] = g.q[k];
        st.rep_cnt[pos * (L + 1) + k] = g.cnt[k];
    }
    st.rep_cnt[pos * (L + 1) + L] = g.nrec;
    st.reps[pos] = (uint32_t)pos;
    st.rep_bucket[pos] = kNoBucket;
}

// ---------------------------------------------------------------------------
// k_sk_group: runs of at most kShortRun equal keys, one thread per run.
// lookup = 0 (compression without a walker list): every group is "absent".
// ---------------------------------------------------------------------------
template <int LR>
__global__ void __launch_bounds__(256) k_sk_group(DevSys s, DevState st, int lookup, int cur) {
    if (halted(st)) return;
    Control *c = st.ctl;
    const long long n = spawn_count(st);
    const uint32_t *key = st.sk_key[cur];
    const uint32_t *val = st.sk_val[cur];
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((n + stride - 1) / stride) * stride;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nround; p += stride) {
        // the run that starts at p, if one does, and its length
        int m = 0;
        bool is_long = false;
        if (p < n) {
            const uint32_t k0 = key[p];
            if (p == 0 || key[p - 1] != k0) {
                m = 1;
                while (p + m < n && key[p + m] == k0) {
                    if (m == kShortRun) {
                        is_long = true;
                        break;
                    }
                    ++m;
                }
            }
        }
        if (is_long) {  // rare: a determinant with many spawns, or a crowded key
            const unsigned long long pos = atomicAdd(&c->n_long, 1ull);
            st.sk_long[pos] = (uint32_t)p;
            m = 0;
        }
        // the elements of the run not yet in a group (bit e: element p + e)
        uint32_t todo = m == 32 ? 0xFFFFFFFFu : ((1u << m) - 1u);
        // one group per lane and pass: every lane takes part in every pass
        // (the appends are warp-wide)
        while (__any_sync(0xffffffffu, todo != 0u)) {
            const bool have = todo != 0u;
            Group g = {{0, 0}, {0u, 0u}, 0u};
            long long lead = 0, slot = -1;
            if (have) {
                const int f = __ffs((int)todo) - 1;
                lead = (long long)val[p + f];
                const long long *rl = st.spawn + lead * R;
                unsigned long long dl[kMaxWords];
                NECI_FOR_WORDS(w, W) dl[w] = (unsigned long long)rl[w];
                uint32_t rest = todo;
                while (rest) {
                    const int e = __ffs((int)rest) - 1;
                    rest &= rest - 1u;
                    const long long *re = st.spawn + (long long)val[p + e] * R;
                    if (e != f && !det_eq(dl, re, W)) continue;
                    todo &= ~(1u << e);
                    group_add(g, re, W, L);
                }
                if (lookup) slot = hash_find(st, dl, W, R, st.sk_h[lead], c);
                if (slot >= 0) group_found(st, slot, g, L);
            }
            const bool absent = have && slot < 0;
            const unsigned long long pos = warp_append1(&c->n_reps, absent);
            if (absent) group_absent(st, pos, lead, g, L);
        }
    }
}

// ---------------------------------------------------------------------------
// k_sk_long: runs longer than kShortRun, one block per run.
// The run's end is found by warp 0 with a 32-way search: probes 1, 32,
// 1024, ... positions apart until one holds another key, then 32-way
// refinement (two probes per factor of 32 in the run's length).  Groups are
// then formed round by round: the first element not yet in a group leads,
// the whole block compares every element of the run with it, marks the
// members (bit 31 of the index) and sums them; the smallest position of an
// element that is neither marked nor a member leads the next round.  A run
// of one determinant (the usual case: one determinant with many spawns, the
// reference above all) takes one round, whose pass is spread over the block.
// ---------------------------------------------------------------------------
constexpr int kLongThreads = 256;
constexpr int kLongItems = 4;  // elements per thread in flight in a pass

template <int LR>
__global__ void __launch_bounds__(kLongThreads) k_sk_long(DevSys s, DevState st, int lookup, int cur) {
    if (halted(st)) return;
    constexpr int NW = kLongThreads / 32;
    __shared__ long long s_p1, s_next[NW];
    __shared__ unsigned long long s_q[NW][2], s_c[NW][2], s_nrec[NW];
    __shared__ uint32_t s_init[NW];
    Control *c = st.ctl;
    const long long n = spawn_count(st);
    const uint32_t *key = st.sk_key[cur];
    uint32_t *val = st.sk_val[cur];
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned long long nlong = min(c->n_long, (unsigned long long)st.max_spawned);
    constexpr long long kNone = 0x7FFFFFFFFFFFFFFFll;
    for (unsigned long long r = blockIdx.x; r < nlong; r += gridDim.x) {  // block-uniform
        const long long p0 = (long long)st.sk_long[r];
        if (wid == 0) {
            const uint32_t k0 = key[p0];
            // key[lo] == k0 throughout; the first position with another key
            // (or n) lies in (lo, lo + 32 * step] once a probe has found one
            long long lo = p0 + kShortRun, step = 1;
            for (;;) {
                const long long q = lo + (long long)(lane + 1) * step;
                const unsigned int m = __ballot_sync(0xffffffffu, q >= n || key[q] != k0);
                if (m) {
                    lo += (long long)(__ffs((int)m) - 1) * step;
                    break;
                }
                lo += 32 * step;
                step *= 32;
            }
            while (step > 1) {  // the probe at lo + step is known to differ
                step /= 32;
                const long long q = lo + (long long)(lane + 1) * step;
                const unsigned int m = __ballot_sync(0xffffffffu, q >= n || key[q] != k0);
                lo += (long long)(__ffs((int)m) - 1) * step;
            }
            if (lane == 0) s_p1 = lo + 1;
        }
        __syncthreads();
        const long long p1 = s_p1;
        long long f = p0;
        for (;;) {  // block-uniform rounds: one group each
            // the lead's index: an unmarked element, so its mark bit is clear
            // (masked all the same: members of this round are marked meanwhile)
            const long long lead = (long long)(val[f] & 0x7FFFFFFFu);
            unsigned long long dl[kMaxWords];
            NECI_FOR_WORDS(w, W) dl[w] = (unsigned long long)st.spawn[lead * R + w];
            Group g = {{0, 0}, {0u, 0u}, 0u};
            long long next = kNone;
            for (long long base = f + threadIdx.x; base < p1; base += kLongThreads * kLongItems) {
                uint32_t v[kLongItems];
#pragma unroll
                for (int j = 0; j < kLongItems; ++j) {
                    const long long q = base + (long long)j * kLongThreads;
                    v[j] = q < p1 ? val[q] : 0x80000000u;  // past the end: treated as marked
                }
#pragma unroll
                for (int j = 0; j < kLongItems; ++j) {
                    if (v[j] & 0x80000000u) continue;
                    const long long q = base + (long long)j * kLongThreads;
                    const long long *re = st.spawn + (long long)v[j] * R;
                    if (!det_eq(dl, re, W)) {
                        next = min(next, q);
                        continue;
                    }
                    val[q] = v[j] | 0x80000000u;
                    group_add(g, re, W, L);
                }
            }
            // the group's sums over the block (two's-complement wrap, as the atomics)
            uint32_t init = 0u;
            NECI_FOR_RUNS(k, L) {
                const unsigned long long qs = warp_sum_u((unsigned long long)g.q[k]);
                const unsigned long long cs = warp_sum_u((unsigned long long)(g.cnt[k] & 0x7FFFFFFFu));
                if (__any_sync(0xffffffffu, (g.cnt[k] & 0x80000000u) != 0u)) init |= 1u << k;
                if (lane == 0) {
                    s_q[wid][k] = qs;
                    s_c[wid][k] = cs;
                }
            }
            const unsigned long long nr = warp_sum_u((unsigned long long)g.nrec);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) next = min(next, __shfl_xor_sync(0xffffffffu, next, o));
            if (lane == 0) {
                s_nrec[wid] = nr;
                s_init[wid] = init;
                s_next[wid] = next;
            }
            __syncthreads();
            next = kNone;
#pragma unroll
            for (int w = 0; w < NW; ++w) next = min(next, s_next[w]);
            if (threadIdx.x == 0) {
                Group t = {{0, 0}, {0u, 0u}, 0u};
                uint32_t ini = 0u;
                for (int w = 0; w < NW; ++w) {
                    NECI_FOR_RUNS(k, L) {
                        t.q[k] = (long long)((unsigned long long)t.q[k] + s_q[w][k]);
                        t.cnt[k] += (uint32_t)s_c[w][k];
                    }
                    t.nrec += (uint32_t)s_nrec[w];
                    ini |= s_init[w];
                }
                NECI_FOR_RUNS(k, L) if (ini & (1u << k)) t.cnt[k] |= 0x80000000u;
                const long long slot = lookup ? hash_find(st, dl, W, R, st.sk_h[lead], c) : -1;
                if (slot >= 0) group_found(st, slot, t, L);
                else group_absent(st, atomicAdd(&c->n_reps, 1ull), lead, t, L);
            }
            __syncthreads();  // the shared sums and s_next are read before the next round writes them
            if (next == kNone) break;
            f = next;
        }
    }
}

// ---------------------------------------------------------------------------
// Launch of the sort form (k_sk_keys, the radix passes, k_sk_group, k_sk_long)
// ---------------------------------------------------------------------------
static int sk_grid(const Engine &e, int per_sm) {
    const long long want = e.st.max_spawned / 1024 + 1, hi = (long long)e.num_sms * per_sm;
    return (int)(want < 8 ? 8 : (want > hi ? hi : want));
}

void launch_sort_keys(Engine &e, cudaStream_t s) {
    const size_t shm = (e.sys.nbasis + 1) * sizeof(int32_t);
    if (e.sys.L == 2) k_sk_keys<2><<<sk_grid(e, 8), 256, shm, s>>>(e.sys, e.st);
    else k_sk_keys<1><<<sk_grid(e, 8), 256, shm, s>>>(e.sys, e.st);
}

// The three radix passes; returns the buffer index that holds the sorted pairs.
int launch_sort_radix(Engine &e, cudaStream_t s) {
    uint32_t *const key[2] = {e.st.sk_key[0], e.st.sk_key[1]};
    uint32_t *const val[2] = {e.st.sk_val[0], e.st.sk_val[1]};
    return radix_sort_pairs<uint32_t>(s, key, val, &e.st.ctl->n_spawned, e.st.max_spawned, kSortKeyBits,
                                      e.st.sk_counts, e.st.sk_blocks);
}

void launch_sort_group(Engine &e, cudaStream_t s, int lookup, int cur) {
    if (e.sys.L == 2) {
        k_sk_group<2><<<sk_grid(e, 8), 256, 0, s>>>(e.sys, e.st, lookup, cur);
        k_sk_long<2><<<e.num_sms * 4, kLongThreads, 0, s>>>(e.sys, e.st, lookup, cur);
    } else {
        k_sk_group<1><<<sk_grid(e, 8), 256, 0, s>>>(e.sys, e.st, lookup, cur);
        k_sk_long<1><<<e.num_sms * 4, kLongThreads, 0, s>>>(e.sys, e.st, lookup, cur);
    }
}

// Blocks of a radix pass over max_spawned elements: chunks of at least 4096
// elements, at most sort_bpsm blocks per SM (2 unless tuned).
int sort_ann_blocks(const Engine &e) {
    const long long want = e.st.max_spawned / 4096 + 1, hi = (long long)e.num_sms * e.sort_bpsm;
    return (int)(want < 1 ? 1 : (want > hi ? hi : want));
}

// ---------------------------------------------------------------------------
// Device selection of the semistochastic core space: the most populated
// determinants (proc_most_populated_states, semi_stoch_procs.F90:1310-1421,
// with core_space_weight = sum over runs of |C|, :1623-1642).  Every slot gets
// the key 2^63 - 1 - bits(weight) (non-negative doubles order like their
// bits, so ascending keys are descending weights) or, for a hole, 2^64 - 1;
// a stable sort of the slots in slot order by that key puts the heaviest
// determinants first and, among equal weights, the lower slot first -- the
// one NECI's strict ">" keeps, since a later determinant of equal weight does
// not displace it.  Occupied means what neci_gpu_download_walkers keeps: a
// sign of magnitude >= 1e-12, or a core flag while a core space is set.
// ---------------------------------------------------------------------------
__global__ void k_cs_keys(DevSys s, DevState st, unsigned long long *key, uint32_t *val, unsigned long long *n_occ) {
    const long long n = slots_in_use(st);
    unsigned long long cnt = 0;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const long long *r = st.dets + j * s.R;
        bool occ = st.n_core > 0 && is_core_flags(r[s.W + s.L]);
        double wgt = 0.0;
        for (int k = 0; k < s.L; ++k) {
            const double c = word_to_double(r[s.W + k]);
            if (fabs(c) >= kEps12) occ = true;
            wgt = k == 0 ? fabs(c) : wgt + fabs(c);
        }
        key[j] = occ ? (0x7FFFFFFFFFFFFFFFull - (unsigned long long)__double_as_longlong(wgt)) : ~0ull;
        val[j] = (uint32_t)j;
        cnt += occ ? 1ull : 0ull;
    }
    if (cnt) atomicAdd(n_occ, cnt);
}

// The determinant words of the first n selected slots.
__global__ void k_cs_gather(DevSys s, DevState st, const uint32_t *slot, long long n, long long *core_dets) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long *r = st.dets + (long long)slot[i] * s.R;
        for (int w = 0; w < s.W; ++w) core_dets[i * s.W + w] = r[w];
    }
}

// Sorts the slots in use by core weight; key/val/counts are scratch of the
// caller (two buffers of max_walkers entries each, 256 * blocks counts);
// returns the buffer index of the sorted slots.
int launch_core_select_sort(Engine &e, unsigned long long *key[2], uint32_t *val[2], uint32_t *counts, int blocks,
                            unsigned long long *n_occ) {
    const int grid = e.num_sms * 4;
    k_cs_keys<<<grid, 256, 0, e.stream>>>(e.sys, e.st, key[0], val[0], n_occ);
    unsigned long long *const k2[2] = {key[0], key[1]};
    uint32_t *const v2[2] = {val[0], val[1]};
    return radix_sort_pairs<unsigned long long>(e.stream, k2, v2, &e.st.ctl->tot_walkers, e.st.max_walkers, 64,
                                                counts, blocks);
}

void launch_core_select_gather(Engine &e, const uint32_t *slot, long long n, long long *core_dets) {
    k_cs_gather<<<e.num_sms * 4, 256, 0, e.stream>>>(e.sys, e.st, slot, n, core_dets);
}

}  // namespace neci
