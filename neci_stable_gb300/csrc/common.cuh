// common.cuh -- device helpers shared by the step kernels (kernels.cu) and
// the spawn kernel (spawn.cu): block reductions into the step's counters,
// warp-aggregated appends, and the walker hash (hash_table_lookup,
// AddNewHashDet, RemoveHashDet).
#pragma once

#include "engine.cuh"

namespace neci {

// ---------------------------------------------------------------------------
// Reduction helpers.
// ---------------------------------------------------------------------------
__device__ inline double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ inline unsigned long long warp_sum_u(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NV doubles into global atomics (one atomic per value per
// block).  The values are per run, run-minor (v[2i + run]); with one run the
// odd entries are skipped.  Every thread's values are staged in shared
// memory and each warp sums whole values (8 adds per lane, then 5 shuffle
// levels), so a block issues about a quarter of the FP64 adds of a shuffle
// tree per warp.  blockDim.x <= 256.
template <int NV>
__device__ inline void block_add(const double (&v)[NV], double *const (&dst)[NV], int L) {
    __shared__ double red[NV][256];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int m = 0; m < NV; ++m)
        if ((m & 1) < L) red[m][t] = v[m];
    __syncthreads();
#pragma unroll
    for (int m = 0; m < NV; ++m) {  // value m is summed by warp m mod nw
        if (m % nw != wid || (m & 1) >= L) continue;
        double s = 0.0;
        for (int i = lane; i < (int)blockDim.x; i += 32) s += red[m][i];
        s = warp_sum(s);
        if (lane == 0 && s != 0.0) atomicAdd(dst[m], s);
    }
    __syncthreads();
}

template <int NV>
__device__ inline void block_add_u(unsigned long long (&v)[NV], unsigned long long *const (&dst)[NV]) {
    __shared__ unsigned long long red[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const unsigned long long s = warp_sum_u(v[k]);
        if (lane == 0) red[k][wid] = s;
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            unsigned long long s = lane < nw ? red[k][lane] : 0ull;
            s = warp_sum_u(s);
            if (lane == 0 && s != 0ull) atomicAdd(dst[k], s);
        }
    }
    __syncthreads();
}

// Warp-aggregated append of `want` items: returns this lane's first index.
// Every lane of the warp must call it (all loops that use it run a
// warp-uniform number of times).
__device__ inline unsigned long long warp_append(unsigned long long *counter, unsigned int want) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    unsigned int incl = want;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const unsigned int total = __shfl_sync(0xffffffffu, incl, 31);
    unsigned long long base = 0;
    if (lane == 31 && total) base = atomicAdd(counter, (unsigned long long)total);
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + incl - want;
}

// warp_append of at most one item per lane: the positions follow from a
// ballot (the same as warp_append's for want in {0, 1}).
__device__ inline unsigned long long warp_append1(unsigned long long *counter, bool want) {
    const unsigned int lane = threadIdx.x & 31;
    const unsigned int m = __ballot_sync(0xffffffffu, want);
    unsigned long long base = 0;
    if (lane == 31 && m) base = atomicAdd(counter, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 31);
    return base + __popc(m & ((1u << lane) - 1u));
}

__device__ inline void set_err(Control *c, int code) { atomicCAS(&c->err, 0, code); }

__device__ inline void load_rh2(const DevSys &s, int32_t *sh) {
    for (int i = threadIdx.x; i <= s.nbasis; i += blockDim.x) sh[i] = s.random_hash2[i];
    __syncthreads();
}

// Remove slot j from the walker hash (RemoveHashDet, load_balancer.fpp:631).
// The caller counts the tombstone and adds its count to Control::n_tomb once
// per block (one atomic per removal would serialise millions of them per
// step on one address).
__device__ inline void hash_remove(const DevState &st, long long j) {
    const uint32_t b = st.slot_bucket[j];
    st.hash[b] = kTomb;
}

// Look a determinant up: returns slot or -1.
__device__ inline long long hash_find(const DevState &st, const unsigned long long *d, int W, int R,
                                      unsigned long long h, Control *ctl) {
    const unsigned long long mask = st.hash_n - 1;
    unsigned long long b = hash_bucket(h, st.hash_n);
    for (int p = 0; p < kProbeLimit; ++p) {
        const uint32_t e = st.hash[b];
        if (e == kEmpty) return -1;
        if (e != kTomb) {
            const long long slot = (long long)e - 1;
            if (det_eq(d, st.dets + slot * R, W)) return slot;
        }
        b = (b + 1) & mask;
    }
    set_err(ctl, NECI_GPU_ERR_HASH_FULL);
    return -1;
}

// Insert a determinant known to be absent.  Returns 1 if it took a
// tombstone's bucket (the caller takes one off its tombstone count).
__device__ inline int hash_insert(const DevState &st, long long slot, unsigned long long h, Control *ctl) {
    const unsigned long long mask = st.hash_n - 1;
    unsigned long long b = hash_bucket(h, st.hash_n);
    for (int p = 0; p < kProbeLimit; ++p) {
        const uint32_t e = st.hash[b];
        if (e == kEmpty || e == kTomb) {
            if (atomicCAS(&st.hash[b], e, (uint32_t)(slot + 1)) == e) {
                st.slot_bucket[slot] = (uint32_t)b;
                return e == kTomb ? 1 : 0;
            }
            continue;  // lost the race for this bucket: look at it again
        }
        b = (b + 1) & mask;
    }
    set_err(ctl, NECI_GPU_ERR_HASH_FULL);
    return 0;
}

// TestInitiator_explicit (fcimc_helper.F90:1142-1240) without ADI, senior
// initiators or an initiator space.
__device__ inline bool test_initiator(const IterParams &p, bool was, double sgn, bool is_ref, bool core) {
    const bool popInit = abs_bits(sgn) > dbl_bits(p.initiator_walk_no);  // |sgn| > InitiatorWalkNo
    if (!was) return popInit;
    if (!is_ref && !(core && p.t_core_inits) && !popInit) return false;
    return true;
}

}  // namespace neci
