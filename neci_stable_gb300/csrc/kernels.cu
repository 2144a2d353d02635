// kernels.cu -- the kernels of one FCIQMC iteration (PerformFCIMCycPar,
// FciMCPar.F90:1177-1920) and the batch utility kernels of the C ABI.
//
// Iteration pipeline (all grid-stride, fixed grids, so one iteration is a
// capturable CUDA graph; counts live in device memory):
//   k_begin        reset per-step counters; rebuild the walker hash if its
//                  tombstone load is high
//   k_sweep        loop_over_determinants (:1294-1758) minus the spawn
//                  attempts: free slots, initiator flags (CalcParentFlag),
//                  E_proj sums (SumEContrib), number of spawns
//                  (decide_num_to_spawn) emitted as one entry per attempt,
//                  core vector gather, and the death step
//                  (perform_death_all_walkers / walker_death)
//   k_expand       attempt entries of heavily populated parents, a block each
//   k_spawn        the spawn attempts (generate_excitation, attempt_create,
//                  create_particle): in spawn.cu
//   k_core         determ_projection_no_death (semi_stoch_procs.F90:290)
//   k_ann_probe    annihilation pass 1: look every spawn up in the walker
//                  hash (hash_table_lookup, hash.F90:294); spawns onto
//                  present determinants are summed into per-slot fixed-
//                  point accumulators, the rest become candidates
//   k_ann_compress pass 2 (CompressSpawnedList, Annihilation.F90:249):
//                  candidates are merged per determinant in a second
//                  open-addressing table keyed on the spawn records
//   k_ann_decide   pass 3 (AnnihilateSpawnedParts not-found branch,
//                  :1191-1290): initiator abort, stochRoundSpawn; the
//                  survivors are listed for
//   k_ann_place    AddNewHashDet: slots, rows, hash buckets, diagonal
//                  elements, one new determinant per thread
//   k_merge_stats  deterministic_annihilation + AnnihilateSpawnedParts
//                  found branch + CalcHashTableStats (load_balancer.fpp:646)
//                  in one sweep over the slots
//   k_final        collect estimators into the step's stats record
#include <cstdio>
#include <type_traits>

#include "engine.cuh"
#include "excitgen.cuh"
#include "internal.h"
#include "stage.cuh"
#include "common.cuh"

namespace neci {

// ===========================================================================
// k_begin: per-step reset (single thread) and optional rehash.
// ===========================================================================
__global__ void k_begin(DevState st) {
    Control *c = st.ctl;
    if (blockIdx.x == 0 && threadIdx.x == 0 && !c->halted) {
        c->n_free = 0; c->free_taken = 0; c->n_att = 0; c->n_spawned = 0; c->n_cand = 0;
        c->n_reps = 0; c->n_new = 0; c->n_attempts = 0; c->n_occupied = 0; c->n_holes = 0; c->n_found = 0;
        c->n_reps_nz = 0;
        c->n_big = 0;
        c->n_huge = 0;
        c->n_long = 0;
        c->n_place = 0;
        c->n_pre = c->tot_walkers;
        for (int k = 0; k < 2; ++k) {
            c->abs_q[k] = 0; c->abs_s[k] = 0;
            c->nborn[k] = c->ndied[k] = c->nannihil[k] = c->naborted[k] = c->nremoved[k] = 0.0;
            c->tot_parts[k] = c->tot_parts_old[k] = c->noat_hf[k] = c->hf_cyc[k] = c->enum_cyc[k] = c->norm[k] = 0.0;
        }
        c->err = 0;
        c->rehash = 0;
    }
}

// Rehash: clear every bucket, then reinsert live slots (run only when the
// tombstone share is high; the flag is decided on the host from n_tomb).
__global__ void k_hash_clear(DevState st) {
    if (halted(st)) return;
    if (!st.ctl->rehash) return;
    for (unsigned long long b = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; b < st.hash_n;
         b += (unsigned long long)gridDim.x * blockDim.x)
        st.hash[b] = kEmpty;
    if (blockIdx.x == 0 && threadIdx.x == 0) st.ctl->n_tomb = 0;
}
__global__ void k_hash_fill(DevSys s, DevState st) {
    if (halted(st)) return;
    if (!st.ctl->rehash) return;
    extern __shared__ int32_t sh_rh2[];
    load_rh2(s, sh_rh2);
    const long long n = slots_in_use(st);
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const long long *r = st.dets + j * s.R;
        bool occ = is_core_flags(r[s.W + s.L]);
        NECI_FOR_RUNS(k, s.L) occ = occ || fabs(word_to_double(r[s.W + k])) >= kEps12;
        if (!occ) continue;
        unsigned long long d[kMaxWords];
        NECI_FOR_WORDS(w, s.W) d[w] = (unsigned long long)r[w];
        hash_insert(st, j, neci_hash(d, s.W, sh_rh2), st.ctl);
    }
}

// ===========================================================================
// Compaction of the walker list (run at the start of a step when the
// previous one left more holes than occupied slots).  The K occupied slots
// (or core slots) keep their order; those at or above K move into the holes
// below K, the r-th of them into the r-th hole, so that slots 0..K-1 hold the
// whole list.  TotWalkers becomes K and the walker hash is rebuilt.  Results
// do not depend on slots: every random stream is keyed by the determinant.
// ===========================================================================
__device__ inline bool slot_kept(const DevSys &s, const DevState &st, long long j) {
    const long long *r = st.dets + j * s.R;
    if (st.n_core > 0 && is_core_flags(r[s.W + s.L])) return true;
    NECI_FOR_RUNS(k, s.L)
        if (abs_bits(word_to_double(r[s.W + k])) >= dbl_bits(kEps12)) return true;
    return false;
}

// Exclusive position of slot j among the kept slots of its tile, and the
// tile's count (blockDim.x == kCompactTile).
__device__ inline unsigned int tile_rank(bool keep, unsigned int &count) {
    __shared__ unsigned int warp_n[kCompactTile / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned int bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_n[wid] = __popc(bal);
    __syncthreads();
    unsigned int before = 0, total = 0;
    for (int w = 0; w < kCompactTile / 32; ++w) {
        const unsigned int c = warp_n[w];
        if (w < wid) before += c;
        total += c;
    }
    __syncthreads();
    count = total;
    return before + __popc(bal & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(kCompactTile) k_compact_count(DevSys s, DevState st) {
    if (halted(st)) return;
    if (!st.ctl->compact) return;
    const long long n = slots_in_use(st);
    const long long ntiles = (n + kCompactTile - 1) / kCompactTile;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long j = t * kCompactTile + threadIdx.x;
        unsigned int count;
        (void)tile_rank(j < n && slot_kept(s, st, j), count);
        if (threadIdx.x == 0) st.tile_count[t] = count;
    }
}

// One block: exclusive scan of the tile counts; K = the kept total.
__global__ void __launch_bounds__(kCompactTile) k_compact_scan(DevState st) {
    if (halted(st)) return;
    if (!st.ctl->compact) return;
    const long long n = slots_in_use(st);
    const long long ntiles = (n + kCompactTile - 1) / kCompactTile;
    __shared__ unsigned int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long base = 0; base < ntiles; base += kCompactTile) {
        const long long t = base + threadIdx.x;
        const unsigned int c = t < ntiles ? st.tile_count[t] : 0u;
        // block-wide exclusive scan of c
        __shared__ unsigned int buf[kCompactTile];
        buf[threadIdx.x] = c;
        __syncthreads();
        for (int o = 1; o < kCompactTile; o <<= 1) {
            const unsigned int v = threadIdx.x >= (unsigned)o ? buf[threadIdx.x - o] : 0u;
            __syncthreads();
            buf[threadIdx.x] += v;
            __syncthreads();
        }
        const unsigned int incl = buf[threadIdx.x];
        if (t < ntiles) st.tile_off[t] = carry + incl - c;
        __syncthreads();
        if (threadIdx.x == kCompactTile - 1) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) st.ctl->compact_k = carry;
}

// Holes below K by rank; the number of kept slots below K.
__global__ void __launch_bounds__(kCompactTile) k_compact_holes(DevSys s, DevState st) {
    if (halted(st)) return;
    if (!st.ctl->compact) return;
    const long long n = slots_in_use(st);
    const long long K = (long long)st.ctl->compact_k;
    const long long ntiles = (n + kCompactTile - 1) / kCompactTile;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long j = t * kCompactTile + threadIdx.x;
        const bool keep = j < n && slot_kept(s, st, j);
        unsigned int count;
        const long long pos = (long long)st.tile_off[t] + tile_rank(keep, count);
        if (j < K && !keep) st.hole_at_rank[j - pos] = (int32_t)j;
        // the kept position of every slot that will move (the free list is
        // scratch until the sweep refills it)
        if (j >= K && keep) st.free_list[j] = (int32_t)pos;
        if (j == K) st.ctl->compact_pos_k = (unsigned long long)pos;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && K >= n) st.ctl->compact_pos_k = (unsigned long long)K;
}

// Every kept slot at or above K moves into the hole of its rank.  Only rows
// at or above K are read, and only holes below K are written.
__global__ void k_compact_move(DevSys s, DevState st) {
    if (halted(st)) return;
    if (!st.ctl->compact) return;
    const long long n = slots_in_use(st);
    const long long K = (long long)st.ctl->compact_k;
    const long long pos_k = (long long)st.ctl->compact_pos_k;
    for (long long j = K + blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
         j += (long long)gridDim.x * blockDim.x) {
        if (!slot_kept(s, st, j)) continue;
        const long long to = st.hole_at_rank[st.free_list[j] - pos_k];
        const long long *src = st.dets + j * s.R;
        long long *dst = st.dets + to * s.R;
        for (int w = 0; w < s.R; ++w) dst[w] = src[w];
        st.diagH[to] = st.diagH[j];
        st.offdiagH[to] = st.offdiagH[j];
        if (st.n_core > 0) {
            const int ci = st.core_of_slot[j];
            st.core_of_slot[to] = ci;
            st.core_of_slot[j] = -1;
            if (ci >= 0) st.core_slot[ci] = to;
        }
    }
}

// Closes the compaction: TotWalkers = K, the hash is rebuilt next.
__global__ void k_compact_done(DevState st) {
    if (halted(st)) return;
    Control *c = st.ctl;
    if (!c->compact) return;
    c->tot_walkers = c->compact_k;
    c->rehash = 1;
    c->compact = 0;
}

// ===========================================================================
// k_sweep
// ===========================================================================
// a / b (IEEE round-to-nearest) as one inline PTX instruction, which the
// compiler does not hoist out of its branch: a division written beside a
// cheap alternative would otherwise be computed for every slot (it expands
// to a long FP64 sequence).
__device__ inline double div_dbl(double a, double b) {
    double r;
    asm("div.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}

// The rare end of walker_death for one run, idie > |C| (more died than
// there were): fmax(idie - |C|, 0) to the born count and, for an initiator
// run whose determinant survives, the abort of the sign change
// (fcimc_helper.F90:2352-2363).  Out of line (and so never executed
// speculatively) with the accumulators passed through.
struct DeathOver {
    double born, ab, cp;
};
__device__ __noinline__ DeathOver death_over(double c, double idie, double cp, double born, double ab, bool abort_ok) {
    const double aC = fabs(c);
    if (!le_nonneg(idie, aC)) born += idie - aC;
    if (abort_ok && is_positive(cp) != is_positive(c)) {
        ab += fabs(cp);
        cp = 0.0;
    }
    return {born, ab, cp};
}

// decide_num_to_spawn (fcimc_helper.F90:2160-2174) in FP64, for AvMCExcits
// != 1 or |C| >= 2^31: the run's spawn-stream draw decides the extra attempt.
// Out of line, so that the fast sweep does not carry its FP64 instructions.
__device__ __noinline__ unsigned int spawn_count_fp64(double c, double av, unsigned long long dkey, long long iter,
                                                      int run) {
    Stream rs(dkey, iter, P_NSPAWN, run, 0);
    const double pa = c * av;
    unsigned int ns = abs((int)pa);
    if (fabs(fabs(pa) - (double)ns) > kEps12) {
        const double pe = fabs(pa) - (double)ns;
        if (bern(rs, pe)) ++ns;
    }
    return ns;
}

// attempt_die_normal with integer walkers (fcimc_pointed_fns.F90:573-705):
// fac |C| rounded stochastically with the determinant's death stream, whose
// draws are taken one per run in run order.  Out of line as above.
__device__ __noinline__ double death_integer(double fac, double c, unsigned long long dkey, long long iter, int run) {
    Stream rd(dkey, iter, P_DEATH, 0, 0);
    for (int k = 0; k < run; ++k) (void)rd.next64();
    double rat = fac * fabs(c);
    double idie = trunc(rat);
    rat -= idie;
    if (bern(rd, fabs(rat))) idie += nearbyint(fsign(1.0, rat));
    return idie;
}

// LR: lenof_sign of the instance (1, or 2 for a replica pair).  FAST: the
// instance for real coefficients with AvMCExcits = 1 (sweep_fast).  GB300
// runs FP64 instructions at about one lane per clock per SM (1/128 of the
// FP32 rate) and a predicated one
// holds the pipe like an executed one, so the FP64 instructions of paths a
// warp rarely takes sit behind branches (warp votes) or out of line.
template <int LR, bool FAST>
__global__ void __launch_bounds__(256, 4) k_sweep(DevSys s, DevState st, const IterParams *pp) {
    if (halted(st)) return;
    const IterParams p = *pp;
    Control *c = st.ctl;
    const long long n = slots_in_use(st);
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    double acc_old[2] = {0.0, 0.0}, acc_hf[2] = {0.0, 0.0}, acc_en[2] = {0.0, 0.0};
    double acc_died[2] = {0.0, 0.0}, acc_born[2] = {0.0, 0.0}, acc_ab[2] = {0.0, 0.0};
    double death_max = 0.0;  // max_death_cpt of this thread's determinants (tau search)
    unsigned long long acc_att = 0, acc_tomb = 0;
    // Tiles of kStageTile slots (one per block and round) are staged into
    // shared memory by TMA bulk copies, the next tile's while this one is
    // processed: rows, diagH and offdiagH of the tile.  Writes go to global.
    extern __shared__ __align__(16) unsigned char sweep_smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int stage_ok[2];  // by round parity
    // the round's appends: per-warp counts of free slots and attempts, and
    // the block's first positions
    __shared__ unsigned int s_wfree[kStageTile / 32], s_watt[kStageTile / 32], s_wbig[kStageTile / 32];
    __shared__ unsigned long long s_base_free, s_base_att, s_base_big;
    const size_t stage_bytes = (size_t)kStageTile * (R + 2) * 8;
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nrounds = (n + (long long)gridDim.x * kStageTile - 1) / ((long long)gridDim.x * kStageTile);
    auto issue = [&](long long k) {  // thread 0: the copies of round k's tile
        const long long tile = blockIdx.x + k * gridDim.x;
        const int rows = stage_rows(tile, n);
        if (rows == 0) return;
        unsigned char *base = sweep_smem + (k & 1) * stage_bytes;
        const uint32_t br = (uint32_t)rows * R * 8, bd = (uint32_t)rows * 8;
        fence_proxy_async_smem();
        mbar_expect_tx(&bars[k & 1], br + 2 * bd);
        bulk_g2s(base, st.dets + tile * kStageTile * R, br, &bars[k & 1]);
        bulk_g2s(base + (size_t)kStageTile * R * 8, st.diagH + tile * kStageTile, bd, &bars[k & 1]);
        bulk_g2s(base + (size_t)kStageTile * (R + 1) * 8, st.offdiagH + tile * kStageTile, bd, &bars[k & 1]);
    };
    // Round kr: wait for tile kr, one barrier, then the copy of tile kr + 1
    // into the other buffer: every thread has passed the barrier, so none is
    // still in round kr - 1, the buffer's last reader.  The barrier also
    // keeps the appends' per-warp counts of round kr - 1 until all have read
    // them, so a round needs no barrier at its end.
    if (threadIdx.x == 0 && nrounds > 0) issue(0);
    for (long long kr = 0; kr < nrounds; ++kr) {
        const long long tile = blockIdx.x + kr * gridDim.x;
        const unsigned char *sbase = sweep_smem + (kr & 1) * stage_bytes;
        if (threadIdx.x == 0)
            stage_ok[kr & 1] =
                stage_rows(tile, n) > 0 ? (mbar_wait_bounded(&bars[kr & 1], (uint32_t)((kr >> 1) & 1)) ? 1 : 0) : 1;
        __syncthreads();
        if (!stage_ok[kr & 1]) {
            // a copy that never completed: report it, give it a last
            // bounded wait (it is the only one in flight), and leave
            if (threadIdx.x == 0) {
                set_err(c, NECI_GPU_ERR_TIMEOUT);
                (void)mbar_wait_bounded(&bars[kr & 1], (uint32_t)((kr >> 1) & 1));
            }
            __syncthreads();
            return;
        }
        if (threadIdx.x == 0 && kr + 1 < nrounds) issue(kr + 1);
        const long long j = tile * kStageTile + threadIdx.x;
        bool live = j < n;
        long long *r = st.dets + (live ? j : 0) * R;  // the global row (writes)
        const long long *sr = (const long long *)sbase + (size_t)threadIdx.x * R;  // its staged copy (reads)
        const double *sdiag = (const double *)(sbase + (size_t)kStageTile * R * 8);
        const double *soffd = (const double *)(sbase + (size_t)kStageTile * (R + 1) * 8);
        unsigned long long d[kMaxWords];
        double C[2] = {0.0, 0.0};
        long long flags = 0;
        bool core = false, occ = false;
        if (live) {
            NECI_FOR_WORDS(w, W) d[w] = (unsigned long long)sr[w];
            NECI_FOR_RUNS(k, L) C[k] = word_to_double(sr[W + k]);
            flags = sr[W + L];
            core = st.n_core > 0 && is_core_flags(flags);
            NECI_FOR_RUNS(k, L) {
                acc_old[k] += abs_dbl(C[k]);
                if (abs_bits(C[k]) >= dbl_bits(kEps12)) occ = true;
            }
            if (core) {
                const int ci = st.core_of_slot[j];
                NECI_FOR_RUNS(k, L) st.core_x[(long long)ci * L + k] = C[k];
                if (p.precision == NECI_PREC_MIXED)
                    NECI_FOR_RUNS(k, L) st.core_x32[(long long)ci * L + k] = (float)C[k];
            }
        }
        // holes go to the free list (FciMCPar.F90:1415-1427)
        const bool hole = live && !occ && !core;
        unsigned int nsp[2] = {0, 0};
        bool neg[2] = {false, false};
        bool out_zero = true;
        if (live && occ) {
            const int exl = excit_level(s.ilut_ref, d, W);
            const bool is_ref = exl == 0;
            if (p.t_trunc_initiator) {
                long long nf = flags;
                NECI_FOR_RUNS(k, L) {
                    const int b = init_flag_bit(k);
                    const bool now = test_initiator(p, test_bit(flags, b), C[k], is_ref, core);
                    if (now) nf |= (1ll << b); else nf &= ~(1ll << b);
                }
                if (nf != flags) { r[W + L] = nf; flags = nf; }
            }
            // offdiagH is zero beyond the double excitations of the
            // reference; adding that +-0 product changes no sum, so it is
            // skipped
            const double odh = soffd[threadIdx.x];
            const bool has_odh = abs_bits(odh) != 0;
            // behind a vote: most warps hold no connection of the reference
            if (__any_sync(__activemask(), has_odh))
                NECI_FOR_RUNS(k, L) if (has_odh) acc_en[k] += odh * C[k];
            if (__any_sync(__activemask(), is_ref))
                if (is_ref) NECI_FOR_RUNS(k, L) acc_hf[k] += C[k];
            const unsigned long long dkey = det_key(d, W, p.seed);
            // the key of the spawn attempts' streams, read by k_spawn for
            // every attempt of this slot instead of hashing the row again
            st.dkey[j] = dkey;
            NECI_FOR_RUNS(k, L) {
                // decide_num_to_spawn (fcimc_helper.F90:2160-2174)
                uint32_t whole;
                bool extra;
                uint64_t thr;
                unsigned int ns;
                if ((FAST || p.av_unit) && split_count(C[k], whole, extra, thr)) {
                    Stream rs(dkey, p.iter, P_NSPAWN, k, 0);
                    ns = whole + (extra && rs.next64() < thr);
                } else {
                    ns = spawn_count_fp64(C[k], p.av_mc_excits, dkey, p.iter, k);
                }
                nsp[k] = ns;
                neg[k] = is_negative(C[k]);
                acc_att += ns;
            }
            // walker_death + attempt_die_normal (fcimc_helper.F90:2279-2407,
            // fcimc_pointed_fns.F90:573-705)
            const double Kii = sdiag[threadIdx.x];
            double cp[2] = {0.0, 0.0}, id[2] = {0.0, 0.0};
            bool any = false, over = false;
            NECI_FOR_RUNS(k, L) {
                const double kd = Kii - p.diag_sft[k];
                const double fac = p.tau * kd;
                // log_death_magnitude: the largest K_ii - S >= 0 (non-negative
                // doubles order like their bit patterns)
                if (s.tau_search && !(dbl_bits(kd) >> 63) && dbl_bits(kd) > dbl_bits(death_max)) death_max = kd;
                if (gt_pos(fac, 2.0)) set_err(c, NECI_GPU_ERR_UNSTABLE);
                double idie;
                if (FAST || p.t_all_real_coeff) idie = fac * abs_dbl(C[k]);
                else idie = death_integer(fac, C[k], dkey, p.iter, k);
                id[k] = idie;
                // fmin(idie, |C|) to the died; idie > |C| (more died than
                // there were) is handled below
                const double aC = abs_dbl(C[k]);
                const bool le = le_nonneg(idie, aC);
                acc_died[k] += le ? idie : aC;
                if (!le) over = true;
                // C - idie * sign(1, C) with Fortran's sign (+1 for C = -0.0); both products are exact
                const bool nonneg = !(dbl_bits(C[k]) >> 63) || abs_bits(C[k]) == 0;
                cp[k] = C[k] + (nonneg ? neg_dbl(idie) : idie);  // a - b is a + (-b), exactly
                if (abs_bits(cp[k]) > dbl_bits(kEps12)) any = true;
            }
            // idie > |C| in a run: fmax(idie - |C|, 0) to the born, and the
            // sign change it makes is aborted for initiator runs; the sign
            // changes only then (at idie = |C| the new sign is +0 and the
            // abort changes nothing)
            if (over) {
                const bool abort_ok = p.t_trunc_initiator && any;
                NECI_FOR_RUNS(k, L) {
                    const DeathOver o = death_over(C[k], id[k], cp[k], acc_born[k], acc_ab[k], abort_ok);
                    acc_born[k] = o.born;
                    acc_ab[k] = o.ab;
                    cp[k] = o.cp;
                }
                if (abort_ok) {
                    any = false;
                    NECI_FOR_RUNS(k, L) if (abs_bits(cp[k]) > dbl_bits(kEps12)) any = true;
                }
            }
            if (any || core) {
                NECI_FOR_RUNS(k, L) {
                    r[W + k] = double_to_word(cp[k]);
                    out_zero = out_zero && abs_bits(cp[k]) == 0;
                }
            } else {
                hash_remove(st, j);
                ++acc_tomb;
                r[W + L] = flags | 1ll;  // flag_removed
                NECI_FOR_RUNS(k, L) r[W + k] = double_to_word(0.0);
            }
        }
        // the signs just written are all zero
        const bool freed = live && occ && !core && out_zero;
        // The round's three appends, free slots, spawn-attempt entries and
        // k_expand's chunks, with one atomic per counter for the whole block
        // (all issued before any result is read): per-warp atomics on these
        // addresses serialise in one L2 slice, tens of thousands to millions
        // per step.  One entry per attempt; a parent with more than
        // kBigAttempts attempts is handed to k_expand in chunks of at most
        // kExpandChunk attempts, each written by a warp there.
        {
            const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
            const bool want = hole || freed;
            if (live) st.hole_mark[j] = want ? 1 : 0;
            const unsigned int mf = __ballot_sync(0xffffffffu, want);
            unsigned int nat = 0, nbig = 0;
            NECI_FOR_RUNS(k, L) {
                nat += nsp[k];
                if (nsp[k] > (unsigned int)kBigAttempts && nsp[k] <= (unsigned int)kHugeAttempts)
                    nbig += (nsp[k] + kExpandChunk - 1) / kExpandChunk;
            }
            unsigned int incl = nat, bincl = nbig;  // inclusive scans of the warp's attempts and chunks
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned int y = __shfl_up_sync(0xffffffffu, incl, o);
                const unsigned int z = __shfl_up_sync(0xffffffffu, bincl, o);
                if (lane >= o) {
                    incl += y;
                    bincl += z;
                }
            }
            if (lane == 31) {
                s_wfree[wid] = __popc(mf);
                s_watt[wid] = incl;
                s_wbig[wid] = bincl;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                unsigned int tf = 0, ta = 0, tb = 0;
                for (int w = 0; w < kStageTile / 32; ++w) {
                    tf += s_wfree[w];
                    ta += s_watt[w];
                    tb += s_wbig[w];
                }
                s_base_free = tf ? atomicAdd(&c->n_free, (unsigned long long)tf) : 0ull;
                s_base_att = ta ? atomicAdd(&c->n_att, (unsigned long long)ta) : 0ull;
                s_base_big = tb ? atomicAdd(&c->n_big, (unsigned long long)tb) : 0ull;
            }
            __syncthreads();
            unsigned long long bf = s_base_free, ba = s_base_att, bb = s_base_big;
            for (int w = 0; w < wid; ++w) {
                bf += s_wfree[w];
                ba += s_watt[w];
                bb += s_wbig[w];
            }
            if (want) st.free_list[bf + __popc(mf & ((1u << lane) - 1u))] = (int32_t)j;
            const unsigned long long base = ba + incl - nat;
            // this lane's chunks for k_expand: every entry below max_big is
            // written (with no attempts where the lane's entries do not fit),
            // so that k_expand reads none from an earlier step
            if (nbig) {
                unsigned long long cb = bb + bincl - nbig;
                const bool fits = base + nat <= (unsigned long long)st.max_att;
                if (cb + nbig > (unsigned long long)st.max_big) set_err(c, NECI_GPU_ERR_SPAWN_FULL);
                unsigned long long q = base;
                NECI_FOR_RUNS(k, L) {
                    if (nsp[k] > (unsigned int)kBigAttempts && nsp[k] <= (unsigned int)kHugeAttempts) {
                        const unsigned long long head = (unsigned long long)j | ((unsigned long long)k << 32) |
                                                        ((unsigned long long)neg[k] << 33);
                        for (unsigned int a0 = 0; a0 < nsp[k] && cb < (unsigned long long)st.max_big;
                             a0 += kExpandChunk, ++cb) {
                            st.big[3 * cb] = head | ((unsigned long long)a0 << 34);
                            st.big[3 * cb + 1] = fits ? min((unsigned int)kExpandChunk, nsp[k] - a0) : 0u;
                            st.big[3 * cb + 2] = q + a0;
                        }
                    }
                    q += nsp[k];
                }
            }
            if (nat) {
                if (base + nat > (unsigned long long)st.max_att) {
                    set_err(c, NECI_GPU_ERR_SPAWN_FULL);
                } else {
                    unsigned long long q = base;
                    NECI_FOR_RUNS(k, L) {
                        const unsigned long long head = (unsigned long long)j | ((unsigned long long)k << 32) |
                                                        ((unsigned long long)neg[k] << 33);
                        if (nsp[k] > (unsigned int)kHugeAttempts) {
                            const unsigned long long b = atomicAdd(&c->n_huge, 1ull);
                            if (b < (unsigned long long)kMaxHuge) {
                                st.huge[3 * b] = head;
                                st.huge[3 * b + 1] = nsp[k];
                                st.huge[3 * b + 2] = q;
                            } else {
                                set_err(c, NECI_GPU_ERR_SPAWN_FULL);
                            }
                        } else if (nsp[k] > (unsigned int)kBigAttempts) {
                            // its chunks for k_expand are written above
                        } else {
                            for (unsigned int a = 0; a < nsp[k]; ++a) st.att[q + a] = head | ((unsigned long long)a << 34);
                        }
                        q += nsp[k];
                    }
                }
            }
        }
    }
    const double v[12] = {acc_old[0], acc_old[1], acc_hf[0], acc_hf[1], acc_en[0], acc_en[1], acc_died[0],
                          acc_died[1], acc_born[0], acc_born[1], acc_ab[0], acc_ab[1]};
    double *const dst[12] = {&c->tot_parts_old[0], &c->tot_parts_old[1], &c->hf_cyc[0], &c->hf_cyc[1],
                             &c->enum_cyc[0], &c->enum_cyc[1], &c->ndied[0], &c->ndied[1],
                             &c->nborn[0], &c->nborn[1], &c->naborted[0], &c->naborted[1]};
    block_add<12>(v, dst, L);
    unsigned long long u[2] = {acc_att, acc_tomb};
    unsigned long long *const du[2] = {&c->n_attempts, &c->n_tomb};
    block_add_u<2>(u, du);
    if (s.tau_search) {
        // non-negative doubles order like their bit patterns
        unsigned long long b = (unsigned long long)__double_as_longlong(death_max);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, b, o);
            b = y > b ? y : b;
        }
        if ((threadIdx.x & 31) == 0 && b) atomicMax(&c->tau_death, b);
    }
}

// ===========================================================================
// k_expand: attempt entries of heavily populated parents, one warp per chunk
// of at most kExpandChunk attempts of a parent (the whole grid per parent for
// the few with more than kHugeAttempts).
// ===========================================================================
__global__ void k_expand(DevState st) {
    if (halted(st)) return;
    // parents with more than kHugeAttempts attempts: the whole grid per parent
    const unsigned long long nh = min(st.ctl->n_huge, (unsigned long long)kMaxHuge);
    for (unsigned long long b = 0; b < nh; ++b) {
        const unsigned long long head = st.huge[3 * b], n = st.huge[3 * b + 1], base = st.huge[3 * b + 2];
        for (unsigned long long a = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; a < n;
             a += (unsigned long long)gridDim.x * blockDim.x)
            st.att[base + a] = head | (a << 34);
    }
    // the others (33 to 65536 attempts): a warp per chunk; the chunk's head
    // carries its first attempt index, so its entry a is head + (a << 34)
    const unsigned long long nb = min(st.ctl->n_big, (unsigned long long)st.max_big);
    const unsigned long long warp = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    const unsigned long long lane = threadIdx.x & 31;
    for (unsigned long long b = warp; b < nb; b += nwarps) {
        const unsigned long long head = st.big[3 * b];
        const unsigned long long n = st.big[3 * b + 1];
        const unsigned long long base = st.big[3 * b + 2];
        for (unsigned long long a = lane; a < n; a += 32) st.att[base + a] = head + (a << 34);
    }
}

// ===========================================================================
// k_core: y = -tau H_offdiag x over the core rows (determ_projection_no_death,
// semi_stoch_procs.F90:290-365).  The rows are cut into segments of at most
// core_segment_len(G, per_lane) elements, and each segment is summed by a group of G
// lanes (a power of two chosen at set-up from the mean row length,
// core_group_size): lane l of the group accumulates the segment's elements
// l, l+G, l+2G, ... in order, and the group's G partial sums are added in a
// fixed tree (offsets G/2, G/4, ..., 1).  A row of one segment gets
// y = tau * (the tree's sum) at once; the segments of a longer row leave
// their sums in core_seg_y, and k_core_sum adds them in segment order, so
// that a row with tens of thousands of elements (the reference's, in a
// molecular core) is spread over many groups instead of holding one.
// FP64: fused multiply-adds acc = fma(-H_ij, x_j, acc), which the oracle
// restates in the same order, so the projection is bit-exact.  Mixed
// precision: FP32 values and products with compensated (TwoSum) FP32
// accumulation per lane, each lane's hi + lo then summed in FP64 by the same
// tree.  kCoreDepth elements of a lane are loaded before their products are
// accumulated (in element order), so that a lane keeps that many independent
// loads and gathers in flight.
// ===========================================================================
// Elements a lane loads before it accumulates them (in element order): its
// column indices and values first, then the gathers of x; and the resident
// blocks of 256 threads per SM the kernel is compiled for.
#ifndef NECI_CORE_DEPTH
#define NECI_CORE_DEPTH 8
#endif
#ifndef NECI_CORE_BLOCKS_PER_SM
#define NECI_CORE_BLOCKS_PER_SM 4
#endif
constexpr int kCoreDepth = NECI_CORE_DEPTH;

template <int G, bool MIXED>
__global__ void __launch_bounds__(256, NECI_CORE_BLOCKS_PER_SM) k_core(DevSys s, DevState st, const IterParams *pp) {
    if (halted(st)) return;
    using VT = typename std::conditional<MIXED, float, double>::type;
    const int L = s.L;
    const double tau = pp->tau;
    const int gl = threadIdx.x & (G - 1);
    const long long grp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) / G;
    const long long ngrp = ((long long)gridDim.x * blockDim.x) / G;
    const long long nseg = st.n_core_seg;
    // every lane runs the same number of rounds (the tree's shuffles are warp-wide)
    const long long nround = ((nseg + ngrp - 1) / ngrp) * ngrp;
    const int32_t *col = st.core_col;
    const VT *val = MIXED ? (const VT *)st.core_val32 : (const VT *)st.core_val;
    // x in the precision of the products: the FP32 copy the sweep wrote in a
    // mixed-precision step (the same rounding as converting here)
    const VT *xv = MIXED ? (const VT *)st.core_x32 : (const VT *)st.core_x;
    for (long long sg = grp; sg < nround; sg += ngrp) {
        const bool valid = sg < nseg;
        CoreSeg seg = {0, 0, 0};
        if (valid) seg = st.core_seg[sg];
        const long long e1 = seg.e0 + seg.len;
        double acc[2] = {0.0, 0.0};
        float hi[2] = {0.0f, 0.0f}, lo[2] = {0.0f, 0.0f};
        auto add = [&](int k, VT v, VT x) {
            if (!MIXED) {
                acc[k] = fma(-(double)v, (double)x, acc[k]);
            } else {
                const float term = -__fmul_rn((float)v, (float)x);
                const float t = __fadd_rn(hi[k], term);
                lo[k] = fabsf(hi[k]) >= fabsf(term) ? __fadd_rn(lo[k], __fadd_rn(__fsub_rn(hi[k], t), term))
                                                    : __fadd_rn(lo[k], __fadd_rn(__fsub_rn(term, t), hi[k]));
                hi[k] = t;
            }
        };
        // kCoreDepth elements of the lane per pass, the last pass predicated
        // (its elements past the segment's end are neither loaded nor added)
        for (long long e = seg.e0 + gl; e < e1; e += kCoreDepth * G) {
            const long long left = (e1 - e + G - 1) / G;  // the lane's elements from e on
            const int nv = left < kCoreDepth ? (int)left : kCoreDepth;
            const int32_t *cp = col + e;
            const VT *vp = val + e;
            int cc[kCoreDepth];
            VT vv[kCoreDepth];
#pragma unroll
            for (int j = 0; j < kCoreDepth; ++j) {
                cc[j] = j < nv ? cp[j * G] : 0;
                vv[j] = j < nv ? vp[j * G] : (VT)0;
            }
            NECI_FOR_RUNS(k, L) {
                VT xx[kCoreDepth];
#pragma unroll
                for (int j = 0; j < kCoreDepth; ++j) xx[j] = j < nv ? xv[cc[j] * L + k] : (VT)0;
#pragma unroll
                for (int j = 0; j < kCoreDepth; ++j)
                    if (j < nv) add(k, vv[j], xx[j]);
            }
        }
        const long long row = seg.row & 0x7FFFFFFF;
        const bool single = seg.row >= 0;
        NECI_FOR_RUNS(k, L) {
            double t = MIXED ? (double)hi[k] + (double)lo[k] : acc[k];
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o, G);
            if (gl == 0 && valid) {
                if (single) st.core_y[row * L + k] = t * tau;
                else st.core_seg_y[sg * L + k] = t;
            }
        }
    }
}

// The rows of more than one segment: their segments' sums added in segment
// order, then multiplied by tau (one thread per row).
__global__ void __launch_bounds__(256) k_core_sum(DevSys s, DevState st, const IterParams *pp) {
    if (halted(st)) return;
    const int L = s.L;
    const double tau = pp->tau;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < st.n_core_multi;
         m += (long long)gridDim.x * blockDim.x) {
        const long long row = st.core_multi[m];
        const long long f = st.core_seg_first[row], fn = st.core_seg_first[row + 1];
        NECI_FOR_RUNS(k, L) {
            double t = st.core_seg_y[f * L + k];
            for (long long sg = f + 1; sg < fn; ++sg) t += st.core_seg_y[sg * L + k];
            st.core_y[row * L + k] = t * tau;
        }
    }
}

// ===========================================================================
// Annihilation pass 1: probe the walker hash with every spawn record.
// ===========================================================================
// LR: lenof_sign of the instance (1, or 2 for a replica pair).
template <int LR>
__global__ void __launch_bounds__(256) k_ann_probe(DevSys s, DevState st) {
    if (halted(st)) return;
    extern __shared__ int32_t sh_rh2[];
    // each warp gathers its candidates in shared memory and appends them to
    // the global list when more than kWarpFlush are held (and at the end): an
    // append per iteration would make every iteration wait for an atomic's
    // round trip
    constexpr int kWarpBuf = 256, kWarpFlush = kWarpBuf - 32;
    __shared__ uint32_t sc_i[8][kWarpBuf];
    __shared__ unsigned long long sc_h[8][kWarpBuf];
    load_rh2(s, sh_rh2);
    Control *c = st.ctl;
    const long long n = (long long)min(c->n_spawned, (unsigned long long)st.max_spawned);
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;  // blockDim.x = 256
    unsigned long long aq[2] = {0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((n + stride - 1) / stride) * stride;
    int wn = 0;  // the warp's buffered candidates, the same in every lane
    auto flush = [&]() {
        __syncwarp();
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&c->n_cand, (unsigned long long)wn);
        base = __shfl_sync(0xffffffffu, base, 0);
        for (int k = lane; k < wn; k += 32) {
            st.cand[base + k] = sc_i[wid][k];
            st.cand_h[base + k] = sc_h[wid][k];
        }
        __syncwarp();
        wn = 0;
    };
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nround; i += stride) {
        bool cand = false;
        unsigned long long h = 0;
        if (i < n) {
            const long long *rec = st.spawn + i * R;
            unsigned long long d[kMaxWords];
            NECI_FOR_WORDS(w, W) d[w] = (unsigned long long)rec[w];
            long long q[2] = {0, 0};
            NECI_FOR_RUNS(k, L) q[k] = rec[W + k];
            const long long fl = rec[W + L];
            NECI_FOR_RUNS(k, L) aq[k] += (unsigned long long)(q[k] < 0 ? -q[k] : q[k]);
            h = neci_hash(d, W, sh_rh2);
            const long long slot = hash_find(st, d, W, R, h, c);
            if (slot >= 0) {
                NECI_FOR_RUNS(k, L) {
                    if (q[k] == 0) continue;
                    atomicAdd((unsigned long long *)&st.acc[slot * L + k], (unsigned long long)q[k]);
                    const uint32_t add = 1u;
                    atomicAdd(&st.meta[slot * L + k], add);
                    if (test_bit(fl, init_flag_bit(k))) atomicOr(&st.meta[slot * L + k], 0x80000000u);
                }
            } else {
                cand = true;
            }
        }
        const unsigned int m = __ballot_sync(0xffffffffu, cand);
        if (cand) {
            const int k = wn + __popc(m & ((1u << lane) - 1u));
            sc_i[wid][k] = (uint32_t)i;
            sc_h[wid][k] = h;
        }
        wn += __popc(m);
        if (wn > kWarpFlush) flush();
    }
    if (wn > 0) flush();
    unsigned long long *const dst[2] = {&c->abs_q[0], &c->abs_q[1]};
    block_add_u<2>(aq, dst);
}

// ===========================================================================
// Annihilation pass 2: merge candidates per determinant.
// ===========================================================================
// LR: lenof_sign of the instance (1, or 2 for a replica pair).
template <int LR>
__global__ void __launch_bounds__(256) k_ann_compress(DevSys s, DevState st) {
    if (halted(st)) return;
    Control *c = st.ctl;
    // the appends count past the allocation when it overflows (SPAWN_FULL is
    // reported at the end of the step): only the entries written are read
    const long long n = (long long)min(c->n_cand, (unsigned long long)st.max_spawned);
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    // The table in use is sized to this step's candidates (a power of two at
    // least 2^comp_shift times their number, twice by default), not to the
    // allocation: at tens of millions
    // of spawns it stays in L2 instead of scattering the probes over
    // gigabytes of DRAM.  Its buckets are cleared through rep_bucket.
    unsigned long long hn = 1024;
    while (hn < ((unsigned long long)n << st.comp_shift) && hn < st.spawn_hash_n) hn <<= 1;
    const unsigned long long mask = (hn < st.spawn_hash_n ? hn : st.spawn_hash_n) - 1;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((n + stride - 1) / stride) * stride;
    // each warp gathers the representatives it elects in shared memory and
    // appends them when more than kWarpFlush are held (and at the end), so
    // that an iteration does not wait for an atomic's round trip
    constexpr int kWarpBuf = 256, kWarpFlush = kWarpBuf - 32;
    __shared__ uint32_t sr_i[8][kWarpBuf], sr_b[8][kWarpBuf];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;  // blockDim.x = 256
    int wn = 0;  // the warp's buffered representatives, the same in every lane
    auto flush = [&]() {
        __syncwarp();
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&c->n_reps, (unsigned long long)wn);
        base = __shfl_sync(0xffffffffu, base, 0);
        for (int k = lane; k < wn; k += 32) {
            st.reps[base + k] = sr_i[wid][k];
            st.rep_bucket[base + k] = sr_b[wid][k];
        }
        __syncwarp();
        wn = 0;
    };
    for (long long ci = blockIdx.x * (long long)blockDim.x + threadIdx.x; ci < nround; ci += stride) {
        bool won = false;
        uint32_t won_bucket = 0;
        if (ci < n) {
            const long long i = st.cand[ci];
            const long long *rec = st.spawn + i * R;
            unsigned long long d[kMaxWords];
            NECI_FOR_WORDS(w, W) d[w] = (unsigned long long)rec[w];
            unsigned long long b = splitmix64(st.cand_h[ci]) & mask;
            long long owner = -1;
            for (int p = 0; p < kProbeLimit; ++p) {
                const uint32_t e = atomicCAS(&st.spawn_hash[b], kEmpty, (uint32_t)(ci + 1));
                if (e == kEmpty) { owner = ci; won = true; won_bucket = (uint32_t)b; break; }
                const long long other = (long long)e - 1;
                if (det_eq(d, st.spawn + (long long)st.cand[other] * R, W)) { owner = other; break; }
                b = (b + 1) & mask;
            }
            if (owner < 0) {
                set_err(c, NECI_GPU_ERR_HASH_FULL);
            } else {
                const long long fl = rec[W + L];
                atomicAdd(&st.rep_cnt[owner * (L + 1) + L], 1u);  // records in the block
                NECI_FOR_RUNS(k, L) {
                    // FindResidualParticle ORs a record's initiator bit of a
                    // run into the block whatever its amplitude in that run
                    if (test_bit(fl, init_flag_bit(k))) atomicOr(&st.rep_cnt[owner * (L + 1) + k], 0x80000000u);
                    const long long q = rec[W + k];
                    if (q == 0) continue;
                    atomicAdd((unsigned long long *)&st.rep_q[owner * L + k], (unsigned long long)q);
                    atomicAdd(&st.rep_cnt[owner * (L + 1) + k], 1u);
                }
            }
        }
        const unsigned int m = __ballot_sync(0xffffffffu, won);
        if (won) {
            const int k = wn + __popc(m & ((1u << lane) - 1u));
            sr_i[wid][k] = (uint32_t)ci;
            sr_b[wid][k] = won_bucket;
        }
        wn += __popc(m);
        if (wn > kWarpFlush) flush();
    }
    if (wn > 0) flush();
}

// ===========================================================================
// Annihilation pass 3: unique new determinants -> CurrentDets, in two
// kernels.  k_ann_decide takes every unique determinant not in the list
// (AnnihilateSpawnedParts' not-found branch with the compressed flags of
// CompressSpawnedList/FindResidualParticle): its summed amplitude, the
// initiator abort, stochRoundSpawn, and appends the survivors to a list.
// k_ann_place gives each survivor a slot (AddNewHashDet), writes its row and
// hash bucket and computes H_jj - Hii and <D0|H|D_j>, one determinant per
// thread: the O(nel^2) diagonal sum runs on GB300's FP64 pipe (about one lane per
// clock per SM), and
// spread over the lanes of the decisions it would hold every lane of a warp
// that had one survivor.
// ===========================================================================
// The high half of a survivor's flag word that stands for "the flag word of
// its one record"; a flag word computed from the counts holds initiator bits
// only, so its high half is never this.
constexpr uint32_t kOwnFlags = 0xFFFFFFFFu;

// LR: lenof_sign of the instance (1, or 2 for a replica pair).
template <int LR>
__global__ void __launch_bounds__(256) k_ann_decide(DevSys s, DevState st, const IterParams *pp) {
    if (halted(st)) return;
    const IterParams p = *pp;
    Control *c = st.ctl;
    // the appends count past the allocation when it overflows (SPAWN_FULL is
    // reported at the end of the step): only the entries written are read
    const long long n = (long long)min(c->n_reps, (unsigned long long)st.max_spawned);
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    double a_ab[2] = {0, 0}, a_rm[2] = {0, 0}, a_born[2] = {0, 0};
    unsigned long long a_s[2] = {0, 0}, a_nz = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((n + stride - 1) / stride) * stride;
    for (long long ri = blockIdx.x * (long long)blockDim.x + threadIdx.x; ri < nround; ri += stride) {
        bool want = false;
        long long ci = 0;
        double ss[2] = {0.0, 0.0};
        long long flags = 0;
        uint32_t nrec = 0;
        if (ri < n) {
            ci = st.reps[ri];
            const uint32_t rb = st.rep_bucket[ri];
            if (rb != kNoBucket) st.spawn_hash[rb] = kEmpty;  // leave the table clean
            long long q[2] = {0, 0};
            uint32_t cnt[2] = {0, 0};
            NECI_FOR_RUNS(k, L) {
                q[k] = st.rep_q[ci * L + k];
                cnt[k] = st.rep_cnt[ci * (L + 1) + k];
            }
            nrec = st.rep_cnt[ci * (L + 1) + L];
            // compressed flags (CompressSpawnedList / FindResidualParticle):
            // a block of one record keeps that record's flag word, read by
            // k_ann_place for the survivors only; its initiator bit in a run
            // with a non-zero amplitude is the one in the run's count, so the
            // counts decide the abort for every block without the record
            if (p.t_trunc_initiator)
                NECI_FOR_RUNS(k, L) {
                    const bool coh = p.t_init_coherent_rule && (cnt[k] & 0x7FFFFFFFu) >= 2u;
                    if (coh || (cnt[k] & 0x80000000u)) flags |= 1ll << init_flag_bit(k);
                }
            bool zero = true;
            NECI_FOR_RUNS(k, L) {
                if (q[k] != 0) zero = false;
                a_s[k] += (unsigned long long)(q[k] < 0 ? -q[k] : q[k]);
            }
            a_nz += zero ? 0ull : 1ull;
            if (!zero) {
                ss[0] = from_fixed(q[0]);
                ss[1] = from_fixed(q[1]);
                if (p.t_trunc_initiator)
                    NECI_FOR_RUNS(k, L)
                        if (!test_bit(flags, init_flag_bit(k))) { a_ab[k] += fabs(ss[k]); ss[k] = 0.0; }
                bool unocc = true;
                NECI_FOR_RUNS(k, L) if (abs_bits(ss[k]) >= dbl_bits(kEps12)) unocc = false;
                if (!unocc) {
                    const long long *rec = st.spawn + (long long)st.cand[ci] * R;
                    unsigned long long d[kMaxWords];
                    NECI_FOR_WORDS(w, W) d[w] = (unsigned long long)rec[w];
                    const unsigned long long dkey = det_key(d, W, p.seed);
                    NECI_FOR_RUNS(k, L) {
                        // stochRoundSpawn (Annihilation.F90:1354-1418)
                        const double a = abs_dbl(ss[k]);
                        if (abs_bits(a) > dbl_bits(kEps12) && abs_bits(a) < dbl_bits(p.occupied_thresh)) {
                            Stream rng(dkey, p.iter, P_ANN_ROUND, k, 0);
                            const double pRemove =
                                1.0 - (dbl_bits(p.occupied_thresh) == dbl_bits(1.0) ? a : div_dbl(a, p.occupied_thresh));
                            if (bern(rng, pRemove)) { a_rm[k] += a; ss[k] = 0.0; }
                            else { a_born[k] += p.occupied_thresh - a; ss[k] = fsign(p.occupied_thresh, ss[k]); }
                        }
                    }
                    NECI_FOR_RUNS(k, L) if (abs_bits(ss[k]) >= dbl_bits(kEps12)) want = true;
                }
            }
            // the sums are consumed: cleared for the next step, or, for a
            // survivor, replaced by its signs (as double bits) and its flag
            // word (low half in the record count's place, high half in the
            // first run's count; kOwnFlags there for a block of one record,
            // whose own flag word k_ann_place reads) for k_ann_place, which
            // clears them
            NECI_FOR_RUNS(k, L) {
                st.rep_q[ci * L + k] = want ? double_to_word(ss[k]) : 0ll;
                st.rep_cnt[ci * (L + 1) + k] = 0u;
            }
            if (want) st.rep_cnt[ci * (L + 1)] = nrec == 1 ? kOwnFlags : (uint32_t)((unsigned long long)flags >> 32);
            st.rep_cnt[ci * (L + 1) + L] = want ? (uint32_t)flags : 0u;
        }
        const unsigned long long pos = warp_append1(&c->n_place, want);
        if (want) {
            if (pos < (unsigned long long)st.max_spawned) st.place[pos] = (uint32_t)ci;
            else set_err(c, NECI_GPU_ERR_SPAWN_FULL);
        }
    }
    double v[6] = {a_ab[0], a_ab[1], a_rm[0], a_rm[1], a_born[0], a_born[1]};
    double *const dst[6] = {&c->naborted[0], &c->naborted[1], &c->nremoved[0], &c->nremoved[1],
                            &c->nborn[0], &c->nborn[1]};
    block_add<6>(v, dst, L);
    unsigned long long u[3] = {a_s[0], a_s[1], a_nz};
    unsigned long long *const du[3] = {&c->abs_s[0], &c->abs_s[1], &c->n_reps_nz};
    block_add_u<3>(u, du);
}

// split: the merge sweep skips the new determinants (it runs beside this
// kernel), so their |C| and C^2 (TotParts, norm) and the reference's sign
// are taken here.
template <int LR>
__global__ void __launch_bounds__(128) k_ann_place(DevSys s, DevState st, int split) {
    if (halted(st)) return;
    Control *c = st.ctl;
    double a_tp[2] = {0.0, 0.0}, a_norm[2] = {0.0, 0.0};
    const long long n = (long long)min(c->n_place, (unsigned long long)st.max_spawned);
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((n + stride - 1) / stride) * stride;
    long long a_tomb = 0;  // tombstones taken over by the insertions (a negative count)
    unsigned long long a_new = 0;
    for (long long pi = blockIdx.x * (long long)blockDim.x + threadIdx.x; pi < nround; pi += stride) {
        const bool want = pi < n;
        // the determinant, its signs and flag word (cleared from the sums'
        // slots) and its hash
        unsigned long long d[kMaxWords], h = 0;
        long long ws[2] = {0, 0}, flags = 0;
        NECI_FOR_WORDS(w, W) d[w] = 0ull;
        if (want) {
            const long long ci = st.place[pi];
            const long long *rec = st.spawn + (long long)st.cand[ci] * R;
            NECI_FOR_WORDS(w, W) d[w] = (unsigned long long)rec[w];
            h = st.cand_h[ci];
            NECI_FOR_RUNS(k, L) {
                ws[k] = st.rep_q[ci * L + k];
                st.rep_q[ci * L + k] = 0;
            }
            const uint32_t hi = st.rep_cnt[ci * (L + 1)];
            flags = hi == kOwnFlags ? rec[W + L]
                                    : (long long)(((unsigned long long)hi << 32) | st.rep_cnt[ci * (L + 1) + L]);
            st.rep_cnt[ci * (L + 1)] = 0u;
            st.rep_cnt[ci * (L + 1) + L] = 0u;
        }
        // Slots for the warp's determinants: the next holes of the free list
        // (one atomic on its cursor), then fresh slots at the end of the list
        // (one atomic on TotWalkers) when the holes run out.  The matrix
        // elements are computed while the atomics are in flight.
        const unsigned int ballot = __ballot_sync(0xffffffffu, want);
        const unsigned int nwant = __popc(ballot);
        const unsigned int rank = __popc(ballot & ((1u << lane) - 1u));
        const int leader = nwant ? __ffs(ballot) - 1 : 0;
        unsigned long long t0 = 0, f0 = 0;
        const unsigned long long nfree = c->n_free;
        if (nwant && lane == leader) {
            t0 = atomicAdd(&c->free_taken, (unsigned long long)nwant);
            const unsigned long long from_free = t0 >= nfree ? 0ull : min(nfree - t0, (unsigned long long)nwant);
            if (nwant > from_free) f0 = atomicAdd(&c->tot_walkers, (unsigned long long)(nwant - from_free));
        }
        double dh = 0.0, odh = 0.0;
        if (want) {
            dh = diag_helement(s, d) - s.hii;
            const int ic = excit_level(s.ilut_ref, d, W);
            odh = (ic >= 1 && ic <= 2) ? offdiag_helement(s, s.ilut_ref, d, ic) : 0.0;
        }
        if (nwant) {
            t0 = __shfl_sync(0xffffffffu, t0, leader);
            f0 = __shfl_sync(0xffffffffu, f0, leader);
        }
        if (!want) continue;
        const unsigned long long t = t0 + rank;
        const unsigned long long first_fresh = t0 >= nfree ? t0 : nfree;  // the first t that gets a fresh slot
        const long long slot = t < nfree ? (long long)st.free_list[t] : (long long)(f0 + (t - first_fresh));
        if (slot + 1 >= st.max_walkers) {
            set_err(c, NECI_GPU_ERR_LIST_FULL);
            continue;
        }
        long long *o = st.dets + slot * R;
        NECI_FOR_WORDS(w, W) o[w] = (long long)d[w];
        NECI_FOR_RUNS(k, L) o[W + k] = ws[k];
        o[W + L] = flags & ~1ll;
        st.diagH[slot] = dh;
        st.offdiagH[slot] = odh;
        if (st.n_core > 0) st.core_of_slot[slot] = -1;
        a_tomb -= hash_insert(st, slot, h, c);
        ++a_new;
        if (split) {
            bool is_ref = true;
            NECI_FOR_WORDS(w, W) if (d[w] != s.ilut_ref[w]) is_ref = false;
            NECI_FOR_RUNS(k, L) {
                const double v = word_to_double(ws[k]);
                a_tp[k] += fabs(v);
                a_norm[k] = fma(v, v, a_norm[k]);  // a statistic: one rounding, one FP64 instruction
                if (is_ref) c->noat_hf[k] = v;
            }
        }
    }
    unsigned long long u[2] = {(unsigned long long)a_tomb, a_new};  // two's complement for -count
    unsigned long long *const du[2] = {&c->n_tomb, &c->n_new};
    block_add_u<2>(u, du);
    if (split) {
        double v[4] = {a_tp[0], a_tp[1], a_norm[0], a_norm[1]};
        double *const dst[4] = {&c->tot_parts[0], &c->tot_parts[1], &c->norm[0], &c->norm[1]};
        block_add<4>(v, dst, L);
    }
}

// ===========================================================================
// k_merge_stats: deterministic annihilation, found-branch merge and
// CalcHashTableStats in one sweep.
// ===========================================================================
// LR: lenof_sign of the instance (1, or 2 for a replica pair).
template <int LR>
__global__ void __launch_bounds__(256, 4) k_merge_stats(DevSys s, DevState st, const IterParams *pp, int with_core,
                                                        int split) {
    if (halted(st)) return;
    const IterParams p = *pp;
    Control *c = st.ctl;
    // split: the slots the step began with, less those its sweep freed
    // (k_ann_place fills some of them and counts its own determinants), so
    // that the placement may run at the same time
    const long long n = (long long)min(split ? c->n_pre : c->tot_walkers, (unsigned long long)st.max_walkers);
    const int W = s.W, R = s.R;
    constexpr int L = LR;
    double a_born[2] = {0, 0}, a_ann[2] = {0, 0}, a_ab[2] = {0, 0}, a_rm[2] = {0, 0};
    double a_tp[2] = {0, 0}, a_norm[2] = {0, 0};
    unsigned long long a_s[2] = {0, 0}, a_occ = 0, a_holes = 0, a_found = 0, a_tomb = 0;
    // Tiles staged into shared memory by TMA bulk copies as in k_sweep: the
    // rows, the per-slot spawn counts (meta) and the per-slot spawn sums
    // (acc) of the tile, and in a step (split) the sweep's free-list marks,
    // so that no global load waits in a slot's path.
    extern __shared__ __align__(16) unsigned char merge_smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int stage_ok[2];  // by round parity
    // rows, meta, acc and (split) the free-list marks of a tile
    const size_t stage_bytes = (size_t)kStageTile * (R * 8 + L * 4 + L * 8 + 1);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const long long nrounds = (n + (long long)gridDim.x * kStageTile - 1) / ((long long)gridDim.x * kStageTile);
    auto issue = [&](long long k) {  // thread 0: the copies of round k's tile
        const long long tile = blockIdx.x + k * gridDim.x;
        const int rows = stage_rows(tile, n);
        if (rows == 0) return;
        unsigned char *base = merge_smem + (k & 1) * stage_bytes;
        const uint32_t br = (uint32_t)rows * R * 8, bm = (uint32_t)rows * L * 4, ba = (uint32_t)rows * L * 8;
        // the one-byte marks move in multiples of 16 slots (the array is
        // allocated 16 slots longer)
        const uint32_t bh = split ? (uint32_t)((rows + 15) & ~15) : 0u;
        fence_proxy_async_smem();
        mbar_expect_tx(&bars[k & 1], br + bm + ba + bh);
        bulk_g2s(base, st.dets + tile * kStageTile * R, br, &bars[k & 1]);
        bulk_g2s(base + (size_t)kStageTile * R * 8, st.meta + tile * kStageTile * L, bm, &bars[k & 1]);
        bulk_g2s(base + (size_t)kStageTile * (R * 8 + L * 4), st.acc + tile * kStageTile * L, ba, &bars[k & 1]);
        if (bh) bulk_g2s(base + (size_t)kStageTile * (R * 8 + L * 12), st.hole_mark + tile * kStageTile, bh, &bars[k & 1]);
    };
    // one slot: its row (global, for writes), staged row, meta and acc
    auto body = [&](long long j, const long long *sr, const uint32_t *sm, const long long *sa) {
        long long *r = st.dets + j * R;
        const long long flags = sr[W + L];
        const bool core = st.n_core > 0 && is_core_flags(flags);
        double C[2] = {0.0, 0.0};
        NECI_FOR_RUNS(k, L) C[k] = word_to_double(sr[W + k]);
        bool changed = false;
        // deterministic_annihilation (Annihilation.F90:930-963)
        if (core && with_core) {
            const int ci = st.core_of_slot[j];
            NECI_FOR_RUNS(k, L) {
                const double y = st.core_y[(long long)ci * L + k];
                a_born[k] += fabs(y);
                if (prod_negative(C[k], y)) a_ann[k] += 2.0 * min_abs(C[k], y);
                C[k] = y + C[k];
            }
            changed = true;
        }
        // AnnihilateSpawnedParts, found branch (Annihilation.F90:1000-1140)
        uint32_t m[2] = {0, 0};
        bool has = false;
        NECI_FOR_RUNS(k, L) {
            m[k] = sm[k];
            if (m[k]) has = true;
        }
        if (has) {
            double S[2] = {0.0, 0.0};
            bool nz = false;  // a block of the compressed list (CompressSpawnedList drops zero sums)
            NECI_FOR_RUNS(k, L) {
                const long long q = sa[k];
                st.acc[j * L + k] = 0;
                st.meta[j * L + k] = 0;
                a_s[k] += (unsigned long long)(q < 0 ? -q : q);
                S[k] = from_fixed(q);
                nz = nz || q != 0;
            }
            a_found += nz ? 1ull : 0ull;
            NECI_FOR_RUNS(k, L) {
                if (abs_bits(C[k]) < dbl_bits(kEps12) && p.t_trunc_initiator) {
                    const bool sp_init = (m[k] & 0x80000000u) ||
                                         (p.t_init_coherent_rule && (m[k] & 0x7FFFFFFFu) >= 2u);
                    if (!sp_init && !core) { a_ab[k] += fabs(S[k]); S[k] = 0.0; }
                }
                if (prod_negative(C[k], S[k])) a_ann[k] += 2.0 * min_abs(C[k], S[k]);
            }
            NECI_FOR_RUNS(k, L) C[k] = S[k] + C[k];
            changed = true;
            if (!core) {
                bool unocc = true;
                NECI_FOR_RUNS(k, L) if (abs_bits(C[k]) >= dbl_bits(kEps12)) unocc = false;
                if (unocc) {
                    hash_remove(st, j);
                    ++a_tomb;
                    r[W + L] = flags | 1ll;
                }
            }
        }
        // CalcHashTableStats (load_balancer.fpp:646-806)
        bool occ = false;
        NECI_FOR_RUNS(k, L) if (abs_bits(C[k]) >= dbl_bits(kEps12)) occ = true;
        if (!occ && !core) {
            if (changed) NECI_FOR_RUNS(k, L) r[W + k] = double_to_word(C[k]);
            ++a_holes;
            return;
        }
        if (!core) {
            NECI_FOR_RUNS(k, L) {
                const double a = abs_dbl(C[k]);
                if (abs_bits(a) > dbl_bits(kEps12) && abs_bits(a) < dbl_bits(p.occupied_thresh)) {
                    unsigned long long d[kMaxWords];
                    NECI_FOR_WORDS(w, W) d[w] = (unsigned long long)sr[w];
                    Stream rng(det_key(d, W, p.seed), p.iter, P_STATS_ROUND, k, 0);
                    // (T - a) / T; a division by T = 1 (the default) is exact and skipped
                    const double tma = p.occupied_thresh - a;
                    const double pRemove =
                        dbl_bits(p.occupied_thresh) == dbl_bits(1.0) ? tma : div_dbl(tma, p.occupied_thresh);
                    if (bern(rng, pRemove)) {
                        a_rm[k] += a;
                        C[k] = 0.0;
                        bool unocc = true;
                        NECI_FOR_RUNS(k2, L) if (abs_bits(C[k2]) >= dbl_bits(kEps12)) unocc = false;
                        if (unocc) {
                            hash_remove(st, j);
                            ++a_tomb;
                            r[W + L] = flags | 1ll;
                        }
                    } else {
                        a_born[k] += tma;
                        C[k] = fsign(p.occupied_thresh, C[k]);
                    }
                    changed = true;
                }
            }
        }
        if (changed) NECI_FOR_RUNS(k, L) r[W + k] = double_to_word(C[k]);
        occ = false;
        NECI_FOR_RUNS(k, L) {
            a_tp[k] += abs_dbl(C[k]);
            a_norm[k] = fma(C[k], C[k], a_norm[k]);  // a statistic: one rounding, one FP64 instruction
            if (abs_bits(C[k]) >= dbl_bits(kEps12)) occ = true;
        }
        if (occ || core) {
            ++a_occ;
            bool is_ref = true;
            NECI_FOR_WORDS(w, W) if ((unsigned long long)sr[w] != s.ilut_ref[w]) is_ref = false;
            if (is_ref) NECI_FOR_RUNS(k, L) c->noat_hf[k] = C[k];
        } else {
            ++a_holes;
        }
        };
    // Round kr: wait for tile kr, one barrier, then the copy of tile kr + 1
    // into the other buffer, which no thread reads any more (as in k_sweep).
    if (threadIdx.x == 0 && nrounds > 0) issue(0);
    for (long long kr = 0; kr < nrounds; ++kr) {
        const long long tile = blockIdx.x + kr * gridDim.x;
        const unsigned char *sbase = merge_smem + (kr & 1) * stage_bytes;
        if (threadIdx.x == 0)
            stage_ok[kr & 1] =
                stage_rows(tile, n) > 0 ? (mbar_wait_bounded(&bars[kr & 1], (uint32_t)((kr >> 1) & 1)) ? 1 : 0) : 1;
        __syncthreads();
        if (!stage_ok[kr & 1]) {
            if (threadIdx.x == 0) {
                set_err(c, NECI_GPU_ERR_TIMEOUT);
                (void)mbar_wait_bounded(&bars[kr & 1], (uint32_t)((kr >> 1) & 1));  // the only copy in flight
            }
            __syncthreads();
            return;
        }
        if (threadIdx.x == 0 && kr + 1 < nrounds) issue(kr + 1);
        const long long j = tile * kStageTile + threadIdx.x;
        if (j < n && !(split && sbase[(size_t)kStageTile * (R * 8 + L * 12) + threadIdx.x]))
            body(j, (const long long *)sbase + (size_t)threadIdx.x * R,
                 (const uint32_t *)(sbase + (size_t)kStageTile * R * 8) + (size_t)threadIdx.x * L,
                 (const long long *)(sbase + (size_t)kStageTile * (R * 8 + L * 4)) + (size_t)threadIdx.x * L);
    }
    double v[12] = {a_born[0], a_born[1], a_ann[0], a_ann[1], a_ab[0], a_ab[1], a_rm[0], a_rm[1],
                    a_tp[0], a_tp[1], a_norm[0], a_norm[1]};
    double *const dst[12] = {&c->nborn[0], &c->nborn[1], &c->nannihil[0], &c->nannihil[1],
                             &c->naborted[0], &c->naborted[1], &c->nremoved[0], &c->nremoved[1],
                             &c->tot_parts[0], &c->tot_parts[1], &c->norm[0], &c->norm[1]};
    block_add<12>(v, dst, L);
    unsigned long long u[6] = {a_s[0], a_s[1], a_occ, a_holes, a_found, a_tomb};
    unsigned long long *const du[6] = {&c->abs_s[0], &c->abs_s[1], &c->n_occupied, &c->n_holes, &c->n_found,
                                       &c->n_tomb};
    block_add_u<6>(u, du);
}

// ===========================================================================
// Stochastic 2-RDM of a replica pair (run 1 = bra, run 2 = ket), sampled
// every step while enabled.  Off-diagonal: each spawn of run s from D_i
// onto D_j that is occupied after annihilation adds
//   1/2 w_i C_j^(other run) <D_j| a+_p a+_q a_s a_r |D_i>
// (DiDj_Found_FillRDM, rdm_filling.F90:423-611, with the instantaneous
// C_j of the next iteration as there); w_i has expectation C_i per child
// (rdm_parent_weight).  Diagonal: every occupied D_i adds C_i^1 C_i^2 to
// Gamma(pq, pq) for its occupied pairs p < q (fill_spawn_rdm_diag,
// rdm_filling.F90:769-789, with instantaneous rather than averaged signs).
// The host symmetrises Gamma and normalises it by its trace.
// ===========================================================================
__device__ inline long long rdm_pair(int p, int q) { return (long long)(q - 1) * (q - 2) / 2 + (p - 1); }

// Add_RDM_From_IJ_Pair (rdm_filling.F90:696-767) with nI = parent (ket) and
// nJ = child (bra): a single i -> a adds to Gamma(ka, ki) for every other
// occupied k of nI (fill_spawn_rdm_singles, :791-817), a double ij -> ab to
// Gamma(ab, ij); both carry the excitation's fermionic sign.
__device__ inline void rdm_add_pair(const DevSys &s, const DevState &st, const unsigned long long *par,
                                    const unsigned long long *chi, double c) {
    int src[2] = {0, 0}, tgt[2] = {0, 0}, ns = 0, nt = 0;
    NECI_FOR_WORDS(w, s.W) {
        unsigned long long x = par[w] & ~chi[w], y = chi[w] & ~par[w];
        while (x) { if (ns < 2) src[ns] = w * 64 + __ffsll((long long)x); ++ns; x &= x - 1; }
        while (y) { if (nt < 2) tgt[nt] = w * 64 + __ffsll((long long)y); ++nt; y &= y - 1; }
    }
    if (ns != nt || ns < 1 || ns > 2) return;
    if (ns == 1) {
        const int i = src[0], a = tgt[0];
        const bool par_odd = occ_between(par, s.W, min(i, a), max(i, a)) & 1;
        const double full = par_odd ? -c : c;
        NECI_FOR_WORDS(w, s.W) {
            unsigned long long x = par[w];
            while (x) {
                const int k = w * 64 + __ffsll((long long)x);
                x &= x - 1;
                if (k == i) continue;
                const double sg = ((k < a) == (k < i)) ? full : -full;
                const long long bra = k < a ? rdm_pair(k, a) : rdm_pair(a, k);
                const long long ket = k < i ? rdm_pair(k, i) : rdm_pair(i, k);
                atomicAdd(&st.rdm2[bra * s.npair + ket], sg);
            }
        }
        return;
    }
    // the parity of i -> a then j -> b (sorted pairing), as successive singles
    unsigned long long t[kMaxWords];
    NECI_FOR_WORDS(w, s.W) t[w] = par[w];
    int np = occ_between(t, s.W, min(src[0], tgt[0]), max(src[0], tgt[0]));
    flip_orb(t, src[0]);
    flip_orb(t, tgt[0]);
    np += occ_between(t, s.W, min(src[1], tgt[1]), max(src[1], tgt[1]));
    atomicAdd(&st.rdm2[rdm_pair(tgt[0], tgt[1]) * s.npair + rdm_pair(src[0], src[1])], (np & 1) ? -c : c);
}

__global__ void __launch_bounds__(256) k_rdm_offdiag(DevSys s, DevState st) {
    if (halted(st)) return;
    extern __shared__ int32_t sh_rh2[];
    load_rh2(s, sh_rh2);
    Control *c = st.ctl;
    const long long n = (long long)min(c->n_spawned, (unsigned long long)st.max_spawned);
    const int W = s.W, L = s.L, R = s.R;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long *rec = st.spawn + i * R;
        const long long *par = st.spawn_par + i * (W + 1);
        const double w = word_to_double(par[W]);
        const int run = rec[W] != 0 ? 0 : 1;
        unsigned long long d[kMaxWords], pd[kMaxWords];
        NECI_FOR_WORDS(k, W) {
            d[k] = (unsigned long long)rec[k];
            pd[k] = (unsigned long long)par[k];
        }
        const long long slot = hash_find(st, d, W, R, neci_hash(d, W, sh_rh2), c);
        if (slot < 0) continue;
        const double cj = word_to_double(st.dets[slot * R + W + (1 - run)]);
        if (cj == 0.0) continue;
        rdm_add_pair(s, st, pd, d, 0.5 * w * cj);
        (void)L;
    }
}

// Pairs of core determinants (fill_RDM_offdiag_deterministic,
// rdm_filling.F90:947-1111): spawns between core determinants do not happen
// (the deterministic projection replaces them), so every stored off-diagonal
// element (i, j) of the core Hamiltonian adds, with parent i and child j,
//   1/2 (x_i^1 C_j^2 + x_i^2 C_j^1),
// the expectation of what the two runs' spawns from i onto j would add:
// x_i the parent's amplitudes at the start of the step (the core vector), C_j
// the child's after annihilation.  NECI adds C_i^2 C_j^1 per ordered pair,
// with averaged signs; over both orders the sums agree, and the host
// symmetrises.  One warp per segment of a core row (the segments of k_core).
__global__ void __launch_bounds__(256) k_rdm_core(DevSys s, DevState st) {
    if (halted(st)) return;
    const int W = s.W, R = s.R;
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long sg = warp; sg < st.n_core_seg; sg += nwarps) {
        const CoreSeg seg = st.core_seg[sg];
        const long long i = seg.row & 0x7FFFFFFF;
        const long long e0 = seg.e0, e1 = seg.e0 + seg.len;
        unsigned long long pd[kMaxWords];
        NECI_FOR_WORDS(w, W) pd[w] = (unsigned long long)st.core_dets[i * W + w];
        const double x1 = st.core_x[i * 2], x2 = st.core_x[i * 2 + 1];
        for (long long e = e0 + lane; e < e1; e += 32) {
            const long long j = st.core_col[e];
            const long long *rj = st.dets + st.core_slot[j] * R;
            const double c = 0.5 * (x1 * word_to_double(rj[W + 1]) + x2 * word_to_double(rj[W]));
            if (c == 0.0) continue;
            unsigned long long cd[kMaxWords];
            NECI_FOR_WORDS(w, W) cd[w] = (unsigned long long)st.core_dets[j * W + w];
            rdm_add_pair(s, st, pd, cd, c);
        }
    }
}

// Diagonal terms; per-block sums in shared memory when npair doubles fit.
// The lanes of a warp hold determinants that share most of their orbitals
// (those near the reference), so walking their pairs in one order would
// send all lanes' atomics to the same sum at once; each lane walks the list
// of electron pairs from its own starting point instead.  (The sums are
// atomics, whose order is not defined in either case.)
__global__ void __launch_bounds__(256) k_rdm_diag(DevSys s, DevState st, int use_shared) {
    if (halted(st)) return;
    extern __shared__ double sh_diag[];
    // the electron pairs (a, b), b < a, as a | b << 8
    __shared__ uint16_t pairs[kMaxNel * (kMaxNel - 1) / 2];
    const long long npair = s.npair;
    const int P = s.nel * (s.nel - 1) / 2;
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
        // the largest a with a (a - 1) / 2 <= k, from a float estimate
        int a = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)k)) * 0.5f);
        while (a > 1 && a * (a - 1) / 2 > k) --a;
        while ((a + 1) * a / 2 <= k) ++a;
        pairs[k] = (uint16_t)(a | ((k - a * (a - 1) / 2) << 8));
    }
    if (use_shared)
        for (long long k = threadIdx.x; k < npair; k += blockDim.x) sh_diag[k] = 0.0;
    __syncthreads();
    const int start = P > 0 ? (int)((threadIdx.x * 7u) % (unsigned)P) : 0;
    const long long n = (long long)min(st.ctl->tot_walkers, (unsigned long long)st.max_walkers);
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const long long *r = st.dets + j * s.R;
        const double prod = word_to_double(r[s.W]) * word_to_double(r[s.W + 1]);
        if (prod == 0.0) continue;
        uint8_t nI[kMaxNel];
        unsigned long long d[kMaxWords];
        NECI_FOR_WORDS(w, s.W) d[w] = (unsigned long long)r[w];
        if (decode(d, s.W, nI) != s.nel) continue;  // every row holds nel electrons (checked at upload)
        int k = start;
        for (int t = 0; t < P; ++t) {
            const uint32_t ab = pairs[k];
            const long long pq = rdm_pair(nI[ab >> 8], nI[ab & 0xFFu]);
            if (use_shared) atomicAdd(&sh_diag[pq], prod);
            else atomicAdd(&st.rdm2[pq * npair + pq], prod);
            if (++k == P) k = 0;
        }
    }
    if (use_shared) {
        __syncthreads();
        for (long long k = threadIdx.x; k < npair; k += blockDim.x)
            if (sh_diag[k] != 0.0) atomicAdd(&st.rdm2[k * npair + k], sh_diag[k]);
    }
}

// ===========================================================================
// k_final: write the step's stats record.
// ===========================================================================
// The record goes to out[*pos] (and *pos advances, up to max_out - 1) when
// pos is given: the step graph is the same for every step of a batch, and
// each step's record lands in its own place.
// split: the merge sweep counted the slots the step began with less the
// freed ones; the new determinants are occupied, and the freed slots the
// placement did not fill are holes.
__global__ void k_final(DevState st, neci_gpu_iter_stats *base, int *pos, int max_out, IterParams *pp,
                        int advance_iter, long long n_core, int split) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    neci_gpu_iter_stats *out = base;
    if (pos) {
        const int k = *pos;
        out = base + (k < max_out ? k : max_out - 1);
        *pos = k + 1;
    }
    Control *c = st.ctl;
    if (c->halted) {
        // a previous step failed: report its status again, change nothing
        neci_gpu_iter_stats r{};
        r.err = c->halted;
        *out = r;
        return;
    }
    if (c->tot_walkers > (unsigned long long)st.max_walkers) c->tot_walkers = (unsigned long long)st.max_walkers;
    if (split) {
        const unsigned long long used = c->free_taken < c->n_free ? c->free_taken : c->n_free;
        c->n_occupied += c->n_new;
        c->n_holes += c->n_free - used;
    }
    neci_gpu_iter_stats r;
    for (int k = 0; k < 2; ++k) {
        r.nborn[k] = c->nborn[k];
        r.ndied[k] = c->ndied[k];
        // compression annihilation: sum |q| - sum |sum q| over unique dets
        const long long dq = (long long)(c->abs_q[k] - c->abs_s[k]);
        r.nannihil[k] = c->nannihil[k] + (double)dq * 0x1.0p-32;
        r.naborted[k] = c->naborted[k];
        r.nremoved[k] = c->nremoved[k];
        r.tot_parts[k] = c->tot_parts[k];
        r.tot_parts_old[k] = c->tot_parts_old[k];
        r.noat_hf[k] = c->noat_hf[k];
        r.hf_cyc[k] = c->hf_cyc[k];
        r.enum_cyc[k] = c->enum_cyc[k];
        r.norm_psi_sq[k] = c->norm[k];
    }
    r.tot_walkers = (long long)c->tot_walkers;
    r.n_occupied = (long long)c->n_occupied;
    r.holes_in_list = (long long)c->n_holes;
    r.n_attempts = (long long)c->n_attempts;
    r.n_spawned = (long long)c->n_spawned;
    // the length of the compressed spawn list: unique determinants whose
    // spawns do not sum to zero
    r.n_unique = (long long)(c->n_reps_nz + c->n_found);
    r.n_new = (long long)c->n_new;
    r.n_core = n_core;
    r.err = c->err;
    r.reserved = 0;
    *out = r;
    if (advance_iter) pp->iter += 1;
    // rebuild the walker hash before the next step when live entries plus
    // tombstones pass 70% of the buckets
    c->rehash = (c->n_occupied + c->n_tomb) * 10ull > st.hash_n * 7ull ? 1 : 0;
    // compact the list before the next step when holes outnumber occupied slots
    c->compact = (c->tot_walkers > (unsigned long long)(4 * kCompactTile) && c->n_holes * 2ull > c->tot_walkers) ? 1 : 0;
    // a failed step halts the ones after it (in the same graph batch)
    if (c->err) c->halted = c->err;
}

// ===========================================================================
// Host-side launch helpers (declared in internal.h).
// ===========================================================================
// Grids are sized to the context's capacity, so that small contexts run
// side by side (neci_gpu_iterate_batch) instead of each filling the GPU.
static int clamp_grid(long long want, int hi) { return (int)(want < 8 ? 8 : (want > hi ? hi : want)); }
static int grid_slots(const Engine &e) { return clamp_grid(e.st.max_walkers / 2048 + 1, e.num_sms * 4); }
static int grid_spawns(const Engine &e, int threads, int occ = 0) {
    return clamp_grid(e.st.max_spawned / (threads * 4) + 1, e.num_sms * (occ > 0 ? occ : (threads == 128 ? 8 : 4)));
}
static int grid_for(const Engine &e, int threads) {
    (void)threads;
    return grid_slots(e);
}

void launch_begin(Engine &e, cudaStream_t s) { k_begin<<<1, 32, 0, s>>>(e.st); }

void launch_compact(Engine &e, cudaStream_t s) {
    const int grid = clamp_grid(e.st.max_walkers / kCompactTile + 1, e.num_sms * 2);
    k_compact_count<<<grid, kCompactTile, 0, s>>>(e.sys, e.st);
    k_compact_scan<<<1, kCompactTile, 0, s>>>(e.st);
    k_compact_holes<<<grid, kCompactTile, 0, s>>>(e.sys, e.st);
    k_compact_move<<<grid_slots(e), 256, 0, s>>>(e.sys, e.st);
    k_compact_done<<<1, 32, 0, s>>>(e.st);
}

void launch_rehash(Engine &e, cudaStream_t s) {
    k_hash_clear<<<grid_for(e, 256), 256, 0, s>>>(e.st);
    k_hash_fill<<<grid_for(e, 256), 256, (e.sys.nbasis + 1) * sizeof(int32_t), s>>>(e.sys, e.st);
}

// Dynamic shared memory of the staged sweeps: two stages of a tile.
static size_t sweep_smem_bytes(const Engine &e) { return 2ull * kStageTile * (e.sys.R + 2) * 8; }
static size_t merge_smem_bytes(const Engine &e) { return 2ull * kStageTile * (e.sys.R * 8 + e.sys.L * 12 + 1); }

int configure_kernels(Engine &e) {
    // The stages and the block reductions' shared arrays pass the default
    // 48 KB per block.  The limit is an attribute of the kernel for the whole
    // process, so it is raised to the largest row any context can have
    // (kMaxWords det words, two signs, a flag word), never lowered.
    const int rmax = kMaxWords + 2 + 1;
    const int sweep_max = 2 * kStageTile * (rmax + 2) * 8;
    const int merge_max = 2 * kStageTile * (rmax * 8 + 2 * 12 + 1);
    if (cudaFuncSetAttribute(k_sweep<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sweep_max) != cudaSuccess ||
        cudaFuncSetAttribute(k_sweep<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sweep_max) != cudaSuccess ||
        cudaFuncSetAttribute(k_sweep<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sweep_max) != cudaSuccess ||
        cudaFuncSetAttribute(k_sweep<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sweep_max) != cudaSuccess)
        return 1;
    if (cudaFuncSetAttribute(k_merge_stats<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, merge_max) != cudaSuccess)
        return 1;
    if (cudaFuncSetAttribute(k_merge_stats<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, merge_max) != cudaSuccess)
        return 1;
    // resident blocks per SM of each instance (the smaller of the two run counts)
    auto occ = [](const void *f1, const void *f2, int threads, size_t smem) {
        int a = 0, b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, f1, threads, smem) != cudaSuccess) a = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f2, threads, smem) != cudaSuccess) b = 1;
        const int m = a < b ? a : b;
        return m < 1 ? 1 : m;
    };
    const size_t rh2 = (size_t)(kMaxWords * 64 + 1) * sizeof(int32_t);
    e.occ_probe = occ((const void *)k_ann_probe<1>, (const void *)k_ann_probe<2>, 256, rh2);
    e.occ_compress = occ((const void *)k_ann_compress<1>, (const void *)k_ann_compress<2>, 256, 0);
    e.occ_insert = occ((const void *)k_ann_decide<1>, (const void *)k_ann_decide<2>, 256, 0);
    e.occ_place = occ((const void *)k_ann_place<1>, (const void *)k_ann_place<2>, 128, 0);
    e.occ_expand = occ((const void *)k_expand, (const void *)k_expand, 256, 0);
    (void)cudaGetLastError();
    return 0;
}

void launch_sweep(Engine &e, cudaStream_t s) {
    const int grid = grid_for(e, 256);
    const size_t shm = sweep_smem_bytes(e);
    const bool fast = sweep_fast(*e.h_params);
    if (e.sys.L == 2) {
        if (fast) k_sweep<2, true><<<grid, kStageTile, shm, s>>>(e.sys, e.st, e.d_params);
        else k_sweep<2, false><<<grid, kStageTile, shm, s>>>(e.sys, e.st, e.d_params);
    } else {
        if (fast) k_sweep<1, true><<<grid, kStageTile, shm, s>>>(e.sys, e.st, e.d_params);
        else k_sweep<1, false><<<grid, kStageTile, shm, s>>>(e.sys, e.st, e.d_params);
    }
}
void launch_expand(Engine &e, cudaStream_t s) { k_expand<<<grid_spawns(e, 256, e.occ_expand), 256, 0, s>>>(e.st); }
template <int G>
static void launch_core_g(Engine &e, cudaStream_t s) {
    const int grid = clamp_grid(e.st.n_core_seg * G / 256 + 1, e.num_sms * 8);
    if (e.h_params->precision == NECI_PREC_MIXED) k_core<G, true><<<grid, 256, 0, s>>>(e.sys, e.st, e.d_params);
    else k_core<G, false><<<grid, 256, 0, s>>>(e.sys, e.st, e.d_params);
    // launched whether or not a row has several segments, so that a step's
    // launches do not depend on the core's row lengths
    k_core_sum<<<clamp_grid(e.st.n_core_multi / 256 + 1, e.num_sms), 256, 0, s>>>(e.sys, e.st, e.d_params);
}
void launch_core(Engine &e, cudaStream_t s) {
    if (e.st.n_core <= 0) return;
    switch (e.st.core_group) {
        case 1: launch_core_g<1>(e, s); break;
        case 2: launch_core_g<2>(e, s); break;
        case 4: launch_core_g<4>(e, s); break;
        case 8: launch_core_g<8>(e, s); break;
        case 16: launch_core_g<16>(e, s); break;
        default: launch_core_g<32>(e, s); break;
    }
}
void launch_ann_probe(Engine &e, cudaStream_t s) {
    const size_t shm = (e.sys.nbasis + 1) * sizeof(int32_t);
    if (e.sys.L == 2) k_ann_probe<2><<<grid_spawns(e, 256, e.occ_probe), 256, shm, s>>>(e.sys, e.st);
    else k_ann_probe<1><<<grid_spawns(e, 256, e.occ_probe), 256, shm, s>>>(e.sys, e.st);
}
void launch_ann_compress(Engine &e, cudaStream_t s) {
    if (e.sys.L == 2) k_ann_compress<2><<<grid_spawns(e, 256, e.occ_compress), 256, 0, s>>>(e.sys, e.st);
    else k_ann_compress<1><<<grid_spawns(e, 256, e.occ_compress), 256, 0, s>>>(e.sys, e.st);
}
void launch_ann_insert(Engine &e, cudaStream_t s, int split) {
    // new determinants are a small part of the spawns: the placement's grid
    // (one determinant per thread and round) is sized to a fraction of the
    // spawn capacity, so that a small instance of a batch launches few blocks
    const int gp = clamp_grid(e.st.max_spawned / 1024 + 1, e.num_sms * e.occ_place);
    if (e.sys.L == 2) {
        k_ann_decide<2><<<grid_spawns(e, 256, e.occ_insert), 256, 0, s>>>(e.sys, e.st, e.d_params);
        k_ann_place<2><<<gp, 128, 0, s>>>(e.sys, e.st, split);
    } else {
        k_ann_decide<1><<<grid_spawns(e, 256, e.occ_insert), 256, 0, s>>>(e.sys, e.st, e.d_params);
        k_ann_place<1><<<gp, 128, 0, s>>>(e.sys, e.st, split);
    }
}
// Blocks per SM of the merge sweep when it runs beside the placement
// (split): e.merge_bpsm, two unless the merge sweep is the longer branch, so
// that the placement's blocks find registers on every SM.
void launch_merge_stats(Engine &e, cudaStream_t s, int with_core, int split) {
    const int grid = split ? clamp_grid(e.st.max_walkers / 2048 + 1, e.num_sms * e.merge_bpsm) : grid_for(e, 256);
    if (e.sys.L == 2)
        k_merge_stats<2><<<grid, kStageTile, merge_smem_bytes(e), s>>>(e.sys, e.st, e.d_params, with_core, split);
    else
        k_merge_stats<1><<<grid, kStageTile, merge_smem_bytes(e), s>>>(e.sys, e.st, e.d_params, with_core, split);
}
void launch_rdm(Engine &e, cudaStream_t s) {
    if (!e.sys.rdm) return;
    k_rdm_offdiag<<<grid_spawns(e, 256), 256, (e.sys.nbasis + 1) * sizeof(int32_t), s>>>(e.sys, e.st);
    if (e.st.n_core > 0) k_rdm_core<<<clamp_grid(e.st.n_core_seg / 8 + 1, e.num_sms * 8), 256, 0, s>>>(e.sys, e.st);
    const size_t shm = (size_t)e.sys.npair * sizeof(double);
    const int use_shared = shm <= 48 * 1024 ? 1 : 0;  // the default dynamic shared-memory limit
    // at least 64 slots per thread: every block ends by adding its npair
    // shared sums to the global 2-RDM, so the blocks are kept few
    const int grid = clamp_grid(e.st.max_walkers / (256 * 64) + 1, e.num_sms);
    k_rdm_diag<<<grid, 256, use_shared ? shm : 0, s>>>(e.sys, e.st, use_shared);
}

void launch_final(Engine &e, cudaStream_t s, neci_gpu_iter_stats *out, int *pos, int advance_iter, int split) {
    k_final<<<1, 32, 0, s>>>(e.st, out, pos, e.max_stats, e.d_params, advance_iter, e.st.n_core, split);
}

}  // namespace neci
