// engine.cuh -- device data layout and device functions of the FCIQMC engine.
//
// Walker rows are NECI CurrentDets rows (bit_rep_data.F90:10-17): W det
// words, L signs (real(dp) bits), one flag word; R = W + L + 1 int64 words.
// Spawn records carry the same words, except that the L sign words hold the
// amplitude in 64-bit fixed point (NECI_SPAWN_FIXED_BITS fractional bits)
// while spawns are being summed.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/neci_gpu.h"
#include "bitsplit.h"

namespace neci {

constexpr int kMaxWords = 4;      // nBasis <= 255 (NIfD <= 3)
// A loop over the words 0..W-1 of a determinant, unrolled over kMaxWords.
#define NECI_FOR_WORDS(w, W) _Pragma("unroll") for (int w = 0; w < kMaxWords; ++w) if (w < (W))
constexpr int kMaxRuns = 2;  // lenof_sign: one run or a replica pair
// A loop over the runs 0..L-1, unrolled over kMaxRuns: per-run arrays
// indexed by it stay in registers.
#define NECI_FOR_RUNS(k, L) _Pragma("unroll") for (int k = 0; k < kMaxRuns; ++k) if (k < (L))
constexpr int kMaxNel = 64;
constexpr int kMaxNeigh = 8;
constexpr int kBigAttempts = 32;  // parents with more attempts are expanded by k_expand
constexpr int kHugeAttempts = 1 << 16;  // ... and with more than this by the whole grid
constexpr int kExpandChunk = 512;  // k_expand's work item: at most this many attempts of one parent
constexpr int kMaxHuge = 4096;
constexpr int kCompactTile = 1024;        // slots per block of the compaction scans
constexpr int kProbeLimit = 1 << 16;
constexpr uint32_t kEmpty = 0u;
constexpr uint32_t kTomb = 0xFFFFFFFFu;
// rep_bucket of a unique new determinant that holds no compression-table
// bucket (the sort form of the annihilation merges without the table)
constexpr uint32_t kNoBucket = 0xFFFFFFFFu;
constexpr double kEps12 = 1e-12;

enum Purpose : uint32_t { P_NSPAWN = 1, P_ATTEMPT = 2, P_DEATH = 3, P_ANN_ROUND = 4, P_STATS_ROUND = 5 };

// Per-iteration counters and estimator sums (one instance in device memory).
struct Control {
    unsigned long long tot_walkers;     // slots in use (TotWalkers)
    unsigned long long n_free;          // holes pushed this step
    unsigned long long free_taken;      // holes reused by new determinants
    unsigned long long n_att;           // spawn attempt entries
    unsigned long long n_spawned;       // spawn records
    unsigned long long n_cand;          // spawns onto determinants not in the list
    unsigned long long n_reps;          // unique new determinants
    unsigned long long n_new;           // determinants inserted
    unsigned long long n_attempts;      // spawn attempts
    unsigned long long n_occupied;
    unsigned long long n_holes;
    unsigned long long n_tomb;          // hash tombstones
    unsigned long long n_found;         // unique spawned determinants already present, with a
                                        // non-zero summed amplitude
    unsigned long long n_reps_nz;       // unique new determinants with a non-zero summed amplitude
    unsigned long long n_big;           // parents expanded by k_expand
    unsigned long long n_huge;          // parents expanded by the whole grid
    unsigned long long n_long;          // sort annihilation: runs of equal keys left to k_sk_long
    unsigned long long n_place;         // new determinants k_ann_decide leaves to k_ann_place
    unsigned long long n_pre;           // slots in use before this step's new determinants
    unsigned long long abs_q[2];        // sum |q| of all spawn records (fixed point)
    unsigned long long abs_s[2];        // sum |sum q| of the unique spawned determinants
    int err;
    int halted;                         // status of a failed step: later steps do nothing until
                                        // the walker list is uploaded again
    int rehash;                         // rebuild the walker hash at the next step
    int compact;                        // compact the walker list at the next step
    unsigned long long compact_k;       // occupied slots kept by the compaction
    unsigned long long compact_pos_k;   // occupied slots below compact_k
    double nborn[2], ndied[2], nannihil[2], naborted[2], nremoved[2];
    double tot_parts[2], tot_parts_old[2], noat_hf[2], hf_cyc[2], enum_cyc[2], norm[2];
    // tau search (log_spawn_magnitude / log_death_magnitude): kept across
    // steps until the host resets them.  Maxima are the bit patterns of
    // non-negative doubles, which order like the values.
    unsigned long long tau_gamma[4];    // per TauClass
    unsigned long long tau_cnt[4];
    unsigned long long tau_death;       // max_death_cpt
};

// One segment of a core row: its first element, its length, its row, and
// whether the row has other segments (one 16-byte load).
struct __align__(16) CoreSeg {
    long long e0;
    int32_t len;
    int32_t row;  // bit 31: the row has more than one segment
};

// Excitation classes of the conventional tau search
// (tau_search_conventional.F90:138-258).
enum TauClass : int { TC_SING = 0, TC_DOUB = 1, TC_PAR = 2, TC_OPP = 3 };
constexpr unsigned int kTauCntThreshold = 50;  // cnt_threshold

// System description as seen by the kernels (passed by value).
// One slot of a PCHB alias table (per (ij, type) and slot), the fields a
// draw reads in one 32-byte sector: the slot's threshold and alias, and the
// probability, 1/probability and target pair of the slot itself.  A draw that
// keeps its slot reads one record, one that takes the alias a second.
struct __align__(32) AliasRec {
    unsigned long long thr;  // prob_thresh(bias)
    double prob, inv;        // p(ab | ij, type) and its reciprocal
    int32_t alias;           // 1-based alias slot
    int32_t tgt;             // tgt_pair of this slot: (small << 16) | large
};
__device__ inline AliasRec load_alias(const AliasRec *p) {
    const ulonglong2 *q = reinterpret_cast<const ulonglong2 *>(p);
    const ulonglong2 x = __ldg(q), y = __ldg(q + 1);
    AliasRec r;
    r.thr = x.x;
    r.prob = __longlong_as_double((long long)x.y);
    r.inv = __longlong_as_double((long long)y.x);
    r.alias = (int32_t)(uint32_t)(y.y & 0xFFFFFFFFull);
    r.tgt = (int32_t)(uint32_t)(y.y >> 32);
    return r;
}

struct DevSys {
    int nel, nbasis, W, L, R, system, excitgen, max_neigh, nsites, nOccAlpha, nOccBeta, nBI;
    double uhub, bhub, ecore, p_singles, p_parallel, hii;
    long long ijMax, abMax;
    unsigned long long ilut_ref[kMaxWords];
    const int32_t *random_hash2;   // [nbasis + 1], 1-based
    const double *tmat;            // TMat2D column-major
    const double *umat;            // UMAT, UMatInd - 1
    const int32_t *neighbours;     // [nsites * max_neigh], 1-based site, 0 = none
    const double *pexch;           // [ijMax]
    const double *alias_bias;      // [(ij-1)*3 + type-1][abMax]
    const int32_t *alias_alias;
    const double *alias_prob;
    const uint8_t *alias_present;  // [(ij-1)*3 + type-1]
    const struct AliasRec *alias_rec;  // [(ij-1)*3 + type-1][abMax]: one 32 B record per slot
    const int32_t *tgt_pair;       // [abMax+1]: (small << 16) | large
    // hoisted constants of the generators
    double pgen_par, pgen_opp, p_doubles, p_elec;        // pBias/par, (1-pBias)/AB, 1-pSingles, 1/nel
    unsigned long long thr_singles, thr_bias;           // prob_thresh(pSingles), prob_thresh(pParallel)
    const unsigned long long *alias_thr;                 // prob_thresh(bias) of each alias entry
    const unsigned long long *pexch_thr;                 // prob_thresh(pExch(ij))
    // single-precision copies for the mixed-precision spawn amplitudes
    float f_pgen_par, f_pgen_opp, f_p_doubles, f_p_singles, f_p_elec;
    float f_inv_nalpha;  // 1/nOccAlpha (0 without alpha electrons): pair index -> (alpha, beta) positions
    const float *umat32, *tmat32, *alias_prob32, *pexch32;
    // Coulomb and Coulomb-minus-exchange rows of the single-excitation
    // elements: [((i-1) n + (a-1)) n + (k-1)] = <ik|ak> (jrow) and
    // <ik|ak> - <ik|ka> (jkrow) for spatial orbitals i, a, k of n = nBI;
    // FP32 copies are the FP64 values rounded once
    const double *jrow, *jkrow;
    const float *jrow32, *jkrow32;
    // Coulomb and exchange integrals of spatial orbital pairs for the
    // diagonal element: jmat[(i-1) n + (j-1)] = <ij|ij>, kmat[...] = <ij|ji>,
    // the UMAT values sltcnd_0 reads, in n^2 doubles each (L1-resident for
    // n up to about 64)
    const double *jmat, *kmat;
    // 1/p_gen of a uniform single with `count` allowed (electron, hole)
    // pairs: [count] = count * (1 / pSingles), FP64 and FP32
    const double *inv_single;
    const float *inv_single32;
    // reciprocals: the spawn amplitude multiplies by 1/p_gen built from them
    double inv_par, inv_opp, inv_pdoub, inv_psingles;
    float f_inv_par, f_inv_opp, f_inv_pdoub, f_inv_psingles;
    // uniform generator (C1): r < pDoubles picks a double; the double's
    // pgen and 1/pgen per iSpn (1 beta/beta, 2 alpha/beta, 3 alpha/alpha)
    unsigned long long thr_doubles;
    double pgen_unif[3], inv_unif[3];
    float f_pgen_unif[3], f_inv_unif[3];
    const double *alias_inv, *pexch_inv, *pnoexch_inv;   // 1/prob, 1/pExch, 1/(1-pExch)
    const float *alias_inv32, *pexch_inv32, *pnoexch_inv32;
    // tau search: on/off, and per TauClass the factor that unbiases p_gen
    // (pSingles, pDoubles, pDoubles pParallel, pDoubles (1 - pParallel))
    int tau_search;
    double tau_fac[4];
    float f_tau_fac[4];
    // stochastic 2-RDM of a replica pair: on/off and the number of spin-orbital
    // pairs p < q (the 2-RDM is npair x npair)
    int rdm;
    long long npair;
};

// Resident walker state (device pointers).
struct DevState {
    long long *dets;               // CurrentDets rows
    double *diagH, *offdiagH;      // global_det_data diagH - Hii, offdiagH
    uint32_t *hash;                // walker hash: slot+1, kEmpty, kTomb
    unsigned long long hash_n;     // buckets (power of two)
    uint32_t *slot_bucket;         // bucket holding each slot
    uint8_t *hole_mark;            // 1: the slot went to this step's free list (k_sweep)
    unsigned long long *dkey;      // det_key of each slot with spawn attempts this step (k_sweep)
    int32_t *free_list;
    long long max_walkers, max_spawned, max_att;
    long long *spawn;              // spawn records
    unsigned long long *att;       // attempts: slot | run << 32 | neg << 33 | attempt << 34
    unsigned long long *big;       // chunks of at most kExpandChunk attempts of one parent, as triples:
                                   // slot | run << 32 | neg << 33 | first attempt << 34, attempts, first entry
    unsigned long long *huge;      // the same for parents with more than kHugeAttempts attempts
    long long max_big;
    long long *acc;                // per slot*L fixed-point spawn sums (found determinants)
    uint32_t *meta;                // per slot*L spawn counts | initiator bit 31
    uint32_t *cand;                // record index of spawns onto absent determinants
    unsigned long long *cand_h;    // their 64-bit NECI hash
    uint32_t *spawn_hash;          // compression table: candidate position + 1
    unsigned long long spawn_hash_n;
    int comp_shift;                // the table in use holds >= 2^comp_shift buckets per candidate
    uint32_t *reps;                // candidate position of each unique new determinant
    uint32_t *place;               // candidate positions of the new determinants to place
    uint32_t *rep_bucket;
    long long *rep_q;              // per candidate*L fixed-point sums
    uint32_t *rep_cnt;             // per candidate*L counts | initiator bit 31
    // semistochastic core
    long long n_core;
    int32_t *core_of_slot;         // core index or -1
    long long *core_slot;
    // compaction of the walker list: occupied slots per tile of kCompactTile,
    // their exclusive prefix, and the holes below the kept count by rank
    uint32_t *tile_count, *tile_off;
    int32_t *hole_at_rank;
    // 2-RDM sampling: the parent of every spawn record (W det words, then the
    // unbiasing weight as double bits), and the dense 2-RDM
    // rdm2[pair(p,q) * npair + pair(r,s)] = <a+_p a+_q a_s a_r>, p<q, r<s
    long long *spawn_par;
    double *rdm2;
    double *core_x, *core_y;
    float *core_x32;               // core_x rounded to FP32, written in mixed-precision steps
    long long *core_rowptr;
    int core_group;                // lanes that sum one core row (core_group_size)
    // segments of the core rows, core_segment_len elements at most: each
    // segment's range and row, each row's first segment (n_core + 1 entries),
    // the partial sums of the segments of rows with more than one, and those
    // rows
    long long n_core_seg, n_core_multi;
    long long core_seg_len;        // elements of a segment, core_segment_len
    struct CoreSeg *core_seg;
    long long *core_seg_first;
    double *core_seg_y;
    int32_t *core_multi;
    long long *core_dets;          // W words of each core determinant (2-RDM core pairs)
    // sort form of the annihilation: 32-bit sort keys and record indices
    // (two buffers each, ping-ponged by the radix passes), the 64-bit NECI
    // hash of every record, per-block digit counts of a radix pass, and the
    // starts of runs of equal keys longer than kShortRun
    uint32_t *sk_key[2], *sk_val[2];
    unsigned long long *sk_h;
    uint32_t *sk_counts;
    uint32_t *sk_long;
    int sk_blocks;                 // blocks of a radix pass (the counts hold 256 per block)
    int sk_hb;                     // log2 of the walker-hash length
    int32_t *core_col;
    double *core_val;
    float *core_val32;
    Control *ctl;
};

// Lanes that sum one row of the core Hamiltonian in k_core: the smallest
// power of two G with NECI_CORE_LANE_ELEMS * G at least the mean row length,
// at most 32 (so a lane takes about that many elements of a row); 1 sums a
// row in one thread.
#ifndef NECI_CORE_LANE_ELEMS
#define NECI_CORE_LANE_ELEMS 4
#endif
__host__ __device__ inline int core_group_size(long long nnz, long long n_core) {
    int g = 1;
    while (g < 32 && (long long)NECI_CORE_LANE_ELEMS * g * n_core < nnz) g <<= 1;
    return g;
}

// Elements of a core row that one group of G lanes sums as one segment
// (per_lane each, 64 unless set by NECI_OPT_CORE_SEGMENT).  A longer row is
// split into segments from its start; their partial sums are added in
// segment order, so that a row of any length is spread over several groups
// in a defined order.
constexpr int kCoreSegmentPerLane = 64;
__host__ __device__ constexpr long long core_segment_len(int G, int per_lane) { return (long long)per_lane * G; }

// Slots in use, never above the allocation (a step that overflowed the list
// leaves TotWalkers above it).
__device__ inline long long slots_in_use(const DevState &st) {
    const unsigned long long n = st.ctl->tot_walkers;
    return (long long)(n < (unsigned long long)st.max_walkers ? n : (unsigned long long)st.max_walkers);
}
__device__ inline bool halted(const DevState &st) { return st.ctl->halted != 0; }

struct IterParams {
    double tau, diag_sft[2], initiator_walk_no, occupied_thresh, real_spawn_cutoff, av_mc_excits;
    int t_trunc_initiator, t_init_coherent_rule, t_all_real_coeff, t_real_spawn_cutoff, t_core_inits, precision;
    unsigned long long seed;
    long long iter;
    // derived on the host: 1/RealSpawnCutoff, 1/AvMCExcits and FP32 copies
    double inv_cutoff, inv_av;
    float f_tau, f_inv_av, f_cutoff, f_inv_cutoff;
    unsigned long long cutoff_q;  // RealSpawnCutoff in fixed point
    int av_unit;                  // AvMCExcits == 1: the spawn count is split in integers
};

// The sweep's fast instance serves steps with real coefficients and
// AvMCExcits = 1, the instance for any parameters the others.
__host__ __device__ inline bool sweep_fast(const IterParams &p) { return p.t_all_real_coeff && p.av_unit; }

// ---------------------------------------------------------------------------
// Philox-4x32-10 (Salmon et al., SC11) and the per-determinant stream.
// ---------------------------------------------------------------------------
__host__ __device__ inline void philox_block(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned long long p0 = (unsigned long long)0xD2511F53u * c0;
        const unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Two Philox-4x32-10 blocks of one key, computed side by side: the rounds of
// the two counters are independent, so their multiply-xor chains overlap
// instead of following each other (each block equals philox_block's).
__host__ __device__ inline void philox_pair(const uint32_t ctr_a[4], const uint32_t ctr_b[4], const uint32_t key[2],
                                            uint32_t out_a[4], uint32_t out_b[4]) {
    uint32_t a0 = ctr_a[0], a1 = ctr_a[1], a2 = ctr_a[2], a3 = ctr_a[3];
    uint32_t b0 = ctr_b[0], b1 = ctr_b[1], b2 = ctr_b[2], b3 = ctr_b[3];
    uint32_t k0 = key[0], k1 = key[1];
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned long long pa0 = (unsigned long long)0xD2511F53u * a0;
        const unsigned long long pa1 = (unsigned long long)0xCD9E8D57u * a2;
        const unsigned long long pb0 = (unsigned long long)0xD2511F53u * b0;
        const unsigned long long pb1 = (unsigned long long)0xCD9E8D57u * b2;
        a0 = (uint32_t)(pa1 >> 32) ^ a1 ^ k0;
        a1 = (uint32_t)pa1;
        a2 = (uint32_t)(pa0 >> 32) ^ a3 ^ k1;
        a3 = (uint32_t)pa0;
        b0 = (uint32_t)(pb1 >> 32) ^ b1 ^ k0;
        b1 = (uint32_t)pb1;
        b2 = (uint32_t)(pb0 >> 32) ^ b3 ^ k1;
        b3 = (uint32_t)pb0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out_a[0] = a0; out_a[1] = a1; out_a[2] = a2; out_a[3] = a3;
    out_b[0] = b0; out_b[1] = b1; out_b[2] = b2; out_b[3] = b3;
}

__host__ __device__ inline unsigned long long splitmix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    unsigned long long z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Key of a determinant's random streams.  Words at or above nset (those
// past the last orbital) are zero and are not read.
__host__ __device__ inline unsigned long long det_key(const unsigned long long *det, int W, unsigned long long seed,
                                                      int nset = kMaxWords) {
    unsigned long long h = seed ^ 0x6A09E667F3BCC909ull;
    NECI_FOR_WORDS(i, W) h = splitmix64(h ^ (i < nset ? det[i] : 0ull));
    return h;
}

// One stream of 64-bit draws for (determinant, iteration, purpose, run,
// attempt).  Every draw consumes one 64-bit value; a Philox block gives two.
// The draws not yet taken are buf[4 - have .. 3].
struct Stream {
    uint32_t key[2];
    uint32_t ctr[4];
    unsigned long long buf[4];
    int have;
    __device__ inline Stream(unsigned long long dkey, long long iter, uint32_t purpose, uint32_t run, uint32_t attempt) {
        key[0] = (uint32_t)dkey;
        key[1] = (uint32_t)(dkey >> 32);
        ctr[0] = attempt;
        ctr[1] = 0;
        ctr[2] = (uint32_t)iter;
        ctr[3] = purpose | (run << 8) | ((uint32_t)((unsigned long long)iter >> 32) << 16);
        have = 0;
    }
    __device__ inline unsigned long long next64() {
        if (have == 0) {
            uint32_t o[4];
            philox_block(ctr, key, o);
            ctr[1] += 1;
            buf[2] = ((unsigned long long)o[1] << 32) | o[0];
            buf[3] = ((unsigned long long)o[3] << 32) | o[2];
            have = 2;
        }
        // buf[4 - have] by selects: an array indexed at run time would live
        // in local memory
        const unsigned long long v = have == 4 ? buf[0] : (have == 3 ? buf[1] : (have == 2 ? buf[2] : buf[3]));
        --have;
        return v;
    }
    // When no draw is left, the next two blocks at once (philox_pair): a
    // caller that will take four more draws gets them with the two blocks'
    // round chains overlapped.  The draws are the same as one block at a time.
    __device__ inline void fill_pair() {
        if (have != 0) return;
        uint32_t c2[4] = {ctr[0], ctr[1] + 1u, ctr[2], ctr[3]};
        uint32_t o[4], q[4];
        philox_pair(ctr, c2, key, o, q);
        ctr[1] += 2;
        buf[0] = ((unsigned long long)o[1] << 32) | o[0];
        buf[1] = ((unsigned long long)o[3] << 32) | o[2];
        buf[2] = ((unsigned long long)q[1] << 32) | q[0];
        buf[3] = ((unsigned long long)q[3] << 32) | q[2];
        have = 4;
    }
    // genrand_real2 equivalent: a double in [0, 1) from 53 bits
    __device__ inline double next() { return (double)(next64() >> 11) * 0x1.0p-53; }
    // The state after the stream's first draw, given its second draw (the
    // rest of the first Philox block): the next draw returns `second`.
    __device__ inline void resume_second(unsigned long long second) {
        ctr[1] = 1;
        buf[3] = second;
        have = 1;
    }
};

// Probability p as a 64-bit threshold: draw r < thresh(p)  <=>  r/2^64 < p.
// (unsigned long long)(p * 2^64) for 0 < p < 1, 0 for p <= 0, all ones for
// p >= 1; taken on the bits of p (prob_thresh_bits), no FP64 instructions.
__host__ __device__ inline unsigned long long prob_thresh(double p) { return prob_thresh_bits(p); }
// Bernoulli(p) from one draw (p >= 1 is always true: the threshold is all
// ones only then).
__device__ inline bool bern(Stream &r, double p) {
    const unsigned long long x = r.next64();
    const unsigned long long t = prob_thresh_bits(p);
    return t == ~0ull || x < t;
}
// Bernoulli(p) for a float p from the top 32 bits of one draw.
__device__ inline bool bern_f(Stream &r, float p) {
    const unsigned int x = (unsigned int)(r.next64() >> 32);
    if (p >= 1.0f) return true;
    if (!(p > 0.0f)) return false;
    return x < (unsigned int)(p * 4294967296.0f);
}
// Uniform integer in [0, n) (multiply-high of one draw).
__device__ inline unsigned int uniform_index(Stream &r, unsigned int n) {
    return (unsigned int)__umul64hi(r.next64(), (unsigned long long)n);
}

// ---------------------------------------------------------------------------
// Fixed point and sign words.
// ---------------------------------------------------------------------------
__device__ inline long long to_fixed(double x, int *overflow) {
    const double s = x * 4294967296.0;  // 2^NECI_SPAWN_FIXED_BITS
    if (!(fabs(s) < 9.2e18)) { *overflow = 1; return 0; }
    return __double2ll_rn(s);
}
// q 2^-32 as a double: the conversion rounds once, then the scaling by 2^-32
// is exact and done on the exponent field (|q| >= 1 keeps it far from the
// subnormal range), not as an FP64 multiply.
__device__ inline double from_fixed(long long q) {
    const double v = __ll2double_rn(q);
    return q == 0 ? 0.0 : __longlong_as_double(__double_as_longlong(v) - (32ll << 52));
}
__device__ inline double word_to_double(long long w) { return __longlong_as_double(w); }
__device__ inline long long double_to_word(double d) { return __double_as_longlong(d); }
// |x| and -x on the high word, in integer instructions: materialised as FP64
// operations they would take a slot of GB300's FP64 pipe each (about one lane
// per clock per SM).
__device__ inline double abs_dbl(double x) { return __hiloint2double(__double2hiint(x) & 0x7FFFFFFF, __double2loint(x)); }
// fmin(|a|, |b|) for finite a, b, on the bit patterns.
__device__ inline double min_abs(double a, double b) { return abs_bits(a) < abs_bits(b) ? abs_dbl(a) : abs_dbl(b); }
__device__ inline double neg_dbl(double x) {
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
// Fortran sign(a, b): |a| for b >= 0 (and for b = -0.0), else -|a|.
__device__ inline double fsign(double a, double b) { return is_negative(b) ? neg_dbl(abs_dbl(a)) : abs_dbl(a); }

__device__ inline int init_flag_bit(int run) { return run == 0 ? NECI_FLAG_INITIATOR_1 : NECI_FLAG_INITIATOR_2; }
__device__ inline bool test_bit(long long f, int b) { return ((unsigned long long)f >> b) & 1ull; }
__device__ inline bool is_core_flags(long long f) { return test_bit(f, NECI_FLAG_DETERMINISTIC_1); }

// ---------------------------------------------------------------------------
// Bit strings.
// ---------------------------------------------------------------------------
// The loops over determinant words run over kMaxWords with a guard and are
// unrolled, and a word is picked by orbital through selects, never by a
// run-time index: a determinant copied into a thread's array then stays in
// registers (an array indexed at run time is placed in local memory).
__device__ inline int excit_level(const unsigned long long *a, const unsigned long long *b, int W) {
    int ic = 0;
#pragma unroll
    for (int i = 0; i < kMaxWords; ++i)
        if (i < W) ic += __popcll(a[i] & ~b[i]);
    return ic;
}
__device__ inline bool det_eq(const unsigned long long *a, const long long *b, int W) {
    bool eq = true;
#pragma unroll
    for (int i = 0; i < kMaxWords; ++i)
        if (i < W) eq = eq && (long long)a[i] == b[i];
    return eq;
}
// The word holding orbital orb (1-based).
__device__ inline unsigned long long orb_word(const unsigned long long *d, int orb) {
    const int w = (orb - 1) >> 6;
    unsigned long long r = 0;
#pragma unroll
    for (int k = 0; k < kMaxWords; ++k)
        if (w == k) r = d[k];
    return r;
}
__device__ inline bool orb_occ(const unsigned long long *d, int orb) { return (orb_word(d, orb) >> ((orb - 1) & 63)) & 1ull; }
__device__ inline void flip_orb(unsigned long long *d, int orb) {
    const int w = (orb - 1) >> 6;
    const unsigned long long m = 1ull << ((orb - 1) & 63);
#pragma unroll
    for (int k = 0; k < kMaxWords; ++k)
        if (w == k) d[k] ^= m;
}
// Occupied orbitals strictly between orbitals lo < hi.
__device__ inline int occ_between(const unsigned long long *d, int W, int lo, int hi) {
    int n = 0;
#pragma unroll
    for (int w = 0; w < kMaxWords; ++w) {
        if (w >= W) break;
        const int base = w * 64;  // orbital base+1 is bit 0
        // bits for orbitals lo+1 .. hi-1 -> bit positions lo .. hi-2
        const int b0 = lo - base, b1 = hi - 2 - base;  // inclusive range in this word
        if (b1 < 0 || b0 > 63) continue;
        const int s = b0 < 0 ? 0 : b0, e = b1 > 63 ? 63 : b1;
        if (s > e) continue;
        const unsigned long long mask = (e - s == 63) ? ~0ull : (((1ull << (e - s + 1)) - 1ull) << s);
        n += __popcll(d[w] & mask);
    }
    return n;
}
// Bit position (0-based) of the (k+1)-th set bit of x, k < popcount(x).
__device__ inline int select_bit(unsigned long long x, int k) {
    int pos = 0;
    int t = __popc((unsigned int)x);
    if (k >= t) { k -= t; x >>= 32; pos += 32; }
    t = __popc((unsigned int)(x & 0xFFFFull));
    if (k >= t) { k -= t; x >>= 16; pos += 16; }
    t = __popc((unsigned int)(x & 0xFFull));
    if (k >= t) { k -= t; x >>= 8; pos += 8; }
    t = __popc((unsigned int)(x & 0xFull));
    if (k >= t) { k -= t; x >>= 4; pos += 4; }
    t = __popc((unsigned int)(x & 0x3ull));
    if (k >= t) { k -= t; x >>= 2; pos += 2; }
    t = (int)(x & 1ull);
    if (k >= t) { pos += 1; }
    return pos;
}
// Orbital (1-based) of the n-th (1-based) set bit of (d & pattern), counting
// from orbital 1 upwards: the n-th electron of that spin class in nI order;
// 0 if there are fewer.  The word is found first, so a single bit select
// runs.
__device__ inline int nth_orbital(const unsigned long long *d, int W, unsigned long long pattern, int n) {
    unsigned long long x = 0;
    int wsel = -1;
#pragma unroll
    for (int w = 0; w < kMaxWords; ++w) {
        if (w < W && wsel < 0) {
            const unsigned long long y = d[w] & pattern;
            const int c = __popcll(y);
            if (n <= c) { x = y; wsel = w; }
            else n -= c;
        }
    }
    if (wsel < 0) return 0;
    return wsel * 64 + select_bit(x, n - 1) + 1;
}
constexpr unsigned long long kAllBits = ~0ull;
constexpr unsigned long long kAlphaBits = 0xAAAAAAAAAAAAAAAAull;  // even orbitals
constexpr unsigned long long kBetaBits = 0x5555555555555555ull;   // odd orbitals

// decode_bit_det: ascending occupied orbitals.
__device__ inline int decode(const unsigned long long *d, int W, uint8_t *nI) {
    int n = 0;
#pragma unroll
    for (int w = 0; w < kMaxWords; ++w) {
        if (w >= W) break;
        unsigned long long x = d[w];
        while (x) {
            const int b = __ffsll((long long)x) - 1;
            nI[n++] = (uint8_t)(w * 64 + b + 1);
            x &= x - 1;
        }
    }
    return n;
}

// FindWalkerHash (hash.F90:23-38): full 64-bit value before the modulo.
__device__ inline unsigned long long neci_hash(const unsigned long long *d, int W, const int32_t *rh2) {
    unsigned long long hash = 0;
    int i = 0;
#pragma unroll
    for (int w = 0; w < kMaxWords; ++w) {
        if (w >= W) break;
        unsigned long long x = d[w];
        while (x) {
            const int b = __ffsll((long long)x) - 1;
            const int orb = w * 64 + b + 1;
            ++i;
            const long long term = (long long)(int32_t)(rh2[orb] * i);
            hash = 1099511628211ull * hash + (unsigned long long)term;
            x &= x - 1;
        }
    }
    return hash;
}
// abs(mod(h, n)) with Fortran's sign-of-dividend mod, 0-based.
__device__ inline unsigned long long hash_mod(unsigned long long hash, unsigned long long n) {
    const long long h = (long long)hash;
    const unsigned long long mag = h < 0 ? (0ull - (unsigned long long)h) : (unsigned long long)h;
    return mag % n;
}
// hash_mod for a table length n that is a power of two (the walker hash):
// abs(mod(h, n)) is the magnitude's low bits, with no 64-bit division.
__device__ inline unsigned long long hash_bucket(unsigned long long hash, unsigned long long n) {
    const long long h = (long long)hash;
    const unsigned long long mag = h < 0 ? (0ull - (unsigned long long)h) : (unsigned long long)h;
    return mag & (n - 1);
}

// ---------------------------------------------------------------------------
// Integrals.
// ---------------------------------------------------------------------------
__device__ inline double tmat_el(const DevSys &s, int i, int j) {
    return __ldg(&s.tmat[(size_t)(j - 1) * s.nbasis + (i - 1)]);
}
// UMatInd (UMatCache.F90:257-306) in 32-bit arithmetic: with at most 128
// spatial orbitals (kMaxWords) a pair index is at most 8256 and the result
// at most 34,084,896.
__device__ inline int umat_ind(int I, int J, int K, int L) {
    const int A = I > K ? I * (I - 1) / 2 + K : K * (K - 1) / 2 + I;
    const int B = J > L ? J * (J - 1) / 2 + L : L * (L - 1) / 2 + J;
    return A > B ? A * (A - 1) / 2 + B : B * (B - 1) / 2 + A;
}
__device__ inline double umat_el(const DevSys &s, int i, int j, int k, int l) {
    return __ldg(&s.umat[umat_ind(i, j, k, l) - 1]);
}
__device__ inline int spat(int orb) { return (orb + 1) >> 1; }
__device__ inline bool beta(int orb) { return orb & 1; }

// sltcnd_1_kernel (sltcnd.fpp:643-679): over the occupied k != src in
// ascending order, one add per k of the Coulomb term <ik|ak> or, for k of
// the source's spin, of the precombined <ik|ak> - <ik|ka>; then h_ia.  The
// reference adds all Coulomb terms before subtracting the exchange terms;
// the reassociation moves the element by rounding only.  The terms come from
// the rows of (id1, id2): jrow[k] = <id1 k|id2 k>, jkrow[k] = jrow[k] -
// <id1 k|k id2>.
__device__ inline double sltcnd_1(const DevSys &s, const unsigned long long *d, int src, int tgt) {
    double hel = 0.0;
    const int id1 = spat(src), id2 = spat(tgt);
    if (beta(src) == beta(tgt)) {
        const size_t row = ((size_t)(id1 - 1) * s.nBI + (id2 - 1)) * s.nBI - 1;
        const double *jr = s.jrow + row, *jkr = s.jkrow + row;
        const unsigned long long same = beta(src) ? 0x5555555555555555ull : 0xAAAAAAAAAAAAAAAAull;
        NECI_FOR_WORDS(w, s.W) {
            unsigned long long x = d[w];
            while (x) {
                const int b = __ffsll((long long)x) - 1;
                const int o = w * 64 + b + 1;
                x &= x - 1;
                if (o != src) hel += __ldg(((same >> b) & 1ull) ? &jkr[spat(o)] : &jr[spat(o)]);
            }
        }
    }
    hel += tmat_el(s, src, tgt);
    return hel;
}
// sltcnd_2_kernel (sltcnd.fpp:690-711), ex sorted: i<j, a<b.
__device__ inline double sltcnd_2(const DevSys &s, int i, int j, int a, int b) {
    double hel = 0.0;
    if (beta(i) == beta(a) && beta(j) == beta(b)) hel = umat_el(s, spat(i), spat(j), spat(a), spat(b));
    if (beta(i) == beta(b) && beta(j) == beta(a)) hel -= umat_el(s, spat(i), spat(j), spat(b), spat(a));
    return hel;
}
// sltcnd_0_base (sltcnd.fpp:585-622), same summation order as NECI, taken
// over the occupied bits in ascending order (nI order) instead of a decoded
// nI array: the one-electron sum, then for each electron i the Coulomb sum
// over j > i added to hel_doub, while the exchange terms of the same pairs,
// in the same (i, j) order, go to their own sum.
__device__ inline double sltcnd_0(const DevSys &s, const unsigned long long *d, int W) {
    double hel_sing = 0.0;
    NECI_FOR_WORDS(w, W) {
        unsigned long long x = d[w];
        while (x) {
            const int o = w * 64 + __ffsll((long long)x);
            x &= x - 1;
            hel_sing += tmat_el(s, o, o);
        }
    }
    double hel_doub = 0.0, hel_tmp = 0.0;
    NECI_FOR_WORDS(wi, W) {
        unsigned long long xi = d[wi];
        while (xi) {
            const int oi = wi * 64 + __ffsll((long long)xi);
            xi &= xi - 1;
            double t = 0.0;
            const size_t ri = (size_t)(spat(oi) - 1) * s.nBI - 1;
            NECI_FOR_WORDS(wj, W) {
                if (wj < wi) continue;
                unsigned long long xj = wj == wi ? xi : d[wj];  // the electrons after i
                while (xj) {
                    const int oj = wj * 64 + __ffsll((long long)xj);
                    xj &= xj - 1;
                    t += __ldg(&s.jmat[ri + spat(oj)]);  // <ij|ij>
                    if (beta(oi) == beta(oj)) hel_tmp -= __ldg(&s.kmat[ri + spat(oj)]);  // <ij|ji>
                }
            }
            hel_doub += t;  // the last electron adds t = 0
        }
    }
    return hel_doub + hel_tmp + hel_sing;
}

__device__ inline double diag_helement(const DevSys &s, const unsigned long long *d) {
    if (s.system == NECI_SYS_HUBBARD_REAL_SPACE) {
        // U * number of doubly occupied sites: beta bit 2k and alpha bit 2k+1.
        int n = 0;
        NECI_FOR_WORDS(w, s.W) n += __popcll(d[w] & (d[w] >> 1) & 0x5555555555555555ull);
        return s.uhub * n;
    }
    return sltcnd_0(s, d, s.W) + s.ecore;
}

// <D_a|H|D_b> for a != b, given the excitation level.
__device__ inline double offdiag_helement(const DevSys &s, const unsigned long long *a, const unsigned long long *b, int ic) {
    if (ic == 1) {
        int src = 0, tgt = 0;
        NECI_FOR_WORDS(w, s.W) {
            const unsigned long long x = a[w] & ~b[w], y = b[w] & ~a[w];
            if (x) src = w * 64 + __ffsll((long long)x);
            if (y) tgt = w * 64 + __ffsll((long long)y);
        }
        const int lo = src < tgt ? src : tgt, hi = src < tgt ? tgt : src;
        const bool par = occ_between(a, s.W, lo, hi) & 1;
        double hel = (s.system == NECI_SYS_HUBBARD_REAL_SPACE) ? tmat_el(s, src, tgt) : sltcnd_1(s, a, src, tgt);
        return par ? -hel : hel;
    }
    if (ic == 2 && s.system == NECI_SYS_MOLECULAR) {
        int src[2], tgt[2], ns = 0, nt = 0;
        NECI_FOR_WORDS(w, s.W) {
            unsigned long long x = a[w] & ~b[w], y = b[w] & ~a[w];
            while (x) { src[ns++] = w * 64 + __ffsll((long long)x); x &= x - 1; }
            while (y) { tgt[nt++] = w * 64 + __ffsll((long long)y); y &= y - 1; }
        }
        // parity of i->a then j->b (sorted pairing), as successive singles
        unsigned long long t[kMaxWords];
        NECI_FOR_WORDS(w, s.W) t[w] = a[w];
        int lo = min(src[0], tgt[0]), hi = max(src[0], tgt[0]);
        int np = occ_between(t, s.W, lo, hi);
        flip_orb(t, src[0]);
        flip_orb(t, tgt[0]);
        lo = min(src[1], tgt[1]);
        hi = max(src[1], tgt[1]);
        np += occ_between(t, s.W, lo, hi);
        const double hel = sltcnd_2(s, src[0], src[1], tgt[0], tgt[1]);
        return (np & 1) ? -hel : hel;
    }
    return 0.0;
}

}  // namespace neci
