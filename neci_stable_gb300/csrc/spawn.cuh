// spawn.cuh -- the spawn attempts of a step (FciMCPar.F90:1600-1745,
// loop_over_walkers): generate_excitation, attempt_create and
// create_particle for every attempt entry the sweep wrote, one attempt per
// thread per round.  Instantiated per precision of the amplitude (one
// translation unit each: spawn_fp64.cu, spawn_fp32.cu), excitation generator
// and number of determinant words.
#pragma once

#include "common.cuh"
#include "excitgen.cuh"
#include "internal.h"

namespace neci {

// ===========================================================================
// k_spawn
// ===========================================================================
template <typename Real>
__device__ inline Real prm(double d, float f) { return sizeof(Real) == 8 ? (Real)d : (Real)f; }

// attempt_create_normal (fcimc_pointed_fns.F90:178-494) for one generated
// excitation: the child amplitude -tau H_ij sign(C) / (p_gen AvMCExcits),
// taken as -tau H_ij sign(C) (1/p_gen) (1/AvMCExcits) in precision Real and
// converted to fixed point, then rounded there in integer arithmetic:
// RealSpawnCutoff rounding (|n| < cutoff -> +-cutoff with probability
// |n|/cutoff) or stochastic_round (lib/util_mod.fpp:182) to an integer
// walker.  Returns 0 for no child.
// In FP64 the product is formed as ((tau H_ij) (1/p_gen)) (1/AvMCExcits)
// and its sign applied afterwards: multiplying by -1, by the walker sign and
// by 1/AvMCExcits = 1 are exact, so the value is the reference order's, with
// two multiplies where it has five; the scaling by 2^32 and the rounding to
// an integer are done on the bits (fixed32_from_double).
template <typename Real>
__device__ inline long long spawn_amplitude(const IterParams &p, Real hel, Real invp, bool neg, Stream &rng, int &ovf,
                                            unsigned long long &aq_out) {
    long long q;
    if (sizeof(Real) == 8) {
        double v = (p.tau * (double)hel) * (double)invp;
        if (!p.av_unit) v = v * p.inv_av;
        int64_t qq;
        if (!fixed32_from_double(v, qq)) { ovf = 1; return 0; }
        q = neg ? qq : -qq;  // -tau H sign(C): positive for a negative parent
    } else {
        const Real ww = neg ? (Real)-1 : (Real)1;
        const Real nsp = -prm<Real>(p.tau, p.f_tau) * hel * ww * invp * prm<Real>(p.inv_av, p.f_inv_av);
        const float sc = (float)nsp * 4294967296.0f;
        if (!(fabsf(sc) < 9.2e18f)) { ovf = 1; return 0; }
        q = __float2ll_rn(sc);
    }
    const unsigned long long aq = (unsigned long long)(q < 0 ? -q : q);
    aq_out = aq;
    if (p.t_all_real_coeff) {
        if (p.t_real_spawn_cutoff && aq < p.cutoff_q) {
            // keep with probability |q| / cutoff_q
            const bool keep = __umul64hi(rng.next64(), p.cutoff_q) < aq;
            return keep ? (q < 0 ? -(long long)p.cutoff_q : (long long)p.cutoff_q) : 0ll;
        }
        return q;
    }
    const unsigned long long whole = aq >> 32, frac = aq & 0xFFFFFFFFull;
    unsigned long long m = whole;
    if (frac != 0 && (rng.next64() >> 32) < frac) m += 1;
    const long long v = (long long)(m << 32);
    return q < 0 ? -v : v;
}

// One spawn attempt's parent, unpacked from its 8-byte attempt entry
// (slot | run << 32 | sign bit << 33 | attempt index << 34).
struct Parent {
    unsigned long long d[kMaxWords];
    unsigned long long key;
    unsigned int k;
    int run;
    bool neg, core, pinit;
};
// Words of a CurrentDets row (NIfD + 1): RW where the kernel is instantiated
// for that count, else the system's W.
template <int RW>
__device__ inline int rwords(const DevSys &s) { return RW > 0 ? RW : s.W; }

template <int NW, int RW>
__device__ inline void load_parent(const DevSys &s, const DevState &st, const IterParams &p, unsigned long long w0,
                                   Parent &P) {
    const long long j = (long long)(w0 & 0xFFFFFFFFull);
    P.run = (int)((w0 >> 32) & 1ull);
    P.neg = (w0 >> 33) & 1ull;
    P.k = (unsigned int)(w0 >> 34);
    const long long *r = st.dets + j * s.R;
    NECI_FOR_WORDS(w, nwords<NW>(s)) P.d[w] = (unsigned long long)r[w];
    const long long flags = r[rwords<RW>(s) + s.L];
    P.core = st.n_core > 0 && is_core_flags(flags);
    P.pinit = p.t_trunc_initiator && test_bit(flags, init_flag_bit(P.run));
    // det_key of the row (the words past NW are zero), which the sweep
    // stored for every slot with attempts
    P.key = st.dkey[j];
}

// The stream of an attempt from its entry alone: what the classification of
// an attempt (single or double) needs, without the parent's row.
__device__ inline Stream attempt_stream(const DevState &st, const IterParams &p, unsigned long long w0) {
    const long long j = (long long)(w0 & 0xFFFFFFFFull);
    return Stream(st.dkey[j], p.iter, P_ATTEMPT, (uint32_t)((w0 >> 32) & 1ull), (uint32_t)(w0 >> 34));
}

// Block-local tau-search log of k_spawn: per TauClass the largest gamma (as
// bits) and the logged count, capped near the reference's threshold.
struct TauAcc {
    unsigned long long g[4];
    unsigned int c[4];
};

// log_spawn_magnitude (tau_search_conventional.F90:138-258): gamma =
// |H_ij| / (p_gen / p_class) of one generated excitation, taken as
// |H_ij| (1/p_gen) p_class in precision Real.  Singles and uniform doubles
// count when gamma > 0, parallel and opposite-spin doubles always.
template <typename Real>
__device__ inline void tau_log(const DevSys &s, const Excit<Real> &e, TauAcc *acc) {
    double g;
    if (sizeof(Real) == 8) g = fabs((double)e.hel) * (double)e.invp * s.tau_fac[e.cls];
    else g = (double)(fabsf((float)e.hel) * (float)e.invp * s.f_tau_fac[e.cls]);
    const unsigned long long b = (unsigned long long)__double_as_longlong(g);
    if (b > acc->g[e.cls]) atomicMax(&acc->g[e.cls], b);
    const bool counts = (e.cls == TC_PAR || e.cls == TC_OPP) || g > 0.0;
    if (counts && acc->c[e.cls] <= kTauCntThreshold) atomicAdd(&acc->c[e.cls], 1u);
}

// attempt_create for a generated excitation: the core -> core filter
// (is_core_state, semi_stoch_procs.F90:547; those spawns are done by the
// deterministic projection), the tau-search log and the rounded fixed-point
// amplitude.
template <typename Real, int NW, int RW>
__device__ inline long long attempt_create(const DevSys &s, const DevState &st, const IterParams &p, const Parent &P,
                                           Excit<Real> &e, Stream &rng, const int32_t *sh_rh2, int &ovf,
                                           TauAcc *tacc) {
    if (!e.ok) return 0;
    if (P.core) {
        const long long hs = hash_find(st, e.child, nwords<NW>(s), s.R, neci_hash(e.child, nwords<NW>(s), sh_rh2), st.ctl);
        if (hs >= 0 && is_core_flags(st.dets[hs * s.R + rwords<RW>(s) + s.L])) return 0;
    }
    if (s.tau_search) tau_log<Real>(s, e, tacc);
    return spawn_amplitude<Real>(p, e.hel, e.invp, P.neg, rng, ovf, e.aq);
}

// The unbiasing weight of a spawn's parent for the 2-RDM (the role of
// calc_rdmbiasfac, rdm_general.fpp:1039-1085, for a per-spawn estimator):
// the expected number of non-zero spawns onto a child per attempt is
// p_gen P(nz), where P(nz) is min(1, |n| / RealSpawnCutoff) with real
// coefficients and the cutoff, min(1, |n|) with integer walkers, and 1
// otherwise; the attempts number |C_i| AvMCExcits on average, so
// sign(C_i) / (AvMCExcits p_gen P(nz)) has expectation C_i per child.
// aq is |n| in fixed point before rounding.
__device__ inline double rdm_parent_weight(const IterParams &p, double invp, unsigned long long aq, bool neg) {
    double inv_pnz = 1.0;
    if (p.t_all_real_coeff) {
        if (p.t_real_spawn_cutoff && aq < p.cutoff_q) inv_pnz = (double)p.cutoff_q / (double)aq;
    } else if (aq < (1ull << 32)) {
        inv_pnz = 4294967296.0 / (double)aq;
    }
    const double w = (invp * p.inv_av) * inv_pnz;
    return neg ? -w : w;
}

// The block's sums of the spawns it created, in shared memory: their number
// and sum of |amplitude| per run (n_spawned and abs_q of the step).  Kept out
// of registers, which the spawn loop is short of.
struct SpawnSums {
    unsigned long long *sh;  // [3]: number, |amplitude| of run 0, of run 1
};

// create_particle (fcimc_helper.F90:152-308) with pass 1 of the
// annihilation done at once: the child is looked up in the walker hash
// (hash_table_lookup); one that is occupied takes the found branch of
// AnnihilateSpawnedParts (Annihilation.F90:1000-1140), its fixed-point
// amplitude, record count and initiator bit added to the slot's spawn sums
// (acc, meta), while an absent child becomes a candidate record of the
// compression pass.  The sums are integer atomics, so the order of the spawns
// does not matter.  Done when `fused` (chosen by the host where spawns are
// frequent enough to fill the lookup's lanes, and never with 2-RDM sampling,
// which needs every record and its parent); otherwise every spawn is written
// and pass 1 runs as its own kernel.  Warp-wide (the appends).
template <typename Real, int NW, int RW>
__device__ inline void create_particle(const DevSys &s, const DevState &st, const IterParams &p, long long qv,
                                       const Parent &P, const Excit<Real> &e, const int32_t *sh_rh2, const SpawnSums &ss,
                                       bool fused) {
    long long slot = -1;
    unsigned long long h = 0;
    if (qv != 0 && fused) {
        h = neci_hash(e.child, nwords<NW>(s), sh_rh2);
        slot = hash_find(st, e.child, nwords<NW>(s), s.R, h, st.ctl);
        atomicAdd(&ss.sh[0], 1ull);
        atomicAdd(&ss.sh[1 + P.run], (unsigned long long)(qv < 0 ? -qv : qv));
    }
    if (fused && qv != 0 && slot >= 0) {
        const long long j = slot * s.L + P.run;
        atomicAdd((unsigned long long *)&st.acc[j], (unsigned long long)qv);
        atomicAdd(&st.meta[j], 1u);
        if (P.pinit) atomicOr(&st.meta[j], 0x80000000u);
    }
    const bool rec = qv != 0 && (!fused || slot < 0);
    const unsigned long long pos = warp_append1(fused ? &st.ctl->n_cand : &st.ctl->n_spawned, rec);
    if (!rec) return;
    if (pos >= (unsigned long long)st.max_spawned) {
        set_err(st.ctl, NECI_GPU_ERR_SPAWN_FULL);
        return;
    }
    long long *o = st.spawn + pos * s.R;
    NECI_FOR_WORDS(w, rwords<RW>(s)) o[w] = w < nwords<NW>(s) ? (long long)e.child[w] : 0ll;
    for (int k2 = 0; k2 < s.L; ++k2) o[rwords<RW>(s) + k2] = (k2 == P.run) ? qv : 0ll;
    o[rwords<RW>(s) + s.L] = P.pinit ? (1ll << init_flag_bit(P.run)) : 0ll;
    if (fused) {
        st.cand[pos] = (uint32_t)pos;
        st.cand_h[pos] = h;
        return;
    }
    if (!s.rdm) return;
    // the parent and its unbiased sign for the 2-RDM: sign(C_i) divided
    // by the expected number of non-zero spawns onto this child per unit
    // of |C_i|, AvMCExcits p_gen P(spawn != 0)
    long long *par = st.spawn_par + pos * (rwords<RW>(s) + 1);
    NECI_FOR_WORDS(w, rwords<RW>(s)) par[w] = w < nwords<NW>(s) ? (long long)P.d[w] : 0ll;
    par[rwords<RW>(s)] = double_to_word(rdm_parent_weight(p, (double)e.invp, e.aq, P.neg));
}

// One attempt of class CLS (0: double, 1: single) whose parent and stream
// are loaded: the stream stands after its first draw (the singles/doubles
// choice), so the draws are those of the attempt processed inline.
template <typename Real, int GEN, int CLS, int NW, int RW>
__device__ inline void spawn_class(const DevSys &s, const DevState &st, const IterParams &p, bool valid,
                                   const Parent &P, Stream &rng, const int32_t *sh_rh2, int &ovf, TauAcc *tacc,
                                   const SpawnSums &ss, bool fused) {
    Excit<Real> e;
    e.ok = false;
    long long qv = 0;
    if (valid) {
        if (CLS == 1) gen_uniform_single<Real, NW>(s, P.d, rng, e);
        else if (GEN == NECI_EXGEN_UNIFORM) gen_uniform_double<Real, NW>(s, P.d, rng, e);
        else gen_pchb_double<Real, NW>(s, P.d, rng, e);
        qv = attempt_create<Real, NW, RW>(s, st, p, P, e, rng, sh_rh2, ovf, tacc);
    }
    create_particle<Real, NW, RW>(s, st, p, qv, P, e, sh_rh2, ss, fused);
}

// The parent and stream of a queued attempt: the stream resumes after its
// first draw from the saved second draw.
template <int NW, int RW>
__device__ inline Stream load_queued(const DevSys &s, const DevState &st, const IterParams &p, bool valid,
                                     unsigned long long w0, unsigned long long r1, Parent &P) {
    P.run = 0;
    P.pinit = false;
    P.key = 0;
    P.k = 0;
    if (valid) load_parent<NW, RW>(s, st, p, w0, P);
    Stream rng(P.key, p.iter, P_ATTEMPT, P.run, P.k);
    rng.resume_second(r1);
    return rng;
}

// The spawn attempts (FciMCPar.F90:1600-1745, loop_over_walkers), one
// attempt entry per thread per round; every lane runs the same number of
// rounds, so the record append is warp-wide.  Molecular systems queue their
// attempts by class (single or double) in shared memory and process full
// batches with all lanes: with QD (both classes common, chosen by the host
// from pSingles) both classes are queued; without it the doubles are
// generated at once and only the singles are queued.  Lattice systems
// (singles only) generate every attempt at once.
//
// NW is the number of words that can hold orbitals, ceil(nBasis/64), and RW
// the row's W = nBasis/64 + 1 words (NIfD + 1): one more, always zero, when
// nBasis is a multiple of 64.  Excitations are generated on NW words; the
// determinant key, the records and the row offsets use all RW.  NW = RW = 0
// is the instance for any size, with the counts read from the system.
// Resident blocks of 128 threads per SM the spawn kernel is compiled for:
// its register cap is 65536 / (128 x this).
#ifndef NECI_SPAWN_BLOCKS_PER_SM
#define NECI_SPAWN_BLOCKS_PER_SM 8
#endif

template <typename Real, int GEN, int NW, int RW, bool QD>
__global__ void __launch_bounds__(128, NECI_SPAWN_BLOCKS_PER_SM)
    k_spawn(DevSys s, DevState st, const IterParams *pp, int fuse_probe) {
    if (halted(st)) return;
    // lattice systems only: their singles spawn often enough to fill the
    // lookup's lanes; the molecular instances carry no fused code
    const bool fused = GEN == NECI_EXGEN_RS_HUBBARD && fuse_probe != 0 && !s.rdm;
    extern __shared__ int32_t sh[];
    // per class: attempt entries and their second draws (at most two
    // rounds' worth are held), and each warp's appends of the round (by
    // round parity)
    __shared__ unsigned long long sq[2][256], sr1[2][256];
    __shared__ int wcnt[2][2][4];
    __shared__ unsigned int ring_tail;
    __shared__ unsigned long long sh_sums[3];
    __shared__ TauAcc tacc;
    int32_t *sh_rh2 = sh;
    int32_t *sh_neigh = sh + (s.nbasis + 1);
    for (int i = threadIdx.x; i <= s.nbasis; i += blockDim.x) sh_rh2[i] = s.random_hash2[i];
    if (GEN == NECI_EXGEN_RS_HUBBARD)
        for (int i = threadIdx.x; i < s.nsites * s.max_neigh; i += blockDim.x) sh_neigh[i] = s.neighbours[i];
    if (threadIdx.x < 4) {
        tacc.g[threadIdx.x] = 0ull;
        tacc.c[threadIdx.x] = 0u;
    }
    if (threadIdx.x == 0) ring_tail = 0u;
    if (threadIdx.x < 3) sh_sums[threadIdx.x] = 0ull;
    __syncthreads();
    const IterParams p = *pp;
    const long long nat = (long long)min(st.ctl->n_att, (unsigned long long)st.max_att);
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nround = ((nat + stride - 1) / stride) * stride;
    const int nb = blockDim.x;  // 128: four warps
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int qn[2] = {0, 0};  // queue lengths, the same in every thread
    int ovf = 0;
    const SpawnSums ss = {sh_sums};
    if (GEN == NECI_EXGEN_RS_HUBBARD) {
        // lattice systems (singles only): one attempt per thread per round
        for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nround; q += stride) {
            long long qv = 0;
            Parent P;
            P.run = 0;
            P.pinit = false;
            Excit<Real> e;
            e.ok = false;
            if (q < nat) {
                load_parent<NW, RW>(s, st, p, st.att[q], P);
                Stream rng(P.key, p.iter, P_ATTEMPT, P.run, P.k);
                gen_rs_hubbard<Real, NW>(s, P.d, sh_neigh, rng, e);
                qv = attempt_create<Real, NW, RW>(s, st, p, P, e, rng, sh_rh2, ovf, &tacc);
            }
            create_particle<Real, NW, RW>(s, st, p, qv, P, e, sh_rh2, ss, fused);
        }
    }
    // Molecular systems without QD (singles rare or dominant): a round
    // classifies one attempt per thread (gen_exc_sd: r < pSingles is a
    // single; gen_rand_excit: r < pDoubles is a double), generates a double
    // at once, inline, and appends a single to a ring of 512 entries.  The
    // ring's tail only grows (shared atomics); the round's barrier is a
    // __syncthreads_count, which gives every thread the round's appends, so
    // the queue length and head are kept in registers, the same in every
    // thread.  A full batch (or after the last attempt what is left) is read
    // at once and processed: the next round's appends land at least 128 and
    // less than 512 entries past the head, never on an entry being read.
    if (GEN != NECI_EXGEN_RS_HUBBARD && !QD) {
        unsigned long long *ring = &sq[0][0], *ring_r1 = &sr1[0][0];  // 512 entries each
        unsigned int head = 0;
        int cnt = 0;
        long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        for (;; q += stride) {
            const bool more = q - threadIdx.x < nround;  // the same in the whole block
            if (!more && cnt == 0) break;
            bool single = false;
            unsigned long long w0 = 0, r1 = 0;
            if (more) {
                Parent P;
                P.run = 0;
                P.pinit = false;
                Excit<Real> e;
                e.ok = false;
                long long qv = 0;
                if (q < nat) {
                    w0 = st.att[q];
                    load_parent<NW, RW>(s, st, p, w0, P);
                    Stream rng(P.key, p.iter, P_ATTEMPT, P.run, P.k);
                    const unsigned long long r0 = rng.next64();
                    single = GEN == NECI_EXGEN_UNIFORM ? !(r0 < s.thr_doubles) : r0 < s.thr_singles;
                    if (single) {
                        r1 = rng.next64();
                    } else {
                        if (GEN == NECI_EXGEN_UNIFORM) gen_uniform_double<Real, NW>(s, P.d, rng, e);
                        else gen_pchb_double<Real, NW>(s, P.d, rng, e);
                        qv = attempt_create<Real, NW, RW>(s, st, p, P, e, rng, sh_rh2, ovf, &tacc);
                    }
                }
                create_particle<Real, NW, RW>(s, st, p, qv, P, e, sh_rh2, ss, fused);
            }
            if (single) {
                const unsigned int t = atomicAdd(&ring_tail, 1u) & 511u;
                ring[t] = w0;
                ring_r1[t] = r1;
            }
            cnt += __syncthreads_count(single);
            const int take = cnt >= nb ? nb : (more ? 0 : cnt);
            if (take) {
                const bool v = (int)threadIdx.x < take;
                const unsigned int i = (head + threadIdx.x) & 511u;
                const unsigned long long a = v ? ring[i] : 0ull, b = v ? ring_r1[i] : 0ull;
                head += (unsigned int)take;
                cnt -= take;
                Parent P;
                Stream rng = load_queued<NW, RW>(s, st, p, v, a, b, P);
                spawn_class<Real, GEN, 1, NW, RW>(s, st, p, v, P, rng, sh_rh2, ovf, &tacc, ss, fused);
            }
        }
    }
    // Molecular systems with QD (both classes common): a round classifies
    // one attempt per thread and queues it by class; full batches of a queue
    // are processed with all lanes, so neither class idles the lanes of the
    // other (half of them after the tau search raises pSingles near 1/2).
    // In the rounds after the last attempt the queues are emptied.  Each
    // class is processed by one call site, so its generator is compiled once.
    //
    // Queue appends: each warp posts its counts per class; after one barrier
    // every thread derives the same queue lengths and its own slot, so no
    // shared counter is read and written in the same round.  A round that
    // drains takes a second barrier (its entries visible) and reads its
    // entries at once; the next round writes only after its own first
    // barrier, by which time every thread has read them.
    if (GEN != NECI_EXGEN_RS_HUBBARD && QD) {
        long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        for (int round = 0;; ++round, q += stride) {
            const bool more = q - threadIdx.x < nround;  // the same in the whole block
            if (!more && qn[0] == 0 && qn[1] == 0) break;
            const bool valid = more && q < nat;
            int cls = 0;
            unsigned long long w0 = 0, r1 = 0;
            if (valid) {
                w0 = st.att[q];
                Stream rng = attempt_stream(st, p, w0);
                const unsigned long long r0 = rng.next64();
                r1 = rng.next64();
                cls = (GEN == NECI_EXGEN_UNIFORM ? !(r0 < s.thr_doubles) : r0 < s.thr_singles) ? 1 : 0;
            }
            const bool queued = valid;
            unsigned int m[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                m[c] = __ballot_sync(0xffffffffu, queued && cls == c);
                if (lane == 0) wcnt[round & 1][c][wid] = __popc(m[c]);
            }
            __syncthreads();
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                int before = 0, total = 0;
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    const int x = wcnt[round & 1][c][w];
                    before += w < wid ? x : 0;
                    total += x;
                }
                if (queued && cls == c) {
                    const int pos = qn[c] + before + __popc(m[c] & ((1u << lane) - 1u));
                    sq[c][pos] = w0;
                    sr1[c][pos] = r1;
                }
                qn[c] += total;
            }
            // a full batch, or after the last attempt what is left
            const int t0 = qn[0] >= nb ? nb : (more ? 0 : qn[0]);
            const int t1 = qn[1] >= nb ? nb : (more ? 0 : qn[1]);
            if (t0 || t1) {
                __syncthreads();
                bool v0 = false, v1 = false;
                unsigned long long a0 = 0, b0 = 0, a1 = 0, b1 = 0;
                if (t0) {
                    qn[0] -= t0;
                    v0 = (int)threadIdx.x < t0;
                    if (v0) {
                        a0 = sq[0][qn[0] + threadIdx.x];
                        b0 = sr1[0][qn[0] + threadIdx.x];
                    }
                }
                if (t1) {
                    qn[1] -= t1;
                    v1 = (int)threadIdx.x < t1;
                    if (v1) {
                        a1 = sq[1][qn[1] + threadIdx.x];
                        b1 = sr1[1][qn[1] + threadIdx.x];
                    }
                }
                if (t0) {
                    Parent P;
                    Stream rng = load_queued<NW, RW>(s, st, p, v0, a0, b0, P);
                    spawn_class<Real, GEN, 0, NW, RW>(s, st, p, v0, P, rng, sh_rh2, ovf, &tacc, ss, fused);
                }
                if (t1) {
                    Parent P;
                    Stream rng = load_queued<NW, RW>(s, st, p, v1, a1, b1, P);
                    spawn_class<Real, GEN, 1, NW, RW>(s, st, p, v1, P, rng, sh_rh2, ovf, &tacc, ss, fused);
                }
            }
        }
    }
    if (ovf) set_err(st.ctl, NECI_GPU_ERR_OVERFLOW);
    // n_spawned and abs_q of the spawns created here (with 2-RDM sampling
    // pass 1 counts them)
    __syncthreads();
    if (threadIdx.x == 0) {
        if (sh_sums[0]) atomicAdd(&st.ctl->n_spawned, sh_sums[0]);
        if (sh_sums[1]) atomicAdd(&st.ctl->abs_q[0], sh_sums[1]);
        if (sh_sums[2]) atomicAdd(&st.ctl->abs_q[1], sh_sums[2]);
    }
    if (s.tau_search) {
        __syncthreads();
        if (threadIdx.x < 4) {
            if (tacc.g[threadIdx.x]) atomicMax(&st.ctl->tau_gamma[threadIdx.x], tacc.g[threadIdx.x]);
            if (tacc.c[threadIdx.x]) atomicAdd(&st.ctl->tau_cnt[threadIdx.x], (unsigned long long)tacc.c[threadIdx.x]);
        }
    }
}

// Grids are sized to the context's capacity (as in kernels.cu).
// The grid fills spawn_occ blocks per SM (8, the launch bound, unless tuned).
inline int spawn_grid(const Engine &e, int threads) {
    const long long want = e.st.max_spawned / (threads * 4) + 1, hi = (long long)e.num_sms * e.spawn_occ;
    return (int)(want < 8 ? 8 : (want > hi ? hi : want));
}

// Doubles are queued like singles when both classes are common: the
// fraction of singles between 0.15 and 0.85 (on GB300, at 0.53 queueing
// both made the spawn kernel 17% faster; with rare singles it is slower).
inline int spawn_queue_doubles(const DevSys &s) {
    const double ps = s.excitgen == NECI_EXGEN_UNIFORM ? 1.0 - s.p_doubles : s.p_singles;
    return ps >= 0.15 && ps <= 0.85 ? 1 : 0;
}

template <typename Real, int GEN, bool QD>
void launch_spawn_words(Engine &e, cudaStream_t s, int grid, size_t shm) {
    const int rw = e.sys.W, nw = (e.sys.nbasis + 63) / 64;
    if (rw == 1) k_spawn<Real, GEN, 1, 1, QD><<<grid, 128, shm, s>>>(e.sys, e.st, e.d_params, fused_lookup(e) ? 1 : 0);
    else if (rw == 2 && nw == 1) k_spawn<Real, GEN, 1, 2, QD><<<grid, 128, shm, s>>>(e.sys, e.st, e.d_params, fused_lookup(e) ? 1 : 0);
    else if (rw == 2) k_spawn<Real, GEN, 2, 2, QD><<<grid, 128, shm, s>>>(e.sys, e.st, e.d_params, fused_lookup(e) ? 1 : 0);
    else if (rw == 3 && nw == 2) k_spawn<Real, GEN, 2, 3, QD><<<grid, 128, shm, s>>>(e.sys, e.st, e.d_params, fused_lookup(e) ? 1 : 0);
    else if (rw == 3) k_spawn<Real, GEN, 3, 3, QD><<<grid, 128, shm, s>>>(e.sys, e.st, e.d_params, fused_lookup(e) ? 1 : 0);
    else k_spawn<Real, GEN, 0, 0, QD><<<grid, 128, shm, s>>>(e.sys, e.st, e.d_params, fused_lookup(e) ? 1 : 0);
}

template <typename Real, int GEN>
void launch_spawn_gen(Engine &e, cudaStream_t s, int grid, size_t shm) {
    if (GEN != NECI_EXGEN_RS_HUBBARD && spawn_queue_doubles(e.sys)) launch_spawn_words<Real, GEN, true>(e, s, grid, shm);
    else launch_spawn_words<Real, GEN, false>(e, s, grid, shm);
}

// The spawn kernel for amplitudes in precision Real.
template <typename Real>
void launch_spawn_real(Engine &e, cudaStream_t s) {
    const size_t shm = (size_t)(e.sys.nbasis + 1 + e.sys.nsites * e.sys.max_neigh) * sizeof(int32_t);
    const int grid = spawn_grid(e, 128);
    if (e.sys.excitgen == NECI_EXGEN_RS_HUBBARD) launch_spawn_gen<Real, NECI_EXGEN_RS_HUBBARD>(e, s, grid, shm);
    else if (e.sys.excitgen == NECI_EXGEN_UNIFORM) launch_spawn_gen<Real, NECI_EXGEN_UNIFORM>(e, s, grid, shm);
    else launch_spawn_gen<Real, NECI_EXGEN_PCHB>(e, s, grid, shm);
}

}  // namespace neci
