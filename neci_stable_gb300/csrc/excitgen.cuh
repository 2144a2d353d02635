// excitgen.cuh -- device excitation generators (generate_excitation,
// proc_ptrs.F90:13) in bit-string form, templated on the precision of the
// generation probability and matrix element (double: the FP64 path; float:
// the mixed-precision spawn amplitudes).
//
// Random draws are consumed as 64-bit integers: int(n*r) becomes
// uniform_index(n) (multiply-high), r < p becomes a threshold test; the
// sampled distributions and the returned p_gen are those of NECI's routines,
// with the constant divisions of p_gen hoisted out of the attempt.  GB300
// executes FP64 at about 1/128 of the FP32 rate, so the sampling itself carries no
// FP64 arithmetic.
#pragma once

#include "engine.cuh"

namespace neci {

template <typename Real>
struct Excit {
    unsigned long long child[kMaxWords];
    Real pgen;
    Real invp;  // 1/pgen as a product of reciprocal factors
    Real hel;
    int ic;
    int cls;  // TauClass
    bool ok;
    unsigned long long aq;  // |amplitude| in fixed point before rounding (2-RDM unbiasing)
};

// Words of a determinant: NW where a kernel is instantiated for that count
// (its loops then have fixed trip counts and unused words need no
// registers), else the system's W.
template <int NW>
__device__ inline int nwords(const DevSys &s) { return NW > 0 ? NW : s.W; }

template <typename Real>
__device__ inline Real tmat_r(const DevSys &s, int i, int j);
template <>
__device__ inline double tmat_r<double>(const DevSys &s, int i, int j) { return tmat_el(s, i, j); }
template <>
__device__ inline float tmat_r<float>(const DevSys &s, int i, int j) {
    return __ldg(&s.tmat32[(size_t)(j - 1) * s.nbasis + (i - 1)]);
}
template <typename Real>
__device__ inline Real umat_r(const DevSys &s, int i, int j, int k, int l);
template <>
__device__ inline double umat_r<double>(const DevSys &s, int i, int j, int k, int l) { return umat_el(s, i, j, k, l); }
template <>
__device__ inline float umat_r<float>(const DevSys &s, int i, int j, int k, int l) {
    return __ldg(&s.umat32[umat_ind(i, j, k, l) - 1]);
}

// sltcnd_1_kernel (sltcnd.fpp:643-679) in precision Real, summed as the
// FP64 form (one add per occupied k of jrow[k] or, same spin, jkrow[k]).
template <typename Real, int NW = 0>
__device__ inline Real sltcnd_1_r(const DevSys &s, const unsigned long long *d, int src, int tgt) {
    Real hel = 0;
    const int id1 = spat(src), id2 = spat(tgt);
    if (beta(src) == beta(tgt)) {
        const size_t row = ((size_t)(id1 - 1) * s.nBI + (id2 - 1)) * s.nBI - 1;
        const Real *jr = (sizeof(Real) == 8 ? (const Real *)s.jrow : (const Real *)s.jrow32) + row;
        const Real *jkr = (sizeof(Real) == 8 ? (const Real *)s.jkrow : (const Real *)s.jkrow32) + row;
        const unsigned long long same = beta(src) ? kBetaBits : kAlphaBits;
        // The occupied k other than src in increasing order, four loads in
        // flight at a time and added in that order.
        NECI_FOR_WORDS(w, nwords<NW>(s)) {
            unsigned long long x = d[w];
            if (((src - 1) >> 6) == w) x &= ~(1ull << ((src - 1) & 63));
            while (x) {
                Real v[4];
                bool have[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    have[u] = x != 0ull;
                    v[u] = 0;
                    if (have[u]) {
                        const int b = __ffsll((long long)x) - 1;
                        x &= x - 1;
                        v[u] = __ldg(((same >> b) & 1ull) ? &jkr[spat(w * 64 + b + 1)] : &jr[spat(w * 64 + b + 1)]);
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (have[u]) hel += v[u];
            }
        }
    }
    hel += tmat_r<Real>(s, src, tgt);
    return hel;
}
// sltcnd_2_kernel (sltcnd.fpp:690-711), ex sorted: i<j, a<b.
template <typename Real>
__device__ inline Real sltcnd_2_r(const DevSys &s, int i, int j, int a, int b) {
    Real hel = 0;
    if (beta(i) == beta(a) && beta(j) == beta(b)) hel = umat_r<Real>(s, spat(i), spat(j), spat(a), spat(b));
    if (beta(i) == beta(b) && beta(j) == beta(a)) hel -= umat_r<Real>(s, spat(i), spat(j), spat(b), spat(a));
    return hel;
}

// Child determinant and H_ij of a single src -> tgt.
template <typename Real, int NW = 0>
__device__ inline void finish_single(const DevSys &s, const unsigned long long *d, int src, int tgt, Excit<Real> &e) {
    NECI_FOR_WORDS(w, nwords<NW>(s)) e.child[w] = d[w];
    flip_orb(e.child, src);
    flip_orb(e.child, tgt);
    const int lo = min(src, tgt), hi = max(src, tgt);
    const bool par = occ_between(d, nwords<NW>(s), lo, hi) & 1;  // make_single tParity
    const Real hel = (s.system == NECI_SYS_HUBBARD_REAL_SPACE) ? tmat_r<Real>(s, src, tgt) : sltcnd_1_r<Real, NW>(s, d, src, tgt);
    e.hel = par ? -hel : hel;
}

// gen_excit_rs_hubbard (real_space_hubbard.F90:1938-2030),
// create_cum_list_rs_hubbard (:2080) and pick_from_cum_list
// (lattice_models_utils.F90:150).  The cumulative pick stays in FP64.
template <typename Real, int NW = 0>
__device__ inline void gen_rs_hubbard(const DevSys &s, const unsigned long long *d,
                                      const int32_t *neigh, Stream &rng, Excit<Real> &e) {
    e.ic = 1;
    e.cls = TC_SING;
    e.ok = false;
    const int elec = 1 + (int)uniform_index(rng, (unsigned)s.nel);
    const int src = nth_orbital(d, nwords<NW>(s), kAllBits, elec);  // nI(elec)
    const int site = spat(src);
    const int32_t *nb = neigh + (site - 1) * s.max_neigh;
    // The cumulative list is walked twice (its total, then the pick) instead
    // of being stored: the running sums are the same additions in the same
    // order, so the pick and its probability are those of the stored list.
    double cum_sum = 0.0;
    for (int k = 0; k < s.max_neigh; ++k) {
        const int n = nb[k];
        if (n <= 0) continue;
        const int orb = beta(src) ? 2 * n - 1 : 2 * n;
        cum_sum += orb_occ(d, orb) ? 0.0 : fabs(tmat_el(s, src, orb));
    }
    if (cum_sum < 1e-10) { e.pgen = 0; return; }
    const double r = rng.next() * cum_sum;
    // the first entry with cum >= r, else the last one
    double c = 0.0, c_at = 0.0, c_before = 0.0;
    int orb = 0;
    bool found = false;
    for (int k = 0; k < s.max_neigh && !found; ++k) {
        const int n = nb[k];
        if (n <= 0) continue;
        const int o = beta(src) ? 2 * n - 1 : 2 * n;
        c_before = c;
        c += orb_occ(d, o) ? 0.0 : fabs(tmat_el(s, src, o));
        c_at = c;
        orb = o;
        found = c >= r;
    }
    const double p_orb = (c_at - c_before) / cum_sum;
    const double pg = s.p_elec * p_orb;
    e.pgen = (Real)pg;
    e.invp = (Real)(1.0 / pg);
    finish_single<Real, NW>(s, d, src, orb, e);
    e.ok = true;
}

// The c-th (1-based) unoccupied spin orbital among those of `pattern`, 0 if none.
template <int NW = 0>
__device__ inline int nth_unoccupied(const DevSys &s, const unsigned long long *d, unsigned long long pattern, int c) {
    unsigned long long u[kMaxWords];
    NECI_FOR_WORDS(w, nwords<NW>(s)) {
        const int lo = 64 * w;
        const unsigned long long valid = s.nbasis >= lo + 64 ? ~0ull : (s.nbasis > lo ? (1ull << (s.nbasis - lo)) - 1 : 0ull);
        u[w] = ~d[w] & valid;
    }
    return nth_orbital(u, nwords<NW>(s), pattern, c);
}

// CreateSingleExcit (GenRandSymExcitNUMod.F90:1118-1243), C1 symmetry,
// tCycleOrbs = .false.: the electron by rejection (repeated only while it
// lands in a spin without holes).  The hole is uniform over the unoccupied
// orbitals of the electron's spin, the distribution of the reference's
// rejection loop, but drawn as an index into those orbitals: one draw and a
// bit select where the loop takes a variable number of draws, which made
// the lanes of a warp diverge and their later Philox blocks fall apart.
// Returns the full single pgen, pSingles / (NExcit * (nel - ElecsWNoExcits)).
template <typename Real, int NW = 0>
__device__ inline void gen_uniform_single(const DevSys &s, const unsigned long long *d, Stream &rng, Excit<Real> &e) {
    e.ic = 1;
    e.cls = TC_SING;
    e.ok = false;
    const int norbs = s.nbasis / 2;
    int nalpha = 0, nbeta = 0;
    NECI_FOR_WORDS(w, nwords<NW>(s)) {
        nalpha += __popcll(d[w] & 0xAAAAAAAAAAAAAAAAull);
        nbeta += __popcll(d[w] & 0x5555555555555555ull);
    }
    const int nun_a = norbs - nalpha, nun_b = norbs - nbeta;
    const int elecs_wno = (nun_a == 0 ? nalpha : 0) + (nun_b == 0 ? nbeta : 0);
    if (elecs_wno == s.nel) { e.pgen = 0; return; }
    int eleci = 0, ispn = 0, nexcit = 0, src = 0;
    for (int attempts = 0; attempts <= 250; ++attempts) {
        eleci = (int)uniform_index(rng, (unsigned)s.nel) + 1;
        src = nth_orbital(d, nwords<NW>(s), kAllBits, eleci);  // nI(eleci)
        ispn = beta(src) ? 2 : 1;
        nexcit = (ispn == 1) ? nun_a : nun_b;
        if (nexcit != 0) break;
    }
    if (nexcit == 0) { e.pgen = 0; return; }
    // ispn 1: alpha (even orbitals), 2: beta (odd)
    const int orb = nth_unoccupied<NW>(s, d, ispn == 1 ? kAlphaBits : kBetaBits,
                                       (int)uniform_index(rng, (unsigned)nexcit) + 1);
    if (orb == 0) { e.pgen = 0; return; }
    const int count = nexcit * (s.nel - elecs_wno);
    if (sizeof(Real) == 8) {
        e.pgen = (Real)(s.p_singles / (double)count);
        e.invp = (Real)__ldg(&s.inv_single[count]);  // (double)count * (1 / pSingles)
    } else {
        e.pgen = (Real)(s.f_p_singles / (float)count);
        e.invp = (Real)__ldg(&s.inv_single32[count]);  // (float)count * (float)(1 / pSingles)
    }
    finish_single<Real, NW>(s, d, src, orb, e);
    e.ok = true;
}

// Child determinant and H_ij of the double src0 < src1 -> {o0, o1}:
// make_double (excit_parity.F90:78) pairs the sources with the sorted
// targets, the parity counts the occupied orbitals each move passes.
template <typename Real, int NW = 0>
__device__ inline void finish_double(const DevSys &s, const unsigned long long *d, int src0, int src1, int o0, int o1,
                                     Excit<Real> &e) {
    const int ta = min(o0, o1), tb = max(o0, o1);
    NECI_FOR_WORDS(w, nwords<NW>(s)) e.child[w] = d[w];
    int np = occ_between(e.child, nwords<NW>(s), min(src0, ta), max(src0, ta));
    flip_orb(e.child, src0);
    flip_orb(e.child, ta);
    np += occ_between(e.child, nwords<NW>(s), min(src1, tb), max(src1, tb));
    flip_orb(e.child, src1);
    flip_orb(e.child, tb);
    const Real hel = sltcnd_2_r<Real>(s, src0, src1, ta, tb);
    e.hel = (np & 1) ? -hel : hel;
}

// Position among the electrons of one spin of the pair with triangular
// index idx (pick_biased_elecs' ceiling((1+sqrt(9+8 idx))/2), in integers):
// returns a1 > a2 >= 1 with idx = (a1-1)(a1-2)/2 + a2 - 1.
__device__ inline void tri_pair(int idx, int &a1, int &a2) {
    // smallest a with a(a-1)/2 > idx, from a float estimate corrected exactly
    int a = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)idx)) * 0.5f) + 1;
    while (a > 2 && (a - 1) * (a - 2) / 2 > idx) --a;
    while (a * (a - 1) / 2 <= idx) ++a;
    a1 = a;
    a2 = idx + 1 - ((a - 1) * (a - 2)) / 2;
}

// GAS_doubles_PCHB_gen_exc (gasci_pchb_doubles_spatorb_fastweighted.fpp)
// with UNIF_UNIF particles = pick_biased_elecs
// (excit_gens_int_weighted.F90:722-830).  Returns the full double pgen
// (times pDoubles).
template <typename Real, int NW = 0>
__device__ inline void gen_pchb_double(const DevSys &s, const unsigned long long *d, Stream &rng, Excit<Real> &e) {
    e.ic = 2;
    e.ok = false;
    const bool dbl = sizeof(Real) == 8;
    const int aa = s.nOccAlpha * (s.nOccAlpha - 1) / 2;
    const int bb = s.nOccBeta * (s.nOccBeta - 1) / 2;
    // Both spin cases run the same instructions (selects, no branches), so a
    // warp whose lanes drew different cases stays converged.
    const bool par = rng.next64() < s.thr_bias;
    // the pair index, the exchange draw, the alias draw and the spawn's
    // rounding draw follow: two Philox blocks, computed side by side
    rng.fill_pair();
    e.cls = par ? TC_PAR : TC_OPP;
    const int idx = (int)uniform_index(rng, par ? (unsigned)(aa + bb) : (unsigned)(s.nOccAlpha * s.nOccBeta));
    // parallel pair: positions a1 > a2 among the electrons of one spin
    const bool alpha_pair = idx < aa;
    int a1, a2;
    tri_pair(alpha_pair ? idx : idx - aa, a1, a2);
    // opposite-spin pair: idx = (n_beta - 1) nOccAlpha + (n_alpha - 1)
    int qb = (int)((float)idx * s.f_inv_nalpha);
    qb -= (qb * s.nOccAlpha > idx);
    qb += ((qb + 1) * s.nOccAlpha <= idx);
    const int ra = idx - qb * s.nOccAlpha;
    const unsigned long long spin_mask = alpha_pair ? kAlphaBits : kBetaBits;
    const int o_a = nth_orbital(d, nwords<NW>(s), par ? spin_mask : kAlphaBits, par ? a2 : 1 + ra);
    const int o_b = nth_orbital(d, nwords<NW>(s), par ? spin_mask : kBetaBits, par ? a1 : 1 + qb);
    Real pgen = par ? (dbl ? (Real)s.pgen_par : (Real)s.f_pgen_par) : (dbl ? (Real)s.pgen_opp : (Real)s.f_pgen_opp);
    Real invp = par ? (dbl ? (Real)s.inv_par : (Real)s.f_inv_par) : (dbl ? (Real)s.inv_opp : (Real)s.f_inv_opp);
    // the exchange draw is taken for every pair and used for opposite spins
    const unsigned long long rx = rng.next64();
    // the chosen electrons in nI order, lower orbital first
    const int src0 = min(o_a, o_b), src1 = max(o_a, o_b);
    if (src0 == 0) { e.pgen = 0; return; }
    const long long i1 = spat(src0), j1 = spat(src1);
    const long long ij = i1 < j1 ? i1 + j1 * (j1 - 1) / 2 : j1 + i1 * (i1 - 1) / 2;
    int spin0 = src0 & 1, spin1 = src1 & 1;
    int type = 1;
    if (spin0 != spin1) {
        const bool exch = rx < __ldg(&s.pexch_thr[ij - 1]);
        type = exch ? 3 : 2;
        const Real pe = dbl ? (Real)__ldg(&s.pexch[ij - 1]) : (Real)__ldg(&s.pexch32[ij - 1]);
        pgen *= exch ? pe : ((Real)1 - pe);
        const Real f = dbl ? (Real)__ldg(exch ? &s.pexch_inv[ij - 1] : &s.pnoexch_inv[ij - 1])
                           : (Real)__ldg(exch ? &s.pexch_inv32[ij - 1] : &s.pnoexch_inv32[ij - 1]);
        invp *= f;
        if (exch) { const int t = spin0; spin0 = spin1; spin1 = t; }
    }
    // sample_AliasTable_t (aliasSampling.F90:310-331): slot and fraction
    // from the high and low halves of one 64x(abMax) product.  An empty
    // table (no allowed ab) is not tested for first: its slots keep
    // themselves with probability 0, so the draw ends in the pholes test
    // below with no child, one dependent load fewer on every double.
    const size_t t = (size_t)(ij - 1) * 3 + (type - 1);
    const unsigned long long r = rng.next64();
    const unsigned long long n = (unsigned long long)s.abMax;
    const unsigned long long pos0 = __umul64hi(r, n);
    const unsigned long long frac = r * n;
    const size_t base = t * (size_t)s.abMax;
    int ab, tp;
    Real pholes, ainv;
    if (dbl) {
        // the slot's 32-byte record; a taken alias reads the alias's record
        const AliasRec a = load_alias(&s.alias_rec[base + pos0]);
        if (frac < a.thr || a.thr == ~0ull) {
            ab = (int)pos0 + 1;
            pholes = (Real)a.prob;
            ainv = (Real)a.inv;
            tp = a.tgt;
        } else {
            ab = a.alias;
            const AliasRec b = load_alias(&s.alias_rec[base + ab - 1]);
            pholes = (Real)b.prob;
            ainv = (Real)b.inv;
            tp = b.tgt;
        }
    } else {
        const unsigned long long thr = __ldg(&s.alias_thr[base + pos0]);
        ab = (frac < thr || thr == ~0ull) ? (int)pos0 + 1 : __ldg(&s.alias_alias[base + pos0]);
        pholes = (Real)__ldg(&s.alias_prob32[base + ab - 1]);
        ainv = (Real)__ldg(&s.alias_inv32[base + ab - 1]);
        tp = __ldg(&s.tgt_pair[ab]);
    }
    const int o0 = 2 * (tp >> 16) - spin0, o1 = 2 * (tp & 0xFFFF) - spin1;
    // pholes > 1e-10 (pholes >= 0: compared on the bits in FP64)
    const bool small = dbl ? !(dbl_bits((double)pholes) > dbl_bits(1e-10)) : !(pholes > (Real)1e-10);
    if (o0 == 0 || o1 == 0 || orb_occ(d, o0) || orb_occ(d, o1) || small) { e.pgen = 0; return; }
    finish_double<Real, NW>(s, d, src0, src1, o0, o1, e);
    pgen *= pholes;
    e.pgen = pgen * (dbl ? (Real)s.p_doubles : (Real)s.f_p_doubles);
    invp *= ainv;
    e.invp = invp * (dbl ? (Real)s.inv_pdoub : (Real)s.f_inv_pdoub);
    e.ok = true;
}


// CreateDoubExcit (GenRandSymExcitNUMod.F90:155-205) without spatial
// symmetry (C1: tNoSymGenRandExcits), tCycleOrbs = .false.:
//   PickElecPair (:954)  a uniform electron pair, iSpn = 1 beta/beta,
//                        2 alpha/beta, 3 alpha/alpha
//   FindNumForbiddenOrbsNoSym (:380), PickAOrb (:669) with
//   IsAOrbSymAllowed: the first hole by rejection (cycled when at most 3
//                        are allowed), PickBOrb (:222) the second by rejection
//   FindDoubleProb (:208) pgen, which depends only on iSpn here (all
//                        determinants share the alpha/beta counts), so it is
//                        taken from the host's table of the three cases.
// NECI stops the run where a rejection loop exceeds its limit; here the
// attempt produces no child.
template <typename Real, int NW = 0>
__device__ inline void gen_uniform_double(const DevSys &s, const unsigned long long *d, Stream &rng, Excit<Real> &e) {
    e.ic = 2;
    e.cls = TC_DOUB;
    e.ok = false;
    e.pgen = 0;
    const int nel = s.nel;
    const int ep = nel * (nel - 1) / 2;
    const int X = ep - ((int)uniform_index(rng, (unsigned)ep) + 1);
    // K = int((sqrt(8X + 1) - 1) / 2): the largest K with K(K+1)/2 <= X
    int K = (int)((sqrtf(8.0f * (float)X + 1.0f) - 1.0f) * 0.5f);
    while (K > 0 && K * (K + 1) / 2 > X) --K;
    while ((K + 1) * (K + 2) / 2 <= X) ++K;
    const int src0 = nth_orbital(d, nwords<NW>(s), kAllBits, nel - 1 - K);
    const int src1 = nth_orbital(d, nwords<NW>(s), kAllBits, nel - X + K * (K + 1) / 2);
    if (src0 == 0 || src1 == 0) return;
    const int ispn = beta(src0) != beta(src1) ? 2 : (beta(src0) ? 1 : 3);
    const int nua = s.nBI - s.nOccAlpha, nub = s.nBI - s.nOccBeta;
    int na, forbidden;
    unsigned long long allowed;  // spin orbitals whose partner class has room (IsAOrbSymAllowed)
    if (ispn == 2) {
        na = s.nbasis - nel;
        forbidden = (nua == 0 ? nub : 0) + (nub == 0 ? nua : 0);
        allowed = (nub != 0 ? kAlphaBits : 0ull) | (nua != 0 ? kBetaBits : 0ull);
    } else if (ispn == 1) {
        na = nub;
        forbidden = nub == 1;
        allowed = nub != 1 ? kBetaBits : 0ull;
    } else {
        na = nua;
        forbidden = nua == 1;
        allowed = nua != 1 ? kAlphaBits : 0ull;
    }
    if (na == forbidden) return;
    int orbA = 0;
    if (na - forbidden <= 3) {
        orbA = nth_unoccupied<NW>(s, d, allowed, (int)uniform_index(rng, (unsigned)(na - forbidden)) + 1);
    } else {
        const unsigned n_draw = ispn == 2 ? (unsigned)s.nbasis : (unsigned)s.nBI;
        bool found = false;
        // NECI's counters: at most 252 draws per pick, 20 nBasis + 2 picks
        for (int overall = 0; overall <= 20 * s.nbasis + 1 && !found; ++overall) {
            orbA = 0;
            for (int att = 0; att <= 251; ++att) {
                const int c = (int)uniform_index(rng, n_draw);
                const int o = ispn == 2 ? c + 1 : (ispn == 1 ? 2 * (c + 1) - 1 : 2 * (c + 1));
                if (!orb_occ(d, o)) { orbA = o; break; }
            }
            if (orbA == 0) return;
            found = (allowed >> ((orbA - 1) & 63)) & 1ull;
        }
        if (!found) return;
    }
    if (orbA == 0) return;
    // PickBOrb: the second hole's spin
    const bool b_beta = ispn == 1 || (ispn == 2 && !beta(orbA));
    int orbB = 0;
    for (int att = 0; att <= 1001; ++att) {
        const int c = (int)uniform_index(rng, (unsigned)s.nBI);
        const int o = 2 * (c + 1) - (b_beta ? 1 : 0);
        if (!orb_occ(d, o) && o != orbA) { orbB = o; break; }
    }
    if (orbB == 0) return;
    finish_double<Real, NW>(s, d, src0, src1, orbA, orbB, e);
    const bool dbl = sizeof(Real) == 8;
    e.pgen = dbl ? (Real)s.pgen_unif[ispn - 1] : (Real)s.f_pgen_unif[ispn - 1];
    e.invp = dbl ? (Real)s.inv_unif[ispn - 1] : (Real)s.f_inv_unif[ispn - 1];
    e.ok = true;
}

// gen_exc_sd (excitation_generators.F90:110-133): singles with pSingles.
template <typename Real, int NW = 0>
__device__ inline void generate_excitation(const DevSys &s, const unsigned long long *d, const int32_t *neigh,
                                           Stream &rng, Excit<Real> &e) {
    if (s.excitgen == NECI_EXGEN_RS_HUBBARD) {
        gen_rs_hubbard<Real, NW>(s, d, neigh, rng, e);
        return;
    }
    if (s.excitgen == NECI_EXGEN_UNIFORM) {
        // gen_rand_excit (GenRandSymExcitNUMod.F90:120-147): r < pDoubles -> double
        if (rng.next64() < s.thr_doubles) gen_uniform_double<Real, NW>(s, d, rng, e);
        else gen_uniform_single<Real, NW>(s, d, rng, e);
        return;
    }
    if (rng.next64() < s.thr_singles) gen_uniform_single<Real, NW>(s, d, rng, e);
    else gen_pchb_double<Real, NW>(s, d, rng, e);
}

}  // namespace neci
