// excitgen.cuh -- device excitation generators (generate_excitation,
// proc_ptrs.F90:13) in bit-string form.  Each consumes uniforms from one
// Philox stream in the same order as NECI's routine consumes dSFMT draws.
#pragma once

#include "engine.cuh"

namespace neci {

struct Excit {
    unsigned long long child[kMaxWords];
    double pgen;
    double hel;
    int ic;
    bool ok;
};

// Child determinant and H_ij of a single src -> tgt.
__device__ inline void finish_single(const DevSys &s, const unsigned long long *d, int src, int tgt, Excit &e) {
    for (int w = 0; w < s.W; ++w) e.child[w] = d[w];
    flip_orb(e.child, src);
    flip_orb(e.child, tgt);
    const int lo = min(src, tgt), hi = max(src, tgt);
    const bool par = occ_between(d, s.W, lo, hi) & 1;  // make_single tParity
    const double hel = (s.system == NECI_SYS_HUBBARD_REAL_SPACE) ? tmat_el(s, src, tgt) : sltcnd_1(s, d, src, tgt);
    e.hel = par ? -hel : hel;
}

// gen_excit_rs_hubbard (real_space_hubbard.F90:1938-2030),
// create_cum_list_rs_hubbard (:2080) and pick_from_cum_list
// (lattice_models_utils.F90:150).
__device__ inline void gen_rs_hubbard(const DevSys &s, const unsigned long long *d, const uint8_t *nI,
                                      const int32_t *neigh, Stream &rng, Excit &e) {
    e.ic = 1;
    e.ok = false;
    const int elec = 1 + (int)(rng.next() * s.nel);
    const double p_elec = 1.0 / (double)s.nel;
    const int src = nI[elec - 1];
    const int site = spat(src);
    int orbs[kMaxNeigh];
    double cum[kMaxNeigh];
    int nn = 0;
    double cum_sum = 0.0;
    for (int k = 0; k < s.max_neigh; ++k) {
        const int n = neigh[(site - 1) * s.max_neigh + k];
        if (n <= 0) continue;
        const int orb = beta(src) ? 2 * n - 1 : 2 * n;
        double elem = 0.0;
        if (!orb_occ(d, orb)) elem = fabs(tmat_el(s, src, orb));
        cum_sum += elem;
        orbs[nn] = orb;
        cum[nn] = cum_sum;
        ++nn;
    }
    if (cum_sum < 1e-10) { e.pgen = 0.0; return; }
    const double r = rng.next() * cum_sum;
    int ind = nn;
    for (int k = 0; k < nn; ++k)
        if (cum[k] >= r) { ind = k + 1; break; }
    const double p_orb = (ind == 1) ? cum[0] / cum_sum : (cum[ind - 1] - cum[ind - 2]) / cum_sum;
    const int orb = orbs[ind - 1];
    e.pgen = p_elec * p_orb;
    finish_single(s, d, src, orb, e);
    e.ok = true;
}

// CreateSingleExcit (GenRandSymExcitNUMod.F90:1118-1243), C1 symmetry,
// tCycleOrbs = .false. (rejection for the electron and for the hole).
__device__ inline void gen_uniform_single(const DevSys &s, const unsigned long long *d, const uint8_t *nI,
                                          Stream &rng, Excit &e) {
    e.ic = 1;
    e.ok = false;
    const int norbs = s.nbasis / 2;
    int nalpha = 0, nbeta = 0;
    for (int w = 0; w < s.W; ++w) {
        nalpha += __popcll(d[w] & 0xAAAAAAAAAAAAAAAAull);
        nbeta += __popcll(d[w] & 0x5555555555555555ull);
    }
    const int nun_a = norbs - nalpha, nun_b = norbs - nbeta;
    const int elecs_wno = (nun_a == 0 ? nalpha : 0) + (nun_b == 0 ? nbeta : 0);
    if (elecs_wno == s.nel) { e.pgen = 0.0; return; }
    int eleci = 0, ispn = 0, nexcit = 0;
    for (int attempts = 0; attempts <= 250; ++attempts) {
        eleci = (int)(s.nel * rng.next()) + 1;
        ispn = beta(nI[eleci - 1]) ? 2 : 1;
        nexcit = (ispn == 1) ? nun_a : nun_b;
        if (nexcit != 0) break;
    }
    if (nexcit == 0) { e.pgen = 0.0; return; }
    int orb = 0;
    bool found = false;
    for (int attempts = 0; attempts <= 250; ++attempts) {
        const int chosen = (int)(norbs * rng.next());
        orb = 2 * (chosen + 1) - (ispn - 1);
        if (!orb_occ(d, orb)) { found = true; break; }
    }
    if (!found) { e.pgen = 0.0; return; }
    e.pgen = 1.0 / (double)(nexcit * (s.nel - elecs_wno));
    finish_single(s, d, nI[eleci - 1], orb, e);
    e.ok = true;
}

// GAS_doubles_PCHB_gen_exc (gasci_pchb_doubles_spatorb_fastweighted.fpp)
// with UNIF_UNIF particles = pick_biased_elecs
// (excit_gens_int_weighted.F90:722-830).
__device__ inline void gen_pchb_double(const DevSys &s, const unsigned long long *d, const uint8_t *nI,
                                       Stream &rng, Excit &e) {
    e.ic = 2;
    e.ok = false;
    const int aa = s.nOccAlpha * (s.nOccAlpha - 1) / 2;
    const int bb = s.nOccBeta * (s.nOccBeta - 1) / 2;
    const int par = aa + bb;
    const int ab_pairs = s.nOccAlpha * s.nOccBeta;
    const double pBias = s.p_parallel;
    double r = rng.next();
    int al_req, be_req, al_num[2] = {0, 0}, be_num[2] = {0, 0};
    double pgen;
    if (r < pBias) {
        r = (r / pBias) * par;
        int idx = (int)floor(r);
        if (idx < aa) {
            al_req = 2; be_req = 0;
            al_num[0] = (int)ceil((1.0 + sqrt(9.0 + 8.0 * (double)idx)) / 2.0);
            al_num[1] = idx + 1 - ((al_num[0] - 1) * (al_num[0] - 2)) / 2;
        } else {
            al_req = 0; be_req = 2;
            idx -= aa;
            be_num[0] = (int)ceil((1.0 + sqrt(9.0 + 8.0 * (double)idx)) / 2.0);
            be_num[1] = idx + 1 - ((be_num[0] - 1) * (be_num[0] - 2)) / 2;
        }
        pgen = pBias / (double)par;
    } else {
        al_req = 1; be_req = 1;
        pgen = (1.0 - pBias) / (double)ab_pairs;
        r = ((r - pBias) / (1.0 - pBias)) * ab_pairs;
        const int idx = (int)floor(r);
        al_num[0] = 1 + idx % s.nOccAlpha;
        be_num[0] = 1 + (int)floor(idx / (double)s.nOccAlpha);
    }
    int elecs[2] = {0, 0}, found = 0, al_count = 0, be_count = 0;
    for (int i = 1; i <= s.nel; ++i) {
        if (!beta(nI[i - 1])) {
            ++al_count;
            if (al_req > 0 && al_count == al_num[al_req - 1]) { elecs[found++] = i; --al_req; }
        } else {
            ++be_count;
            if (be_req > 0 && be_count == be_num[be_req - 1]) { elecs[found++] = i; --be_req; }
        }
        if (al_req == 0 && be_req == 0) break;
    }
    if (found < 2) { e.pgen = 0.0; return; }
    const int src0 = nI[elecs[0] - 1], src1 = nI[elecs[1] - 1];
    const long long i1 = spat(src0), j1 = spat(src1);
    const long long ij = i1 < j1 ? i1 + j1 * (j1 - 1) / 2 : j1 + i1 * (i1 - 1) / 2;
    int spin0 = src0 & 1, spin1 = src1 & 1;
    int type;
    if (spin0 == spin1) {
        type = 1;
    } else {
        const double pe = __ldg(&s.pexch[ij - 1]);
        if (rng.next() < pe) {
            type = 3;
            pgen *= pe;
            const int t = spin0; spin0 = spin1; spin1 = t;
        } else {
            type = 2;
            pgen *= (1.0 - pe);
        }
    }
    // sample_AliasTable_t (aliasSampling.F90:310-331)
    const size_t t = (size_t)(ij - 1) * 3 + (type - 1);
    if (!__ldg(&s.alias_present[t])) { e.pgen = 0.0; return; }
    const double ra = rng.next();
    const int pos = (int)((double)s.abMax * ra) + 1;
    const double bias = fmax((double)s.abMax * ra + 1.0 - pos, 0.0);
    const size_t base = t * (size_t)s.abMax;
    int ab;
    if (bias < __ldg(&s.alias_bias[base + pos - 1])) ab = pos;
    else ab = __ldg(&s.alias_alias[base + pos - 1]);
    const double pholes = __ldg(&s.alias_prob[base + ab - 1]);
    const int tp = __ldg(&s.tgt_pair[ab]);
    const int o0 = 2 * (tp >> 16) - spin0, o1 = 2 * (tp & 0xFFFF) - spin1;
    if (o0 == 0 || o1 == 0 || orb_occ(d, o0) || orb_occ(d, o1) || fabs(pholes) < 1e-10) { e.pgen = 0.0; return; }
    const int ta = min(o0, o1), tb = max(o0, o1);
    for (int w = 0; w < s.W; ++w) e.child[w] = d[w];
    // parity of src0 -> ta then src1 -> tb (make_double pairing)
    int np = occ_between(e.child, s.W, min(src0, ta), max(src0, ta));
    flip_orb(e.child, src0);
    flip_orb(e.child, ta);
    np += occ_between(e.child, s.W, min(src1, tb), max(src1, tb));
    flip_orb(e.child, src1);
    flip_orb(e.child, tb);
    const double hel = sltcnd_2(s, src0, src1, ta, tb);
    e.hel = (np & 1) ? -hel : hel;
    e.pgen = pgen * pholes;
    e.ok = true;
}

// gen_exc_sd (excitation_generators.F90:110-133): singles with pSingles.
__device__ inline void generate_excitation(const DevSys &s, const unsigned long long *d, const uint8_t *nI,
                                           const int32_t *neigh, Stream &rng, Excit &e) {
    if (s.excitgen == NECI_EXGEN_RS_HUBBARD) {
        gen_rs_hubbard(s, d, nI, neigh, rng, e);
        return;
    }
    if (rng.next() < s.p_singles) {
        gen_uniform_single(s, d, nI, rng, e);
        e.pgen *= s.p_singles;
    } else {
        gen_pchb_double(s, d, nI, rng, e);
        e.pgen *= (1.0 - s.p_singles);
    }
}

}  // namespace neci
