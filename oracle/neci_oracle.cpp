// neci_oracle.cpp -- CPU restatement of one NECI FCIQMC iteration.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker of the GB300
// engine: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg load it.  It is never on the product path.
//
// It restates NECI's own routines in their own list-based form (decoded
// orbital lists nI, Fortran-style loops) rather than the bit-parallel forms
// the CUDA kernels use, so that a kernel bug does not cancel against the same
// bug here.  Each function cites the reference file:line it follows.
//
// Two deliberate departures from NECI, shared with the engine and stated in
// the engine's design notes:
//   * random numbers come from Philox-4x32-10 keyed by (seed, determinant,
//     iteration, purpose, run, attempt) instead of one dSFMT stream per rank
//     (lib/dSFMT_interface.F90:67), so the draws a determinant sees do not
//     depend on where it sits in CurrentDets;
//   * spawned amplitudes are summed in 64-bit fixed point
//     (NECI_SPAWN_FIXED_BITS fractional bits) so that the compressed spawn
//     list does not depend on summation order (NECI sums in FP64 in the order
//     left by its quicksort, lib/quicksort.F90.template:584).
//
// Pinning: the pieces covered by the reference's own unit tests are checked
// against those known answers in tests/ (CountBits, the real-space Hubbard
// cumulative lists and pgens, the diagonal-element consistency of
// unit_tests/sltcnd, the alias-table and PCHB pgen diagnostics), and the
// whole iteration against exact diagonalisation.  Hashing and annihilation
// of injected spawn lists have no known answers in the reference's tests.
//
// Build: oracle/build_oracle.sh (g++ -O2 -ffp-contract=off, no -ffast-math:
// the floating-point operation order below is the order the engine uses).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "../include/neci_gpu.h"

namespace {

typedef int64_t i64;
typedef uint64_t u64;
typedef uint32_t u32;

// ---------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC11), written from the published round function.
// ---------------------------------------------------------------------------
struct Philox {
    static void round(u32 c[4], const u32 k[2]) {
        const u64 p0 = (u64)0xD2511F53u * c[0];
        const u64 p1 = (u64)0xCD9E8D57u * c[2];
        const u32 hi0 = (u32)(p0 >> 32), lo0 = (u32)p0;
        const u32 hi1 = (u32)(p1 >> 32), lo1 = (u32)p1;
        u32 n[4];
        n[0] = hi1 ^ c[1] ^ k[0];
        n[1] = lo1;
        n[2] = hi0 ^ c[3] ^ k[1];
        n[3] = lo0;
        c[0] = n[0]; c[1] = n[1]; c[2] = n[2]; c[3] = n[3];
    }
    static void block(const u32 ctr[4], const u32 key[2], u32 out[4]) {
        u32 c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
        u32 k[2] = {key[0], key[1]};
        for (int r = 0; r < 10; ++r) {
            round(c, k);
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
        }
        out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
    }
};

// splitmix64 finaliser (Steele, Lea, Flood 2014) used to fold a determinant
// into a 64-bit Philox key.
inline u64 splitmix64(u64 x) {
    x += 0x9E3779B97F4A7C15ull;
    u64 z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

enum Purpose : u32 { P_NSPAWN = 1, P_ATTEMPT = 2, P_DEATH = 3, P_ANN_ROUND = 4, P_STATS_ROUND = 5 };

inline u64 det_key(const i64 *det, int W, u64 seed) {
    u64 h = seed ^ 0x6A09E667F3BCC909ull;
    for (int i = 0; i < W; ++i) h = splitmix64(h ^ (u64)det[i]);
    return h;
}

// Stream of 64-bit draws for one (determinant, iteration, purpose, run,
// attempt).  Each draw consumes one 64-bit value; a Philox block gives two.
// NECI's uses of a uniform r in [0,1) are restated on the integer draws:
// int(n*r) -> uniform_index(n) (multiply-high), r < p -> draw < prob_thresh(p),
// and a genrand_real2 double is (draw >> 11) * 2^-53.
struct Stream {
    u32 key[2];
    u32 ctr[4];
    u64 buf[2];
    int have;
    Stream(u64 dkey, i64 iter, u32 purpose, u32 run, u32 attempt) {
        key[0] = (u32)dkey;
        key[1] = (u32)(dkey >> 32);
        ctr[0] = attempt;
        ctr[1] = 0;
        ctr[2] = (u32)iter;
        ctr[3] = purpose | (run << 8) | ((u32)((u64)iter >> 32) << 16);
        have = 0;
    }
    u64 next64() {
        if (have == 0) {
            u32 o[4];
            Philox::block(ctr, key, o);
            ctr[1] += 1;
            buf[0] = ((u64)o[1] << 32) | o[0];
            buf[1] = ((u64)o[3] << 32) | o[2];
            have = 2;
        }
        return buf[2 - (have--)];
    }
    double next() { return (double)(next64() >> 11) * 0x1.0p-53; }
};

inline u64 prob_thresh(double p) {
    if (!(p > 0.0)) return 0ull;
    if (p >= 1.0) return ~0ull;
    return (u64)(p * 18446744073709551616.0);
}
inline bool bern(Stream &r, double p) {
    const u64 x = r.next64();
    return p >= 1.0 || x < prob_thresh(p);
}
inline bool bern_f(Stream &r, float p) {
    const u32 x = (u32)(r.next64() >> 32);
    if (p >= 1.0f) return true;
    if (!(p > 0.0f)) return false;
    return x < (u32)(p * 4294967296.0f);
}
inline u32 uniform_index(Stream &r, u32 n) {
    return (u32)(((unsigned __int128)r.next64() * (unsigned __int128)n) >> 64);
}

thread_local std::string g_err;

// ---------------------------------------------------------------------------
// Fixed-point spawn amplitudes.
// ---------------------------------------------------------------------------
inline i64 to_fixed(double x) { return (i64)std::llrint(std::ldexp(x, NECI_SPAWN_FIXED_BITS)); }
inline double from_fixed(i64 q) { return std::ldexp((double)q, -NECI_SPAWN_FIXED_BITS); }

inline double as_double(i64 w) { double d; std::memcpy(&d, &w, 8); return d; }
inline i64 as_word(double d) { i64 w; std::memcpy(&w, &d, 8); return w; }

inline double fsign(double a, double b) { return b >= 0.0 ? std::fabs(a) : -std::fabs(a); }  // Fortran sign(a,b)

// Partial sums of one core row in the core projection: the smallest power of
// two G with 4 G at least the mean row length, at most 32 (the engine's
// core_group_size).
static int core_group_size(long long nnz, long long n_core) {
    int g = 1;
    while (g < 32 && 4ll * g * n_core < nnz) g <<= 1;
    return g;
}

// Elements of a core row summed as one segment (the engine's
// core_segment_len): per_lane per partial sum, 64 unless set
// (NECI_OPT_CORE_SEGMENT).
static long long core_segment_len(int G, int per_lane) { return (long long)per_lane * G; }

struct Oracle {
    neci_gpu_system sys{};
    int W = 1, L = 1, R = 3;  // det words, sign words, row words
    int nifd = 0;

    // system data
    std::vector<int32_t> random_hash2;  // 1-based
    std::vector<double> tmat;           // nbasis*nbasis column-major
    std::vector<double> umat;
    std::vector<int32_t> neighbours;    // max_neighbours * nsites, 1-based
    int nsites = 0;
    std::vector<i64> ilut_ref;
    double hii = 0.0;
    int nOccAlpha = 0, nOccBeta = 0;
    double p_doubles = 0.0;             // 1 - pSingles

    // conventional tau search (tau/tau_search_conventional.F90:138-258,
    // tau/tau_main.F90:197-206): class maxima of gamma and max_death_cpt
    // stochastic 2-RDM of a replica pair: Gamma[pair(p,q) * npair + pair(r,s)]
    bool rdm = false;
    i64 npair = 0;
    std::vector<double> rdm2;
    static i64 rdm_pair(int p, int q) { return (i64)(q - 1) * (q - 2) / 2 + (p - 1); }

    bool tau_search = false;
    double tau_gamma[4] = {0.0, 0.0, 0.0, 0.0};  // sing, doub, par, opp
    i64 tau_cnt[4] = {0, 0, 0, 0};
    double tau_death = 0.0;
    // factor that unbiases p_gen for class c: gamma = |H| (1/p_gen) factor
    double tau_factor(int c) const {
        if (c == 0) return sys.system == NECI_SYS_HUBBARD_REAL_SPACE ? 1.0 : sys.p_singles;  // pSingles = 1 on lattices
        if (c == 1) return p_doubles;
        if (c == 2) return p_doubles * sys.p_parallel;
        return p_doubles * (1.0 - sys.p_parallel);
    }

    // PCHB
    bool pchb_ready = false;
    int nBI = 0;
    i64 ijMax = 0, abMax = 0;
    std::vector<double> pexch;                 // ijMax (1-based index ij-1)
    std::vector<double> alias_bias;            // (ij, type) * abMax
    std::vector<int32_t> alias_alias;          // 1-based ab
    std::vector<double> alias_prob;            // probs
    std::vector<char> alias_present;           // (ij, type)
    std::vector<int32_t> tgt1, tgt2;           // tgtOrbs(:, ab)

    // walker list
    std::vector<i64> CurrentDets;
    std::vector<double> diagH, offdiagH;
    std::vector<std::vector<int32_t>> HashIndex;  // 1-based slot indices
    std::vector<int32_t> FreeSlot;
    i64 iStartFreeSlot = 0, iEndFreeSlot = 0;     // 0-based half-open window
    i64 TotWalkers = 0;
    i64 HolesInList = 0;

    // core space
    std::vector<i64> core_slots;      // slot of each core det
    std::vector<i64> core_rowptr, core_col;
    int core_seg_lane = 64;  // elements per partial sum of a core-row segment
    std::vector<double> core_val;     // off-diagonal H_ij
    std::vector<double> core_diag;    // H_ii - Hii

    // ------------------------------------------------------------------ bits
    static int popc(u64 x) { return __builtin_popcountll(x); }
    bool orb_occ(const i64 *ilut, int orb) const {
        return ((u64)ilut[(orb - 1) / 64] >> ((orb - 1) % 64)) & 1ull;
    }
    // decode_bit_det (BitReps.F90:714): sorted list of occupied orbitals.
    void decode_bit_det(const i64 *ilut, std::vector<int> &nI) const {
        nI.clear();
        for (int orb = 1; orb <= sys.nbasis; ++orb)
            if (orb_occ(ilut, orb)) nI.push_back(orb);
    }
    // EncodeBitDet (DetBitOps.F90:540).
    void encode_bit_det(const std::vector<int> &nI, i64 *ilut) const {
        for (int i = 0; i < W; ++i) ilut[i] = 0;
        for (int orb : nI) ilut[(orb - 1) / 64] |= (i64)(1ull << ((orb - 1) % 64));
    }
    // FindBitExcitLevel (DetBitOps.F90:140-178): popcount(I .and. (I .xor. J)).
    int find_bit_excit_level(const i64 *a, const i64 *b) const {
        int ic = 0;
        for (int i = 0; i < W; ++i) ic += popc((u64)a[i] & ((u64)a[i] ^ (u64)b[i]));
        return ic;
    }
    // DetBitEQ (DetBitOps.F90:274).
    bool det_bit_eq(const i64 *a, const i64 *b) const {
        for (int i = 0; i < W; ++i)
            if (a[i] != b[i]) return false;
        return true;
    }
    // ilut_lt (DetBitOps.F90:431): signed int64 lexicographic over 0:NIfD.
    bool ilut_lt(const i64 *a, const i64 *b) const {
        for (int i = 0; i < W; ++i)
            if (a[i] != b[i]) return a[i] < b[i];
        return false;
    }
    static bool is_beta(int orb) { return orb & 1; }
    static int gtID(int orb) { return (orb + 1) / 2; }

    // FindWalkerHash (hash.F90:23-38): int64 arithmetic wraps (two's
    // complement), Fortran mod takes the sign of the dividend.
    i64 find_walker_hash(const std::vector<int> &nI, i64 len) const {
        u64 hash = 0;
        for (size_t i = 0; i < nI.size(); ++i) {
            const i64 term = (i64)((int32_t)(random_hash2[nI[i]] * (int32_t)(i + 1)));
            hash = 1099511628211ull * hash + (u64)term;
        }
        const i64 h = (i64)hash;
        const i64 m = h % len;  // C++ % truncates toward zero == Fortran mod
        return (m < 0 ? -m : m) + 1;
    }

    // ---------------------------------------------------------- integrals
    double get_tmat(int i, int j) const {  // GetTMatEl (OneEInts.F90:188)
        if (tmat.empty()) return 0.0;
        return tmat[(size_t)(j - 1) * sys.nbasis + (i - 1)];
    }
    // UMatInd_base (UMatCache.F90:257-306), Hermitian branch.
    static i64 umat_ind(int I, int J, int K, int L) {
        i64 A, B;
        if (I > K) A = (i64)I * (I - 1) / 2 + K; else A = (i64)K * (K - 1) / 2 + I;
        if (J > L) B = (i64)J * (J - 1) / 2 + L; else B = (i64)L * (L - 1) / 2 + J;
        if (A > B) return A * (A - 1) / 2 + B;
        return B * (B - 1) / 2 + A;
    }
    // get_umat_el_normal (Integrals_neci.F90:1875): <ij|kl> over spatial orbitals.
    double get_umat_el(int i, int j, int k, int l) const {
        if (sys.system == NECI_SYS_HUBBARD_REAL_SPACE) {
            // get_umat_el_hub (real_space_hubbard.F90:2575): on-site U only.
            return (i == j && j == k && k == l) ? sys.uhub : 0.0;
        }
        return umat[(size_t)(umat_ind(i, j, k, l) - 1)];
    }

    // ------------------------------------------------------- excitations
    // make_single (excit_parity.F90:15-60).
    void make_single(const std::vector<int> &nI, std::vector<int> &nJ, int elec, int tgt,
                     int ex[2], bool &tParity) const {
        const int nel = (int)nI.size();
        nJ = nI;
        ex[0] = nI[elec - 1];
        ex[1] = tgt;
        const int src = nI[elec - 1];
        int i;
        if (src < tgt) {
            for (i = elec + 1; i <= nel; ++i) {
                if (tgt < nJ[i - 1]) { nJ[i - 2] = tgt; break; }
                nJ[i - 2] = nJ[i - 1];
            }
            if (i == nel + 1) nJ[nel - 1] = tgt;
        } else {
            for (i = elec - 1; i >= 1; --i) {
                if (tgt > nJ[i - 1]) { nJ[i] = tgt; break; }
                nJ[i] = nJ[i - 1];
            }
            if (i == 0) nJ[0] = tgt;
        }
        tParity = ((elec - i) % 2) == 0;
    }
    // make_double (excit_parity.F90:78-170).
    void make_double(const std::vector<int> &nI, std::vector<int> &nJ, int elec1, int elec2,
                     int tgt1, int tgt2, int ex[2][2], bool &tParity) const {
        const int nel = (int)nI.size();
        int elecs[2] = {std::min(elec1, elec2), std::max(elec1, elec2)};
        const int tgts[2] = {std::min(tgt1, tgt2), std::max(tgt1, tgt2)};
        const int srcs[2] = {nI[elecs[0] - 1], nI[elecs[1] - 1]};
        ex[0][0] = srcs[0]; ex[0][1] = srcs[1];
        ex[1][0] = tgts[0]; ex[1][1] = tgts[1];
        nJ = nI;
        if (srcs[0] < tgts[0] && srcs[1] < tgts[0]) elecs[1] = elecs[1] - 1;
        int pos_moved = 0;
        for (int k = 0; k < 2; ++k) {
            int i;
            if (srcs[k] < tgts[k]) {
                if (elecs[k] == nel) {
                    i = nel + 1;
                    nJ[nel - 1] = tgts[k];
                } else {
                    for (i = elecs[k] + 1; i <= nel; ++i) {
                        if (tgts[k] < nJ[i - 1]) { nJ[i - 2] = tgts[k]; break; }
                        nJ[i - 2] = nJ[i - 1];
                    }
                    if (i == nel + 1) nJ[nel - 1] = tgts[k];
                }
            } else {
                if (elecs[k] == 1) {
                    i = 0;
                    nJ[0] = tgts[k];
                } else {
                    for (i = elecs[k] - 1; i >= 1; --i) {
                        if (tgts[k] > nJ[i - 1]) { nJ[i] = tgts[k]; break; }
                        nJ[i] = nJ[i - 1];
                    }
                    if (i == 0) nJ[0] = tgts[k];
                }
            }
            pos_moved += elecs[k] - i + 1;
        }
        tParity = pos_moved & 1;
    }

    // Excitation between two determinants with NECI's conventions: sorted
    // source and target rows and the parity make_single/make_double give.
    int get_excitation(const std::vector<int> &nI, const std::vector<int> &nJ, int ex[2][2],
                       bool &tParity) const {
        std::vector<int> src, tgt;
        std::vector<int> elec_of;
        for (size_t a = 0; a < nI.size(); ++a)
            if (!std::binary_search(nJ.begin(), nJ.end(), nI[a])) { src.push_back(nI[a]); elec_of.push_back((int)a + 1); }
        for (int b : nJ)
            if (!std::binary_search(nI.begin(), nI.end(), b)) tgt.push_back(b);
        const int ic = (int)src.size();
        std::vector<int> tmp;
        if (ic == 1) {
            int e[2];
            make_single(nI, tmp, elec_of[0], tgt[0], e, tParity);
            ex[0][0] = e[0]; ex[1][0] = e[1];
        } else if (ic == 2) {
            make_double(nI, tmp, elec_of[0], elec_of[1], tgt[0], tgt[1], ex, tParity);
        }
        return ic;
    }

    // ----------------------------------------------------- matrix elements
    // sltcnd_0_base (sltcnd.fpp:585-622); ECore added for diagonal elements
    // (Determinants.F90:550).
    double sltcnd_0(const std::vector<int> &nI) const {
        const int nel = (int)nI.size();
        double hel_sing = 0.0;
        for (int i = 0; i < nel; ++i) hel_sing += get_tmat(nI[i], nI[i]);
        // hel_doub = hel_doub + sum(get_2el(id(i), id(i+1:), id(i), id(i+1:))):
        // the inner array sum is formed first, then added.
        double hel_doub = 0.0;
        for (int i = 0; i < nel - 1; ++i) {
            double s = 0.0;
            for (int j = i + 1; j < nel; ++j)
                s += get_umat_el(gtID(nI[i]), gtID(nI[j]), gtID(nI[i]), gtID(nI[j]));
            hel_doub += s;
        }
        double hel_tmp = 0.0;
        for (int i = 0; i < nel - 1; ++i)
            for (int j = i + 1; j < nel; ++j)
                if (is_beta(nI[i]) == is_beta(nI[j]))
                    hel_tmp -= get_umat_el(gtID(nI[i]), gtID(nI[j]), gtID(nI[j]), gtID(nI[i]));
        return hel_doub + hel_tmp + hel_sing;
    }
    // sltcnd_1_kernel (sltcnd.fpp:643-679): the Coulomb terms <ik|ak> over
    // the occupied k != src, less the exchange terms <ik|ka> over the
    // same-spin ones, plus h_ia.  The reference sums all Coulomb terms, then
    // all exchange terms; here each same-spin k contributes the precombined
    // <ik|ak> - <ik|ka> in one add, in ascending k (a reassociation: the
    // element moves by rounding only, far inside the 1e-12 relative
    // tolerance of matrix elements).
    double coul_exch(int id1, int id2, int o, bool same) const {
        const double j = get_umat_el(id1, gtID(o), id2, gtID(o));
        return same ? j - get_umat_el(id1, gtID(o), gtID(o), id2) : j;
    }
    double sltcnd_1(const std::vector<int> &nI, int src, int tgt) const {
        double hel = 0.0;
        const int id1 = gtID(src), id2 = gtID(tgt);
        if (is_beta(src) == is_beta(tgt)) {
            for (int o : nI)
                if (o != src) hel += coul_exch(id1, id2, o, is_beta(src) == is_beta(o));
        }
        hel += get_tmat(src, tgt);
        return hel;
    }
    // sltcnd_2_kernel (sltcnd.fpp:690-711).
    double sltcnd_2(const int ex[2][2]) const {
        const int i = ex[0][0], j = ex[0][1], a = ex[1][0], b = ex[1][1];
        double hel = 0.0;
        if (is_beta(i) == is_beta(a) && is_beta(j) == is_beta(b))
            hel = get_umat_el(gtID(i), gtID(j), gtID(a), gtID(b));
        if (is_beta(i) == is_beta(b) && is_beta(j) == is_beta(a))
            hel -= get_umat_el(gtID(i), gtID(j), gtID(b), gtID(a));
        return hel;
    }
    // count_double_orbs: doubly occupied sites.
    int count_double_orbs(const std::vector<int> &nI) const {
        int n = 0;
        for (size_t k = 0; k + 1 < nI.size(); ++k)
            if ((nI[k] & 1) && nI[k + 1] == nI[k] + 1) ++n;
        return n;
    }
    // get_diagonal_matel (matel_getter.F90:30).
    double diag_helement(const std::vector<int> &nI) const {
        if (sys.system == NECI_SYS_HUBBARD_REAL_SPACE)
            return sys.uhub * count_double_orbs(nI);  // get_diag_helemen_rs_hub :2303
        return sltcnd_0(nI) + sys.ecore;
    }
    // Off-diagonal element given the excitation (get_helement_det_only).
    double offdiag_from_ex(const std::vector<int> &nI, int ic, const int ex[2][2], bool tParity) const {
        double hel = 0.0;
        if (sys.system == NECI_SYS_HUBBARD_REAL_SPACE) {
            if (ic == 1) hel = get_tmat(ex[0][0], ex[1][0]);  // get_offdiag_helement_rs_hub :2425
            else return 0.0;
        } else {
            if (ic == 1) hel = sltcnd_1(nI, ex[0][0], ex[1][0]);
            else if (ic == 2) hel = sltcnd_2(ex);
            else return 0.0;
        }
        return tParity ? -hel : hel;
    }
    double helement(const i64 *a, const i64 *b) const {
        std::vector<int> nI, nJ;
        decode_bit_det(a, nI);
        decode_bit_det(b, nJ);
        const int ic = find_bit_excit_level(a, b);
        if (ic == 0) return diag_helement(nI);
        if (ic > 2) return 0.0;
        int ex[2][2];
        bool par = false;
        get_excitation(nI, nJ, ex, par);
        return offdiag_from_ex(nI, ic, ex, par);
    }
    // get_off_diagonal_matel (matel_getter.F90:61): <D0|H|D_j>, zero at D0.
    double offdiag_ref(const i64 *det) const {
        const int ic = find_bit_excit_level(ilut_ref.data(), det);
        if (ic == 0 || ic > 2) return 0.0;
        return helement(ilut_ref.data(), det);
    }

    // ------------------------------------------ real-space Hubbard excitgen
    // lattice get_spinorb_neighbors: same-spin spin orbitals of the
    // neighbouring sites.
    void spinorb_neighbours(int src, std::vector<int> &out) const {
        out.clear();
        const int site = gtID(src);
        for (int k = 0; k < sys.max_neighbours; ++k) {
            const int n = neighbours[(size_t)(site - 1) * sys.max_neighbours + k];
            if (n > 0) out.push_back(is_beta(src) ? 2 * n - 1 : 2 * n);
        }
    }
    // create_cum_list_rs_hubbard (real_space_hubbard.F90:2080-2150).
    void create_cum_list(const i64 *ilut, const std::vector<int> &nI, int src,
                         const std::vector<int> &neigh, std::vector<double> &cum, double &cum_sum) const {
        cum.assign(neigh.size(), 0.0);
        cum_sum = 0.0;
        for (size_t i = 0; i < neigh.size(); ++i) {
            double elem = 0.0;
            if (!orb_occ(ilut, neigh[i])) elem = std::fabs(get_tmat(src, neigh[i]));
            cum_sum += elem;
            cum[i] = cum_sum;
        }
        (void)nI;
    }
    // calc_pgen_rs_hubbard (real_space_hubbard.F90:2035-2078).
    double calc_pgen_rs_hubbard(const i64 *ilut, int src, int tgt, int ic) const {
        if (ic != 1) return 0.0;
        std::vector<int> nI, neigh;
        decode_bit_det(ilut, nI);
        spinorb_neighbours(src, neigh);
        double cum_sum = 0.0, cpt = 0.0;
        for (int n : neigh) {
            double elem = 0.0;
            if (!orb_occ(ilut, n)) elem = std::fabs(get_tmat(src, n));
            cum_sum += elem;
            if (n == tgt) cpt = elem;
        }
        if (cum_sum < 1e-10) return 0.0;
        return (1.0 / (double)sys.nel) * (cpt / cum_sum);
    }

    // Excitation generated in precision Real (double: the FP64 path, float:
    // the mixed-precision spawn amplitudes).
    template <typename Real>
    struct Gen {
        std::vector<int> nJ;
        int ic = 0;
        int ex[2][2] = {{0, 0}, {0, 0}};
        bool par = false;
        Real pgen = 0;
        Real invp = 0;  // 1/pgen as the product of reciprocal factors
        Real hel = 0;
    };
    template <typename Real>
    static Real prm(double d) { return sizeof(Real) == 8 ? (Real)d : (Real)(float)d; }
    double tmat_d(int i, int j) const { return get_tmat(i, j); }
    float tmat_f(int i, int j) const { return (float)get_tmat(i, j); }
    template <typename Real> Real tmat_r(int i, int j) const;
    template <typename Real> Real umat_r(int i, int j, int k, int l) const;
    // sltcnd_1_kernel / sltcnd_2_kernel in precision Real (same order).
    template <typename Real>
    Real sltcnd_1_r(const std::vector<int> &nI, int src, int tgt) const {
        Real hel = 0;
        const int id1 = gtID(src), id2 = gtID(tgt);
        if (is_beta(src) == is_beta(tgt)) {
            for (int o : nI)
                if (o != src) hel += (Real)coul_exch(id1, id2, o, is_beta(src) == is_beta(o));
        }
        hel += tmat_r<Real>(src, tgt);
        return hel;
    }
    template <typename Real>
    Real sltcnd_2_r(const int ex[2][2]) const {
        const int i = ex[0][0], j = ex[0][1], a = ex[1][0], b = ex[1][1];
        Real hel = 0;
        if (is_beta(i) == is_beta(a) && is_beta(j) == is_beta(b)) hel = umat_r<Real>(gtID(i), gtID(j), gtID(a), gtID(b));
        if (is_beta(i) == is_beta(b) && is_beta(j) == is_beta(a)) hel -= umat_r<Real>(gtID(i), gtID(j), gtID(b), gtID(a));
        return hel;
    }
    template <typename Real>
    Real offdiag_from_ex_r(const std::vector<int> &nI, int ic, const int ex[2][2], bool tParity) const {
        Real hel = 0;
        if (sys.system == NECI_SYS_HUBBARD_REAL_SPACE) {
            if (ic == 1) hel = tmat_r<Real>(ex[0][0], ex[1][0]);
            else return 0;
        } else {
            if (ic == 1) hel = sltcnd_1_r<Real>(nI, ex[0][0], ex[1][0]);
            else if (ic == 2) hel = sltcnd_2_r<Real>(ex);
            else return 0;
        }
        return tParity ? -hel : hel;
    }

    // gen_excit_rs_hubbard (real_space_hubbard.F90:1938-2030) with
    // pick_from_cum_list (lattice_models_utils.F90:150).
    template <typename Real>
    bool gen_excit_rs_hubbard(const i64 *ilut, const std::vector<int> &nI, Stream &rng, Gen<Real> &g) const {
        const int nel = sys.nel;
        g.ic = 1;
        const int elec = 1 + (int)uniform_index(rng, (u32)nel);
        const double p_elec = 1.0 / (double)nel;
        const int src = nI[elec - 1];
        std::vector<int> neigh;
        spinorb_neighbours(src, neigh);
        std::vector<double> cum;
        double cum_sum;
        create_cum_list(ilut, nI, src, neigh, cum, cum_sum);
        if (cum_sum < 1e-10) { g.pgen = 0; return false; }
        const double r = rng.next() * cum_sum;
        int ind = (int)cum.size();  // binary_search_first_ge
        for (size_t i = 0; i < cum.size(); ++i)
            if (cum[i] >= r) { ind = (int)i + 1; break; }
        double p_orb;
        if (ind == 1) p_orb = cum[0] / cum_sum;
        else p_orb = (cum[ind - 1] - cum[ind - 2]) / cum_sum;
        const int orb = neigh[ind - 1];
        const double pg = p_elec * p_orb;
        g.pgen = (Real)pg;
        g.invp = (Real)(1.0 / pg);
        int e[2];
        make_single(nI, g.nJ, elec, orb, e, g.par);
        g.ex[0][0] = e[0]; g.ex[1][0] = e[1];
        g.hel = offdiag_from_ex_r<Real>(nI, 1, g.ex, g.par);
        return true;
    }

    // CreateSingleExcit (GenRandSymExcitNUMod.F90:1118-1243), C1 symmetry,
    // tCycleOrbs = .false.: the electron by rejection.  The hole is uniform
    // over the unoccupied orbitals of the electron's spin, as the reference's
    // rejection loop makes it (a uniform orbital of that spin, drawn again
    // while occupied), but drawn as an index into those orbitals: one draw
    // where the loop takes a variable number, the same distribution and pgen.
    // pgen returned including pSingles (UniformSingles_t / gen_exc_sd).
    template <typename Real>
    bool create_single_excit(const i64 *ilut, const std::vector<int> &nI, Stream &rng, Gen<Real> &g) const {
        const int nel = sys.nel, norbs = sys.nbasis / 2;
        g.ic = 1;
        int nocc[2] = {0, 0};  // [alpha, beta]
        for (int o : nI) nocc[is_beta(o) ? 1 : 0]++;
        const int nunocc[2] = {norbs - nocc[0], norbs - nocc[1]};
        int elecs_wno = 0;
        for (int o : nI) if (nunocc[is_beta(o) ? 1 : 0] == 0) ++elecs_wno;
        if (elecs_wno == nel) { g.pgen = 0; return false; }
        int eleci = 0, ispn = 0, nexcit = 0;
        for (int attempts = 0; attempts <= 250; ++attempts) {
            eleci = (int)uniform_index(rng, (u32)nel) + 1;
            ispn = is_beta(nI[eleci - 1]) ? 2 : 1;
            nexcit = nunocc[ispn - 1];
            if (nexcit != 0) break;
        }
        if (nexcit == 0) { g.pgen = 0; return false; }
        // the c-th (0-based) unoccupied orbital of spin ispn, in increasing order
        const int c = (int)uniform_index(rng, (u32)nexcit);
        int orb = 0, seen = 0;
        for (int p = 1; p <= norbs && !orb; ++p) {
            const int o = 2 * p - (ispn - 1);
            if (orb_occ(ilut, o)) continue;
            if (seen == c) orb = o;
            ++seen;
        }
        if (!orb) { g.pgen = 0; return false; }
        int e[2];
        make_single(nI, g.nJ, eleci, orb, e, g.par);
        g.ex[0][0] = e[0]; g.ex[1][0] = e[1];
        const int count = nexcit * (nel - elecs_wno);
        if (sizeof(Real) == 8) {
            g.pgen = (Real)(sys.p_singles / (double)count);
            g.invp = (Real)((double)count * (1.0 / sys.p_singles));
        } else {
            g.pgen = (Real)((float)sys.p_singles / (float)count);
            g.invp = (Real)((float)count * (float)(1.0 / sys.p_singles));
        }
        g.hel = offdiag_from_ex_r<Real>(nI, 1, g.ex, g.par);
        return true;
    }
    // Electron pair positions of triangular index idx: ceiling((1+sqrt(9+8
    // idx))/2) of pick_biased_elecs, in integers.
    static void tri_pair(int idx, int &a1, int &a2) {
        int a = 2;
        while (a * (a - 1) / 2 <= idx) ++a;
        a1 = a;
        a2 = idx + 1 - ((a - 1) * (a - 2)) / 2;
    }
    // pick_biased_elecs (excit_gens_int_weighted.F90:722-830) without pAA:
    // parallel pair with probability pParallel, then a uniform pair index.
    template <typename Real>
    void pick_biased_elecs(const std::vector<int> &nI, Stream &rng, int elecs[2], int src[2], Real &pgen, Real &invp) const {
        const int aa = nOccAlpha * (nOccAlpha - 1) / 2;
        const int bb = nOccBeta * (nOccBeta - 1) / 2;
        const int par = aa + bb;
        const int ab = nOccAlpha * nOccBeta;
        int al_req, be_req, al_num[2] = {0, 0}, be_num[2] = {0, 0};
        if (rng.next64() < prob_thresh(sys.p_parallel)) {
            const int idx = (int)uniform_index(rng, (u32)par);
            if (idx < aa) {
                al_req = 2; be_req = 0;
                tri_pair(idx, al_num[0], al_num[1]);
            } else {
                al_req = 0; be_req = 2;
                tri_pair(idx - aa, be_num[0], be_num[1]);
            }
            if (sizeof(Real) == 8) pgen = (Real)(sys.p_parallel / (double)par);
            else pgen = (Real)((float)sys.p_parallel / (float)par);
            invp = prm<Real>((double)par / sys.p_parallel);
        } else {
            al_req = 1; be_req = 1;
            const int idx = (int)uniform_index(rng, (u32)ab);
            al_num[0] = 1 + idx % nOccAlpha;
            be_num[0] = 1 + idx / nOccAlpha;
            if (sizeof(Real) == 8) pgen = (Real)((1.0 - sys.p_parallel) / (double)ab);
            else pgen = (Real)((1.0f - (float)sys.p_parallel) / (float)ab);
            invp = prm<Real>((double)ab / (1.0 - sys.p_parallel));
        }
        int al_count = 0, be_count = 0, found = 0;
        for (int i = 1; i <= sys.nel; ++i) {
            if (!is_beta(nI[i - 1])) {
                ++al_count;
                if (al_req > 0 && al_count == al_num[al_req - 1]) { elecs[found++] = i; --al_req; }
            } else {
                ++be_count;
                if (be_req > 0 && be_count == be_num[be_req - 1]) { elecs[found++] = i; --be_req; }
            }
            if (al_req == 0 && be_req == 0) break;
        }
        src[0] = nI[elecs[0] - 1];
        src[1] = nI[elecs[1] - 1];
    }

    // fuseIndex (lib/util_mod.fpp:432).
    static i64 fuse_index(i64 x, i64 y) { return x < y ? x + y * (y - 1) / 2 : y + x * (x - 1) / 2; }

    // init_AliasTable_t (aliasSampling.F90:209-297).
    void init_alias(const std::vector<double> &arr, double *bias, int32_t *alias) const {
        const int n = (int)arr.size();
        double s = 0.0;
        for (double v : arr) s += v;
        for (int i = 0; i < n; ++i) { bias[i] = arr[i] / s * (double)n; alias[i] = 0; }
        std::vector<int> over(n), under(n);
        int cV = 0, cU = 0;
        auto assign = [&](int i) {  // i 1-based
            if (bias[i - 1] > 1.0) over[cV++] = i; else under[cU++] = i;
        };
        for (int i = 1; i <= n; ++i) assign(i);
        std::reverse(over.begin(), over.begin() + cV);
        while (cV != 0 && cU != 0) {
            const int i = over[cV - 1];
            const int j = under[cU - 1];
            alias[j - 1] = i;
            bias[i - 1] = bias[i - 1] + bias[j - 1] - 1.0;
            --cU; --cV;
            assign(i);
        }
        for (int k = 0; k < cV; ++k) { bias[over[k] - 1] = 1.0; alias[over[k] - 1] = over[k]; }
        for (int k = 0; k < cU; ++k) { bias[under[k] - 1] = 1.0; alias[under[k] - 1] = under[k]; }
    }

    // GAS_doubles_PCHB_compute_samplers for one supergroup (FCI), spatial
    // orbital resolved, FAST_FAST holes
    // (gasci_pchb_doubles_spatorb_fastweighted.fpp compute_samplers).
    int init_pchb() {
        nBI = sys.nbasis / 2;
        ijMax = fuse_index(nBI, nBI);
        abMax = ijMax;
        tgt1.assign(abMax + 1, 0);
        tgt2.assign(abMax + 1, 0);
        for (int a = 1; a <= nBI; ++a)
            for (int b = 1; b <= a; ++b) {
                const i64 ab = fuse_index(a, b);
                tgt1[ab] = b;
                tgt2[ab] = a;
            }
        pexch.assign(ijMax, 0.0);
        std::vector<double> pnoexch(ijMax, 0.0);
        alias_bias.assign((size_t)ijMax * 3 * abMax, 0.0);
        alias_alias.assign((size_t)ijMax * 3 * abMax, 0);
        alias_prob.assign((size_t)ijMax * 3 * abMax, 0.0);
        alias_present.assign((size_t)ijMax * 3, 0);
        std::vector<double> w(abMax);
        auto to_spin_orb = [](int orb, bool is_alpha) { return is_alpha ? 2 * orb : 2 * orb - 1; };
        for (int i_exch = 1; i_exch <= 3; ++i_exch) {
            for (int i = 1; i <= nBI; ++i) {
                for (int j = i; j <= nBI; ++j) {
                    if (i_exch == 1 && i == j) continue;
                    const i64 ij = fuse_index(i, j);
                    std::fill(w.begin(), w.end(), 0.0);
                    int ex[2][2];
                    ex[0][0] = to_spin_orb(i, true);
                    ex[0][1] = to_spin_orb(j, i_exch == 1);
                    for (int a = 1; a <= nBI; ++a) {
                        ex[1][0] = to_spin_orb(a, i_exch == 1 || i_exch == 2);
                        if (ex[1][0] == ex[0][0] || ex[1][0] == ex[0][1]) continue;
                        for (int b = a; b <= nBI; ++b) {
                            if (i_exch == 3 && a == b) continue;
                            const i64 ab = fuse_index(a, b);
                            ex[1][1] = to_spin_orb(b, i_exch == 1 || i_exch == 3);
                            if (ex[1][1] == ex[0][0] || ex[1][1] == ex[0][1] || ex[1][1] == ex[1][0]) continue;
                            w[ab - 1] = std::fabs(sltcnd_2(ex));  // get_PCHB_weight
                        }
                    }
                    double s = 0.0;
                    for (double v : w) s += v;
                    const size_t t = (size_t)(ij - 1) * 3 + (i_exch - 1);
                    if (std::fabs(s) >= 1e-10) {  // near_zero early return (aliasSampling.F90:389)
                        alias_present[t] = 1;
                        init_alias(w, &alias_bias[t * abMax], &alias_alias[t * abMax]);
                        for (i64 k = 0; k < abMax; ++k) alias_prob[t * abMax + k] = w[k] / s;
                    }
                    if (i_exch == 3) pexch[ij - 1] = s;
                    if (i_exch == 2) pnoexch[ij - 1] = s;
                }
            }
        }
        for (i64 k = 0; k < ijMax; ++k) {
            if (std::fabs(pexch[k] + pnoexch[k]) < 1e-10) pexch[k] = 0.0;
            else pexch[k] = pexch[k] / (pexch[k] + pnoexch[k]);
        }
        pchb_ready = true;
        return NECI_GPU_OK;
    }
    // sample_AliasTable_t (aliasSampling.F90:310-331) + AliasSampler_t%sample:
    // slot = int(n r) and the fraction n r - int(n r) from one 64-bit draw.
    template <typename Real>
    void alias_sample(size_t t, Stream &rng, int &ab, Real &prob) const {
        if (!alias_present[t]) { ab = 0; prob = 1; return; }
        const u64 r = rng.next64();
        const unsigned __int128 prod = (unsigned __int128)r * (unsigned __int128)(u64)abMax;
        const u64 pos0 = (u64)(prod >> 64), frac = (u64)prod;
        const u64 thr = prob_thresh(alias_bias[t * abMax + pos0]);
        if (frac < thr || thr == ~0ull) ab = (int)pos0 + 1;
        else ab = alias_alias[t * abMax + pos0];
        const double pr = alias_prob[t * abMax + ab - 1];
        prob = (Real)pr;  // single precision: the same rounding as the device copy
    }
    // GAS_doubles_PCHB_gen_exc (gasci_pchb_doubles_spatorb_fastweighted.fpp);
    // pgen returned including pDoubles.
    template <typename Real>
    bool pchb_doubles(const std::vector<int> &nI, Stream &rng, Gen<Real> &g) const {
        g.ic = 2;
        int elecs[2], src[2];
        Real pgen, invp;
        pick_biased_elecs<Real>(nI, rng, elecs, src, pgen, invp);
        // The exchange draw is taken for every pair and used for
        // opposite-spin pairs only, so that every double consumes the same
        // number of draws (the device generator runs both spin cases as one
        // instruction stream).  The distribution is that of the reference.
        const u64 rx = rng.next64();
        const i64 ij = fuse_index(gtID(src[0]), gtID(src[1]));
        int spin[2] = {src[0] % 2, src[1] % 2};  // getSpinIndex: 0 alpha, 1 beta
        int type;
        if (spin[0] == spin[1]) type = 1;
        else {
            const Real pe = (Real)pexch[ij - 1];
            if (rx < prob_thresh(pexch[ij - 1])) {
                type = 3;
                pgen *= pe;
                invp *= prm<Real>(1.0 / pexch[ij - 1]);
                std::swap(spin[0], spin[1]);
            } else {
                type = 2;
                pgen *= ((Real)1 - pe);
                invp *= prm<Real>(1.0 / (1.0 - pexch[ij - 1]));
            }
        }
        int ab;
        Real pholes;
        const size_t tab = (size_t)(ij - 1) * 3 + (type - 1);
        alias_sample<Real>(tab, rng, ab, pholes);
        if (ab == 0) { g.pgen = 0; return false; }
        int orbs[2] = {2 * tgt1[ab] - spin[0], 2 * tgt2[ab] - spin[1]};
        bool invalid = orbs[0] == 0 || orbs[1] == 0;
        for (int o : nI) if (o == orbs[0] || o == orbs[1]) invalid = true;
        if (!invalid && !(pholes > (Real)1e-10)) invalid = true;
        if (invalid) { g.pgen = 0; return false; }
        make_double(nI, g.nJ, elecs[0], elecs[1], orbs[0], orbs[1], g.ex, g.par);
        pgen *= pholes;
        if (sizeof(Real) == 8) g.pgen = pgen * (Real)(1.0 - sys.p_singles);
        else g.pgen = pgen * (Real)(1.0f - (float)sys.p_singles);
        invp *= prm<Real>(1.0 / alias_prob[tab * abMax + ab - 1]);
        g.invp = invp * prm<Real>(1.0 / (1.0 - sys.p_singles));
        g.hel = offdiag_from_ex_r<Real>(nI, 2, g.ex, g.par);
        return true;
    }
    // Uniform generator (gen_rand_excit) without spatial symmetry: the pgen of
    // a double from CreateDoubExcit's counts for electron-pair spin case iSpn
    // (1 beta/beta, 2 alpha/beta, 3 alpha/alpha).  FindDoubleProb
    // (GenRandSymExcitNUMod.F90:208) with FindNumForbiddenOrbsNoSym (:380),
    // PickAOrb's NExcit (:669) and PickBOrb's NExcit/NExcitOtherWay (:222).
    double uniform_double_pgen(int ispn, int &nexcit_a, int &forbidden, int &nexcit_b, int &other,
                               int spin_a_ms) const {
        const int norbs = sys.nbasis / 2, nel = sys.nel;
        const int cc[2] = {norbs - nOccAlpha, norbs - nOccBeta};  // ClassCountUnocc2: alpha, beta
        forbidden = 0;
        if (ispn == 2) {
            if (cc[0] == 0) forbidden = cc[1];
            if (cc[1] == 0) forbidden += cc[0];
            nexcit_a = sys.nbasis - nel;
            if (spin_a_ms == -1) { nexcit_b = cc[0]; other = cc[1]; }
            else { nexcit_b = cc[1]; other = cc[0]; }
        } else if (ispn == 1) {
            if (cc[1] == 1) forbidden = 1;
            nexcit_a = norbs - nOccBeta;
            nexcit_b = cc[1] - 1; other = cc[1] - 1;
        } else {
            if (cc[0] == 1) forbidden = 1;
            nexcit_a = norbs - nOccAlpha;
            nexcit_b = cc[0] - 1; other = cc[0] - 1;
        }
        if (nexcit_a == forbidden || nexcit_b <= 0 || other <= 0) return 0.0;
        const int elec_pairs = nel * (nel - 1) / 2;
        return p_doubles * ((1.0 / (double)nexcit_b) + (1.0 / (double)other)) /
               (double)(elec_pairs * (nexcit_a - forbidden));
    }
    // IsAOrbSymAllowed (GenRandSymExcitNUMod.F90:873) with tNoSymGenRandExcits.
    bool a_orb_allowed(int ispn, int spin_a_ms) const {
        const int norbs = sys.nbasis / 2;
        const int cc[2] = {norbs - nOccAlpha, norbs - nOccBeta};
        if (ispn == 2) return spin_a_ms == 1 ? cc[1] != 0 : cc[0] != 0;
        if (ispn == 1) return cc[1] != 1;
        return cc[0] != 1;
    }
    // CreateDoubExcit (GenRandSymExcitNUMod.F90:155-205), C1, tCycleOrbs =
    // .false.; where NECI stops the run (a rejection loop past its limit) the
    // attempt makes no child.
    template <typename Real>
    bool create_doub_excit(const i64 *ilut, const std::vector<int> &nI, Stream &rng, Gen<Real> &g) const {
        g.ic = 2;
        const int nel = sys.nel, nbasis = sys.nbasis, norbs = nbasis / 2;
        const int elec_pairs = nel * (nel - 1) / 2;
        // PickElecPair (:954-1025)
        const int ind = (int)uniform_index(rng, (u32)elec_pairs) + 1;
        const int X = elec_pairs - ind;
        const int K = (int)((std::sqrt(8.0 * (double)X + 1.0) - 1.0) / 2.0);
        const int elec1 = nel - 1 - K;
        const int elec2 = nel - X + (K * (K + 1)) / 2;
        const int orb1 = nI[elec1 - 1], orb2 = nI[elec2 - 1];
        const int ms1 = is_beta(orb1) ? -1 : 1, ms2 = is_beta(orb2) ? -1 : 1;
        const int ispn = ms1 * ms2 == -1 ? 2 : (ms1 == 1 ? 3 : 1);
        int nexcit_a, forbidden, nb_, no_;
        uniform_double_pgen(ispn, nexcit_a, forbidden, nb_, no_, 1);
        // PickAOrb (:669-869)
        if (nexcit_a == forbidden) { g.pgen = 0; return false; }
        int orb_a = 0, spin_a = 0;
        for (int overall = 0;; ++overall) {
            if (nexcit_a - forbidden <= 3) {
                const int chosen = (int)uniform_index(rng, (u32)(nexcit_a - forbidden)) + 1;
                int z = 1;
                if (ispn == 2) {
                    for (int i = 0; i < nbasis && !orb_a; ++i) {
                        if (orb_occ(ilut, i + 1)) continue;
                        spin_a = is_beta(i + 1) ? -1 : 1;
                        if (a_orb_allowed(ispn, spin_a)) {
                            if (z == chosen) orb_a = i + 1;
                            ++z;
                        }
                    }
                } else {
                    for (int i = 1; i <= norbs && !orb_a; ++i) {
                        const int o = ispn == 1 ? 2 * i - 1 : 2 * i;
                        if (!orb_occ(ilut, o) && a_orb_allowed(ispn, 0)) {
                            if (z == chosen) orb_a = o;
                            ++z;
                        }
                    }
                }
                if (!orb_a) { g.pgen = 0; return false; }
                break;  // NECI returns here, without the check below
            }
            int attempts = 0, chosen;
            while (true) {
                if (ispn == 2) {
                    chosen = (int)uniform_index(rng, (u32)nbasis) + 1;
                } else {
                    chosen = (int)uniform_index(rng, (u32)norbs) + 1;
                    chosen = ispn == 1 ? 2 * chosen - 1 : 2 * chosen;
                }
                if (!orb_occ(ilut, chosen)) break;
                if (attempts > 250) { g.pgen = 0; return false; }
                ++attempts;
            }
            orb_a = chosen;
            if (ispn == 2) spin_a = is_beta(orb_a) ? -1 : 1;
            if (a_orb_allowed(ispn, spin_a)) break;
            if (overall > nbasis * 20) { g.pgen = 0; return false; }
        }
        // PickBOrb (:222-378), METHOD 2
        int spin_b;  // 1 alpha, 2 beta
        if (ispn == 2) spin_b = spin_a == -1 ? 1 : 2;
        else spin_b = ispn == 1 ? 2 : 1;
        int orb_b, attempts = 0;
        while (true) {
            const int chosen = (int)uniform_index(rng, (u32)norbs);
            orb_b = 2 * (chosen + 1) - (spin_b - 1);
            if (!orb_occ(ilut, orb_b) && orb_b != orb_a) break;
            if (attempts > 1000) { g.pgen = 0; return false; }
            ++attempts;
        }
        make_double(nI, g.nJ, elec1, elec2, orb_a, orb_b, g.ex, g.par);
        const double pg = uniform_double_pgen(ispn, nexcit_a, forbidden, nb_, no_, spin_a);
        g.pgen = (Real)pg;
        g.invp = prm<Real>(1.0 / pg);
        g.hel = offdiag_from_ex_r<Real>(nI, 2, g.ex, g.par);
        return true;
    }

    // gen_exc_sd (excitation_generators.F90:110-133) with UniformSingles_t;
    // gen_rand_excit (GenRandSymExcitNUMod.F90:120-147) for the uniform generator.
    template <typename Real>
    bool generate_excitation(const i64 *ilut, const std::vector<int> &nI, Stream &rng, Gen<Real> &g) const {
        if (sys.excitgen == NECI_EXGEN_RS_HUBBARD) return gen_excit_rs_hubbard<Real>(ilut, nI, rng, g);
        if (sys.excitgen == NECI_EXGEN_UNIFORM) {
            if (rng.next64() < prob_thresh(p_doubles)) return create_doub_excit<Real>(ilut, nI, rng, g);
            return create_single_excit<Real>(ilut, nI, rng, g);
        }
        if (rng.next64() < prob_thresh(sys.p_singles)) return create_single_excit<Real>(ilut, nI, rng, g);
        return pchb_doubles<Real>(nI, rng, g);
    }

    // ------------------------------------------------------------- rows
    i64 *row(i64 j) { return &CurrentDets[(size_t)j * R]; }
    const i64 *row(i64 j) const { return &CurrentDets[(size_t)j * R]; }
    double get_sign(const i64 *r, int run) const { return as_double(r[W + run]); }
    void set_sign(i64 *r, int run, double v) const { r[W + run] = as_word(v); }
    i64 &flags(i64 *r) const { return r[W + L]; }
    static int init_flag(int run) { return run == 0 ? NECI_FLAG_INITIATOR_1 : NECI_FLAG_INITIATOR_2; }
    static int determ_flag(int run) { return run == 0 ? NECI_FLAG_DETERMINISTIC_1 : NECI_FLAG_DETERMINISTIC_2; }
    static bool test_flag(i64 f, int b) { return ((u64)f >> b) & 1ull; }
    static void set_flag(i64 &f, int b, bool v = true) {
        if (v) f |= (i64)(1ull << b); else f &= ~(i64)(1ull << b);
    }
    bool is_unocc(const i64 *r) const {
        for (int k = 0; k < L; ++k) if (std::fabs(get_sign(r, k)) >= 1e-12) return false;
        return true;
    }
    bool is_core(const i64 *r) const { return test_flag(r[W + L], determ_flag(0)); }

    // hash_table_lookup_int_64 (hash.F90:294-341).
    bool hash_lookup(const std::vector<int> &nI, const i64 *det, i64 &slot, i64 &hash_val) const {
        hash_val = find_walker_hash(nI, (i64)HashIndex.size());
        for (int32_t ind : HashIndex[hash_val - 1])
            if (det_bit_eq(det, row(ind - 1))) { slot = ind - 1; return true; }
        return false;
    }
    // RemoveHashDet (load_balancer.fpp:631-644).
    void remove_hash_det(const std::vector<int> &nI, i64 slot) {
        const i64 h = find_walker_hash(nI, (i64)HashIndex.size());
        auto &b = HashIndex[h - 1];
        for (size_t k = 0; k < b.size(); ++k)
            if (b[k] == slot + 1) { b.erase(b.begin() + k); break; }
        FreeSlot[iEndFreeSlot++] = (int32_t)slot;
        set_flag(flags(row(slot)), 0, true);  // flag_removed
    }

    // ------------------------------------------------------ spawn records
    struct Spawn {
        std::vector<i64> det;   // W words
        i64 q[2];               // fixed-point signs
        i64 flags;
    };
};

template <> inline double Oracle::tmat_r<double>(int i, int j) const { return get_tmat(i, j); }
template <> inline float Oracle::tmat_r<float>(int i, int j) const { return (float)get_tmat(i, j); }
template <> inline double Oracle::umat_r<double>(int i, int j, int k, int l) const { return get_umat_el(i, j, k, l); }
template <> inline float Oracle::umat_r<float>(int i, int j, int k, int l) const { return (float)get_umat_el(i, j, k, l); }

struct IterRun;
std::vector<Oracle::Spawn> compress_list(const Oracle &o, const neci_gpu_iter_params &p, std::vector<Oracle::Spawn> &sp,
                                         double *nannihil);

// ===========================================================================
// One iteration (PerformFCIMCycPar, FciMCPar.F90:1177-1920).
// ===========================================================================
struct IterRun {
    Oracle &o;
    const neci_gpu_iter_params &p;
    neci_gpu_iter_stats &st;
    std::vector<Oracle::Spawn> spawns;
    std::vector<double> partial;  // core vector (L per core det)
    int err = 0;
    // spawns whose parents feed the 2-RDM
    struct RdmEvent {
        std::vector<i64> child, parent;
        int run;
        double w;
    };
    std::vector<RdmEvent> rdm_events;

    // The unbiasing weight of a spawn's parent: sign(C_i) / (AvMCExcits p_gen
    // P(spawn != 0)), the role of calc_rdmbiasfac (rdm_general.fpp:1039) for a
    // per-spawn estimator; aq is |n| in fixed point before rounding.
    double rdm_parent_weight(double invp, u64 aq, bool neg) const {
        double inv_pnz = 1.0;
        if (p.t_all_real_coeff) {
            const u64 cutoff_q = (u64)std::llrint(std::ldexp(p.real_spawn_cutoff, NECI_SPAWN_FIXED_BITS));
            if (p.t_real_spawn_cutoff && aq < cutoff_q) inv_pnz = (double)cutoff_q / (double)aq;
        } else if (aq < (1ull << 32)) {
            inv_pnz = 4294967296.0 / (double)aq;
        }
        const double w = (invp * (1.0 / p.av_mc_excits)) * inv_pnz;
        return neg ? -w : w;
    }
    // Add_RDM_From_IJ_Pair (rdm_filling.F90:696-767): nI the ket (parent),
    // nJ the bra (child); singles via fill_spawn_rdm_singles (:791-817).
    void rdm_add_pair(const std::vector<int> &nI, const std::vector<int> &nJ, double c) {
        int ex[2][2] = {{0, 0}, {0, 0}};
        bool tParity = false;
        const int ic = o.get_excitation(nI, nJ, ex, tParity);
        const double full = tParity ? -c : c;
        const i64 np = o.npair;
        if (ic == 1) {
            const int i = ex[0][0], a = ex[1][0];
            for (int k : nI) {
                if (k < i && k < a) o.rdm2[Oracle::rdm_pair(k, a) * np + Oracle::rdm_pair(k, i)] += full;
                else if (k < i && k > a) o.rdm2[Oracle::rdm_pair(a, k) * np + Oracle::rdm_pair(k, i)] += -full;
                else if (k > i && k < a) o.rdm2[Oracle::rdm_pair(k, a) * np + Oracle::rdm_pair(i, k)] += -full;
                else if (k > i && k > a) o.rdm2[Oracle::rdm_pair(a, k) * np + Oracle::rdm_pair(i, k)] += full;
            }
        } else if (ic == 2) {
            o.rdm2[Oracle::rdm_pair(ex[1][0], ex[1][1]) * np + Oracle::rdm_pair(ex[0][0], ex[0][1])] += full;
        }
    }
    // The step's 2-RDM contributions: spawns onto determinants occupied
    // after annihilation (DiDj_Found_FillRDM, rdm_filling.F90:423-611), and
    // the diagonal C_i^1 C_i^2 (fill_spawn_rdm_diag, :769-789).
    void rdm_fill() {
        std::vector<int> nI, nJ;
        for (const RdmEvent &ev : rdm_events) {
            o.decode_bit_det(ev.child.data(), nJ);
            i64 slot, h;
            if (!o.hash_lookup(nJ, ev.child.data(), slot, h)) continue;
            const double cj = o.get_sign(o.row(slot), 1 - ev.run);
            if (cj == 0.0) continue;
            o.decode_bit_det(ev.parent.data(), nI);
            rdm_add_pair(nI, nJ, 0.5 * ev.w * cj);
        }
        // core pairs (fill_RDM_offdiag_deterministic, rdm_filling.F90:947-1111):
        // every stored off-diagonal element (i, j) of the core Hamiltonian, with
        // parent i at its amplitudes before the step and child j after it,
        // adds 1/2 (x_i^1 C_j^2 + x_i^2 C_j^1), what the two runs' spawns from
        // i onto j would add in expectation (those spawns are not made)
        for (size_t i = 0; i < o.core_slots.size(); ++i) {
            o.decode_bit_det(o.row(o.core_slots[i]), nI);
            for (i64 e = o.core_rowptr[i]; e < o.core_rowptr[i + 1]; ++e) {
                const i64 *rj = o.row(o.core_slots[o.core_col[e]]);
                const double c = 0.5 * (partial[i * 2] * o.get_sign(rj, 1) + partial[i * 2 + 1] * o.get_sign(rj, 0));
                if (c == 0.0) continue;
                o.decode_bit_det(rj, nJ);
                rdm_add_pair(nI, nJ, c);
            }
        }
        for (i64 j = 0; j < o.TotWalkers; ++j) {
            const i64 *r = o.row(j);
            const double prod = o.get_sign(r, 0) * o.get_sign(r, 1);
            if (prod == 0.0) continue;
            o.decode_bit_det(r, nI);
            for (size_t a = 1; a < nI.size(); ++a)
                for (size_t b = 0; b < a; ++b) {
                    const i64 pq = Oracle::rdm_pair(nI[b], nI[a]);
                    o.rdm2[pq * o.npair + pq] += prod;
                }
        }
    }
    IterRun(Oracle &o_, const neci_gpu_iter_params &p_, neci_gpu_iter_stats &s_) : o(o_), p(p_), st(s_) {}

    // decide_num_to_spawn (fcimc_helper.F90:2160-2174).
    static int decide_num_to_spawn(double pop, double av, Stream &rng) {
        int n = std::abs((int)(pop * av));
        if (std::fabs(std::fabs(pop * av) - (double)n) > 1e-12) {
            const double pe = std::fabs(pop * av) - (double)n;
            if (bern(rng, pe)) ++n;
        }
        return n;
    }
    // attempt_create_normal (fcimc_pointed_fns.F90:178-494): the child
    // amplitude -tau H_ij sign(C) / (p_gen AvMCExcits) in precision Real,
    // then RealSpawnCutoff rounding (x = n/cutoff taken as n * (1/cutoff)) or
    // stochastic_round (lib/util_mod.fpp:182-203); returned in fixed point.
    // attempt_create_normal (fcimc_pointed_fns.F90:178-494): the child
    // amplitude -tau H_ij sign(C) / (p_gen AvMCExcits), taken as -tau H_ij
    // sign(C) (1/p_gen) (1/AvMCExcits) in precision Real and converted to
    // fixed point; RealSpawnCutoff rounding (|n| < cutoff -> +-cutoff with
    // probability |n|/cutoff) or stochastic_round (lib/util_mod.fpp:182-203)
    // then act on the fixed-point value in integer arithmetic.
    template <typename Real>
    i64 spawn_amplitude(Real hel, Real invp, bool neg, Stream &rng, int &ovf, u64 &aq_out) const {
        const Real ww = neg ? (Real)-1 : (Real)1;
        const Real nsp = -Oracle::prm<Real>(p.tau) * hel * ww * invp * Oracle::prm<Real>(1.0 / p.av_mc_excits);
        i64 q;
        if (sizeof(Real) == 8) {
            const double sc = (double)nsp * 4294967296.0;
            if (!(std::fabs(sc) < 9.2e18)) { ovf = 1; return 0; }
            q = (i64)std::llrint(sc);
        } else {
            const float sc = (float)nsp * 4294967296.0f;
            if (!(std::fabs(sc) < 9.2e18f)) { ovf = 1; return 0; }
            q = (i64)std::llrintf(sc);
        }
        const u64 aq = (u64)(q < 0 ? -q : q);
        aq_out = aq;
        if (p.t_all_real_coeff) {
            const u64 cutoff_q = (u64)std::llrint(std::ldexp(p.real_spawn_cutoff, NECI_SPAWN_FIXED_BITS));
            if (p.t_real_spawn_cutoff && aq < cutoff_q) {
                const u64 mh = (u64)(((unsigned __int128)rng.next64() * (unsigned __int128)cutoff_q) >> 64);
                if (mh < aq) return q < 0 ? -(i64)cutoff_q : (i64)cutoff_q;
                return 0;
            }
            return q;
        }
        const u64 whole = aq >> 32, frac = aq & 0xFFFFFFFFull;
        u64 m = whole;
        if (frac != 0 && (rng.next64() >> 32) < frac) m += 1;
        const i64 v = (i64)(m << 32);
        return q < 0 ? -v : v;
    }
    template <typename Real>
    void attempt(const i64 *r, const std::vector<int> &nI, u64 dkey, int run, int a, bool neg, bool core,
                 bool semistoch, bool parent_init, int &ovf) {
        Stream rng(dkey, p.iter, P_ATTEMPT, run, (u32)a);
        Oracle::Gen<Real> g;
        if (!o.generate_excitation<Real>(r, nI, rng, g)) return;
        std::vector<i64> child(o.W);
        o.encode_bit_det(g.nJ, child.data());
        if (semistoch && core) {
            // is_core_state (semi_stoch_procs.F90:547)
            i64 slot, h;
            if (o.hash_lookup(g.nJ, child.data(), slot, h) && o.is_core(o.row(slot))) return;
        }
        if (o.tau_search) {
            // log_spawn_magnitude: the class of the excitation (singles;
            // uniform doubles; PCHB doubles by the spins of the two sources)
            int c;
            if (g.ic == 1) c = 0;
            else if (o.sys.excitgen == NECI_EXGEN_UNIFORM) c = 1;
            else c = Oracle::is_beta(g.ex[0][0]) == Oracle::is_beta(g.ex[0][1]) ? 2 : 3;
            double gam;
            if (sizeof(Real) == 8) gam = std::fabs((double)g.hel) * (double)g.invp * o.tau_factor(c);
            else gam = (double)(std::fabs((float)g.hel) * (float)g.invp * (float)o.tau_factor(c));
            if (gam > o.tau_gamma[c]) o.tau_gamma[c] = gam;
            if (c >= 2 || gam > 0.0) o.tau_cnt[c] += 1;
        }
        u64 aq = 0;
        const i64 q = spawn_amplitude<Real>(g.hel, g.invp, neg, rng, ovf, aq);
        if (q == 0) return;
        if (o.rdm) {
            RdmEvent ev;
            ev.child = child;
            ev.parent.assign(r, r + o.W);
            ev.run = run;
            ev.w = rdm_parent_weight((double)g.invp, aq, neg);
            rdm_events.push_back(ev);
        }
        // create_particle (fcimc_helper.F90:152-308)
        if ((i64)spawns.size() >= o.sys.max_spawned) { err = NECI_GPU_ERR_SPAWN_FULL; return; }
        Oracle::Spawn s;
        s.det = child;
        s.q[0] = s.q[1] = 0;
        s.q[run] = q;
        s.flags = 0;
        if (p.t_trunc_initiator && parent_init) Oracle::set_flag(s.flags, Oracle::init_flag(run));
        spawns.push_back(s);
    }
    // TestInitiator_explicit (fcimc_helper.F90:1142-1240) with
    // initiator_criterium (:1274) and no ADI / senior / initiator space.
    bool test_initiator(const i64 *r, bool is_init, double sgn, bool is_ref, bool core) const {
        const bool popInit = std::fabs(sgn) > p.initiator_walk_no;
        if (!is_init) return popInit;
        bool staticInit = is_ref;
        if (!staticInit && !(core && p.t_core_inits) && !popInit) return false;
        (void)r;
        return true;
    }

    void run() {
        const int W = o.W, L = o.L;
        const bool semistoch = !o.core_slots.empty();
        o.FreeSlot.assign(o.sys.max_walkers + 16, 0);
        o.iStartFreeSlot = 0;
        o.iEndFreeSlot = 0;
        partial.assign(o.core_slots.size() * L, 0.0);
        std::vector<i64> core_pos(semistoch ? o.TotWalkers : 0, -1);
        for (size_t c = 0; c < o.core_slots.size(); ++c) core_pos[o.core_slots[c]] = (i64)c;

        // TotParts entering the step.
        for (i64 j = 0; j < o.TotWalkers; ++j)
            for (int k = 0; k < L; ++k) st.tot_parts_old[k] += std::fabs(o.get_sign(o.row(j), k));

        std::vector<int> nI, nJ;
        // ---- loop_over_determinants (FciMCPar.F90:1294-1758)
        for (i64 j = 0; j < o.TotWalkers; ++j) {
            i64 *r = o.row(j);
            const bool core = o.is_core(r);
            double sgn[2] = {0.0, 0.0};
            for (int k = 0; k < L; ++k) sgn[k] = o.get_sign(r, k);
            if (core) for (int k = 0; k < L; ++k) partial[core_pos[j] * L + k] = sgn[k];
            if (o.is_unocc(r)) {
                if (core) continue;
                o.FreeSlot[o.iEndFreeSlot++] = (int32_t)j;
                continue;
            }
            const int exlvl = o.find_bit_excit_level(o.ilut_ref.data(), r);
            const bool is_ref = exlvl == 0;
            // CalcParentFlag_det (fcimc_helper.F90:1036-1120)
            if (p.t_trunc_initiator) {
                for (int k = 0; k < L; ++k) {
                    const bool was = Oracle::test_flag(o.flags(r), Oracle::init_flag(k));
                    const bool now = test_initiator(r, was, sgn[k], is_ref, core);
                    Oracle::set_flag(o.flags(r), Oracle::init_flag(k), now);
                }
            }
            // SumEContrib (fcimc_helper.F90:518-800)
            for (int k = 0; k < L; ++k) {
                if (is_ref) { st.hf_cyc[k] += sgn[k]; }
                st.enum_cyc[k] += o.offdiagH[j] * sgn[k];
            }
            o.decode_bit_det(r, nI);
            const u64 dkey = det_key(r, W, p.seed);
            for (int run = 0; run < L; ++run) {
                Stream rs(dkey, p.iter, P_NSPAWN, run, 0);
                const int nspawn = decide_num_to_spawn(sgn[run], p.av_mc_excits, rs);
                st.n_attempts += nspawn;
                const bool parent_init = Oracle::test_flag(o.flags(r), Oracle::init_flag(run));
                int ovf = 0;
                for (int a = 0; a < nspawn; ++a) {
                    if (p.precision == NECI_PREC_MIXED)
                        attempt<float>(r, nI, dkey, run, a, sgn[run] < 0.0, core, semistoch, parent_init, ovf);
                    else
                        attempt<double>(r, nI, dkey, run, a, sgn[run] < 0.0, core, semistoch, parent_init, ovf);
                    if (err) return;
                }
                if (ovf) { err = NECI_GPU_ERR_OVERFLOW; return; }
            }
        }
        st.n_spawned = (i64)spawns.size();

        // ---- determ_projection_no_death (semi_stoch_procs.F90:290-365):
        // y_i = -tau sum_j H_ij x_j.  A row is cut into segments of
        // core_segment_len(G) elements from its start (G from the mean row
        // length, as the engine's core kernel does).  A segment is summed in G
        // partial sums: partial l adds the segment's elements l, l+G, l+2G,
        // ... in order with fused multiply-adds, then the partials are added
        // pairwise, offsets G/2, G/4, ..., 1, into partial 0.  The segments'
        // sums are added in segment order and the total multiplied by tau.
        std::vector<double> y(partial.size(), 0.0);
        if (semistoch) {
            const size_t nc = o.core_slots.size();
            const int G = core_group_size((i64)o.core_val.size(), (i64)nc);
            const i64 S = core_segment_len(G, o.core_seg_lane);
            double part[32];
            for (size_t i = 0; i < nc; ++i) {
                const i64 r0 = o.core_rowptr[i], r1 = o.core_rowptr[i + 1];
                for (int k = 0; k < L; ++k) {
                    double tot = 0.0;
                    for (i64 s0 = r0; s0 == r0 || s0 < r1; s0 += S) {
                        const i64 s1 = std::min(s0 + S, r1);
                        for (int l = 0; l < G; ++l) {
                            part[l] = 0.0;
                            for (i64 e = s0 + l; e < s1; e += G)
                                part[l] = std::fma(-o.core_val[e], partial[o.core_col[e] * L + k], part[l]);
                        }
                        for (int off = G / 2; off > 0; off >>= 1)
                            for (int l = 0; l < off; ++l) part[l] = part[l] + part[l + off];
                        tot = s0 == r0 ? part[0] : tot + part[0];
                    }
                    y[i * L + k] = tot * p.tau;
                }
            }
        }

        // ---- CompressSpawnedList (Annihilation.F90:249-515)
        std::vector<Oracle::Spawn> comp = compress_list(o, p, spawns, st.nannihil);
        st.n_unique = (i64)comp.size();

        // ---- perform_death_all_walkers (fcimc_helper.F90:2253-2275)
        for (i64 j = 0; j < o.TotWalkers; ++j) {
            i64 *r = o.row(j);
            if (o.is_unocc(r)) continue;
            walker_death(j);
        }

        // ---- deterministic_annihilation (Annihilation.F90:930-963)
        for (size_t c = 0; c < o.core_slots.size(); ++c) {
            i64 *r = o.row(o.core_slots[c]);
            for (int k = 0; k < L; ++k) {
                const double cur = o.get_sign(r, k);
                const double sp = y[c * L + k];
                o.set_sign(r, k, sp + cur);
                st.nborn[k] += std::fabs(sp);
                if (cur * sp < 0.0) st.nannihil[k] += 2.0 * std::min(std::fabs(cur), std::fabs(sp));
            }
        }

        // ---- AnnihilateSpawnedParts (Annihilation.F90:965-1352)
        i64 TotWalkersNew = o.TotWalkers;
        for (Oracle::Spawn &s : comp) {
            o.decode_bit_det(s.det.data(), nJ);
            i64 slot = -1, h = 0;
            double ss[2] = {from_fixed(s.q[0]), from_fixed(s.q[1])};
            if (o.hash_lookup(nJ, s.det.data(), slot, h)) {
                i64 *r = o.row(slot);
                double cur[2] = {0.0, 0.0};
                for (int k = 0; k < L; ++k) cur[k] = o.get_sign(r, k);
                const bool determ = o.is_core(r);
                double sum_abs = 0.0;
                for (int k = 0; k < L; ++k) sum_abs += std::fabs(cur[k]);
                if (sum_abs >= 1e-12 || determ) {
                    for (int k = 0; k < L; ++k) {
                        if (std::fabs(cur[k]) < 1e-12 && p.t_trunc_initiator) {
                            if (!Oracle::test_flag(s.flags, Oracle::init_flag(k)) && !determ) {
                                st.naborted[k] += std::fabs(ss[k]);
                                ss[k] = 0.0;
                            }
                        }
                        if (cur[k] * ss[k] < 0.0) st.nannihil[k] += 2.0 * std::min(std::fabs(cur[k]), std::fabs(ss[k]));
                    }
                    for (int k = 0; k < L; ++k) o.set_sign(r, k, ss[k] + cur[k]);
                    if (!determ && o.is_unocc(r)) o.remove_hash_det(nJ, slot);
                }
            } else {
                if (p.t_trunc_initiator) {
                    for (int k = 0; k < L; ++k) {
                        if (!Oracle::test_flag(s.flags, Oracle::init_flag(k))) {  // test_abort_spawn
                            st.naborted[k] += std::fabs(ss[k]);
                            ss[k] = 0.0;
                        }
                    }
                }
                bool unocc = true;
                for (int k = 0; k < L; ++k) if (std::fabs(ss[k]) >= 1e-12) unocc = false;
                if (unocc) continue;
                const u64 dkey = det_key(s.det.data(), W, p.seed);
                for (int k = 0; k < L; ++k) {
                    // stochRoundSpawn (Annihilation.F90:1354-1418)
                    const double a = std::fabs(ss[k]);
                    if (a > 1e-12 && a < p.occupied_thresh) {
                        Stream rng(dkey, p.iter, P_ANN_ROUND, k, 0);
                        const double pRemove = 1.0 - a / p.occupied_thresh;
                        if (bern(rng, pRemove)) {
                            st.nremoved[k] += a;
                            ss[k] = 0.0;
                        } else {
                            st.nborn[k] += p.occupied_thresh - a;
                            ss[k] = fsign(p.occupied_thresh, ss[k]);
                        }
                    }
                }
                unocc = true;
                for (int k = 0; k < L; ++k) if (std::fabs(ss[k]) >= 1e-12) unocc = false;
                if (unocc) continue;
                // AddNewHashDet (load_balancer.fpp:514-629)
                i64 pos;
                if (o.iStartFreeSlot < o.iEndFreeSlot) {
                    pos = o.FreeSlot[o.iStartFreeSlot++];
                } else {
                    TotWalkersNew += 1;
                    pos = TotWalkersNew - 1;
                    if (TotWalkersNew >= o.sys.max_walkers) { err = NECI_GPU_ERR_LIST_FULL; return; }
                }
                i64 *r = o.row(pos);
                for (int w = 0; w < W; ++w) r[w] = s.det[w];
                for (int k = 0; k < L; ++k) o.set_sign(r, k, ss[k]);
                o.flags(r) = s.flags;
                Oracle::set_flag(o.flags(r), 0, false);
                o.diagH[pos] = o.diag_helement(nJ) - o.hii;
                o.offdiagH[pos] = o.offdiag_ref(s.det.data());
                o.HashIndex[h - 1].push_back((int32_t)pos + 1);
                st.n_new += 1;
            }
        }
        o.HolesInList = o.iStartFreeSlot >= o.iEndFreeSlot ? 0 : o.iEndFreeSlot - o.iStartFreeSlot;

        // ---- CalcHashTableStats (load_balancer.fpp:646-806)
        calc_hash_table_stats(TotWalkersNew);
        o.TotWalkers = TotWalkersNew;
        st.tot_walkers = o.TotWalkers;
        st.holes_in_list = o.HolesInList;
        st.n_core = (i64)o.core_slots.size();
        if (o.rdm) rdm_fill();
    }

    // walker_death (fcimc_helper.F90:2279-2407) + attempt_die_normal
    // (fcimc_pointed_fns.F90:573-705).
    void walker_death(i64 j) {
        const int L = o.L;
        i64 *r = o.row(j);
        const bool core = o.is_core(r);
        double sgn[2] = {0.0, 0.0}, iDie[2] = {0.0, 0.0}, copy[2] = {0.0, 0.0};
        for (int k = 0; k < L; ++k) sgn[k] = o.get_sign(r, k);
        const double Kii = o.diagH[j];
        Stream rng(det_key(r, o.W, p.seed), p.iter, P_DEATH, 0, 0);
        for (int k = 0; k < L; ++k) {
            const double fac = p.tau * (Kii - p.diag_sft[k]);
            if (o.tau_search && Kii - p.diag_sft[k] > o.tau_death) o.tau_death = Kii - p.diag_sft[k];  // log_death_magnitude
            if (fac > 2.0) err = NECI_GPU_ERR_UNSTABLE;
            if (p.t_all_real_coeff) {
                iDie[k] = fac * std::fabs(sgn[k]);
            } else {
                double rat = fac * std::fabs(sgn[k]);
                iDie[k] = std::trunc(rat);
                rat -= iDie[k];
                if (bern(rng, std::fabs(rat))) iDie[k] += std::nearbyint(fsign(1.0, rat));
            }
        }
        for (int k = 0; k < L; ++k) {
            st.ndied[k] += std::min(iDie[k], std::fabs(sgn[k]));
            st.nborn[k] += std::max(iDie[k] - std::fabs(sgn[k]), 0.0);
            copy[k] = sgn[k] - iDie[k] * fsign(1.0, sgn[k]);
        }
        bool any_nonzero = false;
        for (int k = 0; k < L; ++k) if (std::fabs(copy[k]) > 1e-12) any_nonzero = true;
        if (p.t_trunc_initiator && any_nonzero) {
            for (int k = 0; k < L; ++k) {
                if ((copy[k] > 0.0) != (sgn[k] > 0.0)) {
                    st.naborted[k] += std::fabs(copy[k]);
                    copy[k] = 0.0;
                }
            }
        }
        any_nonzero = false;
        for (int k = 0; k < L; ++k) if (std::fabs(copy[k]) > 1e-12) any_nonzero = true;
        if (any_nonzero || core) {
            for (int k = 0; k < L; ++k) o.set_sign(r, k, copy[k]);
        } else {
            std::vector<int> nI;
            o.decode_bit_det(r, nI);
            o.remove_hash_det(nI, j);
            for (int k = 0; k < L; ++k) o.set_sign(r, k, 0.0);
        }
    }

    void calc_hash_table_stats(i64 TotWalkersNew) {
        const int L = o.L;
        for (i64 i = 0; i < TotWalkersNew; ++i) {
            i64 *r = o.row(i);
            const bool determ = o.is_core(r);
            if (o.is_unocc(r) && !determ) continue;
            double cur[2] = {0.0, 0.0};
            for (int k = 0; k < L; ++k) cur[k] = o.get_sign(r, k);
            for (int k = 0; k < L; ++k) {
                if (determ) continue;
                const double a = std::fabs(cur[k]);
                if (a > 1e-12 && a < p.occupied_thresh) {
                    Stream rng(det_key(r, o.W, p.seed), p.iter, P_STATS_ROUND, k, 0);
                    const double pRemove = (p.occupied_thresh - a) / p.occupied_thresh;
                    if (bern(rng, pRemove)) {
                        st.nremoved[k] += a;
                        cur[k] = 0.0;
                        o.set_sign(r, k, 0.0);
                        if (o.is_unocc(r)) {
                            std::vector<int> nI;
                            o.decode_bit_det(r, nI);
                            o.remove_hash_det(nI, i);
                            o.HolesInList += 1;
                        }
                    } else {
                        st.nborn[k] += p.occupied_thresh - a;
                        cur[k] = fsign(p.occupied_thresh, cur[k]);
                        o.set_sign(r, k, cur[k]);
                    }
                }
            }
            bool occ = false;
            for (int k = 0; k < L; ++k) {
                st.tot_parts[k] += std::fabs(cur[k]);
                st.norm_psi_sq[k] += cur[k] * cur[k];
                if (std::fabs(cur[k]) >= 1e-12) occ = true;
            }
            if (occ || determ) st.n_occupied += 1;
            if (o.det_bit_eq(r, o.ilut_ref.data()))
                for (int k = 0; k < L; ++k) st.noat_hf[k] = cur[k];
        }
    }
};

// CompressSpawnedList (Annihilation.F90:249-515) + FindResidualParticle
// (:551-634) over a list of spawn records in fixed point.
std::vector<Oracle::Spawn> compress_list(const Oracle &o, const neci_gpu_iter_params &p, std::vector<Oracle::Spawn> &sp,
                                         double *nannihil) {
    std::vector<size_t> order(sp.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return o.ilut_lt(sp[a].det.data(), sp[b].det.data()); });
    std::vector<Oracle::Spawn> comp;
    const int L = o.L;
    size_t b0 = 0;
    while (b0 < order.size()) {
        size_t b1 = b0 + 1;
        while (b1 < order.size() && o.det_bit_eq(sp[order[b0]].det.data(), sp[order[b1]].det.data())) ++b1;
        if (b1 - b0 == 1) {
            const Oracle::Spawn &s = sp[order[b0]];
            bool zero = true;
            for (int k = 0; k < L; ++k) if (s.q[k] != 0) zero = false;
            if (!zero) comp.push_back(s);
        } else {
            Oracle::Spawn cum;
            cum.det = sp[order[b0]].det;
            cum.q[0] = cum.q[1] = 0;
            cum.flags = 0;
            for (size_t i = b0; i < b1; ++i) {
                const Oracle::Spawn &s = sp[order[i]];
                for (int k = 0; k < L; ++k) {
                    if (p.t_trunc_initiator) {
                        if (p.t_init_coherent_rule) {
                            if ((cum.q[k] != 0 && s.q[k] != 0) || Oracle::test_flag(s.flags, Oracle::init_flag(k)))
                                Oracle::set_flag(cum.flags, Oracle::init_flag(k));
                        } else if (Oracle::test_flag(s.flags, Oracle::init_flag(k))) {
                            Oracle::set_flag(cum.flags, Oracle::init_flag(k));
                        }
                    }
                    const double cs = from_fixed(cum.q[k]), ns = from_fixed(s.q[k]);
                    if (cs * ns < 0.0) nannihil[k] += 2.0 * std::min(std::fabs(cs), std::fabs(ns));
                    cum.q[k] += s.q[k];
                }
            }
            bool zero = true;
            for (int k = 0; k < L; ++k) if (cum.q[k] != 0) zero = false;
            if (!zero) comp.push_back(cum);
        }
        b0 = b1;
    }
    return comp;
}

// Inject a spawn list and run compression + death-free annihilation.
int annihilate_injected(Oracle &o, const neci_gpu_iter_params &p, const i64 *spawned, i64 n,
                        neci_gpu_iter_stats &st) {
    IterRun it(o, p, st);
    for (i64 i = 0; i < n; ++i) {
        Oracle::Spawn s;
        const i64 *r = spawned + (size_t)i * o.R;
        s.det.assign(r, r + o.W);
        s.q[0] = s.q[1] = 0;
        for (int k = 0; k < o.L; ++k) s.q[k] = to_fixed(as_double(r[o.W + k]));
        s.flags = r[o.W + o.L];
        it.spawns.push_back(s);
    }
    std::vector<Oracle::Spawn> comp = compress_list(o, p, it.spawns, st.nannihil);
    const int L = o.L;
    st.n_spawned = n;
    st.n_unique = (i64)comp.size();
    for (i64 j = 0; j < o.TotWalkers; ++j)
        for (int k = 0; k < L; ++k) st.tot_parts_old[k] += std::fabs(o.get_sign(o.row(j), k));
    // free slots = current holes (the sweep that would have found them)
    o.FreeSlot.assign(o.sys.max_walkers + 16, 0);
    o.iStartFreeSlot = 0;
    o.iEndFreeSlot = 0;
    for (i64 j = 0; j < o.TotWalkers; ++j)
        if (o.is_unocc(o.row(j)) && !o.is_core(o.row(j))) o.FreeSlot[o.iEndFreeSlot++] = (int32_t)j;
    // annihilate: reuse IterRun's code path by running it on `comp`.
    std::vector<int> nJ;
    i64 TotWalkersNew = o.TotWalkers;
    for (Oracle::Spawn &s : comp) {
        o.decode_bit_det(s.det.data(), nJ);
        i64 slot = -1, h = 0;
        double ss[2] = {from_fixed(s.q[0]), from_fixed(s.q[1])};
        if (o.hash_lookup(nJ, s.det.data(), slot, h)) {
            i64 *r = o.row(slot);
            double cur[2] = {0.0, 0.0};
            for (int k = 0; k < L; ++k) cur[k] = o.get_sign(r, k);
            const bool determ = o.is_core(r);
            double sum_abs = 0.0;
            for (int k = 0; k < L; ++k) sum_abs += std::fabs(cur[k]);
            if (sum_abs >= 1e-12 || determ) {
                for (int k = 0; k < L; ++k) {
                    if (std::fabs(cur[k]) < 1e-12 && p.t_trunc_initiator) {
                        if (!Oracle::test_flag(s.flags, Oracle::init_flag(k)) && !determ) {
                            st.naborted[k] += std::fabs(ss[k]);
                            ss[k] = 0.0;
                        }
                    }
                    if (cur[k] * ss[k] < 0.0) st.nannihil[k] += 2.0 * std::min(std::fabs(cur[k]), std::fabs(ss[k]));
                }
                for (int k = 0; k < L; ++k) o.set_sign(r, k, ss[k] + cur[k]);
                if (!determ && o.is_unocc(r)) o.remove_hash_det(nJ, slot);
            }
        } else {
            if (p.t_trunc_initiator)
                for (int k = 0; k < L; ++k)
                    if (!Oracle::test_flag(s.flags, Oracle::init_flag(k))) { st.naborted[k] += std::fabs(ss[k]); ss[k] = 0.0; }
            bool unocc = true;
            for (int k = 0; k < L; ++k) if (std::fabs(ss[k]) >= 1e-12) unocc = false;
            if (unocc) continue;
            const u64 dkey = det_key(s.det.data(), o.W, p.seed);
            for (int k = 0; k < L; ++k) {
                const double a = std::fabs(ss[k]);
                if (a > 1e-12 && a < p.occupied_thresh) {
                    Stream rng(dkey, p.iter, P_ANN_ROUND, k, 0);
                    const double pRemove = 1.0 - a / p.occupied_thresh;
                    if (bern(rng, pRemove)) { st.nremoved[k] += a; ss[k] = 0.0; }
                    else { st.nborn[k] += p.occupied_thresh - a; ss[k] = fsign(p.occupied_thresh, ss[k]); }
                }
            }
            unocc = true;
            for (int k = 0; k < L; ++k) if (std::fabs(ss[k]) >= 1e-12) unocc = false;
            if (unocc) continue;
            i64 pos;
            if (o.iStartFreeSlot < o.iEndFreeSlot) pos = o.FreeSlot[o.iStartFreeSlot++];
            else {
                TotWalkersNew += 1;
                pos = TotWalkersNew - 1;
                if (TotWalkersNew >= o.sys.max_walkers) return NECI_GPU_ERR_LIST_FULL;
            }
            i64 *r = o.row(pos);
            for (int w = 0; w < o.W; ++w) r[w] = s.det[w];
            for (int k = 0; k < L; ++k) o.set_sign(r, k, ss[k]);
            o.flags(r) = s.flags;
            Oracle::set_flag(o.flags(r), 0, false);
            o.diagH[pos] = o.diag_helement(nJ) - o.hii;
            o.offdiagH[pos] = o.offdiag_ref(s.det.data());
            o.HashIndex[h - 1].push_back((int32_t)pos + 1);
            st.n_new += 1;
        }
    }
    o.HolesInList = o.iStartFreeSlot >= o.iEndFreeSlot ? 0 : o.iEndFreeSlot - o.iStartFreeSlot;
    it.calc_hash_table_stats(TotWalkersNew);
    o.TotWalkers = TotWalkersNew;
    st.tot_walkers = o.TotWalkers;
    st.holes_in_list = o.HolesInList;
    return NECI_GPU_OK;
}

}  // namespace

// ===========================================================================
// C API (mirrors include/neci_gpu.h with an `orc_` prefix).
// ===========================================================================
extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

int32_t orc_init(void **out, const neci_gpu_system *sys) {
    if (!out || !sys) return NECI_GPU_ERR_INVALID;
    Oracle *o = new Oracle();
    o->sys = *sys;
    o->nifd = sys->nifd;
    o->W = sys->nifd + 1;
    o->L = sys->lenof_sign;
    o->R = o->W + o->L + 1;
    o->CurrentDets.assign((size_t)sys->max_walkers * o->R, 0);
    o->diagH.assign(sys->max_walkers, 0.0);
    o->offdiagH.assign(sys->max_walkers, 0.0);
    o->HashIndex.assign(sys->n_walker_hashes, {});
    o->random_hash2.assign(sys->nbasis + 1, 0);
    o->ilut_ref.assign(o->W, 0);
    // pDoubles = 1 - pSingles (CalcApproxpDoubles); gen_rand_excit's singles
    // carry 1 - pDoubles (CreateSingleExcit, GenRandSymExcitNUMod.F90:1264)
    o->p_doubles = 1.0 - sys->p_singles;
    if (sys->excitgen == NECI_EXGEN_UNIFORM) o->sys.p_singles = 1.0 - o->p_doubles;
    *out = o;
    return NECI_GPU_OK;
}
int32_t orc_free(void *h) { delete (Oracle *)h; return NECI_GPU_OK; }

int32_t orc_set_random_hash(void *h, const int32_t *rh) {
    Oracle *o = (Oracle *)h;
    for (int i = 1; i <= o->sys.nbasis; ++i) o->random_hash2[i] = rh[i - 1];
    return NECI_GPU_OK;
}
int32_t orc_set_tmat(void *h, const double *t) {
    Oracle *o = (Oracle *)h;
    o->tmat.assign(t, t + (size_t)o->sys.nbasis * o->sys.nbasis);
    return NECI_GPU_OK;
}
int32_t orc_set_umat(void *h, const double *u, int64_t n) {
    Oracle *o = (Oracle *)h;
    o->umat.assign(u, u + n);
    return NECI_GPU_OK;
}
int32_t orc_set_lattice(void *h, const int32_t *nb, int32_t nsites) {
    Oracle *o = (Oracle *)h;
    o->nsites = nsites;
    o->neighbours.assign(nb, nb + (size_t)nsites * o->sys.max_neighbours);
    return NECI_GPU_OK;
}
int32_t orc_set_reference(void *h, const int64_t *ref, double hii) {
    Oracle *o = (Oracle *)h;
    o->ilut_ref.assign(ref, ref + o->W);
    o->hii = hii;
    std::vector<int> nI;
    o->decode_bit_det(ref, nI);
    o->nOccAlpha = o->nOccBeta = 0;
    for (int x : nI) (x & 1 ? o->nOccBeta : o->nOccAlpha)++;
    return NECI_GPU_OK;
}
int32_t orc_init_pchb(void *h) { return ((Oracle *)h)->init_pchb(); }

int32_t orc_set_excit_biases(void *h, double p_singles, double p_parallel) {
    Oracle *o = (Oracle *)h;
    o->p_doubles = 1.0 - p_singles;
    o->sys.p_singles = o->sys.excitgen == NECI_EXGEN_UNIFORM ? 1.0 - o->p_doubles : p_singles;
    o->sys.p_parallel = p_parallel;
    return NECI_GPU_OK;
}
int32_t orc_set_rdm_sampling(void *h, int32_t on) {
    Oracle *o = (Oracle *)h;
    if (on && o->L != 2) return NECI_GPU_ERR_INVALID;
    if (on && o->rdm2.empty()) {
        o->npair = (i64)o->sys.nbasis * (o->sys.nbasis - 1) / 2;
        o->rdm2.assign((size_t)(o->npair * o->npair), 0.0);
    }
    o->rdm = on != 0;
    return NECI_GPU_OK;
}
int32_t orc_get_rdm(void *h, double *out, int64_t n, int32_t reset) {
    Oracle *o = (Oracle *)h;
    if ((int64_t)o->rdm2.size() != n) return NECI_GPU_ERR_INVALID;
    std::memcpy(out, o->rdm2.data(), (size_t)n * sizeof(double));
    if (reset) std::fill(o->rdm2.begin(), o->rdm2.end(), 0.0);
    return NECI_GPU_OK;
}
int32_t orc_set_tau_search(void *h, int32_t on) {
    ((Oracle *)h)->tau_search = on != 0;
    return NECI_GPU_OK;
}
int32_t orc_get_tau_stats(void *h, neci_gpu_tau_stats *out, int32_t reset) {
    Oracle *o = (Oracle *)h;
    out->gamma_sing = o->tau_gamma[0];
    out->gamma_doub = o->tau_gamma[1];
    out->gamma_par = o->tau_gamma[2];
    out->gamma_opp = o->tau_gamma[3];
    out->max_death_cpt = o->tau_death;
    out->cnt_sing = std::min<i64>(o->tau_cnt[0], 51);
    out->cnt_doub = std::min<i64>(o->tau_cnt[1], 51);
    out->cnt_par = std::min<i64>(o->tau_cnt[2], 51);
    out->cnt_opp = std::min<i64>(o->tau_cnt[3], 51);
    if (reset) {
        for (int c = 0; c < 4; ++c) { o->tau_gamma[c] = 0.0; o->tau_cnt[c] = 0; }
        o->tau_death = 0.0;
    }
    return NECI_GPU_OK;
}

int32_t orc_upload_walkers(void *h, const int64_t *ilut, int64_t nrows, const double *dh, const double *odh) {
    Oracle *o = (Oracle *)h;
    if (nrows >= o->sys.max_walkers) return NECI_GPU_ERR_LIST_FULL;
    // the engine's upload refuses the same rows: nel electrons below nBasis
    for (int64_t j = 0; j < nrows; ++j) {
        const int64_t *r = ilut + (size_t)j * o->R;
        int n = 0;
        for (int w = 0; w < o->W; ++w) {
            const u64 x = (u64)r[w];
            const int below = o->sys.nbasis - 64 * w;
            if ((below <= 0 && x) || (below > 0 && below < 64 && (x >> below))) n = -1;
            if (n >= 0) n += Oracle::popc(x);
        }
        if (n != o->sys.nel) {
            g_err = "upload: row " + std::to_string(j) + " does not hold nel electrons among the nBasis orbitals";
            return NECI_GPU_ERR_INVALID;
        }
    }
    for (auto &b : o->HashIndex) b.clear();
    std::fill(o->CurrentDets.begin(), o->CurrentDets.end(), 0);
    std::memcpy(o->CurrentDets.data(), ilut, (size_t)nrows * o->R * 8);
    std::vector<int> nI;
    for (int64_t j = 0; j < nrows; ++j) {
        const int64_t *r = o->row(j);
        o->decode_bit_det(r, nI);
        o->diagH[j] = dh ? dh[j] : o->diag_helement(nI) - o->hii;
        o->offdiagH[j] = odh ? odh[j] : o->offdiag_ref(r);
        if (!o->is_unocc(r) || o->is_core(r)) {
            const int64_t hv = o->find_walker_hash(nI, (int64_t)o->HashIndex.size());
            o->HashIndex[hv - 1].push_back((int32_t)j + 1);
        }
    }
    o->TotWalkers = nrows;
    return NECI_GPU_OK;
}
int32_t orc_download_walkers(void *h, int64_t *ilut, double *dh, double *odh, int64_t max_rows, int64_t *nrows) {
    Oracle *o = (Oracle *)h;
    int64_t n = 0;
    for (int64_t j = 0; j < o->TotWalkers; ++j) {
        const int64_t *r = o->row(j);
        if (o->is_unocc(r) && !o->is_core(r)) continue;
        if (n >= max_rows) return NECI_GPU_ERR_INVALID;
        std::memcpy(ilut + (size_t)n * o->R, r, (size_t)o->R * 8);
        if (dh) dh[n] = o->diagH[j];
        if (odh) odh[n] = o->offdiagH[j];
        ++n;
    }
    *nrows = n;
    return NECI_GPU_OK;
}
int32_t orc_iterate(void *h, const neci_gpu_iter_params *p, neci_gpu_iter_stats *st) {
    Oracle *o = (Oracle *)h;
    std::memset(st, 0, sizeof(*st));
    IterRun it(*o, *p, *st);
    it.run();
    st->err = it.err;
    return it.err;
}
int32_t orc_annihilate(void *h, const neci_gpu_iter_params *p, const int64_t *spawned, int64_t n,
                       neci_gpu_iter_stats *st) {
    Oracle *o = (Oracle *)h;
    std::memset(st, 0, sizeof(*st));
    const int e = annihilate_injected(*o, *p, spawned, n, *st);
    st->err = e;
    return e;
}
int32_t orc_compress_spawns(void *h, const neci_gpu_iter_params *p, const int64_t *spawned, int64_t n, int64_t *out,
                            int64_t *n_out, double *nannihil) {
    Oracle *o = (Oracle *)h;
    std::vector<Oracle::Spawn> sp;
    for (int64_t i = 0; i < n; ++i) {
        Oracle::Spawn s;
        const int64_t *r = spawned + (size_t)i * o->R;
        s.det.assign(r, r + o->W);
        s.q[0] = s.q[1] = 0;
        for (int k = 0; k < o->L; ++k) s.q[k] = to_fixed(as_double(r[o->W + k]));
        s.flags = r[o->W + o->L];
        sp.push_back(s);
    }
    nannihil[0] = nannihil[1] = 0.0;
    std::vector<Oracle::Spawn> comp = compress_list(*o, *p, sp, nannihil);
    for (size_t i = 0; i < comp.size(); ++i) {
        int64_t *r = out + i * o->R;
        for (int w = 0; w < o->W; ++w) r[w] = comp[i].det[w];
        for (int k = 0; k < o->L; ++k) r[o->W + k] = as_word(from_fixed(comp[i].q[k]));
        r[o->W + o->L] = comp[i].flags;
    }
    *n_out = (int64_t)comp.size();
    return NECI_GPU_OK;
}
int32_t orc_find_walker_hash(void *h, const int64_t *dets, int64_t n, int64_t len, int64_t *out) {
    Oracle *o = (Oracle *)h;
    std::vector<int> nI;
    for (int64_t i = 0; i < n; ++i) {
        o->decode_bit_det(dets + (size_t)i * o->W, nI);
        out[i] = o->find_walker_hash(nI, len);
    }
    return NECI_GPU_OK;
}
int32_t orc_excit_level(void *h, const int64_t *a, const int64_t *b, int64_t n, int32_t *out) {
    Oracle *o = (Oracle *)h;
    for (int64_t i = 0; i < n; ++i) out[i] = o->find_bit_excit_level(a + (size_t)i * o->W, b + (size_t)i * o->W);
    return NECI_GPU_OK;
}
int32_t orc_helement(void *h, const int64_t *a, const int64_t *b, int64_t n, double *out) {
    Oracle *o = (Oracle *)h;
    for (int64_t i = 0; i < n; ++i) out[i] = o->helement(a + (size_t)i * o->W, b + (size_t)i * o->W);
    return NECI_GPU_OK;
}
int32_t orc_gen_excit(void *h, const int64_t *det, int64_t n, uint64_t seed, int64_t iter, int64_t *child,
                      double *pgen, double *hel) {
    Oracle *o = (Oracle *)h;
    std::vector<int> nI, nJ;
    o->decode_bit_det(det, nI);
    const u64 dkey = det_key(det, o->W, seed);
    for (int64_t a = 0; a < n; ++a) {
        Stream rng(dkey, iter, P_ATTEMPT, 0, (u32)a);
        Oracle::Gen<double> g;
        int64_t *c = child + (size_t)a * o->W;
        for (int w = 0; w < o->W; ++w) c[w] = 0;
        if (o->generate_excitation<double>(det, nI, rng, g)) {
            o->encode_bit_det(g.nJ, c);
            pgen[a] = g.pgen;
            hel[a] = g.hel;
        } else {
            pgen[a] = 0.0;
            hel[a] = 0.0;
        }
    }
    return NECI_GPU_OK;
}
// Exact pgen of det -> child for the configured generator (get_pgen
// routines): used by the statistical excitation-generator tests.
int32_t orc_calc_pgen(void *h, const int64_t *det, const int64_t *child, double *out) {
    Oracle *o = (Oracle *)h;
    std::vector<int> nI, nJ;
    o->decode_bit_det(det, nI);
    o->decode_bit_det(child, nJ);
    int ex[2][2];
    bool par;
    const int ic = o->find_bit_excit_level(det, child);
    if (ic < 1 || ic > 2) { *out = 0.0; return NECI_GPU_OK; }
    o->get_excitation(nI, nJ, ex, par);
    if (o->sys.excitgen == NECI_EXGEN_RS_HUBBARD) {
        *out = o->calc_pgen_rs_hubbard(det, ex[0][0], ex[1][0], ic);
        return NECI_GPU_OK;
    }
    if (ic == 1) {
        // calc_pgen_symrandexcit2 singles, C1: 1/(NExcit*(nel-ElecsWNoExcits))
        const int norbs = o->sys.nbasis / 2;
        int nocc[2] = {0, 0};
        for (int x : nI) nocc[x & 1]++;
        const int nun[2] = {norbs - nocc[0], norbs - nocc[1]};
        int wno = 0;
        for (int x : nI) if (nun[x & 1] == 0) ++wno;
        const int nexcit = nun[ex[0][0] & 1];
        *out = o->sys.p_singles / (double)(nexcit * (o->sys.nel - wno));
        return NECI_GPU_OK;
    }
    if (o->sys.excitgen == NECI_EXGEN_UNIFORM) {
        // calc_pgen_symrandexcit2 doubles, C1: FindDoubleProb of the pair's spins
        const bool b0 = ex[0][0] & 1, b1 = ex[0][1] & 1;
        const int ispn = b0 != b1 ? 2 : (b0 ? 1 : 3);
        int na, forb, nb, no;
        *out = o->uniform_double_pgen(ispn, na, forb, nb, no, 1);
        return NECI_GPU_OK;
    }
    // GAS_doubles_PCHB_get_pgen (spatorb_fastweighted.fpp)
    const int aa = o->nOccAlpha * (o->nOccAlpha - 1) / 2, bb = o->nOccBeta * (o->nOccBeta - 1) / 2;
    const bool parallel = (ex[0][0] & 1) == (ex[0][1] & 1);
    double pg = parallel ? o->sys.p_parallel / (double)(aa + bb)
                         : (1.0 - o->sys.p_parallel) / (double)(o->nOccAlpha * o->nOccBeta);
    const int64_t ij = Oracle::fuse_index(Oracle::gtID(ex[0][0]), Oracle::gtID(ex[0][1]));
    const int64_t ab = Oracle::fuse_index(Oracle::gtID(ex[1][0]), Oracle::gtID(ex[1][1]));
    int type;
    if (parallel) type = 1;
    else if (((ex[0][0] & 1) == (ex[1][0] & 1)) || Oracle::gtID(ex[1][0]) == Oracle::gtID(ex[1][1])) {
        type = 2;
        pg *= (1.0 - o->pexch[ij - 1]);
    } else {
        type = 3;
        pg *= o->pexch[ij - 1];
    }
    const size_t t = (size_t)(ij - 1) * 3 + (type - 1);
    pg *= o->alias_present[t] ? o->alias_prob[t * o->abMax + ab - 1] : 0.0;
    *out = pg * (1.0 - o->sys.p_singles);
    return NECI_GPU_OK;
}
int32_t orc_cum_list_rs_hubbard(void *h, const int64_t *ilut, int32_t src, const int32_t *neigh, int32_t nn,
                                double *cum, double *cum_sum) {
    Oracle *o = (Oracle *)h;
    std::vector<int> nI, nb(neigh, neigh + nn);
    o->decode_bit_det(ilut, nI);
    std::vector<double> c;
    o->create_cum_list(ilut, nI, src, nb, c, *cum_sum);
    for (int i = 0; i < nn; ++i) cum[i] = c[i];
    return NECI_GPU_OK;
}
int32_t orc_calc_pgen_rs_hubbard(void *h, const int64_t *ilut, int32_t src, int32_t tgt, int32_t ic, double *out) {
    *out = ((Oracle *)h)->calc_pgen_rs_hubbard(ilut, src, tgt, ic);
    return NECI_GPU_OK;
}
int32_t orc_init_alias(const double *w, int64_t n, double *bias, int32_t *alias) {
    Oracle o;
    std::vector<double> arr(w, w + n);
    o.init_alias(arr, bias, alias);
    return NECI_GPU_OK;
}
int32_t orc_set_core_segment(void *h, int32_t per_lane) {
    if (per_lane < 1 || per_lane > 65536) return NECI_GPU_ERR_INVALID;
    ((Oracle *)h)->core_seg_lane = per_lane;
    return NECI_GPU_OK;
}
int32_t orc_set_core_space(void *h, const int64_t *core, int64_t n_core) {
    Oracle *o = (Oracle *)h;
    o->core_slots.clear();
    std::vector<int> nI;
    for (int64_t c = 0; c < n_core; ++c) {
        const int64_t *d = core + (size_t)c * o->W;
        o->decode_bit_det(d, nI);
        int64_t slot, hv;
        if (!o->hash_lookup(nI, d, slot, hv)) { g_err = "core determinant not in CurrentDets"; return NECI_GPU_ERR_INVALID; }
        o->core_slots.push_back(slot);
        Oracle::set_flag(o->flags(o->row(slot)), Oracle::determ_flag(0));
        if (o->L == 2) Oracle::set_flag(o->flags(o->row(slot)), Oracle::determ_flag(1));
    }
    // calc_determ_hamil_sparse (sparse_arrays.F90:426-570): rows of
    // connected core pairs; the diagonal is kept apart (core_ham_diag).
    o->core_rowptr.assign(n_core + 1, 0);
    o->core_col.clear();
    o->core_val.clear();
    o->core_diag.assign(n_core, 0.0);
    for (int64_t i = 0; i < n_core; ++i) {
        const int64_t *di = core + (size_t)i * o->W;
        for (int64_t j = 0; j < n_core; ++j) {
            const int64_t *dj = core + (size_t)j * o->W;
            const int ic = o->find_bit_excit_level(di, dj);
            if (i == j) { o->core_diag[i] = o->helement(di, dj) - o->hii; continue; }
            if (ic > 2) continue;
            const double hel = o->helement(di, dj);
            if (hel == 0.0) continue;
            o->core_col.push_back(j);
            o->core_val.push_back(hel);
        }
        o->core_rowptr[i + 1] = (int64_t)o->core_col.size();
    }
    return NECI_GPU_OK;
}
int32_t orc_core_nnz(void *h, int64_t *nnz) { *nnz = (int64_t)((Oracle *)h)->core_val.size(); return NECI_GPU_OK; }


// Sparse Hamiltonian over a list of determinants (for exact diagonalisation,
// the role of NECI's Davidson, davidson_neci.F90:65).  Two-call protocol:
// with rowptr only, counts the non-zeros; with all outputs, fills them.
int32_t orc_hamiltonian(void *h, const int64_t *dets, int64_t n, int64_t *rowptr, int64_t *cols, double *vals) {
    Oracle *o = (Oracle *)h;
    const int W = o->W;
    struct Key { std::vector<int64_t> w; bool operator==(const Key &k) const { return w == k.w; } };
    struct KH { size_t operator()(const Key &k) const { u64 x = 0; for (auto v : k.w) x = splitmix64(x ^ (u64)v); return (size_t)x; } };
    std::unordered_map<Key, int64_t, KH> index;
    index.reserve((size_t)n * 2);
    for (int64_t i = 0; i < n; ++i) index[Key{std::vector<int64_t>(dets + i * W, dets + i * W + W)}] = i;
    const bool mol = o->sys.system == NECI_SYS_MOLECULAR;
    int64_t nnz = 0;
    std::vector<int> nI;
    std::vector<int64_t> child(W);
    for (int64_t i = 0; i < n; ++i) {
        if (rowptr) rowptr[i] = nnz;
        const int64_t *d = dets + i * W;
        o->decode_bit_det(d, nI);
        std::vector<std::pair<int64_t, double>> row;
        row.push_back({i, o->helement(d, d)});
        std::vector<int> un;
        for (int orb = 1; orb <= o->sys.nbasis; ++orb) if (!o->orb_occ(d, orb)) un.push_back(orb);
        auto add = [&](void) {
            auto it = index.find(Key{child});
            if (it == index.end()) return;
            const double v = o->helement(d, child.data());
            if (v != 0.0) row.push_back({it->second, v});
        };
        auto flip = [&](int orb) { child[(orb - 1) / 64] ^= (int64_t)(1ull << ((orb - 1) % 64)); };
        for (int a : nI)
            for (int b : un) {
                if ((a & 1) != (b & 1)) continue;
                for (int w = 0; w < W; ++w) child[w] = d[w];
                flip(a); flip(b);
                add();
            }
        if (mol) {
            for (size_t x = 0; x < nI.size(); ++x)
                for (size_t y = x + 1; y < nI.size(); ++y)
                    for (size_t p = 0; p < un.size(); ++p)
                        for (size_t q = p + 1; q < un.size(); ++q) {
                            const int sa = (nI[x] & 1) + (nI[y] & 1), sb = (un[p] & 1) + (un[q] & 1);
                            if (sa != sb) continue;
                            for (int w = 0; w < W; ++w) child[w] = d[w];
                            flip(nI[x]); flip(nI[y]); flip(un[p]); flip(un[q]);
                            add();
                        }
        }
        std::sort(row.begin(), row.end());
        for (auto &e : row) {
            if (cols) { cols[nnz] = e.first; vals[nnz] = e.second; }
            ++nnz;
        }
    }
    if (rowptr) rowptr[n] = nnz;
    return (int32_t)(nnz > 2147483647 ? -1 : 0) == 0 ? NECI_GPU_OK : NECI_GPU_ERR_OVERFLOW;
}
int64_t orc_hamiltonian_nnz(void *h, const int64_t *dets, int64_t n) {
    std::vector<int64_t> rp(n + 1);
    orc_hamiltonian(h, dets, n, rp.data(), nullptr, nullptr);
    return rp[n];
}

// Philox stream access for tests: n doubles of one stream.
int32_t orc_stream(uint64_t dkey, int64_t iter, uint32_t purpose, uint32_t run, uint32_t attempt, int64_t n, double *out) {
    Stream s(dkey, iter, purpose, run, attempt);
    for (int64_t i = 0; i < n; ++i) out[i] = s.next();
    return NECI_GPU_OK;
}
uint64_t orc_det_key(const int64_t *det, int32_t W, uint64_t seed) { return det_key(det, W, seed); }
int32_t orc_philox_block(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
    Philox::block(ctr, key, out);
    return NECI_GPU_OK;
}

}  // extern "C"
