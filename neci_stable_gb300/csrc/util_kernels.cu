// util_kernels.cu -- set-up kernels (walker upload, core space, PCHB alias
// tables) and the batch kernels behind the bit-string / matrix-element entry
// points of the C ABI.
#include "engine.cuh"
#include "excitgen.cuh"
#include "internal.h"

namespace neci {

__device__ inline void set_err_u(Control *c, int code) { atomicCAS(&c->err, 0, code); }

// ---------------------------------------------------------------- batch ops
__global__ void k_util_hash(DevSys s, const long long *dets, long long n, unsigned long long len, long long *out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long d[kMaxWords];
        for (int w = 0; w < s.W; ++w) d[w] = (unsigned long long)dets[i * s.W + w];
        out[i] = (long long)hash_mod(neci_hash(d, s.W, s.random_hash2), len) + 1;
    }
}
__global__ void k_util_excit_level(DevSys s, const long long *a, const long long *b, long long n, int *out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = excit_level((const unsigned long long *)a + i * s.W, (const unsigned long long *)b + i * s.W, s.W);
}
__global__ void k_util_helement(DevSys s, const long long *a, const long long *b, long long n, double *out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long *da = (const unsigned long long *)a + i * s.W;
        const unsigned long long *db = (const unsigned long long *)b + i * s.W;
        const int ic = excit_level(da, db, s.W);
        double h = 0.0;
        if (ic == 0) h = diag_helement(s, da);
        else if (ic <= 2) h = offdiag_helement(s, da, db, ic);
        out[i] = h;
    }
}
__global__ void k_util_gen_excit(DevSys s, const long long *det, long long n, unsigned long long seed, long long iter,
                                 long long *child, double *pgen, double *hel) {
    unsigned long long d[kMaxWords];
    for (int w = 0; w < s.W; ++w) d[w] = (unsigned long long)det[w];
    const unsigned long long dkey = det_key(d, s.W, seed);
    for (long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x; a < n; a += (long long)gridDim.x * blockDim.x) {
        Stream rng(dkey, iter, P_ATTEMPT, 0, (uint32_t)a);
        Excit<double> e;
        generate_excitation<double>(s, d, s.neighbours, rng, e);
        for (int w = 0; w < s.W; ++w) child[a * s.W + w] = e.ok ? (long long)e.child[w] : 0ll;
        pgen[a] = e.ok ? e.pgen : 0.0;
        hel[a] = e.ok ? e.hel : 0.0;
    }
}

// ------------------------------------------------------------------ upload
// After the rows are copied in: diagonal elements, cleared core flags, hash.
__global__ void k_upload_fix(DevSys s, DevState st, long long nrows, int compute_diag) {
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nrows; j += (long long)gridDim.x * blockDim.x) {
        long long *r = st.dets + j * s.R;
        unsigned long long d[kMaxWords];
        for (int w = 0; w < s.W; ++w) d[w] = (unsigned long long)r[w];
        r[s.W + s.L] &= ~((1ll << NECI_FLAG_DETERMINISTIC_1) | (1ll << NECI_FLAG_DETERMINISTIC_2));
        if (compute_diag) {
            st.diagH[j] = diag_helement(s, d) - s.hii;
            const int ic = excit_level(s.ilut_ref, d, s.W);
            st.offdiagH[j] = (ic >= 1 && ic <= 2) ? offdiag_helement(s, s.ilut_ref, d, ic) : 0.0;
        }
        bool occ = false;
        for (int k = 0; k < s.L; ++k) occ = occ || fabs(word_to_double(r[s.W + k])) >= kEps12;
        if (!occ) continue;
        const unsigned long long mask = st.hash_n - 1;
        unsigned long long b = hash_bucket(neci_hash(d, s.W, s.random_hash2), st.hash_n);
        for (int p = 0; p < kProbeLimit; ++p) {
            if (atomicCAS(&st.hash[b], kEmpty, (uint32_t)(j + 1)) == kEmpty) {
                st.slot_bucket[j] = (uint32_t)b;
                break;
            }
            b = (b + 1) & mask;
            if (p == kProbeLimit - 1) set_err_u(st.ctl, NECI_GPU_ERR_HASH_FULL);
        }
    }
}

// Holes of the current list -> free list (the sweep's FreeSlot pass) for an
// injected annihilation; also resets the step counters.
__global__ void k_collect_holes(DevSys s, DevState st) {
    const long long n = slots_in_use(st);
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        const long long *r = st.dets + j * s.R;
        bool occ = false;
        for (int k = 0; k < s.L; ++k) occ = occ || fabs(word_to_double(r[s.W + k])) >= kEps12;
        if (occ || (st.n_core > 0 && is_core_flags(r[s.W + s.L]))) continue;
        const unsigned long long pos = atomicAdd(&st.ctl->n_free, 1ull);
        st.free_list[pos] = (int32_t)j;
    }
}
__global__ void k_tot_parts_old(DevSys s, DevState st) {
    const long long n = slots_in_use(st);
    double a[2] = {0.0, 0.0};
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < s.L; ++k) a[k] += fabs(word_to_double(st.dets[j * s.R + s.W + k]));
    for (int k = 0; k < s.L; ++k)
        if (a[k] != 0.0) atomicAdd(&st.ctl->tot_parts_old[k], a[k]);
}

// SpawnedParts rows with real(dp) signs -> fixed-point records.
__global__ void k_convert_spawns(DevSys s, DevState st, long long n) {
    int ovf = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        long long *r = st.spawn + i * s.R;
        for (int k = 0; k < s.L; ++k) r[s.W + k] = to_fixed(word_to_double(r[s.W + k]), &ovf);
    }
    if (ovf) set_err_u(st.ctl, NECI_GPU_ERR_OVERFLOW);
    if (blockIdx.x == 0 && threadIdx.x == 0) st.ctl->n_spawned = (unsigned long long)n;
}

// Every record is a candidate (compression without a walker list).
__global__ void k_all_cand(DevSys s, DevState st) {
    const long long n = (long long)st.ctl->n_spawned;
    unsigned long long aq[2] = {0, 0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long *r = st.spawn + i * s.R;
        unsigned long long d[kMaxWords];
        for (int w = 0; w < s.W; ++w) d[w] = (unsigned long long)r[w];
        for (int k = 0; k < s.L; ++k) {
            const long long q = r[s.W + k];
            aq[k] += (unsigned long long)(q < 0 ? -q : q);
        }
        st.cand[i] = (uint32_t)i;
        st.cand_h[i] = neci_hash(d, s.W, s.random_hash2);
    }
    for (int k = 0; k < s.L; ++k)
        if (aq[k]) atomicAdd(&st.ctl->abs_q[k], aq[k]);
    if (blockIdx.x == 0 && threadIdx.x == 0) st.ctl->n_cand = (unsigned long long)n;
}

// Compressed list rows (real(dp) signs) of the unique candidates.
__global__ void k_compress_out(DevSys s, DevState st, long long *out, unsigned long long *n_out, int trunc_init,
                               int coherent) {
    const long long n = (long long)st.ctl->n_reps;
    unsigned long long as[2] = {0, 0};
    for (long long ri = blockIdx.x * (long long)blockDim.x + threadIdx.x; ri < n; ri += (long long)gridDim.x * blockDim.x) {
        const long long ci = st.reps[ri];
        const uint32_t rb = st.rep_bucket[ri];
        if (rb != kNoBucket) st.spawn_hash[rb] = kEmpty;
        const long long *rec = st.spawn + (long long)st.cand[ci] * s.R;
        long long q[2] = {0, 0};
        uint32_t cnt[2] = {0, 0};
        for (int k = 0; k < s.L; ++k) {
            q[k] = st.rep_q[ci * s.L + k];
            cnt[k] = st.rep_cnt[ci * (s.L + 1) + k];
            st.rep_q[ci * s.L + k] = 0;
            st.rep_cnt[ci * (s.L + 1) + k] = 0;
            as[k] += (unsigned long long)(q[k] < 0 ? -q[k] : q[k]);
        }
        const uint32_t nrec = st.rep_cnt[ci * (s.L + 1) + s.L];
        st.rep_cnt[ci * (s.L + 1) + s.L] = 0;
        bool zero = true;
        for (int k = 0; k < s.L; ++k) if (q[k] != 0) zero = false;
        if (zero) continue;
        long long flags;
        if (nrec == 1) flags = rec[s.W + s.L];
        else {
            flags = 0;
            if (trunc_init)
                for (int k = 0; k < s.L; ++k) {
                    const bool coh = coherent && (cnt[k] & 0x7FFFFFFFu) >= 2u;
                    if (coh || (cnt[k] & 0x80000000u)) flags |= 1ll << init_flag_bit(k);
                }
        }
        const unsigned long long pos = atomicAdd(n_out, 1ull);
        long long *o = out + pos * s.R;
        for (int w = 0; w < s.W; ++w) o[w] = rec[w];
        for (int k = 0; k < s.L; ++k) o[s.W + k] = double_to_word(from_fixed(q[k]));
        o[s.W + s.L] = flags;
    }
    for (int k = 0; k < s.L; ++k)
        if (as[k]) atomicAdd(&st.ctl->abs_s[k], as[k]);
}

// ------------------------------------------------------------- core space
__global__ void k_core_mark(DevSys s, DevState st, const long long *core_dets, long long n_core) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n_core; c += (long long)gridDim.x * blockDim.x) {
        unsigned long long d[kMaxWords];
        for (int w = 0; w < s.W; ++w) d[w] = (unsigned long long)core_dets[c * s.W + w];
        const unsigned long long mask = st.hash_n - 1;
        unsigned long long b = hash_bucket(neci_hash(d, s.W, s.random_hash2), st.hash_n);
        long long slot = -1;
        for (int p = 0; p < kProbeLimit; ++p) {
            const uint32_t e = st.hash[b];
            if (e == kEmpty) break;
            if (e != kTomb && det_eq(d, st.dets + (long long)(e - 1) * s.R, s.W)) { slot = (long long)e - 1; break; }
            b = (b + 1) & mask;
        }
        if (slot < 0) { set_err_u(st.ctl, NECI_GPU_ERR_INVALID); continue; }
        long long f = st.dets[slot * s.R + s.W + s.L];
        f |= 1ll << NECI_FLAG_DETERMINISTIC_1;
        if (s.L == 2) f |= 1ll << NECI_FLAG_DETERMINISTIC_2;
        st.dets[slot * s.R + s.W + s.L] = f;
        st.core_of_slot[slot] = (int32_t)c;
        st.core_slot[c] = slot;
    }
}
// Clears the deterministic flags of the previous core space.  A former core
// determinant whose signs are all zero was kept only because it was in the
// core: it leaves the walker hash (RemoveHashDet) as the sweep would have
// removed it, so that its slot can become a hole.
__global__ void k_core_unmark(DevSys s, DevState st) {
    const long long n = slots_in_use(st);
    unsigned long long tomb = 0;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n; j += (long long)gridDim.x * blockDim.x) {
        long long *r = st.dets + j * s.R;
        long long f = r[s.W + s.L];
        const long long det_bits = (1ll << NECI_FLAG_DETERMINISTIC_1) | (1ll << NECI_FLAG_DETERMINISTIC_2);
        if (!(f & det_bits)) continue;
        f &= ~det_bits;
        bool occ = false;
        for (int k = 0; k < s.L; ++k) occ = occ || fabs(word_to_double(r[s.W + k])) >= kEps12;
        if (!occ) {
            st.hash[st.slot_bucket[j]] = kTomb;
            f |= 1ll;  // flag_removed
            ++tomb;
        }
        r[s.W + s.L] = f;
    }
    if (tomb) atomicAdd(&st.ctl->n_tomb, tomb);
}

// One warp per core row: connected core determinants (excitation level 1-2).
__global__ void k_core_count(DevSys s, const long long *core_dets, long long n_core, long long *counts) {
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = warp; i < n_core; i += nwarps) {
        const unsigned long long *di = (const unsigned long long *)core_dets + i * s.W;
        long long cnt = 0;
        for (long long j = lane; j < n_core; j += 32) {
            if (j == i) continue;
            const int ic = excit_level(di, (const unsigned long long *)core_dets + j * s.W, s.W);
            if (ic >= 1 && ic <= 2) {
                const double h = offdiag_helement(s, di, (const unsigned long long *)core_dets + j * s.W, ic);
                if (h != 0.0) ++cnt;
            }
        }
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        if (lane == 0) counts[i] = cnt;
    }
}
// Row i written in ascending column order (one thread per row keeps the
// order of the oracle's dense loop).
__global__ void k_core_fill(DevSys s, DevState st, const long long *core_dets, long long n_core) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_core; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long *di = (const unsigned long long *)core_dets + i * s.W;
        long long e = st.core_rowptr[i];
        for (long long j = 0; j < n_core; ++j) {
            if (j == i) continue;
            const unsigned long long *dj = (const unsigned long long *)core_dets + j * s.W;
            const int ic = excit_level(di, dj, s.W);
            if (ic < 1 || ic > 2) continue;
            const double h = offdiag_helement(s, di, dj, ic);
            if (h == 0.0) continue;
            st.core_col[e] = (int32_t)j;
            st.core_val[e] = h;
            st.core_val32[e] = (float)h;
            ++e;
        }
    }
}

// ------------------------------------------------------------ PCHB tables
// One thread per (ij, type): weights |<ij||ab>| over ab, alias table by
// init_AliasTable_t (aliasSampling.F90:209-297), probabilities w / sum(w).
// Uses alias_prob as the weight buffer and `scratch` (2*abMax ints per
// table) for the over/under-full stacks.
// Coulomb and Coulomb-minus-exchange rows of the single-excitation elements
// (the UMAT values sltcnd_1_kernel reads, laid out by (i, a) so that the sum
// over the occupied orbitals k reads one contiguous row).
__global__ void k_build_jk(DevSys s, double *jrow, double *jkrow, float *jrow32, float *jkrow32) {
    const int n = s.nBI;
    const long long total = (long long)n * n * n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(t % n) + 1, a = (int)((t / n) % n) + 1, i = (int)(t / ((long long)n * n)) + 1;
        const double j = s.umat[umat_ind(i, k, a, k) - 1], x = s.umat[umat_ind(i, k, k, a) - 1];
        const double jk = j - x;
        jrow[t] = j;
        jkrow[t] = jk;
        jrow32[t] = (float)j;
        jkrow32[t] = (float)jk;
    }
}

// The Coulomb and exchange tables of the diagonal element (DevSys::jmat, kmat).
__global__ void k_build_jkmat(DevSys s, double *jmat, double *kmat) {
    const int n = s.nBI;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)n * n;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t / n) + 1, j = (int)(t % n) + 1;
        jmat[t] = s.umat[umat_ind(i, j, i, j) - 1];
        kmat[t] = s.umat[umat_ind(i, j, j, i) - 1];
    }
}

__global__ void k_pchb_tables(DevSys s, double *bias, int32_t *alias, double *prob, uint8_t *present,
                              double *wsum, int32_t *scratch) {
    const long long ntab = s.ijMax * 3;
    const long long n = s.abMax;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntab; t += (long long)gridDim.x * blockDim.x) {
        const long long ij = t / 3 + 1;
        const int type = (int)(t % 3) + 1;
        // invert fuseIndex: ij = i + j(j-1)/2 with i <= j
        int j = 1;
        while ((long long)j * (j + 1) / 2 < ij) ++j;
        const int i = (int)(ij - (long long)j * (j - 1) / 2);
        double *w = prob + t * n;
        for (long long k = 0; k < n; ++k) w[k] = 0.0;
        if (!(type == 1 && i == j)) {
            const int e00 = 2 * i;                               // alpha
            const int e01 = (type == 1) ? 2 * j : 2 * j - 1;
            for (int a = 1; a <= s.nBI; ++a) {
                const int e10 = (type == 1 || type == 2) ? 2 * a : 2 * a - 1;
                if (e10 == e00 || e10 == e01) continue;
                for (int b = a; b <= s.nBI; ++b) {
                    if (type == 3 && a == b) continue;
                    const long long ab = (long long)a + (long long)b * (b - 1) / 2;
                    const int e11 = (type == 1 || type == 3) ? 2 * b : 2 * b - 1;
                    if (e11 == e00 || e11 == e01 || e11 == e10) continue;
                    w[ab - 1] = fabs(sltcnd_2(s, e00, e01, e10, e11));
                }
            }
        }
        double sum = 0.0;
        for (long long k = 0; k < n; ++k) sum += w[k];
        wsum[t] = sum;
        double *bs = bias + t * n;
        int32_t *al = alias + t * n;
        if (fabs(sum) < 1e-10) {
            present[t] = 0;
            for (long long k = 0; k < n; ++k) { bs[k] = 0.0; al[k] = 0; w[k] = 0.0; }
            continue;
        }
        present[t] = 1;
        for (long long k = 0; k < n; ++k) { bs[k] = w[k] / sum * (double)n; al[k] = 0; }
        int32_t *over = scratch + (t % (gridDim.x * (long long)blockDim.x)) * 2 * n;  // per-thread stacks
        int32_t *under = over + n;
        long long cV = 0, cU = 0;
        for (long long k = 1; k <= n; ++k) {
            if (bs[k - 1] > 1.0) over[cV++] = (int32_t)k; else under[cU++] = (int32_t)k;
        }
        for (long long a = 0, b = cV - 1; a < b; ++a, --b) { const int32_t x = over[a]; over[a] = over[b]; over[b] = x; }
        while (cV != 0 && cU != 0) {
            const int32_t ii = over[cV - 1];
            const int32_t jj = under[cU - 1];
            al[jj - 1] = ii;
            bs[ii - 1] = bs[ii - 1] + bs[jj - 1] - 1.0;
            --cU; --cV;
            if (bs[ii - 1] > 1.0) over[cV++] = ii; else under[cU++] = ii;
        }
        for (long long k = 0; k < cV; ++k) { bs[over[k] - 1] = 1.0; al[over[k] - 1] = over[k]; }
        for (long long k = 0; k < cU; ++k) { bs[under[k] - 1] = 1.0; al[under[k] - 1] = under[k]; }
        for (long long k = 0; k < n; ++k) w[k] = w[k] / sum;
    }
}
__global__ void k_pchb_pexch(DevSys s, const double *wsum, double *pexch, unsigned long long *pexch_thr, float *pexch32,
                             double *pexch_inv, double *pnoexch_inv, float *pexch_inv32, float *pnoexch_inv32) {
    for (long long ij = blockIdx.x * (long long)blockDim.x + threadIdx.x; ij < s.ijMax; ij += (long long)gridDim.x * blockDim.x) {
        const double ex = wsum[ij * 3 + 2], noex = wsum[ij * 3 + 1];
        const double pe = fabs(ex + noex) < 1e-10 ? 0.0 : ex / (ex + noex);
        pexch[ij] = pe;
        pexch_thr[ij] = prob_thresh(pe);
        pexch32[ij] = (float)pe;
        const double ie = 1.0 / pe, ine = 1.0 / (1.0 - pe);
        pexch_inv[ij] = ie;
        pnoexch_inv[ij] = ine;
        pexch_inv32[ij] = (float)ie;
        pnoexch_inv32[ij] = (float)ine;
    }
}
// Integer thresholds of the alias biases and single-precision probabilities.
// The slots of an empty table (no allowed ab, `present` 0) keep themselves
// (threshold ~0) and have probability 0, so a draw from one reads only its
// own slot and is rejected by the pholes > 1e-10 test: the attempt makes no
// child, as the present flag's early exit in the reference order does.
__global__ void k_pchb_derived(long long n, long long ab_max, const uint8_t *present, const double *bias,
                               const double *prob, unsigned long long *thr, float *prob32, double *inv, float *inv32) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        thr[i] = present[i / ab_max] ? prob_thresh(bias[i]) : ~0ull;
        prob32[i] = (float)prob[i];
        const double v = 1.0 / prob[i];
        inv[i] = v;
        inv32[i] = (float)v;
    }
}

// The interleaved records of the alias tables (AliasRec), from the arrays
// above; slot i's target pair is tgt_pair[i + 1].
__global__ void k_alias_rec(long long n, long long ab_max, const unsigned long long *thr, const double *prob,
                            const double *inv, const int32_t *alias, const int32_t *tgt, AliasRec *out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        AliasRec r;
        r.thr = thr[i];
        r.prob = prob[i];
        r.inv = inv[i];
        r.alias = alias[i];
        r.tgt = tgt[i % ab_max + 1];
        out[i] = r;
    }
}

// ---------------------------------------------------------------- launchers
static int gsz(const Engine &e) { return e.num_sms * 4; }

void launch_util_hash(Engine &e, const long long *dets, long long n, unsigned long long len, long long *out) {
    k_util_hash<<<gsz(e), 256, 0, e.stream>>>(e.sys, dets, n, len, out);
}
void launch_util_excit_level(Engine &e, const long long *a, const long long *b, long long n, int *out) {
    k_util_excit_level<<<gsz(e), 256, 0, e.stream>>>(e.sys, a, b, n, out);
}
void launch_util_helement(Engine &e, const long long *a, const long long *b, long long n, double *out) {
    k_util_helement<<<gsz(e), 256, 0, e.stream>>>(e.sys, a, b, n, out);
}
void launch_util_gen_excit(Engine &e, const long long *det, long long n, unsigned long long seed, long long iter,
                           long long *child, double *pgen, double *hel) {
    k_util_gen_excit<<<gsz(e), 128, 0, e.stream>>>(e.sys, det, n, seed, iter, child, pgen, hel);
}
void launch_upload_fix(Engine &e, long long nrows, int compute_diag) {
    k_upload_fix<<<gsz(e), 128, 0, e.stream>>>(e.sys, e.st, nrows, compute_diag);
}
void launch_collect_holes(Engine &e) {
    k_collect_holes<<<gsz(e), 256, 0, e.stream>>>(e.sys, e.st);
    k_tot_parts_old<<<gsz(e), 256, 0, e.stream>>>(e.sys, e.st);
}
void launch_convert_spawns(Engine &e, long long n) { k_convert_spawns<<<gsz(e), 256, 0, e.stream>>>(e.sys, e.st, n); }
void launch_all_cand(Engine &e) { k_all_cand<<<gsz(e), 256, 0, e.stream>>>(e.sys, e.st); }
void launch_compress_out(Engine &e, long long *out, unsigned long long *n_out) {
    k_compress_out<<<gsz(e), 256, 0, e.stream>>>(e.sys, e.st, out, n_out, e.h_params->t_trunc_initiator,
                                                 e.h_params->t_init_coherent_rule);
}
void launch_core_unmark(Engine &e) { k_core_unmark<<<gsz(e), 256, 0, e.stream>>>(e.sys, e.st); }
void launch_core_mark(Engine &e, const long long *core_dets, long long n_core) {
    k_core_mark<<<gsz(e), 128, 0, e.stream>>>(e.sys, e.st, core_dets, n_core);
}
void launch_core_count(Engine &e, const long long *core_dets, long long n_core, long long *counts) {
    k_core_count<<<gsz(e), 256, 0, e.stream>>>(e.sys, core_dets, n_core, counts);
}
void launch_core_fill(Engine &e, const long long *core_dets, long long n_core) {
    k_core_fill<<<gsz(e), 128, 0, e.stream>>>(e.sys, e.st, core_dets, n_core);
}
void launch_build_jk(Engine &e, double *jrow, double *jkrow, float *jrow32, float *jkrow32) {
    const long long n = e.sys.nBI;
    const int grid = (int)std::min<long long>((n * n * n + 255) / 256, 4096);
    k_build_jk<<<grid, 256, 0, e.stream>>>(e.sys, jrow, jkrow, jrow32, jkrow32);
}
void launch_build_jkmat(Engine &e, double *jmat, double *kmat) {
    const long long n = e.sys.nBI;
    k_build_jkmat<<<(int)std::min<long long>((n * n + 255) / 256, 1024), 256, 0, e.stream>>>(e.sys, jmat, kmat);
}

int launch_pchb_build(Engine &e) {
    const long long ntab = e.sys.ijMax * 3;
    const long long n = e.sys.abMax;
    const int threads = 128;
    const long long max_threads = (long long)gsz(e) * threads;
    const long long nthreads = ntab < max_threads ? ntab : max_threads;
    const int blocks = (int)((nthreads + threads - 1) / threads);
    // the weight sums and the per-thread stacks of the alias construction
    // (hundreds of MB at 100 spatial orbitals): no kernel runs unless both
    // allocations succeeded
    double *wsum = nullptr;
    int32_t *scratch = nullptr;
    if (cudaMalloc(&wsum, ntab * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&scratch, (size_t)blocks * threads * 2 * n * sizeof(int32_t)) != cudaSuccess) {
        const cudaError_t err = cudaGetLastError();  // clears the allocation error
        if (wsum) cudaFree(wsum);
        if (scratch) cudaFree(scratch);
        return err == cudaSuccess ? (int)cudaErrorMemoryAllocation : (int)err;
    }
    k_pchb_tables<<<blocks, threads, 0, e.stream>>>(e.sys, (double *)e.sys.alias_bias, (int32_t *)e.sys.alias_alias,
                                                    (double *)e.sys.alias_prob, (uint8_t *)e.sys.alias_present, wsum,
                                                    scratch);
    k_pchb_pexch<<<gsz(e), 256, 0, e.stream>>>(e.sys, wsum, (double *)e.sys.pexch,
                                               (unsigned long long *)e.sys.pexch_thr, (float *)e.sys.pexch32,
                                               (double *)e.sys.pexch_inv, (double *)e.sys.pnoexch_inv,
                                               (float *)e.sys.pexch_inv32, (float *)e.sys.pnoexch_inv32);
    k_pchb_derived<<<gsz(e), 256, 0, e.stream>>>((long long)ntab * n, n, e.sys.alias_present, e.sys.alias_bias,
                                                 e.sys.alias_prob,
                                                 (unsigned long long *)e.sys.alias_thr, (float *)e.sys.alias_prob32,
                                                 (double *)e.sys.alias_inv, (float *)e.sys.alias_inv32);
    k_alias_rec<<<gsz(e), 256, 0, e.stream>>>((long long)ntab * n, n, e.sys.alias_thr, e.sys.alias_prob,
                                              e.sys.alias_inv, e.sys.alias_alias, e.sys.tgt_pair,
                                              (AliasRec *)e.sys.alias_rec);
    const cudaError_t err = cudaStreamSynchronize(e.stream);
    cudaFree(wsum);
    cudaFree(scratch);
    return (int)err;
}

}  // namespace neci
