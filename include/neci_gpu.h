/*
 * neci_gpu.h -- C ABI of the GB300 FCIQMC iteration engine.
 *
 * The engine replaces one NECI iteration, PerformFCIMCycPar
 * (src/FciMCPar.F90:1177-1920), behind plain C entry points: no C++ or
 * torch types, only pointers, sizes and POD structs, so that a Fortran
 * `iso_c_binding` interface (or ctypes, or cgo) binds it directly.
 *
 * Walker rows keep NECI's CurrentDets/SpawnedParts layout
 * (src/bit_rep_data.F90:10-17, src/BitReps.F90:164-200): for one determinant
 *   words [0 .. nifd]                  occupation bits (spin orbital p, 1-based,
 *                                      is bit (p-1)%64 of word (p-1)/64)
 *   words [nifd+1 .. nifd+lenof_sign]  real(dp) signs, bit-cast into int64
 *   word  [nifd+lenof_sign+1]          flag word (initiator bits 13/14,
 *                                      deterministic bits 19/20)
 * so a row is NIfTot+1 = nifd+lenof_sign+2 int64 words, and arrays of rows are
 * Fortran CurrentDets(0:NIfTot, n) in memory order.
 *
 * All host buffers are caller-allocated; the library never frees or keeps
 * host memory.  Device state (walker list, hash table, spawn buffers,
 * integrals, alias tables, core space) is owned by the context and stays
 * resident in HBM between calls.
 *
 * Every entry point returns an int32 status (NECI_GPU_OK == 0).  Positive
 * codes map onto NECI's integer `err` (src/fcimc_helper.F90:192-195,
 * src/load_balancer.fpp:540-544): the Fortran shim passes a non-zero value to
 * stop_all exactly as PerformFCIMCycPar's caller does (src/FciMCPar.F90:508).
 */
#ifndef NECI_GPU_H
#define NECI_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NECI_GPU_OK               0
#define NECI_GPU_ERR_SPAWN_FULL   1  /* SpawnedParts full: fcimc_helper.F90:483-510       */
#define NECI_GPU_ERR_LIST_FULL    2  /* CurrentDets full: load_balancer.fpp:540-544       */
#define NECI_GPU_ERR_HASH_FULL    3  /* open-addressing probe limit reached               */
#define NECI_GPU_ERR_TIMEOUT      4  /* a bounded device wait ran out                      */
#define NECI_GPU_ERR_UNSUPPORTED  5  /* generator/system not on the device path           */
#define NECI_GPU_ERR_INVALID      6  /* bad argument                                       */
#define NECI_GPU_ERR_CUDA         7  /* CUDA runtime error (see neci_gpu_last_error)      */
#define NECI_GPU_ERR_UNSTABLE     8  /* death probability > 2: fcimc_pointed_fns.F90:640  */
#define NECI_GPU_ERR_OVERFLOW     9  /* fixed-point spawn sum out of range                 */

/* ---- enumerations ------------------------------------------------------ */
#define NECI_SYS_HUBBARD_REAL_SPACE 0  /* real_space_hubbard.F90          */
#define NECI_SYS_MOLECULAR          1  /* FCIDUMP: TMat2D + 8-fold UMAT    */

#define NECI_EXGEN_RS_HUBBARD 0  /* gen_excit_rs_hubbard, real_space_hubbard.F90:1938 */
#define NECI_EXGEN_UNIFORM    1  /* gen_rand_excit (C1), GenRandSymExcitNUMod.F90:72    */
#define NECI_EXGEN_PCHB       2  /* FCI PCHB "delocalised", pchb_excitgen.F90:216       */

#define NECI_PREC_FP64  0  /* all arithmetic in FP64 (NECI semantics)               */
#define NECI_PREC_MIXED 1  /* FP32 spawn amplitudes and core off-diagonal matvec     */

/* flag bits of the flag word (bit_rep_data.F90:82-114, non-PROG_NUMRUNS build) */
#define NECI_FLAG_INITIATOR_1     13
#define NECI_FLAG_INITIATOR_2     14
#define NECI_FLAG_DETERMINISTIC_1 19
#define NECI_FLAG_DETERMINISTIC_2 20

/* Fixed-point scale of spawned amplitudes while they are summed: a spawn of
 * real amplitude x is carried as llrint(x * 2^NECI_SPAWN_FIXED_BITS) so that
 * the sum over all spawns onto one determinant does not depend on order. */
#define NECI_SPAWN_FIXED_BITS 32

/* ---- system description (fixed for the run) -------------------------- */
typedef struct {
    int32_t nel;            /* NEl                                                   */
    int32_t nbasis;         /* nBasis: spin orbitals (odd = beta, even = alpha)      */
    int32_t nifd;           /* NIfD = nBasis/64 (BitReps.F90:174)                    */
    int32_t lenof_sign;     /* 1 (neci) or 2 (dneci replica pair)                    */
    int32_t system;         /* NECI_SYS_*                                            */
    int32_t excitgen;       /* NECI_EXGEN_*                                          */
    int32_t max_neighbours; /* lattice: neighbours per site (0 for molecules)        */
    int32_t reserved;
    double  uhub;           /* Hubbard U (System_neci.F90 `u`)                       */
    double  bhub;           /* Hubbard hopping (System_neci.F90 `b`, t = -b)         */
    double  ecore;          /* FCIDUMP core energy                                   */
    double  p_singles;      /* pSingles (molecular generators)                       */
    double  p_parallel;     /* pParallel of pick_biased_elecs (Calc.F90:402)         */
    int64_t max_walkers;    /* MaxWalkersPart (fcimc_initialisation.fpp:1650)        */
    int64_t max_spawned;    /* MaxSpawned     (fcimc_initialisation.fpp:3678)        */
    int64_t n_walker_hashes;/* buckets of the walker hash table (nWalkerHashes)      */
} neci_gpu_system;

/* ---- per-iteration parameters (FciMCData / CalcData globals) ---------- */
typedef struct {
    double   tau;
    double   diag_sft[2];          /* DiagSft(run)                                   */
    double   initiator_walk_no;    /* InitiatorWalkNo (Calc.F90:326, default 3)      */
    double   occupied_thresh;      /* OccupiedThresh  (Calc.F90:346, default 1)      */
    double   real_spawn_cutoff;    /* RealSpawnCutoff (Calc.F90:345, default 0.95)   */
    double   av_mc_excits;         /* AvMCExcits      (Calc.F90:232, default 1)      */
    int32_t  t_trunc_initiator;    /* tTruncInitiator                                */
    int32_t  t_init_coherent_rule; /* tInitCoherentRule (default on)                 */
    int32_t  t_all_real_coeff;     /* tAllRealCoeff                                  */
    int32_t  t_real_spawn_cutoff;  /* tRealSpawnCutoff                               */
    int32_t  t_core_inits;         /* t_core_inits (Calc.F90:125)                    */
    int32_t  precision;            /* NECI_PREC_*                                    */
    uint64_t seed;                 /* RNG seed (replaces dSFMT's G_VMC_Seed)         */
    int64_t  iter;                 /* iteration number: part of every RNG counter    */
} neci_gpu_iter_params;

/* ---- per-iteration results: iter_data (FciMCData.F90:445-455) + stats - */
typedef struct {
    double  nborn[2];
    double  ndied[2];
    double  nannihil[2];
    double  naborted[2];
    double  nremoved[2];
    double  tot_parts[2];      /* TotParts after the step (load_balancer.fpp:727)    */
    double  tot_parts_old[2];  /* TotParts entering the step (= walker updates)      */
    double  noat_hf[2];        /* InstNoAtHF after the step                          */
    double  hf_cyc[2];         /* HFCyc: E_proj denominator of this step             */
    double  enum_cyc[2];       /* ENumCyc: E_proj numerator of this step             */
    double  norm_psi_sq[2];    /* norm_psi_squared                                   */
    int64_t tot_walkers;       /* TotWalkers: slots in use incl. holes               */
    int64_t n_occupied;        /* occupied determinants after the step               */
    int64_t holes_in_list;     /* HolesInList                                        */
    int64_t n_attempts;        /* spawn attempts made                                */
    int64_t n_spawned;         /* spawn records written (SpawnedParts length)        */
    int64_t n_unique;          /* unique spawned determinants after compression      */
    int64_t n_new;             /* determinants added to CurrentDets                  */
    int64_t n_core;            /* core-space size                                    */
    int32_t err;               /* NECI_GPU_* status of the step                       */
    int32_t reserved;
} neci_gpu_iter_stats;

typedef struct neci_gpu_ctx neci_gpu_ctx;

/* ---- context lifecycle -------------------------------------------------
 * neci_gpu_init replaces the device-relevant half of InitFCIMCCalcPar
 * (fcimc_initialisation.fpp:1640-1760): it allocates CurrentDets
 * (max_walkers rows), the walker hash table, SpawnedParts (max_spawned
 * records) and the per-determinant global data on `device`.             */
int32_t neci_gpu_init(neci_gpu_ctx **ctx, const neci_gpu_system *sys, int32_t device);
int32_t neci_gpu_free(neci_gpu_ctx *ctx);
/* Text of the last error recorded on this thread (never NULL). */
const char *neci_gpu_last_error(void);

/* ---- system data (uploaded once) ----------------------------------------
 * RandomHash2(nBasis) of fcimc_initialisation.fpp:886-905, used by
 * FindWalkerHash (hash.F90:23-38).                                        */
int32_t neci_gpu_set_random_hash(neci_gpu_ctx *ctx, const int32_t *random_hash2);
/* TMat2D(nBasis, nBasis) in Fortran (column-major) order (OneEInts.F90:188). */
int32_t neci_gpu_set_tmat(neci_gpu_ctx *ctx, const double *tmat2d);
/* UMAT, 8-fold packed over spatial orbitals, index UMatInd (UMatCache.F90:257). */
int32_t neci_gpu_set_umat(neci_gpu_ctx *ctx, const double *umat, int64_t umat_len);
/* Real-space lattice: neighbours(max_neighbours, nsites), 1-based site
 * indices, 0 = no neighbour (lattice_mod get_neighbors).                  */
int32_t neci_gpu_set_lattice(neci_gpu_ctx *ctx, const int32_t *neighbours, int32_t nsites);
/* iLutRef(0:NIfD) and Hii = <D0|H|D0> (FciMCData iLutRef, Hii). */
int32_t neci_gpu_set_reference(neci_gpu_ctx *ctx, const int64_t *ilut_ref, double hii);
/* Changes pSingles and pParallel, as the conventional tau search does
 * (update_tau, tau/tau_search_conventional.F90:274-499, which assigns the
 * FciMCData globals pSingles/pDoubles/pParallel).  Takes effect from the
 * next step; needs the reference set.                                    */
int32_t neci_gpu_set_excit_biases(neci_gpu_ctx *ctx, double p_singles, double p_parallel);

/* Builds the PCHB alias tables on the device from UMAT
 * (gasci_pchb_doubles_spatorb_fastweighted.fpp compute_samplers).        */
int32_t neci_gpu_init_pchb(neci_gpu_ctx *ctx);

/* ---- walker list transfer (POPSFILE read/write, host estimators) ------
 * Upload replaces CurrentDets: `ilut` holds nrows rows in CurrentDets layout;
 * diag_h (H_jj - Hii) and offdiag_h (<D0|H|D_j>) may be NULL, in which case
 * the device computes them (get_diagonal_matel / get_off_diagonal_matel).
 * Every row's determinant must hold nel electrons among the nBasis spin
 * orbitals (NECI's EncodeBitDet of an nI array, BitReps.F90:75); a row that
 * does not is refused with NECI_GPU_ERR_INVALID before anything is copied. */
int32_t neci_gpu_upload_walkers(neci_gpu_ctx *ctx, const int64_t *ilut, int64_t nrows,
                                const double *diag_h, const double *offdiag_h);
/* The check the upload applies, on the host and without a context: the index
 * of the first of nrows rows (nifd+1 determinant words, lenof_sign signs and
 * a flag word each) whose determinant does not hold exactly nel set bits
 * below bit nbasis, or -1 when every row does (or the arguments are out of
 * range: nifd 0..3, lenof_sign 1..2, nrows >= 0, and ilut non-NULL for
 * nrows > 0; those give -2). */
int64_t neci_gpu_check_rows(const int64_t *ilut, int64_t nrows, int32_t nifd, int32_t lenof_sign,
                            int32_t nel, int32_t nbasis);
/* Downloads the occupied rows (holes skipped) into `ilut` (max_rows rows) and,
 * if non-NULL, their diag_h/offdiag_h.  *nrows receives the row count.    */
int32_t neci_gpu_download_walkers(neci_gpu_ctx *ctx, int64_t *ilut, double *diag_h,
                                  double *offdiag_h, int64_t max_rows, int64_t *nrows);

/* ---- the hot path ------------------------------------------------------
 * One PerformFCIMCycPar(iter_data, err) (FciMCPar.F90:1177-1920) with the
 * default tDeathBeforeComms = .false. ordering: sweep (initiator flags,
 * E_proj sums, spawning), core projection, compression of the spawns,
 * death, deterministic annihilation, AnnihilateSpawnedParts and
 * CalcHashTableStats.  `stats` receives iter_data and the estimators.    */
int32_t neci_gpu_iterate(neci_gpu_ctx *ctx, const neci_gpu_iter_params *params,
                         neci_gpu_iter_stats *stats);
/* Runs n_iter iterations back to back on the device without host syncs and
 * with the shift held at params->diag_sft; stats receives n_iter records.  */
int32_t neci_gpu_iterate_n(neci_gpu_ctx *ctx, const neci_gpu_iter_params *params,
                           int32_t n_iter, neci_gpu_iter_stats *stats);

/* neci_gpu_iterate_n with the device time of the n_iter steps, measured by
 * CUDA events on the context stream, returned in *device_ms. */
int32_t neci_gpu_iterate_timed(neci_gpu_ctx *ctx, const neci_gpu_iter_params *params,
                               int32_t n_iter, neci_gpu_iter_stats *stats, double *device_ms);

/* Batched steps: n_iter iterations of each of n_ctx independent contexts
 * (one system and walker list each, e.g. instances of different size or
 * replica pairs), all on one device.  A step of the whole batch is one CUDA
 * graph with one branch per context (its step's kernels), launched once per
 * step, so the GPU executes the instances side by side; the graph is kept by
 * the first context and rebuilt when a context's configuration changes.  The
 * result of every instance is the same as when it is stepped alone.  params
 * holds one record per context; stats receives n_iter records per context
 * (context-major); *device_ms (may be NULL) the CUDA-event time of the whole
 * batch.  The reference runs such instances as separate jobs (replicas: the
 * dneci/mneci builds, CMakeLists.txt:97-106). */
int32_t neci_gpu_iterate_batch(neci_gpu_ctx **ctxs, int32_t n_ctx, const neci_gpu_iter_params *params,
                               int32_t n_iter, neci_gpu_iter_stats *stats, double *device_ms);

/* ---- conventional tau search --------------------------------------------
 * With the search on, every step logs, for each generated excitation that
 * reaches attempt_create, gamma = |H_ij| / (p_gen / p_class) into the
 * maximum of its class (log_spawn_magnitude,
 * tau/tau_search_conventional.F90:138-258; classes sing, doub for the
 * uniform generator, par/opp for PCHB's parallel/opposite-spin doubles) and,
 * for every determinant that undergoes death, K_ii - S into max_death_cpt
 * (log_death_magnitude, tau/tau_main.F90:197-206).  The maxima persist over
 * steps until read with reset != 0; the host applies update_tau to them.
 * The counts stop mattering past the reference's threshold of 50 and are
 * reported capped at 51.                                                 */
typedef struct {
    double  gamma_sing;     /* max |H_ij| / (p_gen / pSingles), singles            */
    double  gamma_doub;     /* max |H_ij| / (p_gen / pDoubles), uniform doubles    */
    double  gamma_par;      /* ... / (pDoubles pParallel), same-spin PCHB doubles  */
    double  gamma_opp;      /* ... / (pDoubles (1-pParallel)), opposite-spin       */
    double  max_death_cpt;  /* max(K_ii - S) over the dying determinants, >= 0      */
    int64_t cnt_sing, cnt_doub, cnt_par, cnt_opp;
} neci_gpu_tau_stats;
int32_t neci_gpu_set_tau_search(neci_gpu_ctx *ctx, int32_t on);
int32_t neci_gpu_get_tau_stats(neci_gpu_ctx *ctx, neci_gpu_tau_stats *out, int32_t reset);

/* ---- stochastic 2-RDM of a replica pair (lenof_sign == 2) ---------------
 * While sampling is on, every step adds to a dense spin-orbital 2-RDM
 *   rdm2[pair(p,q) * npair + pair(r,s)] ~ <Psi_1| a+_p a+_q a_s a_r |Psi_2>,
 * p < q, r < s, pair(p,q) = (q-1)(q-2)/2 + (p-1) for 1-based spin orbitals,
 * npair = nBasis (nBasis - 1) / 2:
 *   off-diagonal: each spawn from D_i (run s) onto D_j that is occupied after
 *   annihilation adds 1/2 w_i C_j(other run) <D_j|...|D_i>, w_i having
 *   expectation C_i (DiDj_Found_FillRDM, rdm_filling.F90:423-611, and
 *   Add_RDM_From_IJ_Pair, :696-767; the parent travels with the spawn as in
 *   store_parent_with_spawned, rdm_general.fpp:1087);
 *   diagonal: each occupied D_i adds C_i^1 C_i^2 to Gamma(pq, pq) for its
 *   occupied pairs (fill_spawn_rdm_diag, rdm_filling.F90:769-789).
 * The sums are unnormalised and not yet symmetrised (the host takes
 * (G + G^T) / 2 and divides by the trace, as the reference's output does). */
int32_t neci_gpu_set_rdm_sampling(neci_gpu_ctx *ctx, int32_t on);
/* Copies the accumulated 2-RDM (n_elements == npair^2 doubles) and, if reset
 * != 0, clears it. */
int32_t neci_gpu_get_rdm(neci_gpu_ctx *ctx, double *rdm2, int64_t n_elements, int32_t reset);

/* ---- annihilation of an injected spawn list -----------------------------
 * CompressSpawnedList (Annihilation.F90:249-515) followed by
 * AnnihilateSpawnedParts + CalcHashTableStats (Annihilation.F90:965-1352,
 * load_balancer.fpp:646-806) applied to the resident CurrentDets, without
 * spawning or death.  `spawned` holds n_spawned rows in SpawnedParts layout
 * (same words as a CurrentDets row, real(dp) signs).                     */
int32_t neci_gpu_annihilate(neci_gpu_ctx *ctx, const neci_gpu_iter_params *params,
                            const int64_t *spawned, int64_t n_spawned,
                            neci_gpu_iter_stats *stats);
/* CompressSpawnedList alone: the compressed list (one row per surviving
 * determinant, sorted by ilut_lt, DetBitOps.F90:431) is written to `out`
 * (n_spawned rows at most); *n_out gets its length, nannihil (lenof_sign
 * doubles) the annihilation count of the compression.  The flag rules use
 * tTruncInitiator and tInitCoherentRule of the parameters the context was
 * last given (by a step or neci_gpu_annihilate; both on before the first). */
int32_t neci_gpu_compress_spawns(neci_gpu_ctx *ctx, const int64_t *spawned, int64_t n_spawned,
                                 int64_t *out, int64_t *n_out, double *nannihil);

/* CompressSpawnedList for callers that cannot allocate memory.  This entry
 * point has no counterpart in the reference.  It is for hosts that may not
 * call cudaMalloc (code running inside another program's memory pool, or a
 * process that must not grow its GPU footprint after start-up): it needs no
 * context and allocates nothing, host or device.  Its scratch (hash table and
 * per-determinant sums) is a fixed set of file-scope device arrays, about
 * 10 MB, that every GPU which loads the library holds until the process exits.
 *   d_spawned  n rows in SpawnedParts layout, in device memory (read only)
 *   n          at most 262144 (2^18) rows per call; larger n returns
 *              NECI_GPU_ERR_INVALID with a message in errbuf
 *   d_out      device memory for up to n rows: the compressed list, one row
 *              per determinant with a non-zero summed amplitude, in no
 *              particular order (neci_gpu_compress_spawns returns the same
 *              rows sorted by ilut_lt)
 *   n_out, nannihil (lenof_sign doubles, may be NULL): host memory
 *   stream     cudaStream_t to run on (NULL: the legacy default stream); the
 *              call synchronises it before returning
 *   errbuf     caller-owned buffer for an error message (may be NULL)
 * The current device is used.  The first call on each device looks up the
 * device addresses of the scratch arrays (cudaGetSymbolAddress) and should
 * come before any stream capture.  Every call on a device shares the same
 * scratch: it is cleared at the start of each call, and calls that overlap on
 * the GPU race, so a caller with several streams or threads serialises them.
 * The looked-up addresses are kept for the life of the process: after a
 * cudaDeviceReset the entry point must not be called again. */
int32_t neci_gpu_compress_spawns_noalloc(const int64_t *d_spawned, int64_t n, int32_t nifd,
                                         int32_t lenof_sign, int32_t t_trunc_initiator,
                                         int32_t t_init_coherent_rule, int64_t *d_out, int64_t *n_out,
                                         double *nannihil, void *stream, char *errbuf,
                                         int32_t errbuf_len);

/* ---- bit-string and matrix-element kernels (batch forms) ---------------
 * FindWalkerHash (hash.F90:23-38) of n determinants for a table of
 * table_len buckets: out[i] in 1..table_len.                             */
int32_t neci_gpu_find_walker_hash(neci_gpu_ctx *ctx, const int64_t *dets, int64_t n,
                                  int64_t table_len, int64_t *out);
/* FindBitExcitLevel(iLutI, iLutJ) (DetBitOps.F90:140) for n pairs. */
int32_t neci_gpu_excit_level(neci_gpu_ctx *ctx, const int64_t *dets_i, const int64_t *dets_j,
                             int64_t n, int32_t *out);
/* <D_i|H|D_j> for n pairs (get_helement_det_only, Determinants.F90:508):
 * Slater-Condon for molecules, real_space_hubbard.F90:2196 for lattices. */
int32_t neci_gpu_helement(neci_gpu_ctx *ctx, const int64_t *dets_i, const int64_t *dets_j,
                          int64_t n, double *out);
/* Draws n_samples excitations from one determinant with the configured
 * generator (generate_excitation pointer, proc_ptrs.F90:13): for sample k
 * the child determinant (nifd+1 words, all zero for a null excitation),
 * pgen and H_ij.  The random stream is the one the engine uses for spawn
 * attempt k of that determinant at iteration `iter` with seed `seed`.    */
int32_t neci_gpu_gen_excit(neci_gpu_ctx *ctx, const int64_t *det, int64_t n_samples,
                           uint64_t seed, int64_t iter, int64_t *child, double *pgen,
                           double *hel);

/* ---- semistochastic core space ------------------------------------------
 * Sets the core space (init_semi_stochastic, semi_stoch_gen.F90:103): the
 * n_core determinants must already be in CurrentDets; they are flagged
 * deterministic, and the core Hamiltonian is built on the device as CSR
 * (calc_determ_hamil_sparse, sparse_arrays.F90:426) in FP64, or in FP32
 * with compensated accumulation when precision == NECI_PREC_MIXED.       */
int32_t neci_gpu_set_core_space(neci_gpu_ctx *ctx, const int64_t *core_dets, int64_t n_core,
                                int32_t precision);
/* Selects the core space on the device and sets it as neci_gpu_set_core_space
 * does: the min(n_core, occupied) determinants of CurrentDets with the largest
 * weight sum over runs of |C| (core_space_weight, semi_stoch_procs.F90:1623-1642,
 * in proc_most_populated_states, :1310-1421), in order of decreasing weight.
 * Among equal weights the lower slot wins, as NECI's strict ">" keeps the
 * first determinant it meets.  core_dets (may be NULL) receives the selected
 * determinants (nifd+1 words each, room for n_core rows) and *n_selected
 * (may be NULL) their number.                                              */
int32_t neci_gpu_select_core(neci_gpu_ctx *ctx, int64_t n_core, int32_t precision, int64_t *core_dets,
                             int64_t *n_selected);
/* Number of stored off-diagonal core Hamiltonian elements. */
int32_t neci_gpu_core_nnz(neci_gpu_ctx *ctx, int64_t *nnz);

/* ---- engine variants ------------------------------------------------------
 * Options that choose how a step is computed, never what it computes: the
 * walker lists and estimators are the same bit for bit under every setting
 * of the first two, and NECI_OPT_CORE_SEGMENT changes only the order of the
 * core projection's additions.
 * They have no counterpart in the reference, whose one CPU path has no such
 * choice; the reference routine each variant restates is named below.  A
 * change takes effect from the next step.                                 */
#define NECI_OPT_FUSE_PROBE   0  /* lattice systems: look every child up in the walker
                                    hash inside the spawn kernel (hash_table_lookup,
                                    hash.F90:294).  -1 (default): chosen from the last
                                    step's spawn rate; 0: never; 1: always.  Only with
                                    the hash annihilation and without 2-RDM sampling */
#define NECI_OPT_ANNIHILATION 1  /* NECI_ANN_HASH (default) or NECI_ANN_SORT           */
#define NECI_ANN_HASH 0  /* spawns looked up in the walker hash, the others merged in an
                            open-addressing table                                    */
#define NECI_ANN_SORT 1  /* spawns radix-sorted by a key of their determinant and
                            equal determinants reduced as runs: CompressSpawnedList's
                            sort and FindResidualParticle (Annihilation.F90:273,
                            551-634)                                                  */
#define NECI_OPT_CORE_SEGMENT 2  /* core projection (determ_projection_no_death,
                                    semi_stoch_procs.F90:290-365): elements per lane of
                                    a segment of a core row, 1..65536, default 64.  A
                                    row is summed in segments of G times this many
                                    elements (G lanes per segment), whose sums are added
                                    in order, so that long rows are spread over many
                                    lanes.  The one option that changes the order of
                                    additions, and so the last bits of the projection;
                                    it takes effect at the next neci_gpu_set_core_space
                                    or neci_gpu_select_core.                          */
int32_t neci_gpu_set_option(neci_gpu_ctx *ctx, int32_t option, int32_t value);

/* ---- autotuning -----------------------------------------------------------
 * The launch shapes and the annihilation form of a context, which change the
 * speed of a step and never its results.  No counterpart in the reference,
 * whose CPU loop has no such settings.                                    */
typedef struct {
    int32_t annihilation;         /* NECI_ANN_HASH or NECI_ANN_SORT                            */
    int32_t spawn_blocks_per_sm;  /* blocks of 128 threads per SM in the spawn kernel's grid,
                                     1..16 (8, the default, is every block its registers
                                     allow; more only queue behind the resident ones)         */
    int32_t table_shift;          /* hash form: the compression table of a step holds at least
                                     2^table_shift buckets per spawn onto an absent
                                     determinant (load factor 2^-table_shift), 1..4            */
    int32_t sort_blocks_per_sm;   /* sort form: blocks per SM of a radix pass, 1..4 (each
                                     block sorts a chunk of the spawn list)                    */
    double  ns_per_update;        /* autotuning: device ns per walker update it measured       */
    int32_t reserved[2];
} neci_gpu_tuning;
int32_t neci_gpu_set_tuning(neci_gpu_ctx *ctx, const neci_gpu_tuning *tuning);
int32_t neci_gpu_get_tuning(neci_gpu_ctx *ctx, neci_gpu_tuning *tuning);
/* Times a fixed list of settings on live steps and keeps the fastest: for
 * each setting one step (which captures its step graph) and then
 * steps_per_setting steps timed by CUDA events, whose cost is device time per
 * walker update (TotParts entering the steps).  The steps are ordinary steps
 * of the run, the same under every setting, from params->iter on: stats
 * (max_stats records) receives them and *n_steps their number, by which the
 * caller advances its iteration count.  *chosen (may be NULL) gets the
 * setting kept.  Settings that do not fit in max_stats are not tried.     */
int32_t neci_gpu_autotune(neci_gpu_ctx *ctx, const neci_gpu_iter_params *params, int32_t steps_per_setting,
                          neci_gpu_iter_stats *stats, int32_t max_stats, int32_t *n_steps, neci_gpu_tuning *chosen);

/* ---- timing --------------------------------------------------------------
 * When enabled, every kernel launch of the iteration is bracketed by CUDA
 * events on the context stream; neci_gpu_kernel_times returns per-kernel
 * accumulated milliseconds and launch counts for kernel ids 0..n-1 and
 * resets them.  Names come from neci_gpu_kernel_name.                    */
int32_t neci_gpu_set_profiling(neci_gpu_ctx *ctx, int32_t on);
int32_t neci_gpu_kernel_times(neci_gpu_ctx *ctx, double *ms, int64_t *launches, int32_t n);
const char *neci_gpu_kernel_name(int32_t id);
/* Number of kernel ids. */
int32_t neci_gpu_num_kernels(void);
/* Synchronises the context stream. */
int32_t neci_gpu_sync(neci_gpu_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif /* NECI_GPU_H */
