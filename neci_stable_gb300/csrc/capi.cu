// capi.cu -- the C ABI declared in include/neci_gpu.h.
//
// Host code only: argument checks, device allocation of the resident state,
// host<->device copies and the launch sequence of one iteration (captured
// once into a CUDA graph and replayed every step).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "stage.cuh"

using namespace neci;

namespace {

thread_local std::string g_last_error = "";

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess)                                                                \
            return fail(NECI_GPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

template <typename T>
int dalloc(Engine &e, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t err = cudaMalloc((void **)p, count * sizeof(T));
    if (err != cudaSuccess) return fail(NECI_GPU_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(err));
    e.allocs.push_back((void *)*p);
    err = cudaMemsetAsync(*p, 0, count * sizeof(T), e.stream);
    if (err != cudaSuccess) return fail(NECI_GPU_ERR_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(err));
    return NECI_GPU_OK;
}

// Frees a dalloc'ed array (the context's list forgets it) and clears the pointer.
template <typename T>
void dfree(Engine &e, T *&p) {
    if (!p) return;
    auto it = std::find(e.allocs.begin(), e.allocs.end(), (void *)p);
    if (it != e.allocs.end()) e.allocs.erase(it);
    cudaFree((void *)p);
    p = nullptr;
}

unsigned long long next_pow2(unsigned long long x) {
    unsigned long long p = 1;
    while (p < x) p <<= 1;
    return p;
}

void copy_params(IterParams &d, const neci_gpu_iter_params &p) {
    d.tau = p.tau;
    d.diag_sft[0] = p.diag_sft[0];
    d.diag_sft[1] = p.diag_sft[1];
    d.initiator_walk_no = p.initiator_walk_no;
    d.occupied_thresh = p.occupied_thresh;
    d.real_spawn_cutoff = p.real_spawn_cutoff;
    d.av_mc_excits = p.av_mc_excits;
    d.t_trunc_initiator = p.t_trunc_initiator;
    d.t_init_coherent_rule = p.t_init_coherent_rule;
    d.t_all_real_coeff = p.t_all_real_coeff;
    d.t_real_spawn_cutoff = p.t_real_spawn_cutoff;
    d.t_core_inits = p.t_core_inits;
    d.precision = p.precision;
    d.seed = p.seed;
    d.iter = p.iter;
    d.inv_cutoff = 1.0 / p.real_spawn_cutoff;
    d.inv_av = 1.0 / p.av_mc_excits;
    d.f_tau = (float)p.tau;
    d.f_inv_av = (float)d.inv_av;
    d.f_cutoff = (float)p.real_spawn_cutoff;
    d.f_inv_cutoff = (float)d.inv_cutoff;
    d.cutoff_q = (unsigned long long)std::llrint(std::ldexp(p.real_spawn_cutoff, NECI_SPAWN_FIXED_BITS));
    d.av_unit = p.av_mc_excits == 1.0;
}

const char *kKernelNames[K_NUM] = {"compact",     "rehash",       "begin",        "sweep",      "expand", "spawn",
                                   "core",        "ann_probe",    "ann_compress", "ann_insert", "merge_stats",
                                   "rdm",         "final",        "sort_keys",    "sort_radix", "sort_group"};

// Launch one kernel stage, bracketed by events when profiling.
template <typename F>
int stage(Engine &e, int id, F &&f) {
    if (e.profiling) {
        cudaEventRecord(e.ev[2 * id], e.stream);
        f();
        cudaEventRecord(e.ev[2 * id + 1], e.stream);
        cudaEventSynchronize(e.ev[2 * id + 1]);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e.ev[2 * id], e.ev[2 * id + 1]);
        e.kernel_ms[id] += ms;
        e.kernel_launches[id] += 1;
    } else {
        f();
    }
    return NECI_GPU_OK;
}

// The annihilation passes before the insertion of new determinants.  Hash
// form: pass 1 (the walker-hash lookup of every spawn) as its own kernel
// unless the spawn kernel does it, then the compression of the spawns onto
// absent determinants.  Sort form: keys, radix passes, and the grouping of
// runs of equal keys (looked up in the walker hash when `lookup`; without it
// every group is a new determinant, as the compression alone needs).
void annihilation_passes(Engine &e, int lookup) {
    if (e.ann_mode == NECI_ANN_SORT) {
        int cur = 0;
        stage(e, K_SORT_KEYS, [&] { launch_sort_keys(e, e.stream); });
        stage(e, K_SORT_RADIX, [&] { cur = launch_sort_radix(e, e.stream); });
        stage(e, K_SORT_GROUP, [&] { launch_sort_group(e, e.stream, lookup, cur); });
        return;
    }
    if (!lookup) {
        launch_all_cand(e);
    } else if (!fused_lookup(e)) {
        stage(e, K_ANN_PROBE, [&] { launch_ann_probe(e, e.stream); });
    }
    stage(e, K_ANN_COMPRESS, [&] { launch_ann_compress(e, e.stream); });
}

// The passes of a step's annihilation that write the found branch (acc,
// meta): the probe of the hash form (unless the spawn kernel did it), or the
// sort form with its grouping, which also lists the new determinants.
void lookup_passes(Engine &e) {
    if (e.ann_mode == NECI_ANN_SORT) {
        annihilation_passes(e, 1);
        return;
    }
    if (!fused_lookup(e)) stage(e, K_ANN_PROBE, [&] { launch_ann_probe(e, e.stream); });
}

// The compression of the hash form (the sort form has none left).
void compress_pass(Engine &e) {
    if (e.ann_mode != NECI_ANN_SORT) stage(e, K_ANN_COMPRESS, [&] { launch_ann_compress(e, e.stream); });
}

// The launch sequence of one PerformFCIMCycPar step.  After the walker-hash
// lookup of the spawns (the found branch in acc/meta) the step has two
// independent branches: the determinants not found (compression, decision,
// placement) and the merge sweep over the slots the step began with, which
// skips the slots the sweep freed (the only ones a placement can fill).  The
// placement accounts for its own determinants' statistics, so the two run
// side by side on two streams (in the step graph, two branches), and in
// either order give the same list and the same counts.  With profiling on
// they run one after the other on the step's stream.
void step_sequence(Engine &e, neci_gpu_iter_stats *out, int advance) {
    stage(e, K_REHASH, [&] { launch_rehash(e, e.stream); });
    stage(e, K_BEGIN, [&] { launch_begin(e, e.stream); });
    stage(e, K_SWEEP, [&] { launch_sweep(e, e.stream); });
    stage(e, K_EXPAND, [&] { launch_expand(e, e.stream); });
    stage(e, K_SPAWN, [&] { launch_spawn(e, e.stream); });
    if (e.st.n_core > 0) stage(e, K_CORE, [&] { launch_core(e, e.stream); });
    const int with_core = e.st.n_core > 0 ? 1 : 0;
    lookup_passes(e);
    if (e.profiling) {
        compress_pass(e);
        stage(e, K_ANN_INSERT, [&] { launch_ann_insert(e, e.stream, 1); });
        stage(e, K_MERGE_STATS, [&] { launch_merge_stats(e, e.stream, with_core, 1); });
    } else {
        cudaEventRecord(e.branch_ev, e.stream);
        cudaStreamWaitEvent(e.side, e.branch_ev, 0);
        launch_merge_stats(e, e.side, with_core, 1);
        cudaEventRecord(e.merge_ev, e.side);
        compress_pass(e);
        launch_ann_insert(e, e.stream, 1);
        cudaStreamWaitEvent(e.stream, e.merge_ev, 0);
    }
    if (e.sys.rdm) stage(e, K_RDM, [&] { launch_rdm(e, e.stream); });
    stage(e, K_FINAL, [&] { launch_final(e, e.stream, out, e.d_stat_pos, advance, 1); });
}

// Destroys the cached step graphs (after any change the kernels see by value).
// A value no context's step graphs have had before, in this process: a
// batch graph built on a context that was freed (and whose address was
// reused) can never match a new one.
unsigned long long fresh_graph_version() {
    static std::atomic<unsigned long long> counter{1};
    return counter.fetch_add(1);
}

void drop_graphs(Engine &e) {
    for (int k = 0; k < 2; ++k)
        if (e.graphs[k]) {
            cudaGraphExecDestroy(e.graphs[k]);
            e.graphs[k] = nullptr;
        }
    e.graph = nullptr;
    e.graph_version = fresh_graph_version();
}

// Makes e.graph the step graph of the current precision; one graph per
// precision is kept, so that steps of both precisions can alternate.
int ensure_graph(Engine &e) {
    const bool core = e.st.n_core > 0;
    const int k = e.h_params->precision == NECI_PREC_MIXED ? 1 : 0;
    const bool fast = sweep_fast(*e.h_params);
    if (e.graphs[k] && (e.graph_core[k] != core || e.graph_fast[k] != fast)) {
        cudaGraphExecDestroy(e.graphs[k]);
        e.graphs[k] = nullptr;
    }
    if (!e.graphs[k]) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(e.stream, cudaStreamCaptureModeThreadLocal));
        step_sequence(e, e.d_stats, 1);  // each replay writes the next record (d_stat_pos)
        CK(cudaStreamEndCapture(e.stream, &g));
        CK(cudaGraphInstantiate(&e.graphs[k], g, 0));
        cudaGraphDestroy(g);
        e.graph_core[k] = core;
        e.graph_fast[k] = fast;
    }
    e.graph = e.graphs[k];
    return NECI_GPU_OK;
}

template <typename T>
int batch_io(Engine &e, const T *h, size_t n, T **d) {
    CK(cudaMallocAsync((void **)d, std::max<size_t>(n, 1) * sizeof(T), e.stream));
    if (h && n) CK(cudaMemcpyAsync(*d, h, n * sizeof(T), cudaMemcpyHostToDevice, e.stream));
    return NECI_GPU_OK;
}

int check_ctx(neci_gpu_ctx *ctx) {
    if (!ctx) return fail(NECI_GPU_ERR_INVALID, "null context");
    return NECI_GPU_OK;
}

}  // namespace

struct neci_gpu_ctx {
    Engine e;
};

extern "C" {

const char *neci_gpu_last_error(void) { return g_last_error.c_str(); }

int32_t neci_gpu_num_kernels(void) { return K_NUM; }
const char *neci_gpu_kernel_name(int32_t id) { return (id >= 0 && id < K_NUM) ? kKernelNames[id] : ""; }

int32_t neci_gpu_init(neci_gpu_ctx **out, const neci_gpu_system *sys, int32_t device) {
    if (!out || !sys) return fail(NECI_GPU_ERR_INVALID, "null argument");
    *out = nullptr;
    if (sys->nifd < 0 || sys->nifd + 1 > kMaxWords || sys->nbasis > 64 * (sys->nifd + 1) || sys->nbasis > 255)
        return fail(NECI_GPU_ERR_UNSUPPORTED, "nBasis/NIfD outside the device layout (nBasis <= 255)");
    if (sys->nel < 2 || sys->nel > kMaxNel) return fail(NECI_GPU_ERR_UNSUPPORTED, "nel outside 2..64");
    if (sys->lenof_sign != 1 && sys->lenof_sign != 2) return fail(NECI_GPU_ERR_UNSUPPORTED, "lenof_sign must be 1 or 2");
    if (sys->system == NECI_SYS_HUBBARD_REAL_SPACE) {
        if (sys->excitgen != NECI_EXGEN_RS_HUBBARD) return fail(NECI_GPU_ERR_UNSUPPORTED, "lattice needs rs-hubbard generator");
        if (sys->max_neighbours < 1 || sys->max_neighbours > kMaxNeigh) return fail(NECI_GPU_ERR_UNSUPPORTED, "max_neighbours");
    } else if (sys->system == NECI_SYS_MOLECULAR) {
        if (sys->excitgen != NECI_EXGEN_PCHB && sys->excitgen != NECI_EXGEN_UNIFORM)
            return fail(NECI_GPU_ERR_UNSUPPORTED, "molecular systems run the PCHB or the uniform generator");
    } else {
        return fail(NECI_GPU_ERR_UNSUPPORTED, "unknown system");
    }
    if (sys->max_walkers < 2 || sys->max_spawned < 1 || sys->max_walkers >= (1ll << 31) || sys->max_spawned >= (1ll << 31))
        return fail(NECI_GPU_ERR_INVALID, "max_walkers / max_spawned out of range");
    neci_gpu_ctx *ctx = new neci_gpu_ctx();
    Engine &e = ctx->e;
    e.desc = *sys;
    e.device = device;
    cudaError_t ce = cudaSetDevice(device);
    if (ce != cudaSuccess) { delete ctx; return fail(NECI_GPU_ERR_CUDA, cudaGetErrorString(ce)); }
    cudaDeviceGetAttribute(&e.num_sms, cudaDevAttrMultiProcessorCount, device);
    ce = cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { delete ctx; return fail(NECI_GPU_ERR_CUDA, cudaGetErrorString(ce)); }
    DevSys &s = e.sys;
    s.nel = sys->nel;
    s.nbasis = sys->nbasis;
    s.W = sys->nifd + 1;
    s.L = sys->lenof_sign;
    s.R = s.W + s.L + 1;
    s.system = sys->system;
    s.excitgen = sys->excitgen;
    s.max_neigh = sys->max_neighbours;
    s.uhub = sys->uhub;
    s.bhub = sys->bhub;
    s.ecore = sys->ecore;
    s.p_singles = sys->p_singles;
    s.p_parallel = sys->p_parallel;
    s.nBI = sys->nbasis / 2;
    DevState &st = e.st;
    st.max_walkers = sys->max_walkers;
    st.max_spawned = sys->max_spawned;
    st.max_att = 2 * sys->max_spawned + 1024;
    // a parent with n attempts (kBigAttempts < n <= kHugeAttempts) takes
    // ceil(n / kExpandChunk) entries, at most n / kBigAttempts + n / kExpandChunk
    st.max_big = st.max_att / kBigAttempts + st.max_att / kExpandChunk + 1024;
    st.hash_n = next_pow2(std::max<unsigned long long>((unsigned long long)sys->n_walker_hashes,
                                                       2ull * (unsigned long long)sys->max_walkers));
    st.spawn_hash_n = next_pow2(2ull * (unsigned long long)sys->max_spawned);
    st.comp_shift = 1;
    int rc = NECI_GPU_OK;
#define A(p, n) if (rc == NECI_GPU_OK) rc = dalloc(e, &(p), (n))
    int32_t *rh2 = nullptr;
    A(rh2, (size_t)s.nbasis + 1);
    s.random_hash2 = rh2;
    // the arrays the sweeps stage by TMA bulk copies are kStagePad slots longer
    A(st.dets, (size_t)(st.max_walkers + kStagePad) * s.R);
    A(st.diagH, (size_t)st.max_walkers + kStagePad);
    A(st.offdiagH, (size_t)st.max_walkers + kStagePad);
    A(st.hash, (size_t)st.hash_n);
    A(st.slot_bucket, (size_t)st.max_walkers);
    A(st.free_list, (size_t)st.max_walkers + 1);
    A(st.hole_mark, (size_t)st.max_walkers + 16);  // the merge sweep stages it in multiples of 16 slots
    A(st.dkey, (size_t)st.max_walkers);
    A(st.spawn, (size_t)st.max_spawned * s.R);
    A(st.att, (size_t)st.max_att);
    A(st.big, (size_t)st.max_big * 3);
    A(st.huge, (size_t)kMaxHuge * 3);
    A(st.acc, (size_t)(st.max_walkers + kStagePad) * s.L);
    A(st.meta, (size_t)(st.max_walkers + kStagePad) * s.L);
    A(st.cand, (size_t)st.max_spawned);
    A(st.cand_h, (size_t)st.max_spawned);
    A(st.spawn_hash, (size_t)st.spawn_hash_n);
    A(st.reps, (size_t)st.max_spawned);
    A(st.place, (size_t)st.max_spawned);
    A(st.rep_bucket, (size_t)st.max_spawned);
    A(st.rep_q, (size_t)st.max_spawned * s.L);
    A(st.rep_cnt, (size_t)st.max_spawned * (s.L + 1));
    A(st.tile_count, (size_t)st.max_walkers / kCompactTile + 2);
    A(st.tile_off, (size_t)st.max_walkers / kCompactTile + 2);
    A(st.hole_at_rank, (size_t)st.max_walkers + 1);
    A(st.ctl, 1);
    A(e.d_params, 1);
    e.max_stats = 4096;
    A(e.d_stats, (size_t)e.max_stats + 1);
    A(e.d_stat_pos, 1);
#undef A
    if (rc == NECI_GPU_OK) {
        if (cudaMallocHost(&e.h_params, sizeof(IterParams)) != cudaSuccess ||
            cudaMallocHost(&e.h_stats, sizeof(neci_gpu_iter_stats) * e.max_stats) != cudaSuccess)
            rc = fail(NECI_GPU_ERR_CUDA, "cudaMallocHost failed");
    }
    if (rc == NECI_GPU_OK) {
        std::memset(e.h_params, 0, sizeof(IterParams));
        e.h_params->t_trunc_initiator = 1;  // CompressSpawnedList defaults for an initiator run
        e.h_params->t_init_coherent_rule = 1;
        for (int k = 0; k < 2 * K_NUM; ++k) cudaEventCreate(&e.ev[k]);
        cudaEventCreateWithFlags(&e.fork_ev, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&e.join_ev, cudaEventDisableTiming);
        if (cudaEventCreateWithFlags(&e.branch_ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&e.merge_ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaStreamCreateWithFlags(&e.side, cudaStreamNonBlocking) != cudaSuccess)
            rc = fail(NECI_GPU_ERR_CUDA, "stream or event creation failed");
        e.graph_version = fresh_graph_version();
        if (cudaStreamSynchronize(e.stream) != cudaSuccess) rc = fail(NECI_GPU_ERR_CUDA, "sync after init");
    }
    if (rc == NECI_GPU_OK && configure_kernels(e) != 0)
        rc = fail(NECI_GPU_ERR_CUDA, "cudaFuncSetAttribute (shared memory of the staged sweeps) failed");
    if (rc != NECI_GPU_OK) {
        neci_gpu_free(ctx);
        return rc;
    }
    *out = ctx;
    return NECI_GPU_OK;
}

int32_t neci_gpu_free(neci_gpu_ctx *ctx) {
    if (!ctx) return NECI_GPU_OK;
    Engine &e = ctx->e;
    cudaSetDevice(e.device);
    if (e.stream) cudaStreamSynchronize(e.stream);
    drop_graphs(e);
    if (e.batch_graph) cudaGraphExecDestroy(e.batch_graph);
    if (e.fork_ev) cudaEventDestroy(e.fork_ev);
    if (e.join_ev) cudaEventDestroy(e.join_ev);
    if (e.branch_ev) cudaEventDestroy(e.branch_ev);
    if (e.merge_ev) cudaEventDestroy(e.merge_ev);
    if (e.side) cudaStreamDestroy(e.side);
    for (void *p : e.allocs) cudaFree(p);
    if (e.h_params) cudaFreeHost(e.h_params);
    if (e.h_stats) cudaFreeHost(e.h_stats);
    for (int k = 0; k < 2 * K_NUM; ++k)
        if (e.ev[k]) cudaEventDestroy(e.ev[k]);
    if (e.stream) cudaStreamDestroy(e.stream);
    delete ctx;
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_random_hash(neci_gpu_ctx *ctx, const int32_t *rh) {
    if (int r = check_ctx(ctx)) return r;
    if (!rh) return fail(NECI_GPU_ERR_INVALID, "null RandomHash2");
    Engine &e = ctx->e;
    std::vector<int32_t> h(e.sys.nbasis + 1, 0);
    for (int i = 1; i <= e.sys.nbasis; ++i) h[i] = rh[i - 1];
    CK(cudaMemcpy((void *)e.sys.random_hash2, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_tmat(neci_gpu_ctx *ctx, const double *t) {
    if (int r = check_ctx(ctx)) return r;
    if (!t) return fail(NECI_GPU_ERR_INVALID, "null TMat2D");
    Engine &e = ctx->e;
    double *d = nullptr;
    const size_t n = (size_t)e.sys.nbasis * e.sys.nbasis;
    if (int r = dalloc(e, &d, n)) return r;
    CK(cudaMemcpyAsync(d, t, n * sizeof(double), cudaMemcpyHostToDevice, e.stream));
    std::vector<float> t32(t, t + n);
    float *d32 = nullptr;
    if (int r = dalloc(e, &d32, n)) return r;
    CK(cudaMemcpyAsync(d32, t32.data(), n * sizeof(float), cudaMemcpyHostToDevice, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    e.sys.tmat = d;
    e.sys.tmat32 = d32;
    drop_graphs(e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_umat(neci_gpu_ctx *ctx, const double *u, int64_t len) {
    if (int r = check_ctx(ctx)) return r;
    if (!u || len <= 0) return fail(NECI_GPU_ERR_INVALID, "null UMAT");
    Engine &e = ctx->e;
    const long long P = (long long)e.sys.nBI * (e.sys.nBI + 1) / 2;
    if (len < P * (P + 1) / 2) return fail(NECI_GPU_ERR_INVALID, "UMAT shorter than the 8-fold packed size");
    double *d = nullptr;
    if (int r = dalloc(e, &d, (size_t)len)) return r;
    CK(cudaMemcpyAsync(d, u, (size_t)len * sizeof(double), cudaMemcpyHostToDevice, e.stream));
    std::vector<float> u32(u, u + len);
    float *d32 = nullptr;
    if (int r = dalloc(e, &d32, (size_t)len)) return r;
    CK(cudaMemcpyAsync(d32, u32.data(), (size_t)len * sizeof(float), cudaMemcpyHostToDevice, e.stream));
    e.sys.umat = d;
    e.sys.umat32 = d32;
    // Coulomb and Coulomb-minus-exchange rows of the singles (nBI^3 each,
    // FP64 and FP32)
    const size_t n3 = (size_t)e.sys.nBI * e.sys.nBI * e.sys.nBI;
    double *jr = nullptr, *kr = nullptr;
    float *jr32 = nullptr, *kr32 = nullptr;
    if (int r = dalloc(e, &jr, n3)) return r;
    if (int r = dalloc(e, &kr, n3)) return r;
    if (int r = dalloc(e, &jr32, n3)) return r;
    if (int r = dalloc(e, &kr32, n3)) return r;
    launch_build_jk(e, jr, kr, jr32, kr32);
    double *jm = nullptr, *km = nullptr;
    if (int r = dalloc(e, &jm, (size_t)e.sys.nBI * e.sys.nBI)) return r;
    if (int r = dalloc(e, &km, (size_t)e.sys.nBI * e.sys.nBI)) return r;
    launch_build_jkmat(e, jm, km);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e.stream));
    e.sys.jmat = jm;
    e.sys.kmat = km;
    e.sys.jrow = jr;
    e.sys.jkrow = kr;
    e.sys.jrow32 = jr32;
    e.sys.jkrow32 = kr32;
    drop_graphs(e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_lattice(neci_gpu_ctx *ctx, const int32_t *nb, int32_t nsites) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!nb || nsites * 2 != e.sys.nbasis) return fail(NECI_GPU_ERR_INVALID, "lattice: nsites must be nBasis/2");
    int32_t *d = nullptr;
    const size_t n = (size_t)nsites * e.sys.max_neigh;
    for (size_t i = 0; i < n; ++i)
        if (nb[i] < 0 || nb[i] > nsites) return fail(NECI_GPU_ERR_INVALID, "lattice: neighbour index out of range");
    if (int r = dalloc(e, &d, n)) return r;
    CK(cudaMemcpyAsync(d, nb, n * sizeof(int32_t), cudaMemcpyHostToDevice, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    e.sys.neighbours = d;
    e.sys.nsites = nsites;
    drop_graphs(e);
    return NECI_GPU_OK;
}

// Hoisted constants of the excitation generators from pSingles, pParallel
// and the reference's alpha/beta counts (pick_biased_elecs pgen,
// excit_gens_int_weighted.F90:770-790; pDoubles = 1 - pSingles), and the
// factors of the tau-search log.
static void derive_generator_constants(Engine &e) {
    const int na = e.sys.nOccAlpha, nb = e.sys.nOccBeta;
    DevSys &s = e.sys;
    const int par = na * (na - 1) / 2 + nb * (nb - 1) / 2;
    s.pgen_par = s.p_parallel / (double)par;
    s.pgen_opp = (1.0 - s.p_parallel) / (double)(na * nb);
    s.p_singles = e.desc.p_singles;  // the caller's pSingles (this may run more than once)
    s.p_doubles = 1.0 - s.p_singles;
    if (s.excitgen == NECI_EXGEN_UNIFORM) {
        // gen_rand_excit draws doubles with pDoubles = 1 - pSingles
        // (fcimc_initialisation.fpp CalcApproxpDoubles); a single's pgen
        // carries 1 - pDoubles (CreateSingleExcit, :1264)
        s.p_singles = 1.0 - s.p_doubles;
        s.thr_doubles = prob_thresh(s.p_doubles);
        // FindDoubleProb (GenRandSymExcitNUMod.F90:208) with the C1 counts of
        // FindNumForbiddenOrbsNoSym, PickAOrb and PickBOrb
        const int nua = s.nBI - na, nub = s.nBI - nb, ep = s.nel * (s.nel - 1) / 2;
        for (int ispn = 1; ispn <= 3; ++ispn) {
            int nA, forb, nB, nOther;
            if (ispn == 2) {
                nA = s.nbasis - s.nel;
                forb = (nua == 0 ? nub : 0) + (nub == 0 ? nua : 0);
                nB = nub; nOther = nua;  // the sum below is symmetric in the two
            } else if (ispn == 1) {
                nA = nub; forb = nub == 1; nB = nub - 1; nOther = nub - 1;
            } else {
                nA = nua; forb = nua == 1; nB = nua - 1; nOther = nua - 1;
            }
            double pg = 0.0;
            if (nA > forb && nB > 0 && nOther > 0)
                pg = s.p_doubles * ((1.0 / (double)nB) + (1.0 / (double)nOther)) / (double)(ep * (nA - forb));
            s.pgen_unif[ispn - 1] = pg;
            s.inv_unif[ispn - 1] = pg > 0.0 ? 1.0 / pg : 0.0;
            s.f_pgen_unif[ispn - 1] = (float)pg;
            s.f_inv_unif[ispn - 1] = (float)s.inv_unif[ispn - 1];
        }
    }
    s.p_elec = 1.0 / (double)s.nel;
    s.thr_singles = prob_thresh(s.p_singles);
    s.thr_bias = prob_thresh(s.p_parallel);
    s.f_pgen_par = (float)s.p_parallel / (float)par;
    s.f_pgen_opp = (1.0f - (float)s.p_parallel) / (float)(na * nb);
    s.f_p_doubles = 1.0f - (float)s.p_singles;
    s.f_p_singles = (float)s.p_singles;
    s.f_p_elec = 1.0f / (float)s.nel;
    s.f_inv_nalpha = na > 0 ? 1.0f / (float)na : 0.0f;
    s.inv_par = (double)par / s.p_parallel;
    s.inv_opp = (double)(na * nb) / (1.0 - s.p_parallel);
    s.inv_pdoub = 1.0 / s.p_doubles;
    s.inv_psingles = 1.0 / s.p_singles;
    s.f_inv_par = (float)s.inv_par;
    s.f_inv_opp = (float)s.inv_opp;
    s.f_inv_pdoub = (float)s.inv_pdoub;
    s.f_inv_psingles = (float)s.inv_psingles;
    // gamma = |H_ij| / (p_gen / p_class) (tau_search_conventional.F90:149-202);
    // the real-space Hubbard model runs with pSingles = 1
    // (real_space_hubbard.F90:231)
    s.tau_fac[TC_SING] = s.system == NECI_SYS_HUBBARD_REAL_SPACE ? 1.0 : s.p_singles;
    s.tau_fac[TC_DOUB] = s.p_doubles;
    s.tau_fac[TC_PAR] = s.p_doubles * s.p_parallel;
    s.tau_fac[TC_OPP] = s.p_doubles * (1.0 - s.p_parallel);
    for (int k = 0; k < 4; ++k) s.f_tau_fac[k] = (float)s.tau_fac[k];
    // 1/p_gen of a uniform single by its count of (electron, hole) pairs,
    // count <= nel * nBI: exactly the products the generator formed inline
    const int ncount = s.nel * s.nBI + 1;
    std::vector<double> inv(ncount);
    std::vector<float> inv32(ncount);
    for (int c = 0; c < ncount; ++c) {
        inv[c] = (double)c * s.inv_psingles;
        inv32[c] = (float)c * s.f_inv_psingles;
    }
    if (!e.inv_single) {
        dalloc(e, &e.inv_single, (size_t)ncount);
        dalloc(e, &e.inv_single32, (size_t)ncount);
    }
    if (e.inv_single && e.inv_single32) {
        cudaMemcpyAsync(e.inv_single, inv.data(), ncount * sizeof(double), cudaMemcpyHostToDevice, e.stream);
        cudaMemcpyAsync(e.inv_single32, inv32.data(), ncount * sizeof(float), cudaMemcpyHostToDevice, e.stream);
        cudaStreamSynchronize(e.stream);
    }
    s.inv_single = e.inv_single;
    s.inv_single32 = e.inv_single32;
}

int32_t neci_gpu_set_reference(neci_gpu_ctx *ctx, const int64_t *ref, double hii) {
    if (int r = check_ctx(ctx)) return r;
    if (!ref) return fail(NECI_GPU_ERR_INVALID, "null reference");
    Engine &e = ctx->e;
    int na = 0, nb = 0, ne = 0;
    for (int w = 0; w < kMaxWords; ++w) e.sys.ilut_ref[w] = 0;
    for (int w = 0; w < e.sys.W; ++w) {
        const unsigned long long x = (unsigned long long)ref[w];
        e.sys.ilut_ref[w] = x;
        na += __builtin_popcountll(x & 0xAAAAAAAAAAAAAAAAull);
        nb += __builtin_popcountll(x & 0x5555555555555555ull);
    }
    ne = na + nb;
    if (ne != e.sys.nel) return fail(NECI_GPU_ERR_INVALID, "reference has the wrong electron count");
    e.sys.nOccAlpha = na;
    e.sys.nOccBeta = nb;
    e.sys.hii = hii;
    derive_generator_constants(e);
    e.have_ref = true;
    drop_graphs(e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_excit_biases(neci_gpu_ctx *ctx, double p_singles, double p_parallel) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!(p_singles >= 0.0 && p_singles < 1.0) || !(p_parallel > 0.0 && p_parallel < 1.0))
        return fail(NECI_GPU_ERR_INVALID, "pSingles must lie in [0, 1) and pParallel in (0, 1)");
    if (!e.have_ref) return fail(NECI_GPU_ERR_INVALID, "set the reference first");
    e.desc.p_singles = p_singles;
    e.desc.p_parallel = p_parallel;
    e.sys.p_parallel = p_parallel;
    derive_generator_constants(e);
    drop_graphs(e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_tau_search(neci_gpu_ctx *ctx, int32_t on) {
    if (int r = check_ctx(ctx)) return r;
    ctx->e.sys.tau_search = on ? 1 : 0;
    drop_graphs(ctx->e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_get_tau_stats(neci_gpu_ctx *ctx, neci_gpu_tau_stats *out, int32_t reset) {
    if (int r = check_ctx(ctx)) return r;
    if (!out) return fail(NECI_GPU_ERR_INVALID, "null argument");
    Engine &e = ctx->e;
    unsigned long long h[9];
    CK(cudaMemcpyAsync(h, &e.st.ctl->tau_gamma[0], sizeof(h), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    double g[5];
    std::memcpy(g, h, 4 * sizeof(double));
    std::memcpy(&g[4], &h[8], sizeof(double));
    out->gamma_sing = g[TC_SING];
    out->gamma_doub = g[TC_DOUB];
    out->gamma_par = g[TC_PAR];
    out->gamma_opp = g[TC_OPP];
    out->max_death_cpt = g[4];
    // the counts only decide whether more than cnt_threshold excitations were
    // seen (the reference stops counting there); report them capped alike
    const long long cap = kTauCntThreshold + 1;
    out->cnt_sing = std::min<long long>((long long)h[4 + TC_SING], cap);
    out->cnt_doub = std::min<long long>((long long)h[4 + TC_DOUB], cap);
    out->cnt_par = std::min<long long>((long long)h[4 + TC_PAR], cap);
    out->cnt_opp = std::min<long long>((long long)h[4 + TC_OPP], cap);
    if (reset) {
        CK(cudaMemsetAsync(&e.st.ctl->tau_gamma[0], 0, sizeof(h), e.stream));
        CK(cudaStreamSynchronize(e.stream));
    }
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_rdm_sampling(neci_gpu_ctx *ctx, int32_t on) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (on && e.sys.L != 2) return fail(NECI_GPU_ERR_INVALID, "2-RDM sampling needs a replica pair (lenof_sign 2)");
    if (on && !e.st.rdm2) {
        const long long npair = (long long)e.sys.nbasis * (e.sys.nbasis - 1) / 2;
        if (int r = dalloc(e, &e.st.spawn_par, (size_t)e.st.max_spawned * (e.sys.W + 1))) return r;
        if (int r = dalloc(e, &e.st.rdm2, (size_t)npair * npair)) return r;
        CK(cudaStreamSynchronize(e.stream));
        e.sys.npair = npair;
    }
    e.sys.rdm = on ? 1 : 0;
    drop_graphs(e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_get_rdm(neci_gpu_ctx *ctx, double *rdm2, int64_t n_elements, int32_t reset) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!e.st.rdm2) return fail(NECI_GPU_ERR_INVALID, "2-RDM sampling was never enabled");
    if (!rdm2 || n_elements != e.sys.npair * e.sys.npair)
        return fail(NECI_GPU_ERR_INVALID, "rdm2 must hold npair^2 doubles, npair = nBasis (nBasis - 1) / 2");
    CK(cudaMemcpyAsync(rdm2, e.st.rdm2, (size_t)n_elements * sizeof(double), cudaMemcpyDeviceToHost, e.stream));
    if (reset) CK(cudaMemsetAsync(e.st.rdm2, 0, (size_t)n_elements * sizeof(double), e.stream));
    CK(cudaStreamSynchronize(e.stream));
    return NECI_GPU_OK;
}

int32_t neci_gpu_init_pchb(neci_gpu_ctx *ctx) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (e.sys.system != NECI_SYS_MOLECULAR || !e.sys.umat) return fail(NECI_GPU_ERR_INVALID, "PCHB needs a molecular system with UMAT");
    DevSys &s = e.sys;
    s.ijMax = (long long)s.nBI * (s.nBI + 1) / 2;
    s.abMax = s.ijMax;
    const size_t ntab = (size_t)s.ijMax * 3;
    double *bias, *prob, *pexch;
    int32_t *alias, *tgt;
    uint8_t *present;
    if (int r = dalloc(e, &bias, ntab * s.abMax)) return r;
    if (int r = dalloc(e, &prob, ntab * s.abMax)) return r;
    if (int r = dalloc(e, &alias, ntab * s.abMax)) return r;
    if (int r = dalloc(e, &present, ntab)) return r;
    if (int r = dalloc(e, &pexch, (size_t)s.ijMax)) return r;
    if (int r = dalloc(e, &tgt, (size_t)s.abMax + 1)) return r;
    unsigned long long *athr, *pthr;
    float *prob32, *pexch32;
    if (int r = dalloc(e, &athr, ntab * s.abMax)) return r;
    if (int r = dalloc(e, &prob32, ntab * s.abMax)) return r;
    if (int r = dalloc(e, &pthr, (size_t)s.ijMax)) return r;
    if (int r = dalloc(e, &pexch32, (size_t)s.ijMax)) return r;
    s.alias_thr = athr;
    s.alias_prob32 = prob32;
    s.pexch_thr = pthr;
    s.pexch32 = pexch32;
    double *ainv, *peinv, *pninv;
    float *ainv32, *peinv32, *pninv32;
    if (int r = dalloc(e, &ainv, ntab * s.abMax)) return r;
    if (int r = dalloc(e, &ainv32, ntab * s.abMax)) return r;
    if (int r = dalloc(e, &peinv, (size_t)s.ijMax)) return r;
    if (int r = dalloc(e, &pninv, (size_t)s.ijMax)) return r;
    if (int r = dalloc(e, &peinv32, (size_t)s.ijMax)) return r;
    if (int r = dalloc(e, &pninv32, (size_t)s.ijMax)) return r;
    s.alias_inv = ainv;
    s.alias_inv32 = ainv32;
    s.pexch_inv = peinv;
    s.pnoexch_inv = pninv;
    s.pexch_inv32 = peinv32;
    s.pnoexch_inv32 = pninv32;
    std::vector<int32_t> tp(s.abMax + 1, 0);
    for (int a = 1; a <= s.nBI; ++a)
        for (int b = 1; b <= a; ++b) tp[(long long)b + (long long)a * (a - 1) / 2] = (b << 16) | a;
    CK(cudaMemcpyAsync(tgt, tp.data(), tp.size() * sizeof(int32_t), cudaMemcpyHostToDevice, e.stream));
    s.alias_bias = bias;
    s.alias_prob = prob;
    s.alias_alias = alias;
    s.alias_present = present;
    AliasRec *arec;
    if (int r = dalloc(e, &arec, ntab * s.abMax)) return r;
    s.alias_rec = arec;
    s.pexch = pexch;
    s.tgt_pair = tgt;
    if (const int err = launch_pchb_build(e))
        return fail(NECI_GPU_ERR_CUDA, std::string("PCHB table build: ") + cudaGetErrorString((cudaError_t)err));
    CK(cudaGetLastError());
    e.have_pchb = true;
    drop_graphs(e);
    return NECI_GPU_OK;
}

int64_t neci_gpu_check_rows(const int64_t *ilut, int64_t nrows, int32_t nifd, int32_t lenof_sign, int32_t nel,
                            int32_t nbasis) {
    if (nrows < 0 || (nrows > 0 && !ilut) || nifd < 0 || nifd + 1 > kMaxWords || lenof_sign < 1 || lenof_sign > 2)
        return -2;
    const int W = nifd + 1, R = W + lenof_sign + 1;
    for (int64_t j = 0; j < nrows; ++j) {
        const int64_t *r = ilut + (size_t)j * R;
        int n = 0;
        bool outside = false;
        for (int w = 0; w < W; ++w) {
            const unsigned long long x = (unsigned long long)r[w];
            const int below = nbasis - 64 * w;  // orbitals this word may hold
            if (below <= 0) outside |= x != 0;
            else if (below < 64) outside |= (x >> below) != 0;
            n += __builtin_popcountll(x);
        }
        if (outside || n != nel) return j;
    }
    return -1;
}

int32_t neci_gpu_upload_walkers(neci_gpu_ctx *ctx, const int64_t *ilut, int64_t nrows, const double *dh,
                                const double *odh) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!ilut && nrows > 0) return fail(NECI_GPU_ERR_INVALID, "null rows");
    if (nrows < 0 || nrows >= e.st.max_walkers) return fail(NECI_GPU_ERR_LIST_FULL, "more rows than MaxWalkersPart - 1");
    if (!e.have_ref) return fail(NECI_GPU_ERR_INVALID, "set the reference first");
    // a determinant with the wrong electron count, or an orbital past nBasis,
    // would index the integral and lattice tables out of range on the device
    if (const int64_t bad = neci_gpu_check_rows(ilut, nrows, e.sys.W - 1, e.sys.L, e.sys.nel, e.sys.nbasis); bad != -1)
        return fail(NECI_GPU_ERR_INVALID, "upload: row " + std::to_string(bad) +
                                              " does not hold nel electrons among the nBasis orbitals");
    const int R = e.sys.R;
    CK(cudaMemsetAsync(e.st.dets, 0, (size_t)e.st.max_walkers * R * 8, e.stream));
    CK(cudaMemsetAsync(e.st.hash, 0, (size_t)e.st.hash_n * 4, e.stream));
    CK(cudaMemsetAsync(e.st.acc, 0, (size_t)e.st.max_walkers * e.sys.L * 8, e.stream));
    CK(cudaMemsetAsync(e.st.meta, 0, (size_t)e.st.max_walkers * e.sys.L * 4, e.stream));
    if (nrows > 0) CK(cudaMemcpyAsync(e.st.dets, ilut, (size_t)nrows * R * 8, cudaMemcpyHostToDevice, e.stream));
    const int compute = (dh && odh) ? 0 : 1;
    if (!compute && nrows > 0) {
        CK(cudaMemcpyAsync(e.st.diagH, dh, (size_t)nrows * 8, cudaMemcpyHostToDevice, e.stream));
        CK(cudaMemcpyAsync(e.st.offdiagH, odh, (size_t)nrows * 8, cudaMemcpyHostToDevice, e.stream));
    }
    Control c{};
    c.tot_walkers = (unsigned long long)nrows;
    // the tau-search log at the end of the block outlives the walker list
    CK(cudaMemcpyAsync(e.st.ctl, &c, offsetof(Control, tau_gamma), cudaMemcpyHostToDevice, e.stream));
    // the core space belongs to the previous list
    e.st.n_core = 0;
    if (nrows > 0) launch_upload_fix(e, nrows, compute);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e.stream));
    int err = 0;
    CK(cudaMemcpy(&err, &e.st.ctl->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) return fail(err, "upload: hash table full");
    drop_graphs(e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_download_walkers(neci_gpu_ctx *ctx, int64_t *ilut, double *dh, double *odh, int64_t max_rows,
                                  int64_t *nrows) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!ilut || !nrows) return fail(NECI_GPU_ERR_INVALID, "null output");
    CK(cudaStreamSynchronize(e.stream));
    unsigned long long tw = 0;
    CK(cudaMemcpy(&tw, &e.st.ctl->tot_walkers, sizeof(tw), cudaMemcpyDeviceToHost));
    tw = std::min<unsigned long long>(tw, (unsigned long long)e.st.max_walkers);
    const int R = e.sys.R, W = e.sys.W, L = e.sys.L;
    std::vector<long long> rows((size_t)tw * R);
    std::vector<double> d1(tw), d2(tw);
    if (tw) {
        CK(cudaMemcpy(rows.data(), e.st.dets, (size_t)tw * R * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(d1.data(), e.st.diagH, (size_t)tw * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(d2.data(), e.st.offdiagH, (size_t)tw * 8, cudaMemcpyDeviceToHost));
    }
    long long n = 0;
    for (unsigned long long j = 0; j < tw; ++j) {
        const long long *r = &rows[j * R];
        bool occ = e.st.n_core > 0 && ((r[W + L] >> NECI_FLAG_DETERMINISTIC_1) & 1);
        for (int k = 0; k < L; ++k) {
            double v;
            std::memcpy(&v, &r[W + k], 8);
            if (std::fabs(v) >= 1e-12) occ = true;
        }
        if (!occ) continue;
        if (n >= max_rows) return fail(NECI_GPU_ERR_INVALID, "download: output too small");
        std::memcpy(ilut + (size_t)n * R, r, (size_t)R * 8);
        if (dh) dh[n] = d1[j];
        if (odh) odh[n] = d2[j];
        ++n;
    }
    *nrows = n;
    return NECI_GPU_OK;
}

// What a context still lacks before it can step (nullptr when ready).
static const char *not_ready(const Engine &e) {
    if (!e.have_ref) return "set the reference first";
    if (!e.sys.tmat) return "set TMat2D first";
    if (e.sys.system == NECI_SYS_MOLECULAR && !e.sys.umat) return "set UMAT first";
    if (e.sys.system == NECI_SYS_MOLECULAR && e.sys.excitgen == NECI_EXGEN_PCHB && !e.have_pchb)
        return "call neci_gpu_init_pchb first";
    if (e.sys.system == NECI_SYS_HUBBARD_REAL_SPACE && !e.sys.neighbours) return "set the lattice first";
    return nullptr;
}

// Pass 1 of the annihilation (the hash lookup of every spawn) moves into the
// spawn kernel where spawns are frequent enough for its lookups to fill a
// warp's lanes; where they are rare a separate kernel packs them 32 to a warp.
// On GB300 a spawn rate of 0.41 (the 6x6 Hubbard lattice) made the fused step
// 10% faster, rates of 0.16 and 0.024 (molecules) 3% and 9% slower, so only
// the lattice instances of the spawn kernel carry the fused path.  Decided
// from the last step, with a margin against flipping; a change drops the
// captured step graphs.
static void update_fuse_probe(Engine &e, const neci_gpu_iter_stats &last) {
    if (e.fuse_mode >= 0 || e.ann_mode != NECI_ANN_HASH) return;  // fixed by NECI_OPT_FUSE_PROBE, or no hash passes
    if (e.sys.rdm || e.sys.excitgen != NECI_EXGEN_RS_HUBBARD || last.n_attempts <= 0) return;
    const double rate = (double)last.n_spawned / (double)last.n_attempts;
    const bool want = e.fuse_probe ? rate >= 0.25 : rate >= 0.3;
    if (want != e.fuse_probe) {
        e.fuse_probe = want;
        drop_graphs(e);
    }
}

// The merge sweep's blocks per SM while it runs beside the placement: two
// where the branch of the new determinants is the longer one (many unique
// spawned determinants per slot: n = 24, the Hubbard lattice), four, as
// alone, where the merge sweep is (a large list with few spawns per slot:
// n = 64), with a margin so that the choice does not flap.
static void update_merge_blocks(Engine &e, const neci_gpu_iter_stats &last) {
    if (last.tot_walkers <= 0) return;
    const double r = (double)last.n_unique / (double)last.tot_walkers;
    const int want = e.merge_bpsm == 2 ? (r < 0.10 ? 4 : 2) : (r > 0.20 ? 2 : 4);
    if (want != e.merge_bpsm) {
        e.merge_bpsm = want;
        drop_graphs(e);
    }
}

// Compaction of the walker list runs between calls, before the first step
// of a call whose last step left more holes than occupied slots (the rule
// k_final applies to Control::compact; the compaction kernels check that
// flag and ask for the rebuild of the walker hash, which the next step
// does).  It is not part of the step graph: holes cost only sweep work, and
// the five launches would do nothing in almost every step.
static void update_compact_due(Engine &e, const neci_gpu_iter_stats &last) {
    e.compact_due = last.tot_walkers > 4ll * kCompactTile && 2 * last.holes_in_list > last.tot_walkers;
}
static void compact_if_due(Engine &e, cudaStream_t s) {
    if (!e.compact_due) return;
    stage(e, K_COMPACT, [&] { launch_compact(e, s); });
    e.compact_due = false;
}

static int run_steps(Engine &e, const neci_gpu_iter_params *p, int n_iter, neci_gpu_iter_stats *stats,
                     double *device_ms = nullptr) {
    if (const char *why = not_ready(e)) return fail(NECI_GPU_ERR_INVALID, why);
    if (p->tau <= 0.0 || p->av_mc_excits <= 0.0) return fail(NECI_GPU_ERR_INVALID, "tau and AvMCExcits must be positive");
    copy_params(*e.h_params, *p);
    CK(cudaMemcpyAsync(e.d_params, e.h_params, sizeof(IterParams), cudaMemcpyHostToDevice, e.stream));
    compact_if_due(e, e.stream);
    int done = 0;
    if (device_ms) *device_ms = 0.0;
    while (done < n_iter) {
        if (!e.profiling)
            if (int r = ensure_graph(e)) return r;
        const int batch = std::min(n_iter - done, e.max_stats);
        CK(cudaMemsetAsync(e.d_stat_pos, 0, sizeof(int), e.stream));
        if (device_ms) CK(cudaEventRecord(e.ev[0], e.stream));
        if (e.profiling) {
            for (int i = 0; i < batch; ++i) step_sequence(e, e.d_stats, 1);
        } else {
            for (int i = 0; i < batch; ++i) CK(cudaGraphLaunch(e.graph, e.stream));
        }
        if (device_ms) CK(cudaEventRecord(e.ev[1], e.stream));
        CK(cudaMemcpyAsync(e.h_stats, e.d_stats, sizeof(neci_gpu_iter_stats) * batch, cudaMemcpyDeviceToHost, e.stream));
        CK(cudaStreamSynchronize(e.stream));
        CK(cudaGetLastError());
        if (device_ms) {
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, e.ev[0], e.ev[1]));
            *device_ms += ms;
        }
        std::memcpy(stats + done, e.h_stats, sizeof(neci_gpu_iter_stats) * batch);
        for (int i = 0; i < batch; ++i)
            if (stats[done + i].err) {
                done += i + 1;
                return fail(stats[done - 1].err, "device reported an error in the step");
            }
        done += batch;
        update_fuse_probe(e, stats[done - 1]);
        update_merge_blocks(e, stats[done - 1]);
        update_compact_due(e, stats[done - 1]);
        if (done < n_iter) compact_if_due(e, e.stream);
    }
    return NECI_GPU_OK;
}

int32_t neci_gpu_iterate(neci_gpu_ctx *ctx, const neci_gpu_iter_params *p, neci_gpu_iter_stats *stats) {
    if (int r = check_ctx(ctx)) return r;
    if (!p || !stats) return fail(NECI_GPU_ERR_INVALID, "null argument");
    return run_steps(ctx->e, p, 1, stats);
}

int32_t neci_gpu_iterate_n(neci_gpu_ctx *ctx, const neci_gpu_iter_params *p, int32_t n_iter, neci_gpu_iter_stats *stats) {
    if (int r = check_ctx(ctx)) return r;
    if (!p || !stats || n_iter < 1) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    return run_steps(ctx->e, p, n_iter, stats);
}

int32_t neci_gpu_iterate_timed(neci_gpu_ctx *ctx, const neci_gpu_iter_params *p, int32_t n_iter,
                               neci_gpu_iter_stats *stats, double *device_ms) {
    if (int r = check_ctx(ctx)) return r;
    if (!p || !stats || n_iter < 1 || !device_ms) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    if (ctx->e.profiling) return fail(NECI_GPU_ERR_INVALID, "timed steps need profiling off");
    return run_steps(ctx->e, p, n_iter, stats, device_ms);
}

int32_t neci_gpu_iterate_batch(neci_gpu_ctx **ctxs, int32_t n_ctx, const neci_gpu_iter_params *params, int32_t n_iter,
                               neci_gpu_iter_stats *stats, double *device_ms) {
    if (!ctxs || !params || !stats || n_ctx < 1 || n_iter < 1) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    const int dev = ctxs[0] ? ctxs[0]->e.device : 0;
    for (int c = 0; c < n_ctx; ++c) {
        if (!ctxs[c]) return fail(NECI_GPU_ERR_INVALID, "null context in batch");
        Engine &e = ctxs[c]->e;
        if (e.device != dev) return fail(NECI_GPU_ERR_INVALID, "batched contexts must share one device");
        if (e.profiling) return fail(NECI_GPU_ERR_INVALID, "batched steps need profiling off");
        if (n_iter > e.max_stats) return fail(NECI_GPU_ERR_INVALID, "n_iter above the per-context stats buffer");
        if (const char *why = not_ready(e)) return fail(NECI_GPU_ERR_INVALID, why);
    }
    CK(cudaSetDevice(dev));
    Engine &e0 = ctxs[0]->e;
    // What every branch captures: its context's kernels as its parameters and
    // state choose them (precision, sweep instance, core space; the rest
    // changes the context's graph version)
    std::vector<std::pair<const void *, unsigned long long>> key;
    for (int c = 0; c < n_ctx; ++c) {
        Engine &e = ctxs[c]->e;
        copy_params(*e.h_params, params[c]);
        const unsigned long long v = e.graph_version * 8 + (e.h_params->precision == NECI_PREC_MIXED ? 4 : 0) +
                                     (sweep_fast(*e.h_params) ? 2 : 0) + (e.st.n_core > 0 ? 1 : 0);
        key.push_back({(const void *)ctxs[c], v});
    }
    if (!e0.batch_graph || e0.batch_key != key) {
        // One graph for a step of the whole batch: the first context's stream
        // forks to every other context's stream, each stream captures its
        // context's step, and all join back; the instances run side by side
        // and the batch is one launch per step.
        if (e0.batch_graph) {
            cudaGraphExecDestroy(e0.batch_graph);
            e0.batch_graph = nullptr;
        }
        e0.batch_key.clear();
        CK(cudaStreamBeginCapture(e0.stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaEventRecord(e0.fork_ev, e0.stream);
        for (int c = 1; c < n_ctx && ce == cudaSuccess; ++c) ce = cudaStreamWaitEvent(ctxs[c]->e.stream, e0.fork_ev, 0);
        if (ce == cudaSuccess)
            for (int c = 0; c < n_ctx; ++c) step_sequence(ctxs[c]->e, ctxs[c]->e.d_stats, 1);
        for (int c = 1; c < n_ctx && ce == cudaSuccess; ++c) {
            Engine &e = ctxs[c]->e;
            ce = cudaEventRecord(e.join_ev, e.stream);
            if (ce == cudaSuccess) ce = cudaStreamWaitEvent(e0.stream, e.join_ev, 0);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(e0.stream, &g);  // ends the capture whatever happened
        if (ce == cudaSuccess) ce = ee;
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&e0.batch_graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            e0.batch_graph = nullptr;
            (void)cudaGetLastError();
            return fail(NECI_GPU_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(ce));
        }
        e0.batch_key = key;
    }
    // parameters in, record counters reset, then one launch per step; the
    // whole batch runs in the first context's stream order
    for (int c = 0; c < n_ctx; ++c) {
        Engine &e = ctxs[c]->e;
        CK(cudaMemcpyAsync(e.d_params, e.h_params, sizeof(IterParams), cudaMemcpyHostToDevice, e0.stream));
        CK(cudaMemsetAsync(e.d_stat_pos, 0, sizeof(int), e0.stream));
        compact_if_due(e, e0.stream);
    }
    CK(cudaEventRecord(e0.ev[0], e0.stream));
    for (int i = 0; i < n_iter; ++i) CK(cudaGraphLaunch(e0.batch_graph, e0.stream));
    CK(cudaEventRecord(e0.ev[1], e0.stream));
    for (int c = 0; c < n_ctx; ++c) {
        Engine &e = ctxs[c]->e;
        CK(cudaMemcpyAsync(e.h_stats, e.d_stats, sizeof(neci_gpu_iter_stats) * n_iter, cudaMemcpyDeviceToHost,
                           e0.stream));
    }
    CK(cudaStreamSynchronize(e0.stream));
    CK(cudaGetLastError());
    if (device_ms) {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, e0.ev[0], e0.ev[1]));
        *device_ms = ms;
    }
    int first_err = 0;
    for (int c = 0; c < n_ctx; ++c) {
        Engine &e = ctxs[c]->e;
        std::memcpy(stats + (size_t)c * n_iter, e.h_stats, sizeof(neci_gpu_iter_stats) * n_iter);
        for (int i = 0; i < n_iter && !first_err; ++i) first_err = e.h_stats[i].err;
        if (!first_err) {
            update_fuse_probe(e, e.h_stats[n_iter - 1]);
            update_merge_blocks(e, e.h_stats[n_iter - 1]);
            update_compact_due(e, e.h_stats[n_iter - 1]);
        }
    }
    if (first_err) return fail(first_err, "device reported an error in a batched step");
    return NECI_GPU_OK;
}

static int upload_spawns(Engine &e, const int64_t *sp, int64_t n) {
    if (n < 0 || n > e.st.max_spawned) return fail(NECI_GPU_ERR_SPAWN_FULL, "spawn list longer than MaxSpawned");
    if (n > 0) CK(cudaMemcpyAsync(e.st.spawn, sp, (size_t)n * e.sys.R * 8, cudaMemcpyHostToDevice, e.stream));
    launch_convert_spawns(e, n);
    return NECI_GPU_OK;
}

int32_t neci_gpu_annihilate(neci_gpu_ctx *ctx, const neci_gpu_iter_params *p, const int64_t *spawned, int64_t n,
                            neci_gpu_iter_stats *stats) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!p || !stats || (!spawned && n > 0)) return fail(NECI_GPU_ERR_INVALID, "null argument");
    copy_params(*e.h_params, *p);
    CK(cudaMemcpyAsync(e.d_params, e.h_params, sizeof(IterParams), cudaMemcpyHostToDevice, e.stream));
    launch_rehash(e, e.stream);
    launch_begin(e, e.stream);
    launch_collect_holes(e);
    if (int r = upload_spawns(e, spawned, n)) return r;
    // every record is written: the spawn kernel's fused lookup plays no part
    const bool fused = e.fuse_probe;
    const int mode = e.fuse_mode;
    e.fuse_mode = 0;
    annihilation_passes(e, 1);
    e.fuse_probe = fused;
    e.fuse_mode = mode;
    launch_ann_insert(e, e.stream, 0);
    launch_merge_stats(e, e.stream, 0, 0);
    launch_final(e, e.stream, e.d_stats, nullptr, 0, 0);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(e.h_stats, e.d_stats, sizeof(neci_gpu_iter_stats), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    *stats = e.h_stats[0];
    stats->n_spawned = n;
    if (stats->err) return fail(stats->err, "device reported an error in the annihilation");
    return NECI_GPU_OK;
}

int32_t neci_gpu_compress_spawns(neci_gpu_ctx *ctx, const int64_t *spawned, int64_t n, int64_t *out, int64_t *n_out,
                                 double *nannihil) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if ((!spawned && n > 0) || !out || !n_out) return fail(NECI_GPU_ERR_INVALID, "null argument");
    const int R = e.sys.R, W = e.sys.W, L = e.sys.L;
    launch_begin(e, e.stream);
    if (int r = upload_spawns(e, spawned, n)) return r;
    annihilation_passes(e, 0);
    // the output buffers come from the stream's pool and go back to it on
    // every exit, the early returns of a failed call included
    struct StreamBuffers {
        cudaStream_t s;
        long long *out = nullptr;
        unsigned long long *n = nullptr;
        ~StreamBuffers() {
            if (out) cudaFreeAsync(out, s);
            if (n) cudaFreeAsync(n, s);
        }
    } buf{e.stream};
    CK(cudaMallocAsync(&buf.out, (size_t)std::max<int64_t>(n, 1) * R * 8, e.stream));
    CK(cudaMallocAsync(&buf.n, sizeof(unsigned long long), e.stream));
    long long *const d_out = buf.out;
    unsigned long long *const d_n = buf.n;
    CK(cudaMemsetAsync(d_n, 0, sizeof(unsigned long long), e.stream));
    launch_compress_out(e, d_out, d_n);
    CK(cudaGetLastError());
    unsigned long long hn = 0;
    Control c{};
    CK(cudaMemcpyAsync(&hn, d_n, sizeof(hn), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaMemcpyAsync(&c, e.st.ctl, sizeof(Control), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    std::vector<long long> rows((size_t)hn * R);
    if (hn) CK(cudaMemcpyAsync(rows.data(), d_out, (size_t)hn * R * 8, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    if (c.err) return fail(c.err, "device reported an error in the compression");
    // order of CompressSpawnedList's output: sorted by ilut_lt
    std::vector<size_t> idx(hn);
    for (size_t i = 0; i < hn; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
        for (int w = 0; w < W; ++w)
            if (rows[a * R + w] != rows[b * R + w]) return rows[a * R + w] < rows[b * R + w];
        return false;
    });
    for (size_t i = 0; i < hn; ++i) std::memcpy(out + i * R, &rows[idx[i] * R], (size_t)R * 8);
    *n_out = (int64_t)hn;
    if (nannihil)
        for (int k = 0; k < L; ++k) nannihil[k] = (double)(long long)(c.abs_q[k] - c.abs_s[k]) * 0x1.0p-32;
    return NECI_GPU_OK;
}

int32_t neci_gpu_find_walker_hash(neci_gpu_ctx *ctx, const int64_t *dets, int64_t n, int64_t len, int64_t *out) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (n < 0 || len < 1 || (n > 0 && (!dets || !out))) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    if (n == 0) return NECI_GPU_OK;
    long long *dd, *dout;
    if (int r = batch_io(e, (const long long *)dets, (size_t)n * e.sys.W, &dd)) return r;
    if (int r = batch_io<long long>(e, nullptr, (size_t)n, &dout)) return r;
    launch_util_hash(e, dd, n, (unsigned long long)len, dout);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout, (size_t)n * 8, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaFreeAsync(dd, e.stream));
    CK(cudaFreeAsync(dout, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    return NECI_GPU_OK;
}

int32_t neci_gpu_excit_level(neci_gpu_ctx *ctx, const int64_t *a, const int64_t *b, int64_t n, int32_t *out) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (n < 0 || (n > 0 && (!a || !b || !out))) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    if (n == 0) return NECI_GPU_OK;
    long long *da, *db;
    int *dout;
    if (int r = batch_io(e, (const long long *)a, (size_t)n * e.sys.W, &da)) return r;
    if (int r = batch_io(e, (const long long *)b, (size_t)n * e.sys.W, &db)) return r;
    if (int r = batch_io<int>(e, nullptr, (size_t)n, &dout)) return r;
    launch_util_excit_level(e, da, db, n, dout);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaFreeAsync(da, e.stream));
    CK(cudaFreeAsync(db, e.stream));
    CK(cudaFreeAsync(dout, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    return NECI_GPU_OK;
}

int32_t neci_gpu_helement(neci_gpu_ctx *ctx, const int64_t *a, const int64_t *b, int64_t n, double *out) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (n < 0 || (n > 0 && (!a || !b || !out))) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    if (!e.sys.tmat) return fail(NECI_GPU_ERR_INVALID, "set TMat2D first");
    if (e.sys.system == NECI_SYS_MOLECULAR && !e.sys.umat) return fail(NECI_GPU_ERR_INVALID, "set UMAT first");
    if (n == 0) return NECI_GPU_OK;
    long long *da, *db;
    double *dout;
    if (int r = batch_io(e, (const long long *)a, (size_t)n * e.sys.W, &da)) return r;
    if (int r = batch_io(e, (const long long *)b, (size_t)n * e.sys.W, &db)) return r;
    if (int r = batch_io<double>(e, nullptr, (size_t)n, &dout)) return r;
    launch_util_helement(e, da, db, n, dout);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout, (size_t)n * 8, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaFreeAsync(da, e.stream));
    CK(cudaFreeAsync(db, e.stream));
    CK(cudaFreeAsync(dout, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    return NECI_GPU_OK;
}

int32_t neci_gpu_gen_excit(neci_gpu_ctx *ctx, const int64_t *det, int64_t n, uint64_t seed, int64_t iter,
                           int64_t *child, double *pgen, double *hel) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (n < 0 || !det || (n > 0 && (!child || !pgen || !hel))) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    if (const char *why = not_ready(e)) return fail(NECI_GPU_ERR_INVALID, why);
    if (n == 0) return NECI_GPU_OK;
    int nel = 0;
    for (int w = 0; w < e.sys.W; ++w) nel += __builtin_popcountll((unsigned long long)det[w]);
    if (nel != e.sys.nel) return fail(NECI_GPU_ERR_INVALID, "determinant has the wrong electron count");
    long long *dd, *dc;
    double *dp, *dh;
    if (int r = batch_io(e, (const long long *)det, (size_t)e.sys.W, &dd)) return r;
    if (int r = batch_io<long long>(e, nullptr, (size_t)n * e.sys.W, &dc)) return r;
    if (int r = batch_io<double>(e, nullptr, (size_t)n, &dp)) return r;
    if (int r = batch_io<double>(e, nullptr, (size_t)n, &dh)) return r;
    launch_util_gen_excit(e, dd, n, seed, iter, dc, dp, dh);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(child, dc, (size_t)n * e.sys.W * 8, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaMemcpyAsync(pgen, dp, (size_t)n * 8, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaMemcpyAsync(hel, dh, (size_t)n * 8, cudaMemcpyDeviceToHost, e.stream));
    CK(cudaFreeAsync(dd, e.stream));
    CK(cudaFreeAsync(dc, e.stream));
    CK(cudaFreeAsync(dp, e.stream));
    CK(cudaFreeAsync(dh, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    return NECI_GPU_OK;
}

}  // extern "C"

namespace {

// The core space from n_core determinants (W words each) in device memory:
// the previous core space's arrays are freed and its flags cleared, the new
// determinants are flagged deterministic and the core Hamiltonian is built
// as CSR (calc_determ_hamil_sparse, sparse_arrays.F90:426).
int core_build(Engine &e, const long long *dcore, long long n_core) {
    DevState &st = e.st;
    const int L = e.sys.L;
    // a new core space replaces the old one: its arrays are freed (the step
    // graphs that read them are dropped first) and its flags cleared below
    CK(cudaStreamSynchronize(e.stream));
    drop_graphs(e);
    st.n_core = 0;
    dfree(e, st.core_slot);
    dfree(e, st.core_x);
    dfree(e, st.core_x32);
    dfree(e, st.core_y);
    dfree(e, st.core_rowptr);
    dfree(e, st.core_col);
    dfree(e, st.core_val);
    dfree(e, st.core_val32);
    dfree(e, st.core_dets);
    dfree(e, st.core_seg);
    dfree(e, st.core_seg_first);
    dfree(e, st.core_seg_y);
    dfree(e, st.core_multi);
    st.n_core_seg = st.n_core_multi = 0;
    if (!st.core_of_slot) {
        if (int r = dalloc(e, &st.core_of_slot, (size_t)st.max_walkers)) return r;
    }
    CK(cudaMemsetAsync(st.core_of_slot, 0xFF, (size_t)st.max_walkers * 4, e.stream));
    launch_core_unmark(e);
    // the row counts, a set-up temporary freed on every exit
    struct Temp {
        Engine &e;
        long long *counts = nullptr;
        ~Temp() {
            cudaStreamSynchronize(e.stream);
            dfree(e, counts);
        }
    } tmp{e};
    if (int r = dalloc(e, &st.core_slot, (size_t)n_core)) return r;
    if (int r = dalloc(e, &st.core_x, (size_t)n_core * L)) return r;
    if (int r = dalloc(e, &st.core_x32, (size_t)n_core * L)) return r;
    if (int r = dalloc(e, &st.core_y, (size_t)n_core * L)) return r;
    if (int r = dalloc(e, &st.core_rowptr, (size_t)n_core + 1)) return r;
    if (int r = dalloc(e, &st.core_dets, (size_t)n_core * e.sys.W)) return r;
    CK(cudaMemcpyAsync(st.core_dets, dcore, (size_t)n_core * e.sys.W * 8, cudaMemcpyDeviceToDevice, e.stream));
    if (int r = dalloc(e, &tmp.counts, (size_t)n_core)) return r;
    long long *const counts = tmp.counts;
    CK(cudaMemsetAsync(&st.ctl->err, 0, sizeof(int), e.stream));
    launch_core_mark(e, dcore, n_core);
    launch_core_count(e, dcore, n_core, counts);
    CK(cudaGetLastError());
    std::vector<long long> hc(n_core), rp(n_core + 1, 0);
    CK(cudaMemcpyAsync(hc.data(), counts, (size_t)n_core * 8, cudaMemcpyDeviceToHost, e.stream));
    int err = 0;
    CK(cudaMemcpyAsync(&err, &st.ctl->err, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    if (err) {
        launch_core_unmark(e);
        CK(cudaMemsetAsync(&st.ctl->err, 0, sizeof(int), e.stream));
        return fail(NECI_GPU_ERR_INVALID, "core determinant not in CurrentDets");
    }
    for (long long i = 0; i < n_core; ++i) rp[i + 1] = rp[i] + hc[i];
    const long long nnz = rp[n_core];
    CK(cudaMemcpyAsync(st.core_rowptr, rp.data(), (size_t)(n_core + 1) * 8, cudaMemcpyHostToDevice, e.stream));
    if (int r = dalloc(e, &st.core_col, (size_t)nnz)) return r;
    if (int r = dalloc(e, &st.core_val, (size_t)nnz)) return r;
    if (int r = dalloc(e, &st.core_val32, (size_t)nnz)) return r;
    // segments of the rows: core_segment_len(G, per_lane) elements at most,
    // one for an empty row
    const int G = core_group_size(nnz, n_core);
    const long long S = core_segment_len(G, e.core_seg_lane);
    std::vector<long long> sfirst(n_core + 1, 0);
    std::vector<int32_t> multi;
    for (long long i = 0; i < n_core; ++i) {
        const long long ns = hc[i] > S ? (hc[i] + S - 1) / S : 1;
        sfirst[i + 1] = sfirst[i] + ns;
        if (ns > 1) multi.push_back((int32_t)i);
    }
    const long long nseg = sfirst[n_core];
    std::vector<CoreSeg> segs(nseg);
    for (long long i = 0; i < n_core; ++i)
        for (long long k = sfirst[i]; k < sfirst[i + 1]; ++k) {
            const long long e0 = rp[i] + (k - sfirst[i]) * S;
            const long long e1 = std::min(e0 + S, rp[i + 1]);
            const bool many = sfirst[i + 1] - sfirst[i] > 1;
            segs[k] = CoreSeg{e0, (int32_t)(e1 - e0), (int32_t)((uint32_t)i | (many ? 0x80000000u : 0u))};
        }
    if (int r = dalloc(e, &st.core_seg, (size_t)nseg)) return r;
    if (int r = dalloc(e, &st.core_seg_first, (size_t)n_core + 1)) return r;
    if (int r = dalloc(e, &st.core_seg_y, (size_t)(multi.empty() ? 1 : nseg) * L)) return r;
    if (int r = dalloc(e, &st.core_multi, multi.empty() ? (size_t)1 : multi.size())) return r;
    CK(cudaMemcpyAsync(st.core_seg, segs.data(), (size_t)nseg * sizeof(CoreSeg), cudaMemcpyHostToDevice, e.stream));
    CK(cudaMemcpyAsync(st.core_seg_first, sfirst.data(), (size_t)(n_core + 1) * 8, cudaMemcpyHostToDevice, e.stream));
    if (!multi.empty())
        CK(cudaMemcpyAsync(st.core_multi, multi.data(), multi.size() * 4, cudaMemcpyHostToDevice, e.stream));
    st.n_core = n_core;
    st.core_group = G;
    st.n_core_seg = nseg;
    st.core_seg_len = S;
    st.n_core_multi = (long long)multi.size();
    launch_core_fill(e, dcore, n_core);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e.stream));
    return NECI_GPU_OK;
}

// Allocates the arrays of the sort form of the annihilation (once).
int alloc_sort_buffers(Engine &e) {
    DevState &st = e.st;
    if (st.sk_key[0]) return NECI_GPU_OK;
    const size_t n = (size_t)st.max_spawned;
    st.sk_blocks = sort_ann_blocks(e);
    int hb = 0;
    while ((1ull << hb) < st.hash_n) ++hb;
    st.sk_hb = hb;
    int rc = NECI_GPU_OK;
    if (rc == NECI_GPU_OK) rc = dalloc(e, &st.sk_key[0], n);
    if (rc == NECI_GPU_OK) rc = dalloc(e, &st.sk_key[1], n);
    if (rc == NECI_GPU_OK) rc = dalloc(e, &st.sk_val[0], n);
    if (rc == NECI_GPU_OK) rc = dalloc(e, &st.sk_val[1], n);
    if (rc == NECI_GPU_OK) rc = dalloc(e, &st.sk_h, n);
    // counts for the most blocks a tuning may give a radix pass (4 per SM)
    if (rc == NECI_GPU_OK) rc = dalloc(e, &st.sk_counts, (size_t)kSortBins * (4 * e.num_sms + 1));
    if (rc == NECI_GPU_OK) rc = dalloc(e, &st.sk_long, n / 32 + 2);
    if (rc == NECI_GPU_OK && cudaStreamSynchronize(e.stream) != cudaSuccess) rc = fail(NECI_GPU_ERR_CUDA, "sync");
    if (rc != NECI_GPU_OK) {
        dfree(e, st.sk_key[0]);
        dfree(e, st.sk_key[1]);
        dfree(e, st.sk_val[0]);
        dfree(e, st.sk_val[1]);
        dfree(e, st.sk_h);
        dfree(e, st.sk_counts);
        dfree(e, st.sk_long);
    }
    return rc;
}

// A tuning's settings checked and applied (the step graphs are captured
// again with them).
int apply_tuning(Engine &e, const neci_gpu_tuning &t) {
    if ((t.annihilation != NECI_ANN_HASH && t.annihilation != NECI_ANN_SORT) || t.spawn_blocks_per_sm < 1 ||
        t.spawn_blocks_per_sm > 16 || t.table_shift < 1 || t.table_shift > 4 || t.sort_blocks_per_sm < 1 ||
        t.sort_blocks_per_sm > 4)
        return fail(NECI_GPU_ERR_INVALID, "tuning out of range: annihilation NECI_ANN_*, spawn blocks per SM 1..16, "
                                          "table shift 1..4, sort blocks per SM 1..4");
    e.sort_bpsm = t.sort_blocks_per_sm;
    if (t.annihilation == NECI_ANN_SORT)
        if (int r = alloc_sort_buffers(e)) return r;
    if (e.st.sk_key[0]) e.st.sk_blocks = sort_ann_blocks(e);
    e.ann_mode = t.annihilation;
    e.spawn_occ = t.spawn_blocks_per_sm;
    e.st.comp_shift = t.table_shift;
    drop_graphs(e);
    return NECI_GPU_OK;
}

neci_gpu_tuning current_tuning(const Engine &e) {
    neci_gpu_tuning t{};
    t.annihilation = e.ann_mode;
    t.spawn_blocks_per_sm = e.spawn_occ;
    t.table_shift = e.st.comp_shift;
    t.sort_blocks_per_sm = e.sort_bpsm;
    t.ns_per_update = 0.0;
    return t;
}

}  // namespace

extern "C" {

int32_t neci_gpu_set_tuning(neci_gpu_ctx *ctx, const neci_gpu_tuning *t) {
    if (int r = check_ctx(ctx)) return r;
    if (!t) return fail(NECI_GPU_ERR_INVALID, "null tuning");
    return apply_tuning(ctx->e, *t);
}

int32_t neci_gpu_get_tuning(neci_gpu_ctx *ctx, neci_gpu_tuning *t) {
    if (int r = check_ctx(ctx)) return r;
    if (!t) return fail(NECI_GPU_ERR_INVALID, "null tuning");
    *t = current_tuning(ctx->e);
    return NECI_GPU_OK;
}

int32_t neci_gpu_autotune(neci_gpu_ctx *ctx, const neci_gpu_iter_params *params, int32_t steps_per_setting,
                          neci_gpu_iter_stats *stats, int32_t max_stats, int32_t *n_steps, neci_gpu_tuning *chosen) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!params || !stats || !n_steps || steps_per_setting < 1) return fail(NECI_GPU_ERR_INVALID, "bad argument");
    if (e.profiling) return fail(NECI_GPU_ERR_INVALID, "autotuning needs profiling off");
    // the candidate settings: the hash form with the spawn grid at 8, 6 or 4
    // blocks per SM and the compression table at load 1/2 or 1/4, and the
    // sort form with 1, 2 or 4 radix-pass blocks per SM
    static const neci_gpu_tuning cands[] = {
        {NECI_ANN_HASH, 8, 1, 2, 0.0, {0}}, {NECI_ANN_HASH, 6, 1, 2, 0.0, {0}}, {NECI_ANN_HASH, 4, 1, 2, 0.0, {0}},
        {NECI_ANN_HASH, 8, 2, 2, 0.0, {0}}, {NECI_ANN_SORT, 8, 1, 1, 0.0, {0}}, {NECI_ANN_SORT, 8, 1, 2, 0.0, {0}},
        {NECI_ANN_SORT, 8, 1, 4, 0.0, {0}}};
    const int per = 1 + steps_per_setting;  // one untimed step captures the setting's graph
    neci_gpu_iter_params p = *params;
    const neci_gpu_tuning start = current_tuning(e);
    neci_gpu_tuning best = start;
    double best_cost = -1.0;
    int done = 0;
    for (const neci_gpu_tuning &c : cands) {
        if (done + per > max_stats) break;
        if (apply_tuning(e, c) != NECI_GPU_OK) continue;  // e.g. no memory for the sort form
        if (int r = run_steps(e, &p, 1, stats + done)) { *n_steps = done + 1; return r; }
        p.iter += 1;
        double ms = 0.0;
        if (int r = run_steps(e, &p, steps_per_setting, stats + done + 1, &ms)) { *n_steps = done + per; return r; }
        p.iter += steps_per_setting;
        double upd = 0.0;
        for (int i = 1; i < per; ++i)
            for (int k = 0; k < e.sys.L; ++k) upd += stats[done + i].tot_parts_old[k];
        done += per;
        const double cost = upd > 0.0 ? ms * 1e6 / upd : 0.0;  // ns per walker update
        if (best_cost < 0.0 || cost < best_cost) {
            best_cost = cost;
            best = c;
            best.ns_per_update = cost;
        }
    }
    *n_steps = done;
    if (int r = apply_tuning(e, best_cost < 0.0 ? start : best)) return r;
    if (chosen) *chosen = best;
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_core_space(neci_gpu_ctx *ctx, const int64_t *core, int64_t n_core, int32_t precision) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    (void)precision;  // both value arrays are kept; the step's precision picks one
    if (n_core < 1 || !core || n_core >= (1ll << 31)) return fail(NECI_GPU_ERR_INVALID, "bad core space");
    struct Temp {
        Engine &e;
        long long *dcore = nullptr;
        ~Temp() {
            cudaStreamSynchronize(e.stream);
            dfree(e, dcore);
        }
    } tmp{e};
    if (int r = dalloc(e, &tmp.dcore, (size_t)n_core * e.sys.W)) return r;
    CK(cudaMemcpyAsync(tmp.dcore, core, (size_t)n_core * e.sys.W * 8, cudaMemcpyHostToDevice, e.stream));
    return core_build(e, tmp.dcore, n_core);
}

int32_t neci_gpu_select_core(neci_gpu_ctx *ctx, int64_t n_core, int32_t precision, int64_t *core_dets,
                             int64_t *n_selected) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    (void)precision;
    if (n_core < 1 || n_core >= (1ll << 31)) return fail(NECI_GPU_ERR_INVALID, "bad core size");
    if (!e.have_ref) return fail(NECI_GPU_ERR_INVALID, "set the reference first");
    DevState &st = e.st;
    const size_t n = (size_t)st.max_walkers;
    const int blocks = (int)std::min<long long>((long long)e.num_sms * 2, st.max_walkers / 4096 + 1);
    // the sort's scratch: keys and slots, two buffers each, the digit counts
    // and the occupied count, freed on every exit
    struct Temp {
        Engine &e;
        unsigned long long *key[2] = {nullptr, nullptr}, *n_occ = nullptr;
        uint32_t *val[2] = {nullptr, nullptr}, *counts = nullptr;
        long long *dcore = nullptr;
        ~Temp() {
            cudaStreamSynchronize(e.stream);
            dfree(e, key[0]);
            dfree(e, key[1]);
            dfree(e, val[0]);
            dfree(e, val[1]);
            dfree(e, counts);
            dfree(e, n_occ);
            dfree(e, dcore);
        }
    } t{e};
    if (int r = dalloc(e, &t.key[0], n)) return r;
    if (int r = dalloc(e, &t.key[1], n)) return r;
    if (int r = dalloc(e, &t.val[0], n)) return r;
    if (int r = dalloc(e, &t.val[1], n)) return r;
    if (int r = dalloc(e, &t.counts, (size_t)kSortBins * (blocks + 1))) return r;
    if (int r = dalloc(e, &t.n_occ, 1)) return r;
    const int cur = launch_core_select_sort(e, t.key, t.val, t.counts, blocks, t.n_occ);
    CK(cudaGetLastError());
    unsigned long long occ = 0;
    CK(cudaMemcpyAsync(&occ, t.n_occ, sizeof(occ), cudaMemcpyDeviceToHost, e.stream));
    CK(cudaStreamSynchronize(e.stream));
    const long long nsel = std::min<long long>(n_core, (long long)occ);
    if (n_selected) *n_selected = nsel;
    if (nsel < 1) return fail(NECI_GPU_ERR_INVALID, "no occupied determinant to select");
    if (int r = dalloc(e, &t.dcore, (size_t)nsel * e.sys.W)) return r;
    launch_core_select_gather(e, t.val[cur], nsel, t.dcore);
    CK(cudaGetLastError());
    if (core_dets)
        CK(cudaMemcpyAsync(core_dets, t.dcore, (size_t)nsel * e.sys.W * 8, cudaMemcpyDeviceToHost, e.stream));
    return core_build(e, t.dcore, nsel);
}

int32_t neci_gpu_set_option(neci_gpu_ctx *ctx, int32_t option, int32_t value) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (option == NECI_OPT_FUSE_PROBE) {
        if (value < -1 || value > 1) return fail(NECI_GPU_ERR_INVALID, "NECI_OPT_FUSE_PROBE takes -1, 0 or 1");
        if (value == 1 && e.sys.excitgen != NECI_EXGEN_RS_HUBBARD)
            return fail(NECI_GPU_ERR_UNSUPPORTED, "the fused lookup exists for lattice systems only");
        e.fuse_mode = value;
        drop_graphs(e);
        return NECI_GPU_OK;
    }
    if (option == NECI_OPT_ANNIHILATION) {
        if (value != NECI_ANN_HASH && value != NECI_ANN_SORT)
            return fail(NECI_GPU_ERR_INVALID, "NECI_OPT_ANNIHILATION takes NECI_ANN_HASH or NECI_ANN_SORT");
        if (value == NECI_ANN_SORT)
            if (int r = alloc_sort_buffers(e)) return r;
        e.ann_mode = value;
        drop_graphs(e);
        return NECI_GPU_OK;
    }
    if (option == NECI_OPT_CORE_SEGMENT) {
        if (value < 1 || value > 65536) return fail(NECI_GPU_ERR_INVALID, "NECI_OPT_CORE_SEGMENT takes 1..65536");
        e.core_seg_lane = value;  // used by the next core_build
        return NECI_GPU_OK;
    }
    return fail(NECI_GPU_ERR_INVALID, "unknown option");
}

int32_t neci_gpu_core_nnz(neci_gpu_ctx *ctx, int64_t *nnz) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    if (!nnz) return fail(NECI_GPU_ERR_INVALID, "null argument");
    if (e.st.n_core == 0) { *nnz = 0; return NECI_GPU_OK; }
    long long v = 0;
    CK(cudaMemcpy(&v, e.st.core_rowptr + e.st.n_core, 8, cudaMemcpyDeviceToHost));
    *nnz = v;
    return NECI_GPU_OK;
}

int32_t neci_gpu_set_profiling(neci_gpu_ctx *ctx, int32_t on) {
    if (int r = check_ctx(ctx)) return r;
    ctx->e.profiling = on != 0;
    return NECI_GPU_OK;
}

int32_t neci_gpu_kernel_times(neci_gpu_ctx *ctx, double *ms, int64_t *launches, int32_t n) {
    if (int r = check_ctx(ctx)) return r;
    Engine &e = ctx->e;
    for (int k = 0; k < n && k < K_NUM; ++k) {
        if (ms) ms[k] = e.kernel_ms[k];
        if (launches) launches[k] = e.kernel_launches[k];
        e.kernel_ms[k] = 0.0;
        e.kernel_launches[k] = 0;
    }
    return NECI_GPU_OK;
}

int32_t neci_gpu_sync(neci_gpu_ctx *ctx) {
    if (int r = check_ctx(ctx)) return r;
    CK(cudaStreamSynchronize(ctx->e.stream));
    return NECI_GPU_OK;
}

}  // extern "C"
