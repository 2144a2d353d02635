// internal.h -- host-side engine object shared by the C ABI and the launchers.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/neci_gpu.h"
#include "engine.cuh"

namespace neci {

enum KernelId {
    K_COMPACT = 0,
    K_REHASH,
    K_BEGIN,
    K_SWEEP,
    K_EXPAND,
    K_SPAWN,
    K_CORE,
    K_ANN_PROBE,
    K_ANN_COMPRESS,
    K_ANN_INSERT,
    K_MERGE_STATS,
    K_RDM,
    K_FINAL,
    K_SORT_KEYS,   // sort form of the annihilation: keys, radix passes, grouping
    K_SORT_RADIX,
    K_SORT_GROUP,
    K_NUM
};

struct Engine {
    neci_gpu_system desc{};
    DevSys sys{};
    DevState st{};
    int device = 0;
    int num_sms = 152;
    // resident blocks per SM of the grid-stride spawn-list kernels (their
    // grids fill the GPU once; the latency-bound hash passes want every warp)
    int occ_probe = 4, occ_compress = 4, occ_insert = 4, occ_place = 8, occ_expand = 4;
    // pass 1 of the annihilation runs inside the spawn kernel (chosen from the
    // last step's spawn rate; see update_fuse_probe)
    bool fuse_probe = false;
    // NECI_OPT_FUSE_PROBE: -1 chosen from the spawn rate, 0 never, 1 always
    int fuse_mode = -1;
    // NECI_OPT_ANNIHILATION: NECI_ANN_HASH or NECI_ANN_SORT
    int ann_mode = NECI_ANN_HASH;
    // tuned launch shapes (neci_gpu_tuning): spawn blocks per SM, radix-pass
    // blocks per SM (DevState::comp_shift holds the table load setting)
    int spawn_occ = 8;
    int sort_bpsm = 2;
    int merge_bpsm = 2;  // merge sweep blocks per SM beside the placement (update_merge_blocks)
    bool compact_due = false;  // the last step left more holes than occupied slots
    int core_seg_lane = kCoreSegmentPerLane;  // NECI_OPT_CORE_SEGMENT
    cudaStream_t stream = nullptr;
    IterParams *d_params = nullptr;
    IterParams *h_params = nullptr;          // pinned
    neci_gpu_iter_stats *d_stats = nullptr;  // per-step records
    neci_gpu_iter_stats *h_stats = nullptr;  // pinned
    int max_stats = 0;
    int *d_stat_pos = nullptr;               // the next record a step writes (k_final)
    // changes with every drop of the step graphs (a batch graph built on them
    // is rebuilt)
    unsigned long long graph_version = 0;
    // a batch graph (neci_gpu_iterate_batch) kept by the batch's first
    // context: every instance's step as one branch, and what it was built for
    cudaGraphExec_t batch_graph = nullptr;
    std::vector<std::pair<const void *, unsigned long long>> batch_key;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // the step's two branches after the walker-hash lookup (new determinants;
    // the merge sweep), on stream and side
    cudaStream_t side = nullptr;
    cudaEvent_t branch_ev = nullptr, merge_ev = nullptr;
    std::vector<void *> allocs;
    bool have_ref = false, have_pchb = false;
    double *inv_single = nullptr;  // device table of DevSys::inv_single
    float *inv_single32 = nullptr;
    // CUDA graph of one step per precision (FP64, mixed); `graph` is the one
    // ensure_graph selected for the current parameters
    cudaGraphExec_t graphs[2] = {nullptr, nullptr};
    bool graph_core[2] = {false, false};
    bool graph_fast[2] = {false, false};  // the sweep variant a graph was captured with
    cudaGraphExec_t graph = nullptr;
    // profiling
    bool profiling = false;
    cudaEvent_t ev[2 * K_NUM] = {};
    double kernel_ms[K_NUM] = {};
    long long kernel_launches[K_NUM] = {};
};

// Whether the spawn kernel does pass 1 of the annihilation (the walker-hash
// lookup of every child): lattice systems with the hash annihilation and no
// 2-RDM sampling, as NECI_OPT_FUSE_PROBE (or, by default, the spawn rate) says.
inline bool fused_lookup(const Engine &e) {
    if (e.sys.rdm || e.sys.excitgen != NECI_EXGEN_RS_HUBBARD || e.ann_mode != NECI_ANN_HASH) return false;
    return e.fuse_mode < 0 ? e.fuse_probe : e.fuse_mode == 1;
}

// launchers (kernels.cu)
void launch_begin(Engine &e, cudaStream_t s);
void launch_rehash(Engine &e, cudaStream_t s);
void launch_compact(Engine &e, cudaStream_t s);
void launch_sweep(Engine &e, cudaStream_t s);
// sets the per-kernel launch attributes a context needs (non-zero: failure)
int configure_kernels(Engine &e);
void launch_expand(Engine &e, cudaStream_t s);
void launch_spawn(Engine &e, cudaStream_t s);
void launch_core(Engine &e, cudaStream_t s);
void launch_ann_probe(Engine &e, cudaStream_t s);
void launch_ann_compress(Engine &e, cudaStream_t s);
void launch_ann_insert(Engine &e, cudaStream_t s, int split);
void launch_merge_stats(Engine &e, cudaStream_t s, int with_core, int split);
void launch_final(Engine &e, cudaStream_t s, neci_gpu_iter_stats *out, int *pos, int advance_iter, int split);
void launch_rdm(Engine &e, cudaStream_t s);

// sort form of the annihilation and core selection (sort_kernels.cu)
constexpr int kSortBins = 256;  // digit values of a radix pass (radix.cuh kRadixBins)
void launch_sort_keys(Engine &e, cudaStream_t s);
int launch_sort_radix(Engine &e, cudaStream_t s);
void launch_sort_group(Engine &e, cudaStream_t s, int lookup, int cur);
int sort_ann_blocks(const Engine &e);
int launch_core_select_sort(Engine &e, unsigned long long *key[2], uint32_t *val[2], uint32_t *counts, int blocks,
                            unsigned long long *n_occ);
void launch_core_select_gather(Engine &e, const uint32_t *slot, long long n, long long *core_dets);

// utility launchers (util_kernels.cu)
void launch_util_hash(Engine &e, const long long *dets, long long n, unsigned long long len, long long *out);
void launch_util_excit_level(Engine &e, const long long *a, const long long *b, long long n, int *out);
void launch_util_helement(Engine &e, const long long *a, const long long *b, long long n, double *out);
void launch_util_gen_excit(Engine &e, const long long *det, long long n, unsigned long long seed, long long iter,
                           long long *child, double *pgen, double *hel);
void launch_upload_fix(Engine &e, long long nrows, int compute_diag);
void launch_collect_holes(Engine &e);
void launch_convert_spawns(Engine &e, long long n);
void launch_all_cand(Engine &e);
void launch_compress_out(Engine &e, long long *out, unsigned long long *n_out);
void launch_core_unmark(Engine &e);
void launch_core_mark(Engine &e, const long long *core_dets, long long n_core);
void launch_core_count(Engine &e, const long long *core_dets, long long n_core, long long *counts);
void launch_core_fill(Engine &e, const long long *core_dets, long long n_core);
// PCHB alias tables; returns a cudaError_t value (0: built), and launches
// nothing when its scratch cannot be allocated
int launch_pchb_build(Engine &e);
void launch_build_jk(Engine &e, double *jrow, double *jkrow, float *jrow32, float *jkrow32);
void launch_build_jkmat(Engine &e, double *jmat, double *kmat);

}  // namespace neci
