// mtg_engine.cuh - the engine object behind the opaque mtg_engine handle.
// Internal to the library; shared by the .cu files that implement the ABI.
#pragma once
#include <string>
#include <vector>

#include "../../include/mtg.h"
#include "mtg_internal.cuh"

struct mtg_engine {
    using KParams = mtg::KParams;
    using DevBuffers = mtg::DevBuffers;
    mtg_params p{};
    KParams kp{};
    int nb = 0, nt = 0;
    int cur = 0;            // frame buffer holding the current state
    bool keep_forces = false;
    bool have_state = false;
    bool lists_valid = false;
    bool lists_fresh = false;   // mtg_rebuild_pairs ran after the last step
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;   // second stream of the learned step (M2L)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<int> h_off;
    // device
    int *off = nullptr, *traj = nullptr, *flags = nullptr, *harm = nullptr;
    float *zs = nullptr;
    float4 *frame[2] = {nullptr, nullptr};
    float4 *force = nullptr;
    uint4 *seeds = nullptr;
    int *ljc = nullptr, *lj = nullptr, *lonc = nullptr, *lon = nullptr, *latc = nullptr, *lat = nullptr;
    int *err = nullptr;
    int2 *work = nullptr;
    int nwork = 0;
    int2 *tea_work = nullptr;   // chunks of kTeaChunk beads for the TEA kernels
    int tea_nwork = 0;
    int *work_first = nullptr;
    double *en_partials = nullptr, *en_traj = nullptr, *en_bead = nullptr;
    float4 *tea_r = nullptr, *tea_ci = nullptr;
    float *tea_eps = nullptr, *tea_beta = nullptr;
    double *tea_eps_t = nullptr;
    float4 *tea_part = nullptr;    // kTeaMaxParts * nb partial sums (split TEA kernels)
    float *stage = nullptr;        // 7*nb floats for host <-> device Coord transfers
    void *stage_host = nullptr;    // pinned mirror of stage
    uint8_t *stage_u8 = nullptr;
    int *stage_i = nullptr;
    int device = 0;
    // graphs: [parity]
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_kernels[2] = {0, 0};      // kernel nodes of each captured graph
    long long graph_kernel_launches = 0;      // kernel nodes replayed since the last reset
    int graph_period = 0;
    // per-kernel timing (see mtg_set_kernel_timing)
    bool timing = false;
    std::vector<cudaEvent_t> ev_a, ev_b;
    std::vector<int> ev_kind;
    int graph_slot_base[2] = {0, 0}, graph_slot_count[2] = {0, 0};
    int direct_base = 0, direct_next = 0, capture_next = 0;
    bool capturing = false;
    std::vector<int> used_slots;
    double kt_total[MTG_KERNEL_KINDS] = {0};
    long long kt_count[MTG_KERNEL_KINDS] = {0};
    cudaEvent_t call_a = nullptr, call_b = nullptr;
    // plain steps between rebuilds as one persistent launch (k_step_period)
    bool persistent = false;
    // list rebuild method: 0 auto, 1 brute-force tiles, 2 cell list
    int list_method = 0;
    bool use_cells = false;
    int max_traj_beads = 0;
    int *cell_tbase = nullptr, *cell_tmask = nullptr, *cell_key = nullptr, *cell_cnt = nullptr;
    int *cell_start = nullptr, *cell_cursor = nullptr, *cell_bead = nullptr;
    float4 *cell_pos = nullptr;
    int cell_nbuckets = 0, cell_max_buckets = 0;
    // learned TEA (surrogate.cu)
    struct mtg_surrogate *surr = nullptr;
    int surr_recheck = 0;
    float surr_max_err = 0.01f;
    float *surr_desc = nullptr, *surr_pred = nullptr;
    float4 *surr_stats = nullptr;
    int *surr_gate = nullptr;      // [0] fell back to exact, [1] re-checks done, [2] fallback not yet applied
    double *surr_err = nullptr, *surr_part = nullptr;
    float4 *tea_ci2 = nullptr, *feff_a = nullptr, *feff_b = nullptr;
    float *tea_eps2 = nullptr, *tea_beta2 = nullptr;
    double *tea_eps_t2 = nullptr;
    // stride-step analytics (kernels_updater.cu)
    int *hydro_cand = nullptr, *hydro_rank = nullptr, *hydro_sums = nullptr, *hydro_counts = nullptr;
    int8_t *hydro_events = nullptr;
    int hydro_ncand = -1;
    // stride-step outputs (output.cu)
    struct mtg_output *output = nullptr;
    // far field of learned TEA (tea_ff.cu): partition, lists, proxy data
    bool ff_on = false;
    float ff_theta = 0.85f;
    int ff_refresh = 0;
    long long ff_steps = 0;          // steps since the partition was built
    int *ff_ints = nullptr;          // every int array of the partition, one allocation
    size_t ff_ints_cap = 0;
    float4 *ff_f4 = nullptr;         // boxes, proxy charges, proxy potentials
    size_t ff_f4_cap = 0;
    mtg::FFBuffers ffb{};
    long long ff_near_pairs = 0, ff_proxy_pairs = 0;
    std::vector<int> ff_host;        // the partition as built (for mtg_tea_farfield_layout)
    int ff_sizes[5] = {0, 0, 0, 0, 0};  // leaves, leaf beads, near entries, nodes, far entries
    // device address of the fixed scratch of mtg_energies_noalloc, looked up
    // by this engine's first call (energy_noalloc.cu)
    double *noalloc_scratch = nullptr;

    mtg::CellBuffers cells() const {
        mtg::CellBuffers c{};
        c.nbuckets = cell_nbuckets;
        c.max_buckets = cell_max_buckets;
        c.tbase = cell_tbase;
        c.tmask = cell_tmask;
        c.key = cell_key;
        c.cnt = cell_cnt;
        c.start = cell_start;
        c.cursor = cell_cursor;
        c.cell_bead = cell_bead;
        c.cell_pos = cell_pos;
        return c;
    }

    DevBuffers bufs() const {
        DevBuffers b{};
        b.off = off;
        b.traj = traj;
        b.flags = flags;
        b.harm = harm;
        b.zs = zs;
        b.frame_in = frame[cur];
        b.frame_out = frame[cur ^ 1];
        b.force = force;
        b.seeds = seeds;
        b.ljc = ljc;
        b.lj = lj;
        b.lonc = lonc;
        b.lon = lon;
        b.latc = latc;
        b.lat = lat;
        b.err = err;
        b.tea_part = tea_part;
        b.tea_r = tea_r;
        b.tea_ci = tea_ci;
        b.tea_eps = tea_eps;
        b.tea_beta = tea_beta;
        b.tea_eps_t = tea_eps_t;
        return b;
    }
};


// Records msg as the calling thread's last error (mtg_last_error_string) and
// returns code.
int mtg_internal_fail(int code, const char *msg);
void mtg_internal_close_output(mtg_engine *e);

// learned TEA helpers (surrogate.cu)
int mtg_surrogate_buffers(mtg_engine *e);
void enqueue_surrogate_eps(mtg_engine *e);
void enqueue_surrogate_recheck(mtg_engine *e);
// drops the captured step graphs (after a mode change)
void mtg_internal_reset_graphs(mtg_engine *e);
// far field of learned TEA (tea_ff.cu): rebuilds the partition when due
int mtg_internal_ff_refresh(mtg_engine *e);
void mtg_internal_ff_free(mtg_engine *e);
