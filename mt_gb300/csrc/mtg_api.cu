// mtg_api.cu - the engine object and the C ABI declared in include/mtg.h.
//
// Host orchestration of one batch on one GPU: device buffers owned by the
// engine, one CUDA stream per engine, the step loop replayed from CUDA graphs
// (one graph per pair-list period and frame-buffer parity), device error
// words read back once per call instead of a device synchronisation after
// every launch (the reference's checkCUDAError, src/Cuda.h:120-135).
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mtg.h"
#include "mtg_engine.cuh"

using namespace mtg;

namespace {

thread_local std::string g_last_error = "no error";

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return fail(MTG_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                       \
    } while (0)

// ran2 of the reference seeding (src/ran2.h:18-56) with its function statics
// held in a struct that starts from their initial values.
struct Ran2 {
    int idum2 = 123456789, iy = 0, iv[32] = {0};
    double next(int *idum) {
        const int IM1 = 2147483563, IM2 = 2147483399, IMM1 = IM1 - 1;
        const int IA1 = 40014, IA2 = 40692, IQ1 = 53668, IQ2 = 52774, IR1 = 12211, IR2 = 3791;
        const int NTAB = 32, NDIV = 1 + IMM1 / NTAB;
        int j, k;
        if (*idum <= 0) {
            *idum = (-(*idum) < 1) ? 1 : -(*idum);
            idum2 = *idum;
            for (j = NTAB + 7; j >= 0; j--) {
                k = *idum / IQ1;
                *idum = IA1 * (*idum - k * IQ1) - k * IR1;
                if (*idum < 0) *idum += IM1;
                if (j < NTAB) iv[j] = *idum;
            }
            iy = iv[0];
        }
        k = *idum / IQ1;
        *idum = IA1 * (*idum - k * IQ1) - k * IR1;
        if (*idum < 0) *idum += IM1;
        k = idum2 / IQ2;
        idum2 = IA2 * (idum2 - k * IQ2) - k * IR2;
        if (idum2 < 0) idum2 += IM2;
        j = iy / NDIV;
        iy = iv[j] - idum2;
        iv[j] = *idum;
        if (iy < 1) iy += IMM1;
        const double t = (1.0 / IM1) * iy;
        return t > 1.0 - 1.2e-7 ? 1.0 - 1.2e-7 : t;
    }
};

// generateSeeds (src/HybridTaus.cu:32-48): each component (unsigned)(ran2 *
// UINT_MAX), redrawn while below 128.
void make_seeds(int seed, size_t nstreams, std::vector<uint32_t> &out) {
    Ran2 r;
    out.resize(4 * nstreams);
    for (size_t i = 0; i < 4 * nstreams; i++) {
        uint32_t v;
        do {
            v = (uint32_t)(r.next(&seed) * (double)UINT_MAX);
        } while (v < 128u);
        out[i] = v;
    }
}

template <class T>
int dalloc(T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    CK(cudaMalloc((void **)p, n * sizeof(T)));
    return MTG_OK;
}

}  // namespace

int mtg_internal_fail(int code, const char *msg) { return fail(code, "%s", msg); }

void destroy_graphs(mtg_engine *e);
void mtg_internal_reset_graphs(mtg_engine *e) { destroy_graphs(e); }

namespace {

KParams make_kparams(const mtg_params &p, int nb, int nt, int maxH, int maxLong, int maxLat, int maxLJ) {
    KParams k{};
    k.nb = nb;
    k.nt = nt;
    // integrate_kernel coefficients, evaluated in float as src/compute_cuda.cu:955-961 does
    k.kr = p.dt / p.gammaR;
    k.kfi = p.dt / (p.gammaTheta * p.alpha);
    k.kth = p.dt / p.gammaTheta;
    k.varR = p.varR;
    k.nfi = p.varTheta * sqrtf(p.freeze_temp / p.alpha);
    k.varTheta = p.varTheta;
    k.C = p.C;
    k.B_psi = p.B_psi;
    k.B_fi = p.B_fi;
    k.B_theta = p.B_theta;
    k.psi_0 = p.psi_0;
    k.fi_0 = p.fi_0;
    k.th0_gtp = p.theta0_gtp;
    k.th0_gdp = p.theta0_gdp;
    k.A_long = p.A_long;
    k.D_long = p.D_long;
    k.A_lat = p.A_lat;
    k.D_lat = p.D_lat;
    k.D_lat_seam = p.D_lat / p.seam_coeff;
    k.barrier = p.barrier;
    k.a_bl = p.a_barr_long;
    k.r_bl = p.r_barr_long;
    k.w_bl = p.w_barr_long;
    k.a_bt = p.a_barr_lat;
    k.r_bt = p.r_barr_lat;
    k.w_bt = p.w_barr_lat;
    k.lj_on = p.lj_on;
    k.lj_pref = p.ljscale * p.ljsigma6;
    k.ljcut = p.ljpairscutoff;
    k.is_wall = p.is_wall;
    k.rep_r = p.rep_r;
    k.rep_eps = p.rep_eps;
    k.lb = p.rep_leftborder;
    k.is_assembly = p.is_assembly;
    // lateral binding sites (src/mt.h:44-50), float arithmetic as in the reference
    const float c = cosf((float)(2.0 * M_PI / 13.0)), s = sinf((float)(2.0 * M_PI / 13.0));
    k.p1x = 0.5f * 8.12f * (c - 1.0f);
    k.p1y = 0.5f * 8.12f * s;
    k.p1z = -3.0f * 2.0f / 13.0f;
    k.p2x = k.p1x;
    k.p2y = -k.p1y;
    k.p2z = -k.p1z;
    k.maxH = maxH;
    k.maxLong = maxLong;
    k.maxLat = maxLat;
    k.maxLJ = maxLJ;
    k.step_block = 128;
    k.tea_a = p.tea_a;
    k.tea_var = sqrtf(2.0f * 0.0019872041f * p.Temp * p.gammaR / p.dt);
    return k;
}

int check_params(const mtg_params *p) {
    if (!p) return fail(MTG_E_CONFIG, "params is NULL");
    if (!(p->dt > 0) || !(p->gammaR > 0) || !(p->gammaTheta > 0) || !(p->alpha > 0))
        return fail(MTG_E_CONFIG, "dt, gammaR, gammaTheta and alpha must be positive (call mtg_derive_params)");
    if (p->ljpairsupdatefreq <= 0) return fail(MTG_E_CONFIG, "ljpairsupdatefreq must be positive");
    if (p->hdi_on && p->tea_epsilon_freq <= 0)
        return fail(MTG_E_CONFIG, "tea_epsilon_freq must be positive with tea_on (the reference divides by it)");
    if (p->hdi_on && !(p->tea_a > 0)) return fail(MTG_E_CONFIG, "tea_a must be positive");
    if (p->seam_coeff == 0.0f) return fail(MTG_E_CONFIG, "seam_coeff must be non-zero");
    return MTG_OK;
}

int upload(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
    return MTG_OK;
}

int check_errors(mtg_engine *e) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, e->err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    CK(cudaGetLastError());
    if (h) {
        CK(cudaMemsetAsync(e->err, 0, sizeof(int), e->stream));
        if (h & kErrOverflow) return fail(MTG_E_OVERFLOW, "a neighbour list exceeded its capacity");
        if (h & kErrTeaEps)
            return fail(MTG_E_TEA_EPS, "TEA epsilon out of range (> 1 in capricious mode, > epsmax, or a too diagonal tensor)");
        if (h & kErrNonFinite) return fail(MTG_E_NONFINITE, "non-finite energy total");
        if (h & kErrTimeout) return fail(MTG_E_TIMEOUT, "a bounded wait for the tensor cores ran out");
    }
    return MTG_OK;
}

}  // namespace

void destroy_graphs(mtg_engine *e) {
    for (auto &g : e->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    e->graph_kernels[0] = e->graph_kernels[1] = 0;
    e->direct_base = 0;
    e->graph_slot_count[0] = e->graph_slot_count[1] = 0;
}

namespace {

// Kernel nodes of a captured graph.
long long count_kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) return 0;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
    long long k = 0;
    for (size_t i = 0; i < n; i++) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
    }
    return k;
}

// The list rebuild with the engine's method.
void launch_lists(mtg_engine *e) {
    if (e->use_cells)
        launch_rebuild_cells(e->kp, e->bufs(), e->cells(), e->work, e->nwork, e->stream);
    else
        launch_rebuild(e->kp, e->bufs(), e->work, e->nwork, e->stream);
}

void choose_list_method(mtg_engine *e) {
    const bool cells_ok = e->kp.maxLong <= kCellMaxLong && e->kp.maxLat <= kCellMaxLat && e->cell_tbase;
    if (e->list_method == 1 || !cells_ok)
        e->use_cells = false;
    else if (e->list_method == 2)
        e->use_cells = true;
    else
        e->use_cells = e->max_traj_beads >= 512;
}

// Event slot for one timed launch (created outside any stream capture).
int timing_slot(mtg_engine *e, int kind) {
    int &next = e->capturing ? e->capture_next : e->direct_next;
    const int s = next++;
    while ((int)e->ev_a.size() <= s) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        e->ev_a.push_back(a);
        e->ev_b.push_back(b);
        e->ev_kind.push_back(0);
    }
    e->ev_kind[s] = kind;
    if (!e->capturing) e->used_slots.push_back(s);
    return s;
}

template <class F>
void timed_launch(mtg_engine *e, int kind, F &&launch) {
    if (!e->timing) {
        launch();
        return;
    }
    const int s = timing_slot(e, kind);
    // inside a stream capture a plain record only orders the capture; the
    // External flag makes it an event-record node of the graph
    const unsigned fl = e->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    cudaEventRecordWithFlags(e->ev_a[s], e->stream, fl);
    launch();
    cudaEventRecordWithFlags(e->ev_b[s], e->stream, fl);
}

// Enqueues one step of the loop of compute() (src/compute_cuda.cu:1137-1238)
// minus its host I/O.
void enqueue_step(mtg_engine *e, long long step, bool allow_rebuild = true) {
    const mtg_params &p = e->p;
    if (allow_rebuild && step % p.ljpairsupdatefreq == 0 && (p.lj_on || p.is_assembly)) {
        timed_launch(e, 0, [&] { launch_lists(e); });
        e->lists_valid = true;
    }
    if (p.hdi_on) {
        timed_launch(e, 2, [&] { launch_forces(e->kp, e->bufs(), true, e->stream); });
        // learned TEA with the far field: proxies of this step's F and R.
        // Without per-kernel timing the inner proxies and M2L run on the
        // second stream beside the network and the near pairs, and join
        // before the first kernel that reads the far potentials.
        const bool ff = e->surr && e->ff_on;
        const bool fork = ff && !e->timing && e->side;
        bool joined = true;
        auto join = [&] {
            if (!joined) {
                cudaEventRecord(e->ev_join, e->side);
                cudaStreamWaitEvent(e->stream, e->ev_join, 0);
                joined = true;
            }
        };
        if (fork) {
            launch_ff_p2m_leaves(e->kp, e->bufs(), e->ffb, e->surr_gate, e->stream);
            cudaEventRecord(e->ev_fork, e->stream);
            cudaStreamWaitEvent(e->side, e->ev_fork, 0);
            launch_ff_m2l(e->kp, e->ffb, e->surr_gate, e->side);
            joined = false;
        } else if (ff) {
            timed_launch(e, 8, [&] { launch_ff_proxies(e->kp, e->bufs(), e->ffb, e->surr_gate, e->stream); });
        }
        if (e->surr) {
            // learned TEA: the network replaces the epsilon pass; the exact
            // re-check decides whether it stays in charge
            if (step % p.tea_epsilon_freq == 0) timed_launch(e, 6, [&] { enqueue_surrogate_eps(e); });
            if (e->surr_recheck > 0 && step % e->surr_recheck == 0) {
                join();
                timed_launch(e, 7, [&] { enqueue_surrogate_recheck(e); });
            }
        } else if (step % p.tea_epsilon_freq == 0) {
            timed_launch(e, 3, [&] { launch_tea_eps(e->kp, e->bufs(), e->tea_work, e->tea_nwork, e->stream); });
            timed_launch(e, 4, [&] { launch_tea_beta(e->kp, e->bufs(), p.tea_capricious, p.tea_epsmax, e->stream); });
        }
        if (ff) {
            // the far-field product while the surrogate is in charge, the exact
            // one after a fall-back (each gated on the fall-back flag)
            timed_launch(e, 9, [&] { launch_ff_near(e->kp, e->bufs(), e->ffb, e->surr_gate, e->stream); });
            join();
            timed_launch(e, 11, [&] {
                launch_ff_far(e->kp, e->bufs(), e->ffb, false, nullptr, e->surr_gate, e->stream);
            });
            timed_launch(e, 5, [&] {
                launch_tea_step_gated(e->kp, e->bufs(), e->tea_work, e->tea_nwork, e->surr_gate, e->stream);
            });
        } else {
            timed_launch(e, 5, [&] { launch_tea_step(e->kp, e->bufs(), e->tea_work, e->tea_nwork, e->stream); });
        }
    } else {
        timed_launch(e, 1, [&] { launch_step_plain(e->kp, e->bufs(), e->keep_forces, e->stream); });
    }
    e->cur ^= 1;
}

// The persistent plain path applies (see mtg_tuning::plain_persistent).
bool period_active(const mtg_engine *e) { return e->persistent && !e->p.hdi_on && period_fits(e->max_traj_beads); }

// Enqueues steps step .. step+run-1 of the plain loop as one persistent launch,
// after the pair-list rebuild due at `step`; run never crosses a rebuild.
void enqueue_period_run(mtg_engine *e, long long step, int run, bool allow_rebuild = true) {
    const mtg_params &p = e->p;
    bool in_kernel = false;
    if (allow_rebuild && step % p.ljpairsupdatefreq == 0 && (p.lj_on || p.is_assembly)) {
        // small trajectories rebuild inside the persistent launch (the same lists)
        in_kernel = period_rebuilds(e->max_traj_beads);
        if (!in_kernel) timed_launch(e, 0, [&] { launch_lists(e); });
        e->lists_valid = true;
    }
    timed_launch(e, 10, [&] {
        launch_step_period(e->kp, e->bufs(), e->keep_forces, run, e->max_traj_beads, in_kernel, e->stream);
    });
    if (run & 1) e->cur ^= 1;
}

// Creates event pairs up to slot `upto` (never called during a capture).
void reserve_slots(mtg_engine *e, int upto) {
    while ((int)e->ev_a.size() < upto) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        e->ev_a.push_back(a);
        e->ev_b.push_back(b);
        e->ev_kind.push_back(0);
    }
}

void collect_timing(mtg_engine *e) {
    for (int s : e->used_slots) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e->ev_a[s], e->ev_b[s]) == cudaSuccess) {
            e->kt_total[e->ev_kind[s]] += ms;
            e->kt_count[e->ev_kind[s]]++;
        } else {
            cudaGetLastError();  // a slot without a completed record is skipped
        }
    }
    e->used_slots.clear();
}

long long lcm_ll(long long a, long long b) {
    long long x = a, y = b;
    while (y) {
        const long long t = x % y;
        x = y;
        y = t;
    }
    return a / x * b;
}

}  // namespace

extern "C" {

const char *mtg_last_error_string(void) { return g_last_error.c_str(); }

int mtg_derive_params(mtg_params *p) {
    if (!p) return fail(MTG_E_CONFIG, "params is NULL");
    const float rmon = 2.0f;
    // src/preparator.cpp:209-219 (M_PI in double, stored to float)
    p->gammaR = (float)(6 * M_PI * p->viscosity * (p->hdi_on ? p->tea_a : rmon));
    p->gammaTheta = (float)(8 * M_PI * p->viscosity * pow(rmon, 3));
    p->varR = sqrtf(2.0f * 0.0019872041f * p->Temp * p->dt / p->gammaR);
    p->varTheta = sqrtf(2.0f * 0.0019872041f * p->Temp * p->dt / p->gammaTheta);
    return MTG_OK;
}

int mtg_create_batch(const mtg_params *p, const mtg_batch_topology *t, mtg_engine **out) {
    if (!out) return fail(MTG_E_CONFIG, "out is NULL");
    *out = nullptr;
    int rc = check_params(p);
    if (rc) return rc;
    if (!t || t->ntraj <= 0 || !t->offsets) return fail(MTG_E_CONFIG, "topology needs ntraj > 0 and offsets");
    const int nt = t->ntraj;
    if (t->offsets[0] != 0) return fail(MTG_E_CONFIG, "offsets[0] must be 0");
    for (int i = 0; i < nt; i++)
        if (t->offsets[i + 1] <= t->offsets[i]) return fail(MTG_E_CONFIG, "trajectory %d is empty or offsets decrease", i);
    const long long nbl = t->offsets[nt];
    const int maxH = t->maxHarmonicPerMonomer > 0 ? t->maxHarmonicPerMonomer : 1;
    const int maxLong = t->maxLongitudinalPerMonomer > 0 ? t->maxLongitudinalPerMonomer : 8;
    const int maxLat = t->maxLateralPerMonomer > 0 ? t->maxLateralPerMonomer : 16;
    const int maxLJ = t->maxLJPerMonomer > 0 ? t->maxLJPerMonomer : 256;
    if (nbl * (long long)maxLJ >= INT_MAX || nbl * (long long)maxLat >= INT_MAX || 2 * nbl * 4 >= INT_MAX)
        return fail(MTG_E_CONFIG, "batch too large for 32-bit list indexing");
    if (maxH > 7) return fail(MTG_E_CONFIG, "at most 7 harmonic partners per bead");
    if (!t->harmonicCount || !t->harmonic || !t->fixed || !t->mon_type)
        return fail(MTG_E_CONFIG, "harmonicCount, harmonic, fixed and mon_type are required");
    if (!p->is_assembly && (!t->longitudinalCount || !t->longitudinal || !t->lateralCount || !t->lateral))
        return fail(MTG_E_CONFIG, "static (non-assembly) mode needs the longitudinal and lateral lists");
    const int nb = (int)nbl;

    if (cudaSetDevice(p->device) != cudaSuccess) return fail(MTG_E_CUDA, "cudaSetDevice(%d) failed", p->device);
    auto *e = new mtg_engine();
    e->p = *p;
    e->device = p->device;
    e->nb = nb;
    e->nt = nt;
    e->h_off.assign(t->offsets, t->offsets + nt + 1);
    e->kp = make_kparams(*p, nb, nt, maxH, maxLong, maxLat, maxLJ);

    // host-side per-bead tables
    std::vector<int> traj(nb), flags(nb), harm((size_t)maxH * nb);
    for (int tr = 0; tr < nt; tr++)
        for (int g = t->offsets[tr]; g < t->offsets[tr + 1]; g++) traj[g] = tr;
    for (int g = 0; g < nb; g++) {
        const int hc = t->harmonicCount[g];
        if (hc < 0 || hc > maxH) {
            delete e;
            return fail(MTG_E_CONFIG, "bead %d: harmonicCount %d outside [0, %d]", g, hc, maxH);
        }
        const int n = t->offsets[traj[g] + 1] - t->offsets[traj[g]];
        for (int k = 0; k < maxH; k++) {
            const int v = t->harmonic[(size_t)maxH * g + k];
            const int a = v < 0 ? -v : v;
            if (k < hc && a >= n) {
                delete e;
                return fail(MTG_E_CONFIG, "bead %d: harmonic partner %d outside its trajectory", g, v);
            }
            harm[(size_t)maxH * g + k] = v;
        }
        int f = 0;
        if (t->extra && t->extra[g]) f |= kFlagExtra;
        if (t->fixed[g]) f |= kFlagFixed;
        if (t->mon_type[g] != 0) f |= kFlagBeta;
        if (!t->gtp || t->gtp[g] == 1) f |= kFlagGtp;
        if (t->on_tubule_cur && t->on_tubule_cur[g] != 0) f |= kFlagOnTubule;
        f |= hc << kHarmShift;
        flags[g] = f;
    }
    // work items: chunks of kTile beads, never straddling a trajectory
    std::vector<int2> work;
    std::vector<int> work_first(nt + 1);
    for (int tr = 0; tr < nt; tr++) {
        work_first[tr] = (int)work.size();
        for (int g = t->offsets[tr]; g < t->offsets[tr + 1]; g += kTile) work.push_back(make_int2(tr, g));
    }
    work_first[nt] = (int)work.size();
    e->nwork = (int)work.size();
    std::vector<int2> tea_work;
    for (int tr = 0; tr < nt; tr++)
        for (int g = t->offsets[tr]; g < t->offsets[tr + 1]; g += kTeaChunk) tea_work.push_back(make_int2(tr, g));
    e->tea_nwork = (int)tea_work.size();
    // threads per bead in the all-pairs TEA kernels: enough to fill the GPU
    {
        int dev = p->device, sms = 148;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        // two beads per thread; aim for about two full waves at 64 registers
        const double target = (double)sms * 2048.0;
        int sl = 1;
        while (sl < 8 && (double)nb / 4 * sl < target) sl <<= 1;   // four beads per thread
        e->kp.tea_slices = sl;
        e->kp.tea_jparts = 1;
    }

#define ALLOC(ptr, n)                         \
    do {                                      \
        if ((rc = dalloc(&(ptr), (n))) != 0) { \
            mtg_destroy(e);                   \
            return rc;                        \
        }                                     \
    } while (0)
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete e;
        return fail(MTG_E_CUDA, "cudaStreamCreate failed");
    }
    ALLOC(e->off, nt + 1);
    ALLOC(e->traj, nb);
    ALLOC(e->flags, nb);
    ALLOC(e->harm, (size_t)maxH * nb);
    ALLOC(e->zs, nt);
    ALLOC(e->frame[0], 4 * (size_t)nb);
    ALLOC(e->frame[1], 4 * (size_t)nb);
    ALLOC(e->force, 2 * (size_t)nb);
    ALLOC(e->seeds, 2 * (size_t)nb);
    ALLOC(e->ljc, nb);
    ALLOC(e->lj, (size_t)maxLJ * nb);
    ALLOC(e->lonc, nb);
    ALLOC(e->lon, (size_t)maxLong * nb);
    ALLOC(e->latc, nb);
    ALLOC(e->lat, (size_t)maxLat * nb);
    ALLOC(e->err, 1);
    ALLOC(e->work, e->nwork);
    ALLOC(e->work_first, nt + 1);
    ALLOC(e->en_partials, 7 * (size_t)e->nwork);
    ALLOC(e->en_traj, 7 * (size_t)nt);
    ALLOC(e->stage, 7 * (size_t)nb);
    ALLOC(e->stage_u8, nb);
    ALLOC(e->stage_i, nb);
    if (p->hdi_on) {
        ALLOC(e->tea_work, e->tea_nwork);
        ALLOC(e->tea_r, nb);
        ALLOC(e->tea_ci, nb);
        ALLOC(e->tea_eps, nb);
        ALLOC(e->tea_beta, nt);
        ALLOC(e->tea_eps_t, nt);
        ALLOC(e->tea_part, (size_t)kTeaMaxParts * nb);
    }
    // spatial-hash tables of the cell-list rebuild
    std::vector<int> tbase(nt + 1, 0), tmask(nt, 0);
    for (int tr = 0; tr < nt; tr++) {
        const int n = t->offsets[tr + 1] - t->offsets[tr];
        e->max_traj_beads = n > e->max_traj_beads ? n : e->max_traj_beads;
        int size = 32;
        while (size < n) size <<= 1;
        tbase[tr + 1] = tbase[tr] + size;
        tmask[tr] = size - 1;
        e->cell_max_buckets = size > e->cell_max_buckets ? size : e->cell_max_buckets;
    }
    e->cell_nbuckets = tbase[nt];
    ALLOC(e->cell_tbase, nt + 1);
    ALLOC(e->cell_tmask, nt);
    ALLOC(e->cell_key, nb);
    ALLOC(e->cell_bead, nb);
    ALLOC(e->cell_pos, nb);
    ALLOC(e->cell_cnt, e->cell_nbuckets);
    ALLOC(e->cell_start, e->cell_nbuckets);
    ALLOC(e->cell_cursor, e->cell_nbuckets);
#undef ALLOC
    cudaStream_t s = e->stream;
    if ((rc = upload(e->cell_tbase, tbase.data(), sizeof(int) * (nt + 1), s)) ||
        (rc = upload(e->cell_tmask, tmask.data(), sizeof(int) * nt, s))) {
        mtg_destroy(e);
        return rc;
    }
    choose_list_method(e);
    std::vector<float> zs(nt, 0.f);
    if (t->zs) zs.assign(t->zs, t->zs + nt);
    if ((rc = upload(e->off, t->offsets, sizeof(int) * (nt + 1), s)) || (rc = upload(e->traj, traj.data(), sizeof(int) * nb, s)) ||
        (rc = upload(e->flags, flags.data(), sizeof(int) * nb, s)) ||
        (rc = upload(e->harm, harm.data(), sizeof(int) * harm.size(), s)) ||
        (rc = upload(e->zs, zs.data(), sizeof(float) * nt, s)) ||
        (rc = upload(e->work, work.data(), sizeof(int2) * work.size(), s)) ||
        (rc = upload(e->work_first, work_first.data(), sizeof(int) * (nt + 1), s))) {
        mtg_destroy(e);
        return rc;
    }
    cudaMemsetAsync(e->err, 0, sizeof(int), s);
    cudaMemsetAsync(e->ljc, 0, sizeof(int) * nb, s);
    cudaMemsetAsync(e->lonc, 0, sizeof(int) * nb, s);
    cudaMemsetAsync(e->latc, 0, sizeof(int) * nb, s);
    cudaMemsetAsync(e->force, 0, sizeof(float4) * 2 * nb, s);
    if (p->hdi_on) {
        if ((rc = upload(e->tea_work, tea_work.data(), sizeof(int2) * tea_work.size(), s)) != 0) {
            mtg_destroy(e);
            return rc;
        }
        cudaMemsetAsync(e->tea_ci, 0, sizeof(float4) * nb, s);
        cudaMemsetAsync(e->tea_beta, 0, sizeof(float) * nt, s);
    }
    // static (non-assembly) lists, transposed to k-major
    if (!p->is_assembly) {
        std::vector<int> cnt(nb), lon((size_t)maxLong * nb, 0), lat((size_t)maxLat * nb, 0), cnt2(nb);
        for (int g = 0; g < nb; g++) {
            cnt[g] = t->longitudinalCount[g];
            cnt2[g] = t->lateralCount[g];
            if (cnt[g] < 0 || cnt[g] > maxLong || cnt2[g] < 0 || cnt2[g] > maxLat) {
                mtg_destroy(e);
                return fail(MTG_E_OVERFLOW, "bead %d: static list count exceeds its capacity", g);
            }
            const int n = t->offsets[traj[g] + 1] - t->offsets[traj[g]];
            for (int k = 0; k < cnt[g]; k++) {
                const int v = t->longitudinal[(size_t)maxLong * g + k], a = v < 0 ? -v : v;
                if (a >= n) {
                    mtg_destroy(e);
                    return fail(MTG_E_CONFIG, "bead %d: longitudinal partner %d outside its trajectory", g, v);
                }
                lon[(size_t)k * nb + g] = v;
            }
            for (int k = 0; k < cnt2[g]; k++) {
                const int v = t->lateral[(size_t)maxLat * g + k];
                int a = v < 0 ? -v : v;
                if (a == kZeroCode) a = 0;
                if (a >= n) {
                    mtg_destroy(e);
                    return fail(MTG_E_CONFIG, "bead %d: lateral partner %d outside its trajectory", g, v);
                }
                lat[(size_t)k * nb + g] = v;
            }
        }
        if ((rc = upload(e->lonc, cnt.data(), sizeof(int) * nb, s)) ||
            (rc = upload(e->lon, lon.data(), sizeof(int) * lon.size(), s)) ||
            (rc = upload(e->latc, cnt2.data(), sizeof(int) * nb, s)) ||
            (rc = upload(e->lat, lat.data(), sizeof(int) * lat.size(), s))) {
            mtg_destroy(e);
            return rc;
        }
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            mtg_destroy(e);
            return fail(MTG_E_CUDA, "static list upload failed");
        }
    }
    if ((rc = mtg_seed_rng(e, p->rseed)) != 0) {
        mtg_destroy(e);
        return rc;
    }
    *out = e;
    return MTG_OK;
}

int mtg_create(const mtg_params *p, const mtg_topology *t, mtg_engine **out) {
    if (!out) return fail(MTG_E_CONFIG, "out is NULL");
    *out = nullptr;
    if (!t || t->Ntot <= 0 || t->Ntr <= 0) return fail(MTG_E_CONFIG, "topology needs Ntot > 0 and Ntr > 0");
    if (!t->harmonicCount || !t->harmonic || !t->fixed || !t->mon_type)
        return fail(MTG_E_CONFIG, "harmonicCount, harmonic, fixed and mon_type are required");
    const int N = t->Ntot, R = t->Ntr;
    const int maxH = t->maxHarmonicPerMonomer > 0 ? t->maxHarmonicPerMonomer : 1;
    const size_t nb = (size_t)N * R;
    // replicate the per-template arrays over the trajectories
    std::vector<int> off(R + 1), hc(nb), hh((size_t)maxH * nb), mt(nb);
    std::vector<uint8_t> fx(nb);
    for (int r = 0; r <= R; r++) off[r] = r * N;
    for (int r = 0; r < R; r++)
        for (int i = 0; i < N; i++) {
            const size_t g = (size_t)r * N + i;
            hc[g] = t->harmonicCount[i];
            for (int k = 0; k < maxH; k++) hh[(size_t)maxH * g + k] = t->harmonic[(size_t)maxH * i + k];
            mt[g] = t->mon_type[i];
            fx[g] = t->fixed[i];
        }
    mtg_batch_topology b{};
    b.ntraj = R;
    b.offsets = off.data();
    b.maxHarmonicPerMonomer = maxH;
    b.harmonicCount = hc.data();
    b.harmonic = hh.data();
    b.maxLongitudinalPerMonomer = t->maxLongitudinalPerMonomer;
    b.maxLateralPerMonomer = t->maxLateralPerMonomer;
    b.maxLJPerMonomer = t->maxLJPerMonomer;
    b.longitudinalCount = t->longitudinalCount;
    b.longitudinal = t->longitudinal;
    b.lateralCount = t->lateralCount;
    b.lateral = t->lateral;
    b.fixed = fx.data();
    b.extra = t->extra;
    b.mon_type = mt.data();
    b.gtp = t->gtp;
    b.on_tubule_cur = t->on_tubule_cur;
    b.zs = t->zs;
    return mtg_create_batch(p, &b, out);
}

int mtg_destroy(mtg_engine *e) {
    if (!e) return MTG_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    mtg_internal_close_output(e);
    destroy_graphs(e);
    mtg_internal_ff_free(e);
    void *ptrs[] = {e->off, e->traj, e->flags, e->harm, e->zs, e->frame[0], e->frame[1], e->force, e->seeds,
                    e->ljc, e->lj, e->lonc, e->lon, e->latc, e->lat, e->err, e->work, e->work_first,
                    e->en_partials, e->en_traj, e->en_bead, e->tea_r, e->tea_ci, e->tea_eps, e->tea_beta,
                    e->tea_eps_t, e->stage, e->stage_u8, e->stage_i, e->cell_tbase, e->cell_tmask,
                    e->cell_key, e->cell_bead, e->cell_pos, e->cell_cnt, e->cell_start, e->cell_cursor, e->tea_work,
                    e->surr_desc, e->surr_pred, e->surr_stats, e->surr_gate, e->surr_err, e->surr_part,
                    e->tea_ci2, e->feff_a, e->feff_b, e->tea_eps2, e->tea_beta2, e->tea_eps_t2,
                    e->hydro_cand, e->hydro_rank, e->hydro_sums, e->hydro_counts, e->hydro_events,
                    e->tea_part};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (e->stage_host) cudaFreeHost(e->stage_host);
    for (auto ev : e->ev_a) cudaEventDestroy(ev);
    for (auto ev : e->ev_b) cudaEventDestroy(ev);
    if (e->call_a) cudaEventDestroy(e->call_a);
    if (e->call_b) cudaEventDestroy(e->call_b);
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->side) cudaStreamDestroy(e->side);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    delete e;
    return MTG_OK;
}

int mtg_num_beads(const mtg_engine *e, int *nbeads, int *ntraj) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (nbeads) *nbeads = e->nb;
    if (ntraj) *ntraj = e->nt;
    return MTG_OK;
}

int mtg_list_capacity(const mtg_engine *e, int *max_long, int *max_lat, int *max_lj) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (max_long) *max_long = e->kp.maxLong;
    if (max_lat) *max_lat = e->kp.maxLat;
    if (max_lj) *max_lj = e->kp.maxLJ;
    return MTG_OK;
}

int mtg_seed_rng(mtg_engine *e, int rseed) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    std::vector<uint32_t> s;
    make_seeds(rseed, 2 * (size_t)e->nb, s);
    return mtg_upload_rng(e, s.data());
}

int mtg_generate_seeds(int rseed, long long nstreams, uint32_t *seeds) {
    if (!seeds || nstreams < 0) return fail(MTG_E_CONFIG, "seeds is NULL or nstreams negative");
    std::vector<uint32_t> s;
    make_seeds(rseed, (size_t)nstreams, s);
    std::memcpy(seeds, s.data(), sizeof(uint32_t) * s.size());
    return MTG_OK;
}

int mtg_upload_rng(mtg_engine *e, const uint32_t *seeds) {
    if (!e || !seeds) return fail(MTG_E_CONFIG, "engine or seeds is NULL");
    cudaSetDevice(e->device);
    CK(cudaMemcpyAsync(e->seeds, seeds, sizeof(uint4) * 2 * (size_t)e->nb, cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

int mtg_download_rng(mtg_engine *e, uint32_t *seeds) {
    if (!e || !seeds) return fail(MTG_E_CONFIG, "engine or seeds is NULL");
    cudaSetDevice(e->device);
    CK(cudaMemcpyAsync(seeds, e->seeds, sizeof(uint4) * 2 * (size_t)e->nb, cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

int mtg_upload_state(mtg_engine *e, const float *r) {
    if (!e || !r) return fail(MTG_E_CONFIG, "engine or r is NULL");
    cudaSetDevice(e->device);
    CK(cudaMemcpyAsync(e->stage, r, sizeof(float) * 7 * (size_t)e->nb, cudaMemcpyHostToDevice, e->stream));
    launch_frames_from_coords(e->kp, e->stage, e->frame[e->cur], e->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e->stream));
    e->have_state = true;
    return MTG_OK;
}

int mtg_download_state(mtg_engine *e, float *r, float *f) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    const size_t bytes = sizeof(float) * 7 * (size_t)e->nb;
    if (r) {
        launch_coords_from_frames(e->kp, e->frame[e->cur], e->stage, e->stream);
        CK(cudaMemcpyAsync(r, e->stage, bytes, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    if (f) {
        launch_forces_to_coords(e->kp, e->force, e->stage, e->stream);
        CK(cudaMemcpyAsync(f, e->stage, bytes, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
    }
    CK(cudaGetLastError());
    return MTG_OK;
}

static int set_flag_array(mtg_engine *e, const uint8_t *extra, const int *gtp, const int *ontub) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    const size_t nb = e->nb;
    if (extra) CK(cudaMemcpyAsync(e->stage_u8, extra, nb, cudaMemcpyHostToDevice, e->stream));
    if (gtp || ontub) CK(cudaMemcpyAsync(e->stage_i, gtp ? gtp : ontub, sizeof(int) * nb, cudaMemcpyHostToDevice, e->stream));
    launch_set_flags(e->nb, extra ? e->stage_u8 : nullptr, gtp ? e->stage_i : nullptr, ontub ? e->stage_i : nullptr,
                     e->flags, e->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

int mtg_set_gtp(mtg_engine *e, const int *gtp) {
    if (!gtp) return fail(MTG_E_CONFIG, "gtp is NULL");
    return set_flag_array(e, nullptr, gtp, nullptr);
}
int mtg_set_extra(mtg_engine *e, const uint8_t *extra) {
    if (!extra) return fail(MTG_E_CONFIG, "extra is NULL");
    return set_flag_array(e, extra, nullptr, nullptr);
}
int mtg_set_on_tubule(mtg_engine *e, const int *on_tubule_cur) {
    if (!on_tubule_cur) return fail(MTG_E_CONFIG, "on_tubule_cur is NULL");
    return set_flag_array(e, nullptr, nullptr, on_tubule_cur);
}

int mtg_set_keep_forces(mtg_engine *e, int keep) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (e->keep_forces != (keep != 0)) destroy_graphs(e);
    e->keep_forces = keep != 0;
    return MTG_OK;
}

int mtg_rebuild_pairs(mtg_engine *e) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (!e->have_state) return fail(MTG_E_STATE, "no state uploaded");
    if (e->p.lj_on || e->p.is_assembly) launch_lists(e);
    CK(cudaGetLastError());
    e->lists_valid = true;
    e->lists_fresh = true;
    return check_errors(e);
}

int mtg_download_lists(mtg_engine *e, int *lj_count, int *lj, int *long_count, int *lon, int *lat_count, int *lat) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    const size_t nb = e->nb;
    struct L {
        int *cnt_dev, *arr_dev, cap;
        int *cnt_host, *arr_host;
    } ls[3] = {{e->ljc, e->lj, e->kp.maxLJ, lj_count, lj},
               {e->lonc, e->lon, e->kp.maxLong, long_count, lon},
               {e->latc, e->lat, e->kp.maxLat, lat_count, lat}};
    for (auto &l : ls) {
        if (!l.cnt_host && !l.arr_host) continue;
        std::vector<int> cnt(nb), arr((size_t)l.cap * nb);
        CK(cudaMemcpyAsync(cnt.data(), l.cnt_dev, sizeof(int) * nb, cudaMemcpyDeviceToHost, e->stream));
        CK(cudaMemcpyAsync(arr.data(), l.arr_dev, sizeof(int) * arr.size(), cudaMemcpyDeviceToHost, e->stream));
        CK(cudaStreamSynchronize(e->stream));
        if (l.cnt_host) std::memcpy(l.cnt_host, cnt.data(), sizeof(int) * nb);
        if (l.arr_host) {
            // k-major on the device -> bead-major (reference layout) on the host
            for (size_t g = 0; g < nb; g++)
                for (int k = 0; k < l.cap; k++) l.arr_host[(size_t)l.cap * g + k] = k < cnt[g] ? arr[(size_t)k * nb + g] : 0;
        }
    }
    return MTG_OK;
}

int mtg_compute_forces(mtg_engine *e, float *f) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (!e->have_state) return fail(MTG_E_STATE, "no state uploaded");
    launch_forces(e->kp, e->bufs(), false, e->stream);
    CK(cudaGetLastError());
    int rc = check_errors(e);
    if (rc) return rc;
    return f ? mtg_download_state(e, nullptr, f) : MTG_OK;
}

static int enqueue_range(mtg_engine *e, long long first_step, int nsteps) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (!e->have_state) return fail(MTG_E_STATE, "no state uploaded");
    if (nsteps < 0 || first_step < 0) return fail(MTG_E_CONFIG, "negative step range");
    const mtg_params &p = e->p;
    long long period = p.ljpairsupdatefreq;
    if (p.hdi_on) period = lcm_ll(period, p.tea_epsilon_freq);
    if (p.hdi_on && e->surr && e->surr_recheck > 0) period = lcm_ll(period, e->surr_recheck);
    const bool use_graphs = period <= 256;
    if (e->graph_period != period) {
        destroy_graphs(e);
        e->graph_period = (int)period;
    }
    const int max_launch_per_step = 8;
    int rc = mtg_internal_ff_refresh(e);   // a due far-field partition is rebuilt before any capture
    if (rc) return rc;
    e->direct_next = e->direct_base;
    e->used_slots.clear();
    long long s = first_step;
    const long long end = first_step + nsteps;
    if (e->lists_fresh && s < end && s % p.ljpairsupdatefreq == 0) {
        // the caller rebuilt the lists for this step already (reference order:
        // rebuild, host hooks, forces; src/compute_cuda.cu:1140-1228)
        if (period_active(e))
            enqueue_period_run(e, s, 1, false);
        else
            enqueue_step(e, s, false);
        s++;
    }
    if (nsteps > 0) e->lists_fresh = false;
    while (s < end) {
        if (use_graphs && s % period == 0 && end - s >= period) {
            cudaGraphExec_t &ge = e->graph[e->cur];
            if (!ge) {
                const int cur0 = e->cur;
                if (e->timing) {
                    // graph slots live below direct_base; direct launches above it
                    const int base = e->direct_base;
                    const int count = (int)period * max_launch_per_step;
                    reserve_slots(e, base + count);
                    e->graph_slot_base[cur0] = base;
                    e->graph_slot_count[cur0] = 0;
                    e->direct_base = base + count;
                    e->direct_next = e->direct_base;
                    e->capture_next = base;
                }
                cudaGraph_t g;
                e->capturing = true;
                cudaError_t ce = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
                if (ce == cudaSuccess) {
                    if (period_active(e)) {
                        const long long freq = p.ljpairsupdatefreq;
                        for (long long k = 0; k < period;) {
                            long long run = freq - k % freq;
                            if (k + run > period) run = period - k;
                            enqueue_period_run(e, k, (int)run);
                            k += run;
                        }
                    } else {
                        for (long long k = 0; k < period; k++) enqueue_step(e, k);
                    }
                    ce = cudaStreamEndCapture(e->stream, &g);
                }
                e->capturing = false;
                if (ce != cudaSuccess) return fail(MTG_E_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
                if (e->timing) e->graph_slot_count[cur0] = e->capture_next - e->graph_slot_base[cur0];
                e->cur = cur0;
                e->graph_kernels[cur0] = count_kernel_nodes(g);
                CK(cudaGraphInstantiate(&ge, g, 0));
                cudaGraphDestroy(g);
            }
            if (e->timing)
                for (int k = 0; k < e->graph_slot_count[e->cur]; k++) {
                    const int slot = e->graph_slot_base[e->cur] + k;
                    bool seen = false;
                    for (int u : e->used_slots) seen |= (u == slot);
                    if (!seen) e->used_slots.push_back(slot);
                }
            CK(cudaGraphLaunch(ge, e->stream));
            e->graph_kernel_launches += e->graph_kernels[e->cur];
            if (period & 1) e->cur ^= 1;
            if (p.lj_on || p.is_assembly) e->lists_valid = true;
            s += period;
        } else if (period_active(e)) {
            // outside a graph the persistent path runs up to the next rebuild
            const long long freq = p.ljpairsupdatefreq;
            long long run = freq - s % freq;
            if (s + run > end) run = end - s;
            enqueue_period_run(e, s, (int)run);
            s += run;
        } else {
            enqueue_step(e, s);
            s++;
        }
    }
    CK(cudaGetLastError());
    e->ff_steps += nsteps;
    return MTG_OK;
}

int mtg_step(mtg_engine *e, long long first_step, int nsteps) {
    if (e) cudaSetDevice(e->device);
    int rc = enqueue_range(e, first_step, nsteps);
    if (rc) return rc;
    rc = check_errors(e);
    if (e->timing) collect_timing(e);
    return rc;
}

int mtg_step_timed(mtg_engine *e, long long first_step, int nsteps, float *device_ms) {
    if (!e || !device_ms) return fail(MTG_E_CONFIG, "engine or device_ms is NULL");
    cudaSetDevice(e->device);
    if (!e->call_a) {
        CK(cudaEventCreate(&e->call_a));
        CK(cudaEventCreate(&e->call_b));
    }
    CK(cudaEventRecord(e->call_a, e->stream));
    int rc = enqueue_range(e, first_step, nsteps);
    if (rc) return rc;
    CK(cudaEventRecord(e->call_b, e->stream));
    rc = check_errors(e);
    if (e->timing) collect_timing(e);
    CK(cudaEventElapsedTime(device_ms, e->call_a, e->call_b));
    return rc;
}

int mtg_set_list_method(mtg_engine *e, int method) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    if (method < 0 || method > 2) return fail(MTG_E_CONFIG, "list method must be 0 (auto), 1 (tiles) or 2 (cells)");
    e->list_method = method;
    choose_list_method(e);
    if (method == 2 && !e->use_cells)
        return fail(MTG_E_CONFIG, "the cell-list rebuild supports list capacities up to %d/%d", kCellMaxLong,
                    kCellMaxLat);
    destroy_graphs(e);
    return MTG_OK;
}

int mtg_get_list_method(mtg_engine *e, int *method) {
    if (!e || !method) return fail(MTG_E_CONFIG, "engine or method is NULL");
    *method = e->use_cells ? 2 : 1;
    return MTG_OK;
}

int mtg_get_tuning(mtg_engine *e, mtg_tuning *t) {
    if (!e || !t) return fail(MTG_E_CONFIG, "engine or tuning is NULL");
    t->list_method = e->use_cells ? 2 : 1;
    t->step_block = e->kp.step_block;
    t->tea_slices = e->kp.tea_slices;
    t->tea_jparts = e->kp.tea_jparts;
    t->plain_persistent = e->persistent ? 1 : 0;
    return MTG_OK;
}

int mtg_set_tuning(mtg_engine *e, const mtg_tuning *t) {
    if (!e || !t) return fail(MTG_E_CONFIG, "engine or tuning is NULL");
    if (t->step_block != 64 && t->step_block != 128 && t->step_block != 256)
        return fail(MTG_E_CONFIG, "step_block must be 64, 128 or 256");
    if (t->tea_slices != 1 && t->tea_slices != 2 && t->tea_slices != 4 && t->tea_slices != 8)
        return fail(MTG_E_CONFIG, "tea_slices must be 1, 2, 4 or 8");
    if (t->tea_jparts < 1 || t->tea_jparts > kTeaMaxParts) return fail(MTG_E_CONFIG, "tea_jparts must be 1..4");
    if (t->plain_persistent != 0 && t->plain_persistent != 1) return fail(MTG_E_CONFIG, "plain_persistent must be 0 or 1");
    if (t->plain_persistent && !period_fits(e->max_traj_beads))
        return fail(MTG_E_CONFIG, "plain_persistent needs trajectories of at most %d beads",
                    kPeriodThreads * kPeriodBeads);
    int rc = mtg_set_list_method(e, t->list_method);
    if (rc) return rc;
    if (t->plain_persistent) {
        cudaSetDevice(e->device);
        if (period_prepare(e->max_traj_beads) != 0)
            return fail(MTG_E_CUDA, "the persistent step kernel could not reserve its shared memory");
    }
    e->persistent = t->plain_persistent != 0;
    e->kp.step_block = t->step_block;
    e->kp.tea_slices = t->tea_slices;
    e->kp.tea_jparts = t->tea_jparts;
    destroy_graphs(e);
    return MTG_OK;
}

int mtg_autotune(mtg_engine *e, long long first_step, int trial_steps, mtg_tuning *best, float *best_ms) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    if (!e->have_state) return fail(MTG_E_STATE, "no state uploaded");
    if (trial_steps <= 0) return fail(MTG_E_CONFIG, "trial_steps must be positive");
    cudaSetDevice(e->device);
    // snapshot of everything a trial advances: the state and the noise streams
    const size_t fbytes = sizeof(float4) * 4 * (size_t)e->nb, sbytes = sizeof(uint4) * 2 * (size_t)e->nb;
    void *snap = nullptr;
    CK(cudaMalloc(&snap, fbytes + sbytes));
    CK(cudaMemcpyAsync(snap, e->frame[e->cur], fbytes, cudaMemcpyDeviceToDevice, e->stream));
    CK(cudaMemcpyAsync((char *)snap + fbytes, e->seeds, sbytes, cudaMemcpyDeviceToDevice, e->stream));
    const int cur0 = e->cur;
    mtg_tuning orig;
    mtg_get_tuning(e, &orig);
    std::vector<mtg_tuning> cands;
    const bool cells_ok = e->kp.maxLong <= kCellMaxLong && e->kp.maxLat <= kCellMaxLat;
    const bool lists = e->p.lj_on || e->p.is_assembly;
    for (int lm : {1, 2}) {
        if (lm == 2 && (!cells_ok || !lists)) continue;
        if (lm == 1 && !lists && !cands.empty()) continue;
        if (e->p.hdi_on) {
            for (int sl : {1, 2, 4, 8})
                for (int jp = 1; jp <= kTeaMaxParts; jp++) cands.push_back({lm, orig.step_block, sl, jp, 0});
        } else {
            for (int bs : {64, 128, 256}) cands.push_back({lm, bs, orig.tea_slices, orig.tea_jparts, 0});
            if (period_fits(e->max_traj_beads)) cands.push_back({lm, orig.step_block, orig.tea_slices, orig.tea_jparts, 1});
        }
    }
    float best_t = 3.4e38f;
    mtg_tuning bt = orig;
    int rc = MTG_OK;
    for (const auto &c : cands) {
        if ((rc = mtg_set_tuning(e, &c)) != 0) break;
        float ms = 0.f;
        for (int rep = 0; rep < 2 && rc == MTG_OK; rep++) {  // first run captures the graph
            e->cur = cur0;
            cudaMemcpyAsync(e->frame[e->cur], snap, fbytes, cudaMemcpyDeviceToDevice, e->stream);
            cudaMemcpyAsync(e->seeds, (char *)snap + fbytes, sbytes, cudaMemcpyDeviceToDevice, e->stream);
            rc = mtg_step_timed(e, first_step, trial_steps, &ms);
        }
        if (rc) break;
        if (ms < best_t) {
            best_t = ms;
            bt = c;
        }
    }
    e->cur = cur0;
    cudaMemcpyAsync(e->frame[e->cur], snap, fbytes, cudaMemcpyDeviceToDevice, e->stream);
    cudaMemcpyAsync(e->seeds, (char *)snap + fbytes, sbytes, cudaMemcpyDeviceToDevice, e->stream);
    cudaStreamSynchronize(e->stream);
    cudaFree(snap);
    if (rc) {
        mtg_set_tuning(e, &orig);
        return rc;
    }
    rc = mtg_set_tuning(e, &bt);
    if (best) *best = bt;
    if (best_ms) *best_ms = best_t;
    return rc;
}

int mtg_set_kernel_timing(mtg_engine *e, int on) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (e->timing != (on != 0)) destroy_graphs(e);
    e->timing = on != 0;
    return MTG_OK;
}

int mtg_kernel_times(mtg_engine *e, double *total_ms, long long *launches, int reset) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    for (int k = 0; k < MTG_KERNEL_KINDS; k++) {
        if (total_ms) total_ms[k] = e->kt_total[k];
        if (launches) launches[k] = e->kt_count[k];
        if (reset) {
            e->kt_total[k] = 0;
            e->kt_count[k] = 0;
        }
    }
    return MTG_OK;
}

int mtg_graph_kernel_launches(mtg_engine *e, long long *launches, int reset) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    if (launches) *launches = e->graph_kernel_launches;
    if (reset) e->graph_kernel_launches = 0;
    return MTG_OK;
}

int mtg_host_alloc(void **ptr, size_t bytes) {
    if (!ptr) return fail(MTG_E_CONFIG, "ptr is NULL");
    CK(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocPortable));
    return MTG_OK;
}

int mtg_host_free(void *ptr) {
    if (ptr) CK(cudaFreeHost(ptr));
    return MTG_OK;
}

int mtg_sync(mtg_engine *e) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    return check_errors(e);
}

int mtg_energies(mtg_engine *e, double *per_bead, double *per_traj) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (!e->have_state) return fail(MTG_E_STATE, "no state uploaded");
    int rc;
    if (per_bead && !e->en_bead && (rc = dalloc(&e->en_bead, 7 * (size_t)e->nb)) != 0) return rc;
    launch_energy(e->kp, e->bufs(), per_bead ? e->en_bead : nullptr, e->en_partials, e->work, e->nwork, e->stream);
    launch_energy_totals(e->kp, e->en_partials, e->work_first, e->en_traj, e->err, e->stream);
    CK(cudaGetLastError());
    if (per_traj)
        CK(cudaMemcpyAsync(per_traj, e->en_traj, sizeof(double) * 7 * e->nt, cudaMemcpyDeviceToHost, e->stream));
    if (per_bead)
        CK(cudaMemcpyAsync(per_bead, e->en_bead, sizeof(double) * 7 * (size_t)e->nb, cudaMemcpyDeviceToHost, e->stream));
    return check_errors(e);
}

int mtg_tea_update(mtg_engine *e, double *eps_out, float *beta_out, float *ci_out) {
    if (!e) return fail(MTG_E_CONFIG, "engine is NULL");
    cudaSetDevice(e->device);
    if (!e->p.hdi_on) return fail(MTG_E_STATE, "engine created without hdi_on");
    if (!e->have_state) return fail(MTG_E_STATE, "no state uploaded");
    launch_tea_eps(e->kp, e->bufs(), e->tea_work, e->tea_nwork, e->stream);
    launch_tea_beta(e->kp, e->bufs(), e->p.tea_capricious, e->p.tea_epsmax, e->stream);
    CK(cudaGetLastError());
    if (eps_out) CK(cudaMemcpyAsync(eps_out, e->tea_eps_t, sizeof(double) * e->nt, cudaMemcpyDeviceToHost, e->stream));
    if (beta_out) CK(cudaMemcpyAsync(beta_out, e->tea_beta, sizeof(float) * e->nt, cudaMemcpyDeviceToHost, e->stream));
    if (ci_out) CK(cudaMemcpyAsync(ci_out, e->tea_ci, sizeof(float4) * e->nb, cudaMemcpyDeviceToHost, e->stream));
    return check_errors(e);
}

}  // extern "C"
