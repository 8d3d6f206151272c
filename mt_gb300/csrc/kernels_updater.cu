// kernels_updater.cu - the stride-step analytics of the reference's updater
// as kernels on the device-resident state: microtubule length (mt_length),
// GTP hydrolysis (hydrolyse) and the extra-bead counts of change_conc, so
// that a stride step no longer downloads the coordinates for them.
//
//   mtg_mt_length           src/updater.cpp:154-227  on_tubule flags + counts
//   mtg_hydrolysis_candidates / mtg_hydrolyse
//                           src/updater.cpp:229-257  (the reference draws
//                           rand() for every candidate dimer in loop order;
//                           the caller draws the same numbers and passes them)
//   mtg_count_extra / mtg_set_beads
//                           src/updater.cpp:97-152   counts and placements of
//                           change_conc (its rand() stays with the caller)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "mtg_engine.cuh"

using namespace mtg;

namespace {

constexpr int kFlagOnTubPrev = 1 << 5;   // on_tubule_prev of the reference
// mt_length constants (src/mt.h:23-30): R_MT + R_THRES = 8.12 + 8 r_mon nm
constexpr float kMtRad = 8.12f + 2.0f * 8.0f;

__device__ __forceinline__ int dimer_slots(const int *off, int t) { return (off[t + 1] - off[t]) / 2; }

// rad = |(x, y)| < R_MT + R_THRES, rad > 1, cos(theta) > cos(ANG_THRES): the
// bead is on the tubule (src/updater.cpp:166-168); counts per trajectory.
__global__ void k_mt_length(int nb, const int *traj, const float4 *frame, int *flags, int save_prev, float cos_thres,
                            int *counts) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const float4 p = frame[g];
    const float theta = frame[2 * nb + g].w;
    const float rad = __fsqrt_rn(__fadd_rn(__fmul_rn(p.x, p.x), __fmul_rn(p.y, p.y)));
    const bool on = rad < kMtRad && rad > 1.0f && cosf(theta) > cos_thres;
    int f = flags[g];
    if (save_prev) f = (f & kFlagOnTubule) ? (f | kFlagOnTubPrev) : (f & ~kFlagOnTubPrev);
    f = on ? (f | kFlagOnTubule) : (f & ~kFlagOnTubule);
    flags[g] = f;
    if (on) atomicAdd(&counts[traj[g]], 1);   // integer sums: order-independent
}

// Candidate dimers of the hydrolysis loop (src/updater.cpp:232-235): dimer k
// (beads 2k, 2k+1 of the trajectory) with gtp, not extra, on the tubule now
// and at the previous stride.  Slot k * nt + t: the reference's loop order
// (dimer index outer, trajectory inner).
__global__ void k_hydro_mark(int nt, int max_dimers, const int *off, const int *flags, int *cand) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= max_dimers * nt) return;
    const int k = s / nt, t = s % nt;
    int c = 0;
    if (k < dimer_slots(off, t)) {
        const int f = flags[off[t] + 2 * k];
        c = (f & kFlagGtp) && !(f & kFlagExtra) && (f & kFlagOnTubule) && (f & kFlagOnTubPrev);
    }
    cand[s] = c;
}

// Exclusive scan in three passes: 1024-element blocks, their sums, the offsets.
__global__ void __launch_bounds__(1024) k_scan_blocks(int n, const int *in, int *out, int *block_sums) {
    __shared__ int s_w[32];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int v = i < n ? in[i] : 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += u;
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int y = s_w[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += u;
        }
        s_w[lane] = y;
    }
    __syncthreads();
    const int incl = x + (wid > 0 ? s_w[wid - 1] : 0);
    if (i < n) out[i] = incl - v;
    if (threadIdx.x == 1023) block_sums[blockIdx.x] = incl;
}
__global__ void k_scan_sums(int nblocks, int *block_sums, int *total) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int run = 0;
    for (int b = 0; b < nblocks; b++) {
        const int v = block_sums[b];
        block_sums[b] = run;
        run += v;
    }
    *total = run;
}
__global__ void k_scan_add(int n, int *out, const int *block_sums) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
}

// Hydrolysis of the candidates whose number prob[rank] < 0.02, then the
// return to GTP of the dimers off the tubule now and before
// (src/updater.cpp:232-256).  events[s]: 1 hydrolysed, 2 back to GTP.
__global__ void k_hydro_apply(int nt, int max_dimers, const int *off, int *flags, const int *cand, const int *rank,
                              const double *prob, double threshold, int8_t *events, int *n_events) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= max_dimers * nt) return;
    const int k = s / nt, t = s % nt;
    int8_t ev = 0;
    if (k < dimer_slots(off, t)) {
        const int g = off[t] + 2 * k;
        const int f = flags[g];
        if (cand[s] && prob[rank[s]] < threshold) {
            flags[g] = f & ~kFlagGtp;
            flags[g + 1] &= ~kFlagGtp;
            ev = 1;
        } else if (!(f & kFlagGtp) && !(f & kFlagExtra) && !(f & kFlagOnTubule) && !(f & kFlagOnTubPrev)) {
            flags[g] = f | kFlagGtp;
            flags[g + 1] |= kFlagGtp;
            ev = 2;
        }
    }
    if (events) events[s] = ev;
    if (ev) atomicAdd(&n_events[ev - 1], 1);
}

__global__ void k_count_extra(int nb, const int *traj, const int *flags, int *counts) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < nb && (flags[g] & kFlagExtra)) atomicAdd(&counts[traj[g]], 1);
}

__global__ void k_set_beads(KParams P, int n, const int *idx, const float *c7, const uint8_t *extra, float4 *frame,
                            int *flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int g = idx[i];
    const float *c = c7 + 7 * (size_t)i;
    store_frame(frame, P.nb, g, make_frame(P, c[0], c[1], c[2], c[3], c[4], c[5]));
    if (extra) flags[g] = extra[i] ? (flags[g] | kFlagExtra) : (flags[g] & ~kFlagExtra);
}

__global__ void k_flags_out(int nb, const int *flags, int *gtp, uint8_t *extra, int *on_cur, int *on_prev) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const int f = flags[g];
    if (gtp) gtp[g] = (f & kFlagGtp) ? 1 : 0;
    if (extra) extra[g] = (f & kFlagExtra) ? 1 : 0;
    if (on_cur) on_cur[g] = (f & kFlagOnTubule) ? 1 : 0;
    if (on_prev) on_prev[g] = (f & kFlagOnTubPrev) ? 1 : 0;
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

int cuda_fail(cudaError_t e) { return mtg_internal_fail(MTG_E_CUDA, cudaGetErrorString(e)); }
#define UCK(call)                                   \
    do {                                            \
        cudaError_t e_ = (call);                    \
        if (e_ != cudaSuccess) return cuda_fail(e_); \
    } while (0)

// scratch of the hydrolysis pass: candidate flags, ranks, events, block sums
struct HydroScratch {
    int *cand, *rank, *sums, *counts;   // counts: [0] total candidates, [1..2] events
    int8_t *events;
    double *prob;
    int prob_cap;
};

int max_dimers(const mtg_engine *e) {
    int m = 0;
    for (int t = 0; t < e->nt; t++) m = std::max(m, (e->h_off[t + 1] - e->h_off[t]) / 2);
    return m;
}

}  // namespace

extern "C" {

int mtg_mt_length(mtg_engine *e, int save_prev, int *mt_len) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (!e->have_state) return mtg_internal_fail(MTG_E_STATE, "no state uploaded");
    UCK(cudaSetDevice(e->device));
    int *counts = nullptr;
    UCK(cudaMallocAsync(&counts, sizeof(int) * e->nt, e->stream));
    UCK(cudaMemsetAsync(counts, 0, sizeof(int) * e->nt, e->stream));
    // the threshold cos(ANG_THRES) as the host's libm gives it (the reference
    // evaluates it on the host)
    const float cos_thres = std::cos(1.0f);
    k_mt_length<<<nblk(e->nb, 256), 256, 0, e->stream>>>(e->nb, e->traj, e->frame[e->cur], e->flags, save_prev,
                                                        cos_thres, counts);
    UCK(cudaGetLastError());
    if (mt_len) UCK(cudaMemcpyAsync(mt_len, counts, sizeof(int) * e->nt, cudaMemcpyDeviceToHost, e->stream));
    UCK(cudaFreeAsync(counts, e->stream));
    UCK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

int mtg_hydrolysis_candidates(mtg_engine *e, int *count) {
    if (!e || !count) return mtg_internal_fail(MTG_E_CONFIG, "engine or count is NULL");
    UCK(cudaSetDevice(e->device));
    const int md = max_dimers(e), L = md * e->nt, nb1 = nblk(L, 1024);
    if (!e->hydro_cand) {
        UCK(cudaMalloc(&e->hydro_cand, sizeof(int) * ((size_t)L + 1)));
        UCK(cudaMalloc(&e->hydro_rank, sizeof(int) * ((size_t)L + 1)));
        UCK(cudaMalloc(&e->hydro_sums, sizeof(int) * ((size_t)nb1 + 1)));
        UCK(cudaMalloc(&e->hydro_counts, sizeof(int) * 4));
        UCK(cudaMalloc(&e->hydro_events, (size_t)L + 1));
    }
    if (L == 0) {
        *count = 0;
        return MTG_OK;
    }
    k_hydro_mark<<<nblk(L, 256), 256, 0, e->stream>>>(e->nt, md, e->off, e->flags, e->hydro_cand);
    k_scan_blocks<<<nb1, 1024, 0, e->stream>>>(L, e->hydro_cand, e->hydro_rank, e->hydro_sums);
    k_scan_sums<<<1, 32, 0, e->stream>>>(nb1, e->hydro_sums, e->hydro_counts);
    k_scan_add<<<nb1, 1024, 0, e->stream>>>(L, e->hydro_rank, e->hydro_sums);
    UCK(cudaGetLastError());
    UCK(cudaMemcpyAsync(count, e->hydro_counts, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    UCK(cudaStreamSynchronize(e->stream));
    e->hydro_ncand = *count;
    return MTG_OK;
}

int mtg_hydrolyse(mtg_engine *e, const double *prob, int n, int8_t *events, int *n_hydrolysed, int *n_restored) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (!e->hydro_cand || n != e->hydro_ncand || (n > 0 && !prob))
        return mtg_internal_fail(MTG_E_STATE, "call mtg_hydrolysis_candidates first and pass one number per candidate");
    UCK(cudaSetDevice(e->device));
    const int md = max_dimers(e), L = md * e->nt;
    double *dprob = nullptr;
    UCK(cudaMallocAsync(&dprob, sizeof(double) * ((size_t)n + 1), e->stream));
    if (n > 0) UCK(cudaMemcpyAsync(dprob, prob, sizeof(double) * n, cudaMemcpyHostToDevice, e->stream));
    UCK(cudaMemsetAsync(e->hydro_counts + 1, 0, sizeof(int) * 2, e->stream));
    if (L > 0)
        k_hydro_apply<<<nblk(L, 256), 256, 0, e->stream>>>(e->nt, md, e->off, e->flags, e->hydro_cand, e->hydro_rank,
                                                          dprob, 0.02, events ? e->hydro_events : nullptr,
                                                          e->hydro_counts + 1);
    UCK(cudaGetLastError());
    int ev[2] = {0, 0};
    UCK(cudaMemcpyAsync(ev, e->hydro_counts + 1, sizeof(int) * 2, cudaMemcpyDeviceToHost, e->stream));
    if (events && L > 0) UCK(cudaMemcpyAsync(events, e->hydro_events, L, cudaMemcpyDeviceToHost, e->stream));
    UCK(cudaFreeAsync(dprob, e->stream));
    UCK(cudaStreamSynchronize(e->stream));
    e->hydro_ncand = -1;
    if (n_hydrolysed) *n_hydrolysed = ev[0];
    if (n_restored) *n_restored = ev[1];
    return MTG_OK;
}

int mtg_hydrolysis_slots(const mtg_engine *e, int *max_dimers_out) {
    if (!e || !max_dimers_out) return mtg_internal_fail(MTG_E_CONFIG, "engine or output is NULL");
    *max_dimers_out = max_dimers(e);
    return MTG_OK;
}

int mtg_count_extra(mtg_engine *e, int *n_extra) {
    if (!e || !n_extra) return mtg_internal_fail(MTG_E_CONFIG, "engine or n_extra is NULL");
    UCK(cudaSetDevice(e->device));
    int *counts = nullptr;
    UCK(cudaMallocAsync(&counts, sizeof(int) * e->nt, e->stream));
    UCK(cudaMemsetAsync(counts, 0, sizeof(int) * e->nt, e->stream));
    k_count_extra<<<nblk(e->nb, 256), 256, 0, e->stream>>>(e->nb, e->traj, e->flags, counts);
    UCK(cudaGetLastError());
    UCK(cudaMemcpyAsync(n_extra, counts, sizeof(int) * e->nt, cudaMemcpyDeviceToHost, e->stream));
    UCK(cudaFreeAsync(counts, e->stream));
    UCK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

int mtg_set_beads(mtg_engine *e, const int *idx, const float *coords, const uint8_t *extra, int n) {
    if (!e || (n > 0 && (!idx || !coords))) return mtg_internal_fail(MTG_E_CONFIG, "bad arguments");
    if (n < 0) return mtg_internal_fail(MTG_E_CONFIG, "n must be >= 0");
    for (int i = 0; i < n; i++)
        if (idx[i] < 0 || idx[i] >= e->nb) return mtg_internal_fail(MTG_E_CONFIG, "bead index out of range");
    if (n == 0) return MTG_OK;
    UCK(cudaSetDevice(e->device));
    int *didx = nullptr;
    float *dc = nullptr;
    uint8_t *dx = nullptr;
    UCK(cudaMallocAsync(&didx, sizeof(int) * n, e->stream));
    UCK(cudaMallocAsync(&dc, sizeof(float) * 7 * (size_t)n, e->stream));
    UCK(cudaMemcpyAsync(didx, idx, sizeof(int) * n, cudaMemcpyHostToDevice, e->stream));
    UCK(cudaMemcpyAsync(dc, coords, sizeof(float) * 7 * (size_t)n, cudaMemcpyHostToDevice, e->stream));
    if (extra) {
        UCK(cudaMallocAsync(&dx, n, e->stream));
        UCK(cudaMemcpyAsync(dx, extra, n, cudaMemcpyHostToDevice, e->stream));
    }
    k_set_beads<<<nblk(n, 128), 128, 0, e->stream>>>(e->kp, n, didx, dc, dx, e->frame[e->cur], e->flags);
    UCK(cudaGetLastError());
    UCK(cudaFreeAsync(didx, e->stream));
    UCK(cudaFreeAsync(dc, e->stream));
    if (dx) UCK(cudaFreeAsync(dx, e->stream));
    UCK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

int mtg_download_flags(mtg_engine *e, int *gtp, uint8_t *extra, int *on_tubule_cur, int *on_tubule_prev) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    UCK(cudaSetDevice(e->device));
    const size_t nb = e->nb;
    int *dg = nullptr, *dc = nullptr, *dp = nullptr;
    uint8_t *dx = nullptr;
    if (gtp) UCK(cudaMallocAsync(&dg, sizeof(int) * nb, e->stream));
    if (on_tubule_cur) UCK(cudaMallocAsync(&dc, sizeof(int) * nb, e->stream));
    if (on_tubule_prev) UCK(cudaMallocAsync(&dp, sizeof(int) * nb, e->stream));
    if (extra) UCK(cudaMallocAsync(&dx, nb, e->stream));
    k_flags_out<<<nblk(e->nb, 256), 256, 0, e->stream>>>(e->nb, e->flags, dg, dx, dc, dp);
    UCK(cudaGetLastError());
    if (gtp) UCK(cudaMemcpyAsync(gtp, dg, sizeof(int) * nb, cudaMemcpyDeviceToHost, e->stream));
    if (on_tubule_cur) UCK(cudaMemcpyAsync(on_tubule_cur, dc, sizeof(int) * nb, cudaMemcpyDeviceToHost, e->stream));
    if (on_tubule_prev) UCK(cudaMemcpyAsync(on_tubule_prev, dp, sizeof(int) * nb, cudaMemcpyDeviceToHost, e->stream));
    if (extra) UCK(cudaMemcpyAsync(extra, dx, nb, cudaMemcpyDeviceToHost, e->stream));
    for (void *q : {(void *)dg, (void *)dc, (void *)dp, (void *)dx})
        if (q) UCK(cudaFreeAsync(q, e->stream));
    UCK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

}  // extern "C"
