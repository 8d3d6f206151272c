// tea_ff.cu - the partition behind the far-field approximation of the
// learned TEA mobility product (kernels in kernels_tea.cu), and its C ABI.
//
// Every trajectory's non-extra beads are split by a k-d bisection (longest
// extent, median rounded to a multiple of kFFLeaf while more than two leaves'
// worth remain) into leaves of at most kFFLeaf beads.  For each target leaf I
// a source leaf J of the same trajectory is far when the leaves' centres are
// farther apart than (r_I + r_J + 2 margin) / theta and their spheres are
// more than 4a + 2 margin apart (r: largest distance of a bead from its box
// centre); every other leaf, I included, is near.  The partition is built on
// the host from the current positions when the far field is switched on and
// again every `refresh_every` steps; the boxes and proxies follow the beads
// at every step, so a partition only has to stay a good grouping, which it
// does for thousands of steps (beads move about 0.02 nm per step).  No
// reference counterpart: the reference sums all pairs of a trajectory
// (src/bdhitea_kernel.cu:174-180) and leaves its listed variant unbuilt
// (src/mt.h:118).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mtg_engine.cuh"

using namespace mtg;

namespace {

constexpr float kFFMargin = 1.0f;   // nm added to each radius in the far test

#define FCK(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return mtg_internal_fail(MTG_E_CUDA, cudaGetErrorString(e_));        \
    } while (0)

struct Partition {
    std::vector<int> leaf_start{0}, leaf_bead, leaf_traj, near_start{0}, near, far_start{0}, far, rest;
    long long near_pairs = 0, proxy_pairs = 0;
};

void kd_split(const std::vector<float4> &x, int *ids, int n, std::vector<std::pair<int *, int>> &leaves) {
    if (n <= kFFLeaf) {
        leaves.push_back({ids, n});
        return;
    }
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int k = 0; k < n; k++) {
        const float4 p = x[ids[k]];
        const float v[3] = {p.x, p.y, p.z};
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], v[d]);
            hi[d] = std::max(hi[d], v[d]);
        }
    }
    int ax = 0;
    for (int d = 1; d < 3; d++)
        if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    const int k = n > 2 * kFFLeaf ? std::max(kFFLeaf, (n / 2) / kFFLeaf * kFFLeaf) : n / 2;
    auto coord = [&](int g) { return ax == 0 ? x[g].x : (ax == 1 ? x[g].y : x[g].z); };
    std::nth_element(ids, ids + k, ids + n, [&](int a, int b) {
        const float va = coord(a), vb = coord(b);
        return va < vb || (va == vb && a < b);
    });
    kd_split(x, ids, k, leaves);
    kd_split(x, ids + k, n - k, leaves);
}

void build_partition(const mtg_engine *e, const std::vector<float4> &x, const std::vector<int> &flags, float theta,
                     Partition &P) {
    const float a = e->p.tea_a;
    for (int t = 0; t < e->nt; t++) {
        std::vector<int> ids;
        for (int g = e->h_off[t]; g < e->h_off[t + 1]; g++) {
            if (flags[g] & kFlagExtra)
                P.rest.push_back(g);
            else
                ids.push_back(g);
        }
        if (ids.empty()) continue;
        std::vector<std::pair<int *, int>> leaves;
        kd_split(x, ids.data(), (int)ids.size(), leaves);
        const int first = (int)P.leaf_traj.size();
        std::vector<float> cx, cy, cz, rr;
        std::vector<int> cnt;
        for (auto &l : leaves) {
            float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
            for (int k = 0; k < l.second; k++) {
                const float4 p = x[l.first[k]];
                lo[0] = std::min(lo[0], p.x), hi[0] = std::max(hi[0], p.x);
                lo[1] = std::min(lo[1], p.y), hi[1] = std::max(hi[1], p.y);
                lo[2] = std::min(lo[2], p.z), hi[2] = std::max(hi[2], p.z);
            }
            const float c[3] = {0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2])};
            float r = 0.f;
            for (int k = 0; k < l.second; k++) {
                const float4 p = x[l.first[k]];
                r = std::max(r, std::sqrt((p.x - c[0]) * (p.x - c[0]) + (p.y - c[1]) * (p.y - c[1]) +
                                          (p.z - c[2]) * (p.z - c[2])));
            }
            cx.push_back(c[0]), cy.push_back(c[1]), cz.push_back(c[2]), rr.push_back(r), cnt.push_back(l.second);
            P.leaf_bead.insert(P.leaf_bead.end(), l.first, l.first + l.second);
            P.leaf_start.push_back((int)P.leaf_bead.size());
            P.leaf_traj.push_back(t);
        }
        const int nl = (int)leaves.size();
        for (int I = 0; I < nl; I++) {
            for (int J = 0; J < nl; J++) {
                const float dx = cx[J] - cx[I], dy = cy[J] - cy[I], dz = cz[J] - cz[I];
                const float d = std::sqrt(dx * dx + dy * dy + dz * dz);
                const bool far = I != J && d * theta > rr[I] + rr[J] + 2.0f * kFFMargin &&
                                 d - rr[I] - rr[J] > 4.0f * a + 2.0f * kFFMargin;
                if (far) {
                    P.far.push_back(first + J);
                    P.proxy_pairs += 64;
                } else {
                    P.near.push_back(first + J);
                    P.near_pairs += (long long)cnt[I] * cnt[J] - (I == J ? cnt[I] : 0);
                }
            }
            P.near_start.push_back((int)P.near.size());
            P.far_start.push_back((int)P.far.size());
        }
    }
}

}  // namespace

void mtg_internal_ff_free(mtg_engine *e) {
    if (e->ff_ints) cudaFree(e->ff_ints);
    if (e->ff_f4) cudaFree(e->ff_f4);
    e->ff_ints = nullptr;
    e->ff_f4 = nullptr;
    e->ff_ints_cap = e->ff_f4_cap = 0;
    e->ffb = FFBuffers{};
}

// Builds the partition from the current state and uploads it.
static int ff_build(mtg_engine *e) {
    const int nb = e->nb;
    std::vector<float4> x(nb);
    std::vector<int> flags(nb);
    FCK(cudaMemcpyAsync(x.data(), e->frame[e->cur], sizeof(float4) * nb, cudaMemcpyDeviceToHost, e->stream));
    FCK(cudaMemcpyAsync(flags.data(), e->flags, sizeof(int) * nb, cudaMemcpyDeviceToHost, e->stream));
    FCK(cudaStreamSynchronize(e->stream));
    Partition P;
    build_partition(e, x, flags, e->ff_theta, P);
    const int nleaf = (int)P.leaf_traj.size();
    const std::vector<int> *parts[] = {&P.leaf_start, &P.leaf_bead, &P.leaf_traj, &P.near_start, &P.near,
                                       &P.far_start, &P.far, &P.rest};
    size_t nints = 0;
    for (auto *v : parts) nints += v->size() + 1;
    const size_t nf4 = (size_t)(2 + 16 + 24) * std::max(nleaf, 1) + (size_t)kFFPackF4 * (nleaf + 1);
    if (nints > e->ff_ints_cap) {
        if (e->ff_ints) cudaFree(e->ff_ints);
        e->ff_ints = nullptr;
        FCK(cudaMalloc(&e->ff_ints, sizeof(int) * nints));
        e->ff_ints_cap = nints;
    }
    if (nf4 > e->ff_f4_cap) {
        if (e->ff_f4) cudaFree(e->ff_f4);
        e->ff_f4 = nullptr;
        FCK(cudaMalloc(&e->ff_f4, sizeof(float4) * nf4));
        e->ff_f4_cap = nf4;
    }
    std::vector<int> host;
    host.reserve(nints);
    int *dev[8];
    for (int k = 0; k < 8; k++) {
        dev[k] = e->ff_ints + host.size();
        host.insert(host.end(), parts[k]->begin(), parts[k]->end());
        host.push_back(0);   // keeps every array non-empty
    }
    FCK(cudaMemcpyAsync(e->ff_ints, host.data(), sizeof(int) * host.size(), cudaMemcpyHostToDevice, e->stream));
    FCK(cudaMemsetAsync(e->ff_f4, 0, sizeof(float4) * nf4, e->stream));
    FCK(cudaStreamSynchronize(e->stream));
    FFBuffers &F = e->ffb;
    F.nleaf = nleaf;
    F.nrest = (int)P.rest.size();
    F.leaf_start = dev[0];
    F.leaf_bead = dev[1];
    F.leaf_traj = dev[2];
    F.near_start = dev[3];
    F.near = dev[4];
    F.far_start = dev[5];
    F.far = dev[6];
    F.rest = dev[7];
    F.box = e->ff_f4;
    F.q = e->ff_f4 + 2 * (size_t)nleaf;
    F.phi = e->ff_f4 + 18 * (size_t)nleaf;
    F.pack = e->ff_f4 + 42 * (size_t)std::max(nleaf, 1);
    e->ff_near_pairs = P.near_pairs;
    e->ff_proxy_pairs = P.proxy_pairs;
    e->ff_sizes[0] = nleaf;
    e->ff_sizes[1] = (int)P.leaf_bead.size();
    e->ff_sizes[2] = (int)P.near.size();
    e->ff_sizes[3] = (int)P.far.size();
    e->ff_host.clear();
    for (int k = 0; k < 7; k++) e->ff_host.insert(e->ff_host.end(), parts[k]->begin(), parts[k]->end());
    e->ff_steps = 0;
    mtg_internal_reset_graphs(e);   // the graphs hold the old lists and sizes
    return MTG_OK;
}

int mtg_internal_ff_refresh(mtg_engine *e) {
    if (!e->ff_on || !e->surr || e->ff_refresh <= 0 || e->ff_steps < e->ff_refresh) return MTG_OK;
    return ff_build(e);
}

extern "C" {

int mtg_set_tea_farfield(mtg_engine *e, int on, float theta, int refresh_every) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (on && !e->p.hdi_on) return mtg_internal_fail(MTG_E_STATE, "the far field approximates TEA: create with hdi_on");
    if (on && !(theta > 0.0f && theta <= 1.0f)) return mtg_internal_fail(MTG_E_CONFIG, "theta must be in (0, 1]");
    if (refresh_every < 0) return mtg_internal_fail(MTG_E_CONFIG, "refresh_every must be >= 0");
    if (on && !e->have_state) return mtg_internal_fail(MTG_E_STATE, "no state uploaded");
    FCK(cudaSetDevice(e->device));
    mtg_internal_reset_graphs(e);
    e->ff_on = on != 0;
    if (!e->ff_on) return MTG_OK;
    e->ff_theta = theta;
    e->ff_refresh = refresh_every;
    return ff_build(e);
}

int mtg_tea_farfield_stats(mtg_engine *e, int *nleaves, long long *near_pairs, long long *proxy_pairs) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (nleaves) *nleaves = e->ff_on ? e->ffb.nleaf : 0;
    if (near_pairs) *near_pairs = e->ff_on ? e->ff_near_pairs : 0;
    if (proxy_pairs) *proxy_pairs = e->ff_on ? e->ff_proxy_pairs : 0;
    return MTG_OK;
}

int mtg_tea_farfield_layout(mtg_engine *e, int *sizes, int *leaf_start, int *leaf_bead, int *near_start, int *near,
                            int *far_start, int *far) {
    if (!e || !sizes) return mtg_internal_fail(MTG_E_CONFIG, "engine or sizes is NULL");
    if (!e->ff_on) return mtg_internal_fail(MTG_E_STATE, "the far field is off");
    std::memcpy(sizes, e->ff_sizes, sizeof e->ff_sizes);
    const int nl = e->ff_sizes[0];
    int *outs[7] = {leaf_start, leaf_bead, nullptr, near_start, near, far_start, far};
    const size_t lens[7] = {(size_t)nl + 1, (size_t)e->ff_sizes[1], (size_t)nl, (size_t)nl + 1,
                            (size_t)e->ff_sizes[2], (size_t)nl + 1, (size_t)e->ff_sizes[3]};
    size_t at = 0;
    for (int k = 0; k < 7; k++) {
        if (outs[k]) std::memcpy(outs[k], e->ff_host.data() + at, sizeof(int) * lens[k]);
        at += lens[k];
    }
    return MTG_OK;
}

int mtg_tea_effective_forces(mtg_engine *e, float *feff_exact, float *feff_ff, float *rforce) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (!e->p.hdi_on) return mtg_internal_fail(MTG_E_STATE, "engine created without hdi_on");
    if (!e->have_state) return mtg_internal_fail(MTG_E_STATE, "no state uploaded");
    if (feff_ff && !e->ff_on) return mtg_internal_fail(MTG_E_STATE, "the far field is off");
    FCK(cudaSetDevice(e->device));
    // the pair lists of the current state (the far-field step corrects
    // overlapping pairs from the LJ list)
    if (e->p.lj_on || e->p.is_assembly) {
        const int rc = mtg_rebuild_pairs(e);
        if (rc) return rc;
    }
    const size_t nb = e->nb;
    float4 *buf = nullptr;
    FCK(cudaMalloc(&buf, sizeof(float4) * 2 * nb));
    const DevBuffers B = e->bufs();
    launch_forces(e->kp, B, true, e->stream);
    if (feff_exact) launch_tea_feff(e->kp, B, e->tea_work, e->tea_nwork, buf, nullptr, e->stream);
    if (feff_ff) {
        launch_ff_proxies(e->kp, B, e->ffb, nullptr, e->stream);
        launch_ff_step(e->kp, B, e->ffb, true, buf + nb, nullptr, e->stream);
    }
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess && feff_exact)
        err = cudaMemcpyAsync(feff_exact, buf, sizeof(float4) * nb, cudaMemcpyDeviceToHost, e->stream);
    if (err == cudaSuccess && feff_ff)
        err = cudaMemcpyAsync(feff_ff, buf + nb, sizeof(float4) * nb, cudaMemcpyDeviceToHost, e->stream);
    if (err == cudaSuccess && rforce)
        err = cudaMemcpyAsync(rforce, e->tea_r, sizeof(float4) * nb, cudaMemcpyDeviceToHost, e->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
    cudaFree(buf);
    if (err != cudaSuccess) return mtg_internal_fail(MTG_E_CUDA, cudaGetErrorString(err));
    return mtg_sync(e);
}

}  // extern "C"
