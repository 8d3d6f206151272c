// tea_ff.cu - the tree behind the far-field approximation of the learned
// TEA mobility product (kernels in kernels_tea.cu), and its C ABI.
//
// Every trajectory's non-extra beads are split by a k-d bisection (longest
// extent, median rounded to a multiple of kFFLeaf while more than two leaves'
// worth remain) into a binary tree with leaves of at most kFFLeaf beads; each
// node has a centre c (of its bounding box) and a radius r (largest distance
// of a bead from c).  A dual traversal of the tree against itself, from the
// pair (root, root), sorts every ordered bead pair of the trajectory into
// exactly one of: a node pair (N, J), N != J, that is well separated --
// the centres farther apart than (r_N + r_J + 2 margin) / theta' and the
// spheres more than 4a + 2 margin apart, with theta' = theta for two leaves
// and theta * kFFNodeTheta when an internal node is involved -- whose
// interaction goes through the proxies (far list of N); a pair of leaves
// that is not (near list of the target leaf); otherwise the node with the
// larger radius is split and its two children are visited.  The tree is built
// on the host from the current positions when the far field is switched on and
// again every `refresh_every` steps; the boxes and proxies follow the beads
// at every step, so a tree only has to stay a good grouping, which it does
// for thousands of steps (beads move about 0.02 nm per step).  The scheme is
// a black-box fast multipole method with degree-2 Chebyshev interpolation
// (Fong and Darve, J. Comput. Phys. 228 (2009) 8712), with node charges and
// target potentials evaluated directly at every level instead of through
// M2M / L2L translations (which, for trilinear interpolation, give the
// same values).  No reference counterpart: the reference sums all pairs of a
// trajectory (src/bdhitea_kernel.cu:174-180) and leaves its listed variant
// unbuilt (src/mt.h:118).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mtg_engine.cuh"

using namespace mtg;

namespace {

constexpr float kFFMargin = 1.0f;      // nm added to each radius in the far test
constexpr float kFFNodeTheta = 0.7f;   // theta factor for pairs that involve an internal node

#define FCK(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return mtg_internal_fail(MTG_E_CUDA, cudaGetErrorString(e_));        \
    } while (0)

struct Partition {
    std::vector<int> leaf_start{0}, leaf_bead, leaf_traj, near_start{0}, near, rest;
    std::vector<int> node_range, node_leaves, node_parent, far_start{0}, far, tgt, anc_start{0}, anc;
    long long near_pairs = 0, proxy_pairs = 0;
};

struct TreeNode {
    int beg, end;            // positions in the trajectory's bead order
    int child[2];            // -1 for a leaf
    int parent;
    float c[3], r;
};

// Splits ids[beg, end) in place (leaves end up contiguous in depth-first
// order) and appends the nodes, parent before children.
int kd_build(const std::vector<float4> &x, std::vector<int> &ids, int beg, int end, int parent,
             std::vector<TreeNode> &T) {
    const int me = (int)T.size();
    T.push_back(TreeNode{beg, end, {-1, -1}, parent, {0.f, 0.f, 0.f}, 0.f});
    const int n = end - beg;
    float lo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, hi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int k = beg; k < end; k++) {
        const float4 p = x[ids[k]];
        const float v[3] = {p.x, p.y, p.z};
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], v[d]);
            hi[d] = std::max(hi[d], v[d]);
        }
    }
    const float c[3] = {0.5f * (lo[0] + hi[0]), 0.5f * (lo[1] + hi[1]), 0.5f * (lo[2] + hi[2])};
    float r = 0.f;
    for (int k = beg; k < end; k++) {
        const float4 p = x[ids[k]];
        r = std::max(r, std::sqrt((p.x - c[0]) * (p.x - c[0]) + (p.y - c[1]) * (p.y - c[1]) +
                                  (p.z - c[2]) * (p.z - c[2])));
    }
    for (int d = 0; d < 3; d++) T[me].c[d] = c[d];
    T[me].r = r;
    if (n <= kFFLeaf) return me;
    int ax = 0;
    for (int d = 1; d < 3; d++)
        if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    const int k = n > 2 * kFFLeaf ? std::max(kFFLeaf, (n / 2) / kFFLeaf * kFFLeaf) : n / 2;
    auto coord = [&](int g) { return ax == 0 ? x[g].x : (ax == 1 ? x[g].y : x[g].z); };
    int *base = ids.data() + beg;
    std::nth_element(base, base + k, base + n, [&](int a, int b) {
        const float va = coord(a), vb = coord(b);
        return va < vb || (va == vb && a < b);
    });
    const int l = kd_build(x, ids, beg, beg + k, me, T);
    const int rr = kd_build(x, ids, beg + k, end, me, T);
    T[me].child[0] = l;
    T[me].child[1] = rr;
    return me;
}

void build_partition(const mtg_engine *e, const std::vector<float4> &x, const std::vector<int> &flags, float theta,
                     Partition &P) {
    const float a = e->p.tea_a;
    // internal nodes get their ids at the end (after every leaf, larger first):
    // until then a node reference is a leaf id (>= 0) or -(1 + internal index)
    struct Internal {
        int beg, end, parent, leaf0, leaf1;
    };
    std::vector<Internal> internal;
    std::vector<std::pair<int, int>> farpairs;   // (target, source) references
    std::vector<int> leaf_parent;                // reference of each leaf's parent
    std::vector<std::vector<int>> leaf_anc;      // references of each leaf's nodes with a far list
    for (int t = 0; t < e->nt; t++) {
        std::vector<int> ids;
        for (int g = e->h_off[t]; g < e->h_off[t + 1]; g++) {
            if (flags[g] & kFlagExtra)
                P.rest.push_back(g);
            else
                ids.push_back(g);
        }
        if (ids.empty()) continue;
        std::vector<TreeNode> T;
        kd_build(x, ids, 0, (int)ids.size(), -1, T);
        const int base = (int)P.leaf_bead.size();
        P.leaf_bead.insert(P.leaf_bead.end(), ids.begin(), ids.end());
        // references of this trajectory's nodes
        std::vector<int> ref(T.size());
        for (size_t k = 0; k < T.size(); k++) {
            if (T[k].child[0] < 0) {
                ref[k] = (int)P.leaf_traj.size();
                P.leaf_traj.push_back(t);
                P.leaf_start.push_back(base + T[k].end);
            } else {
                ref[k] = -(1 + (int)internal.size());
                internal.push_back({base + T[k].beg, base + T[k].end, 0, 0, 0});
            }
        }
        for (size_t k = 0; k < T.size(); k++) {
            const int pr = T[k].parent < 0 ? -1 - (1 << 30) : ref[T[k].parent];
            if (ref[k] >= 0)
                leaf_parent.push_back(pr);
            else
                internal[-ref[k] - 1].parent = pr;
        }
        // leaf ranges of the internal nodes (children come after their parent in T)
        std::vector<int> lf0(T.size()), lf1(T.size());
        for (int k = (int)T.size() - 1; k >= 0; k--) {
            if (ref[k] >= 0) {
                lf0[k] = ref[k];
                lf1[k] = ref[k] + 1;
            } else {
                lf0[k] = lf0[T[k].child[0]];
                lf1[k] = lf1[T[k].child[1]];
                internal[-ref[k] - 1].leaf0 = lf0[k];
                internal[-ref[k] - 1].leaf1 = lf1[k];
            }
        }
        // dual traversal
        std::vector<char> has_far(T.size(), 0);
        std::vector<std::vector<int>> nearl(T.size());
        std::vector<std::pair<int, int>> stack{{0, 0}};
        while (!stack.empty()) {
            const auto [I, J] = stack.back();
            stack.pop_back();
            const TreeNode &A = T[I], &B = T[J];
            const bool leaves = A.child[0] < 0 && B.child[0] < 0;
            const float th = leaves ? theta : theta * kFFNodeTheta;
            const float dx = B.c[0] - A.c[0], dy = B.c[1] - A.c[1], dz = B.c[2] - A.c[2];
            const float d = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (I != J && d * th > A.r + B.r + 2.0f * kFFMargin && d - A.r - B.r > 4.0f * a + 2.0f * kFFMargin) {
                farpairs.push_back({ref[I], ref[J]});
                has_far[I] = 1;
                P.proxy_pairs += 64;
            } else if (leaves) {
                nearl[I].push_back(J);
                const long long ni = A.end - A.beg, nj = B.end - B.beg;
                P.near_pairs += ni * nj - (I == J ? ni : 0);
            } else if (B.child[0] < 0 || (A.child[0] >= 0 && A.r >= B.r)) {
                stack.push_back({A.child[1], J});
                stack.push_back({A.child[0], J});
            } else {
                stack.push_back({I, B.child[1]});
                stack.push_back({I, B.child[0]});
            }
        }
        for (size_t k = 0; k < T.size(); k++) {
            if (T[k].child[0] >= 0) continue;
            std::vector<int> nl;
            for (int J : nearl[k]) nl.push_back(ref[J]);
            std::sort(nl.begin(), nl.end());
            P.near.insert(P.near.end(), nl.begin(), nl.end());
            P.near_start.push_back((int)P.near.size());
            std::vector<int> an;
            for (int N = (int)k; N >= 0; N = T[N].parent)
                if (has_far[N]) an.push_back(ref[N]);
            leaf_anc.push_back(an);
        }
    }
    // final ids: leaves 0 .. nleaf-1, then the internal nodes by decreasing size
    const int nleaf = (int)P.leaf_traj.size();
    std::vector<int> order(internal.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int u, int v) {
        return internal[u].end - internal[u].beg > internal[v].end - internal[v].beg;
    });
    std::vector<int> idof(internal.size());
    for (size_t k = 0; k < order.size(); k++) idof[order[k]] = nleaf + (int)k;
    auto fin = [&](int r) { return r >= 0 ? r : (r == -1 - (1 << 30) ? -1 : idof[-r - 1]); };
    const int nnode = nleaf + (int)internal.size();
    P.node_range.resize(2 * (size_t)nnode);
    P.node_leaves.resize(2 * (size_t)nnode);
    P.node_parent.resize(nnode);
    for (int L = 0; L < nleaf; L++) {
        P.node_range[2 * L] = P.leaf_start[L];
        P.node_range[2 * L + 1] = P.leaf_start[L + 1];
        P.node_leaves[2 * L] = L;
        P.node_leaves[2 * L + 1] = L + 1;
        P.node_parent[L] = fin(leaf_parent[L]);
    }
    for (size_t k = 0; k < internal.size(); k++) {
        const int N = idof[k];
        P.node_range[2 * N] = internal[k].beg;
        P.node_range[2 * N + 1] = internal[k].end;
        P.node_leaves[2 * N] = internal[k].leaf0;
        P.node_leaves[2 * N + 1] = internal[k].leaf1;
        P.node_parent[N] = fin(internal[k].parent);
    }
    // far lists grouped by target node, in traversal order
    std::vector<int> cnt(nnode + 1, 0);
    for (auto &fp : farpairs) cnt[fin(fp.first) + 1]++;
    for (int N = 0; N < nnode; N++) cnt[N + 1] += cnt[N];
    P.far_start.assign(cnt.begin(), cnt.end());
    P.far.resize(farpairs.size());
    for (auto &fp : farpairs) P.far[cnt[fin(fp.first)]++] = fin(fp.second);
    for (int N = 0; N < nnode; N++)
        if (P.far_start[N + 1] > P.far_start[N]) P.tgt.push_back(N);
    for (int L = 0; L < nleaf; L++) {
        for (int r : leaf_anc[L]) P.anc.push_back(fin(r));
        P.anc_start.push_back((int)P.anc.size());
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

// Builds the tree from the current state and uploads it.
static int ff_build(mtg_engine *e) {
    const int nb = e->nb;
    std::vector<float4> x(nb);
    std::vector<int> flags(nb);
    FCK(cudaMemcpyAsync(x.data(), e->frame[e->cur], sizeof(float4) * nb, cudaMemcpyDeviceToHost, e->stream));
    FCK(cudaMemcpyAsync(flags.data(), e->flags, sizeof(int) * nb, cudaMemcpyDeviceToHost, e->stream));
    FCK(cudaStreamSynchronize(e->stream));
    Partition P;
    build_partition(e, x, flags, e->ff_theta, P);
    const int nleaf = (int)P.leaf_traj.size(), nnode = (int)P.node_parent.size();
    // inner nodes the P2M kernel visits: far sources or targets (ids are larger nodes first)
    std::vector<char> used(nnode, 0);
    for (int N = 0; N < nnode; N++)
        if (P.far_start[N + 1] > P.far_start[N]) used[N] = 1;
    for (int J : P.far) used[J] = 1;
    std::vector<int> inner;
    for (int N = nleaf; N < nnode; N++)
        if (used[N]) inner.push_back(N);
    int max_anc = 0;
    for (int L = 0; L < nleaf; L++) max_anc = std::max(max_anc, P.anc_start[L + 1] - P.anc_start[L]);
    if (max_anc > kFFMaxAnc)
        return mtg_internal_fail(MTG_E_CONFIG, "far-field tree deeper than the step kernel's ancestor limit");
    enum { kLeafStart, kLeafBead, kLeafTraj, kNearStart, kNear, kNodeRange, kNodeLeaves, kFarStart, kFar, kTgt,
           kInner, kAncStart, kAnc, kRest, kParts };
    const std::vector<int> *parts[kParts] = {&P.leaf_start, &P.leaf_bead, &P.leaf_traj, &P.near_start, &P.near,
                                             &P.node_range, &P.node_leaves, &P.far_start, &P.far, &P.tgt, &inner,
                                             &P.anc_start, &P.anc, &P.rest};
    size_t nints = 0;
    for (auto *v : parts) nints += v->size() + 1;
    const size_t nn1 = (size_t)std::max(nnode, 1);
    const size_t nf4 = (size_t)(2 + 16 + 24) * nn1 + (size_t)kFFPackF4 * (nleaf + 1) + P.leaf_bead.size();
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
    int *dev[kParts];
    for (int k = 0; k < kParts; k++) {
        dev[k] = e->ff_ints + host.size();
        host.insert(host.end(), parts[k]->begin(), parts[k]->end());
        host.push_back(0);   // keeps every array non-empty
    }
    FCK(cudaMemcpyAsync(e->ff_ints, host.data(), sizeof(int) * host.size(), cudaMemcpyHostToDevice, e->stream));
    FCK(cudaMemsetAsync(e->ff_f4, 0, sizeof(float4) * nf4, e->stream));
    FCK(cudaStreamSynchronize(e->stream));
    FFBuffers &F = e->ffb;
    F.nleaf = nleaf;
    F.nnode = nnode;
    F.ntgt = (int)P.tgt.size();
    F.ninner = (int)inner.size();
    F.nrest = (int)P.rest.size();
    F.max_anc = max_anc;
    F.leaf_start = dev[kLeafStart];
    F.leaf_bead = dev[kLeafBead];
    F.leaf_traj = dev[kLeafTraj];
    F.near_start = dev[kNearStart];
    F.near = dev[kNear];
    F.node_range = dev[kNodeRange];
    F.node_leaves = dev[kNodeLeaves];
    F.far_start = dev[kFarStart];
    F.far = dev[kFar];
    F.tgt = dev[kTgt];
    F.inner = dev[kInner];
    F.anc_start = dev[kAncStart];
    F.anc = dev[kAnc];
    F.rest = dev[kRest];
    F.box = e->ff_f4;
    F.q = e->ff_f4 + 2 * nn1;
    F.phi = e->ff_f4 + 18 * nn1;
    F.pack = e->ff_f4 + 42 * nn1;
    F.nearsum = F.pack + (size_t)kFFPackF4 * (nleaf + 1);
    e->ff_near_pairs = P.near_pairs;
    e->ff_proxy_pairs = P.proxy_pairs;
    e->ff_sizes[0] = nleaf;
    e->ff_sizes[1] = (int)P.leaf_bead.size();
    e->ff_sizes[2] = (int)P.near.size();
    e->ff_sizes[3] = nnode;
    e->ff_sizes[4] = (int)P.far.size();
    // the layout as mtg_tea_farfield_layout returns it
    e->ff_host.clear();
    for (const std::vector<int> *v : {&P.leaf_start, &P.leaf_bead, &P.near_start, &P.near, &P.node_range,
                                      &P.node_parent, &P.far_start, &P.far})
        e->ff_host.insert(e->ff_host.end(), v->begin(), v->end());
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
    if (!e->side) FCK(cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking));
    if (!e->ev_fork) FCK(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
    if (!e->ev_join) FCK(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
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
                            int *node_range, int *node_parent, int *far_start, int *far) {
    if (!e || !sizes) return mtg_internal_fail(MTG_E_CONFIG, "engine or sizes is NULL");
    if (!e->ff_on) return mtg_internal_fail(MTG_E_STATE, "the far field is off");
    std::memcpy(sizes, e->ff_sizes, sizeof e->ff_sizes);
    const size_t nl = e->ff_sizes[0], nn = e->ff_sizes[3];
    int *outs[8] = {leaf_start, leaf_bead, near_start, near, node_range, node_parent, far_start, far};
    const size_t lens[8] = {nl + 1, (size_t)e->ff_sizes[1], nl + 1, (size_t)e->ff_sizes[2], 2 * nn, nn, nn + 1,
                            (size_t)e->ff_sizes[4]};
    size_t at = 0;
    for (int k = 0; k < 8; k++) {
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
