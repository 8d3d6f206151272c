// Host check of the learned mode's far-field tree (mt_gb300/csrc/tea_ff.cu,
// compiled into this program with stand-ins for the device-side functions it
// never calls here): for the trajectories of a dumped batch, every ordered
// pair of active beads is covered exactly once (a near leaf pair, or one far
// node pair), each leaf's ancestor list holds exactly its ancestors with a
// far list, node ranges nest in their parents, leaves hold at most kFFLeaf
// beads, internal nodes come larger first, and node leaf ranges match node
// bead ranges.  Usage: tree_check <batch.bin> <theta> [trajectories to check]
#include "../../mt_gb300/csrc/tea_ff.cu"

// stand-ins: never called by the host check
extern "C" int mtg_rebuild_pairs(mtg_engine *) { return 0; }
int mtg_internal_fail(int c, const char *) { return c; }
extern "C" int mtg_sync(mtg_engine *) { return 0; }
void mtg_internal_reset_graphs(mtg_engine *) {}
namespace mtg {
void launch_forces(const KParams &, const DevBuffers &, bool, cudaStream_t) {}
void launch_tea_feff(const KParams &, const DevBuffers &, const int2 *, int, float4 *, const int *, cudaStream_t) {}
void launch_ff_proxies(const KParams &, const DevBuffers &, const FFBuffers &, const int *, cudaStream_t) {}
void launch_ff_step(const KParams &, const DevBuffers &, const FFBuffers &, bool, float4 *, const int *, cudaStream_t) {}
}
#include <cstdio>
#include <cstdlib>
int main(int argc, char **argv) {
    const char *path = argv[1];
    float theta = atof(argv[2]);
    FILE *f = fopen(path, "rb");
    int nb, nt;
    fread(&nb, 4, 1, f); fread(&nt, 4, 1, f);
    std::vector<int> off(nt + 1), flags(nb);
    std::vector<float4> x(nb);
    fread(off.data(), 4, nt + 1, f);
    fread(flags.data(), 4, nb, f);
    fread(x.data(), 16, nb, f);
    fclose(f);
    mtg_engine e;
    e.nb = nb; e.nt = nt; e.h_off = off; e.p.tea_a = 2.0f;
    Partition P;
    build_partition(&e, x, flags, theta, P);
    const int nleaf = P.leaf_traj.size(), nn = P.node_parent.size();
    printf("leaves %d nodes %d near %lld proxy %lld far entries %zu tgt %zu anc %zu\n", nleaf, nn, P.near_pairs,
           P.proxy_pairs, P.far.size(), P.tgt.size(), P.anc.size());
    // position of each bead in leaf_bead order
    std::vector<int> pos(nb, -1);
    for (size_t k = 0; k < P.leaf_bead.size(); k++) pos[P.leaf_bead[k]] = k;
    long long bad = 0, checked = 0;
    const int ncheck = argc > 3 ? atoi(argv[3]) : 2;
    for (int t = 0; t < std::min(nt, ncheck); t++) {
        std::vector<int> act;
        for (int g = off[t]; g < off[t + 1]; g++) if (!(flags[g] & kFlagExtra)) act.push_back(g);
        const int n = act.size();
        std::vector<unsigned char> cov((size_t)n * n, 0);
        std::vector<int> li(nb, -1);  // local index by bead
        for (int k = 0; k < n; k++) li[act[k]] = k;
        auto mark = [&](int tn, int sn) {
            for (int a = P.node_range[2 * tn]; a < P.node_range[2 * tn + 1]; a++)
                for (int b = P.node_range[2 * sn]; b < P.node_range[2 * sn + 1]; b++) {
                    const int i = li[P.leaf_bead[a]], j = li[P.leaf_bead[b]];
                    if (i < 0 || j < 0) { bad++; continue; }
                    if (i != j) cov[(size_t)i * n + j]++;
                }
        };
        for (int L = 0; L < nleaf; L++) {
            if (P.leaf_traj[L] != t) continue;
            for (int k = P.near_start[L]; k < P.near_start[L + 1]; k++) mark(L, P.near[k]);
        }
        for (int N = 0; N < nn; N++) {
            const int b0 = P.node_range[2 * N];
            if (li[P.leaf_bead[b0]] < 0) continue;   // other trajectory
            for (int k = P.far_start[N]; k < P.far_start[N + 1]; k++) mark(N, P.far[k]);
        }
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                if (i == j) continue;
                checked++;
                if (cov[(size_t)i * n + j] != 1) bad++;
            }
        // ancestors: leaf L's anc list = nodes with far lists on its path
        for (int L = 0; L < nleaf; L++) {
            if (P.leaf_traj[L] != t) continue;
            std::vector<int> expect;
            for (int N = L; N >= 0; N = P.node_parent[N])
                if (P.far_start[N + 1] > P.far_start[N]) expect.push_back(N);
            std::vector<int> got(P.anc.begin() + P.anc_start[L], P.anc.begin() + P.anc_start[L + 1]);
            if (expect != got) bad++;
        }
    }
    // node ranges nest in their parents; internal ids ordered by size
    for (int N = 0; N < nn; N++) {
        const int p = P.node_parent[N];
        if (p >= 0 && (P.node_range[2 * N] < P.node_range[2 * p] || P.node_range[2 * N + 1] > P.node_range[2 * p + 1])) bad++;
        if (N > nleaf && P.node_range[2 * N + 1] - P.node_range[2 * N] > P.node_range[2 * N - 1] - P.node_range[2 * N - 2]) bad++;
        if (N < nleaf && P.node_range[2 * N + 1] - P.node_range[2 * N] > kFFLeaf) bad++;
        if (P.leaf_start[P.node_leaves[2 * N]] != P.node_range[2 * N] ||
            P.leaf_start[P.node_leaves[2 * N + 1]] != P.node_range[2 * N + 1]) bad++;
    }
    printf("checked %lld pairs, bad %lld\n", checked, bad);
    return bad != 0;
}
