// kernels_cells.cu - neighbour-list rebuild through a per-trajectory spatial
// hash (cell list), producing the same lists as the brute-force kernel.
//
// Cells are cubes of edge `reach` (the largest list cutoff, or the 6.6 nm
// prefilter of the assembly lists), so every partner lies in the 27 cells
// around a bead.  Each trajectory owns a hash table of next_pow2(max(32, N))
// buckets; colliding cells share a bucket and only add candidates.
//   1. k_cell_count : bucket of every bead, bucket populations
//   2. k_cell_scan  : one CTA per trajectory, exclusive scan of its table
//   3. k_cell_fill  : beads scattered into bucket order
//   4. k_cell_lists : a warp per bead: candidates from the 27 cells' buckets
//      (each bucket visited once), the reference's list tests, hits ordered
//      by rank so each list is in ascending j (orientation 0 before 1 for the
//      lateral list), exactly the order of the reference's j loops
//      (src/compute_cuda.cu:564-661, :927-936).
#include "mtg_internal.cuh"

namespace mtg {

namespace {

constexpr float kPairReach = 6.6f;  // see kPairPrefilter in kernels_lists.cu

__global__ void k_cell_count(KParams P, const float4 *pos, const int *traj, const int *tbase, const int *tmask,
                             float inv_cell, int *key, int *cnt) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.nb) return;
    const float4 p = pos[g];
    const int t = traj[g];
    const uint32_t h = cell_hash(cell_coord(p.x, inv_cell), cell_coord(p.y, inv_cell), cell_coord(p.z, inv_cell));
    const int k = tbase[t] + (int)(h & (uint32_t)tmask[t]);
    key[g] = k;
    atomicAdd(&cnt[k], 1);
}

// Exclusive scan of each trajectory's table; start and cursor get the result.
__global__ void __launch_bounds__(1024) k_cell_scan(const int *tbase, const int *cnt, int *start, int *cursor) {
    const int t = blockIdx.x;
    const int b0 = tbase[t], n = tbase[t + 1] - tbase[t];
    __shared__ int s_part[1024];
    __shared__ int s_warp[32];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    int local = 0;
    for (int i = lo; i < hi; i++) local += cnt[b0 + i];
    // block exclusive scan of `local`
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int v = local;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) s_warp[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    int run = (v - local) + (wid > 0 ? s_warp[wid - 1] : 0);
    s_part[threadIdx.x] = run;
    for (int i = lo; i < hi; i++) {
        start[b0 + i] = run;
        cursor[b0 + i] = run;
        run += cnt[b0 + i];
    }
}

// Bucket-ordered bead lists; positions are relative to the trajectory's
// first bead, so slots of trajectory t start at off[t].
__global__ void k_cell_fill(int nb, const int *traj, const int *off, const int *key, int *cursor, int *cell_bead) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const int slot = atomicAdd(&cursor[key[g]], 1);
    cell_bead[off[traj[g]] + slot] = g;
}

// Warp per bead: the 27 neighbour cells' buckets are deduplicated across
// lanes, their candidates tested 32 at a time, the hits compacted in order
// of discovery into per-warp shared buffers, then written out at their rank
// (the number of smaller keys), i.e. in ascending j.
constexpr int kListWarps = 8;
constexpr int kWarpLJ = 256;   // per-warp LJ hit buffer; larger capacities use the tiled rebuild

__device__ __forceinline__ void warp_append(int *buf, int &n, int cap, bool hit, int key, bool &overflow) {
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (m) {
        const int lane = threadIdx.x & 31;
        const int pos = n + __popc(m & ((1u << lane) - 1u));
        if (hit) {
            if (pos < cap)
                buf[pos] = key;
            else
                overflow = true;
        }
        n += __popc(m);
    }
}

// writes buf[0..n) (distinct keys) to out[rank * stride] in ascending order
__device__ __forceinline__ void warp_rank_store(const int *buf, int n, int *out, int stride, int mode, int h0) {
    const int lane = threadIdx.x & 31;
    for (int k = lane; k < n; k += 32) {
        const int v = buf[k];
        int rank = 0;
        for (int m = 0; m < n; m++) rank += buf[m] < v;
        int val = v;
        if (mode == 1) {                      // longitudinal: sign from the harmonic partner side
            val = h0 < 0 ? v : -v;
        } else if (mode == 2) {               // lateral: key 2j + orientation
            const int j = v >> 1;
            const int code = j != 0 ? j : kZeroCode;
            val = (v & 1) ? code : -code;
        }
        out[(size_t)rank * stride] = val;
    }
}

__global__ void __launch_bounds__(kListWarps * 32) k_cell_lists(KParams P, DevBuffers B, const int2 *work,
                                                                const int *tbase, const int *tmask, const int *start,
                                                                const int *cnt, const int *cell_bead, float inv_cell) {
    __shared__ int s_lj[kListWarps][kWarpLJ];
    __shared__ int s_lo[kListWarps][kCellMaxLong];
    __shared__ int s_la[kListWarps][kCellMaxLat];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int nb = P.nb;
    const float4 *fr = B.frame_in;
    const int tb = tbase[traj];
    const uint32_t mask = (uint32_t)tmask[traj];
    const int capLJ = min(P.maxLJ, kWarpLJ);
    // the CTA's kTile beads, kTile / kListWarps per warp
    for (int g = w.y + wid; g < min(w.y + kTile, end); g += kListWarps) {
        const int flags = B.flags[g];
        const bool extra_i = (flags & kFlagExtra) != 0;
        const bool do_lj = P.lj_on && !extra_i;
        const bool do_pairs = P.is_assembly && !extra_i;
        if (!do_lj && !do_pairs) {
            if (lane == 0) {
                if (P.lj_on) B.ljc[g] = 0;
                if (P.is_assembly) {
                    B.lonc[g] = 0;
                    B.latc[g] = 0;
                }
            }
            continue;
        }
        const float4 pi = fr[g], ui = fr[nb + g], li1 = fr[2 * nb + g], li2 = fr[3 * nb + g];
        const int il = g - base;
        const int h0 = B.harm[g * P.maxH];
        const float rmon = h0 < 0 ? -2.0f : 2.0f;
        const int hpart = h0 < 0 ? -h0 : h0;
        const float3 wi = make_float3(ui.x * rmon, ui.y * rmon, ui.z * rmon);
        const int cx = cell_coord(pi.x, inv_cell), cy = cell_coord(pi.y, inv_cell), cz = cell_coord(pi.z, inv_cell);
        // lanes 0..26 own one neighbour cell each; duplicate buckets are dropped
        int bkt = -1;
        if (lane < 27) bkt = tb + (int)(cell_hash(cx + lane % 3 - 1, cy + (lane / 3) % 3 - 1, cz + lane / 9 - 1) & mask);
        bool dup = false;
        for (int k = 0; k < 27; k++) {
            const int other = __shfl_sync(0xffffffffu, bkt, k);
            dup |= (k < lane) && (other == bkt);
        }
        unsigned todo = __ballot_sync(0xffffffffu, lane < 27 && !dup);
        int nlj = 0, nlo = 0, nla = 0;
        bool overflow = false;
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int b = __shfl_sync(0xffffffffu, bkt, src);
            const int s0 = base + start[b], s1 = s0 + cnt[b];
            for (int s = s0; s < s1; s += 32) {
                const int sidx = s + lane;
                const bool have = sidx < s1;
                int jl = -1;
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                float cd = 3.0e38f;
                int jg = 0;
                if (have) {
                    jg = cell_bead[sidx];
                    jl = jg - base;
                    q = fr[jg];
                    cd = centre_dist(pi, q);
                }
                warp_append(s_lj[wid], nlj, capLJ, do_lj && have && jl != il && cd < P.ljcut, jl, overflow);
                bool lo_hit = false, la0 = false, la1 = false;
                if (do_pairs && have && cd < kPairReach && jl != hpart) {
                    const int fj = B.flags[jg];
                    if (((flags ^ fj) & kFlagBeta) != 0) {
                        const float4 uj = fr[nb + jg];
                        lo_hit = norm3_rn(site_delta(pi, q, wi, make_float3(-uj.x * rmon, -uj.y * rmon, -uj.z * rmon))) <
                                 2.5f;
                    }
                    if (jl != il) {
                        const float4 l1 = fr[2 * nb + jg], l2 = fr[3 * nb + jg];
                        la0 = norm3_rn(site_delta(pi, q, f3(li1), f3(l2))) < 2.5f;
                        la1 = norm3_rn(site_delta(pi, q, f3(li2), f3(l1))) < 2.5f;
                    }
                }
                warp_append(s_lo[wid], nlo, P.maxLong, lo_hit, jl, overflow);
                warp_append(s_la[wid], nla, P.maxLat, la0, 2 * jl, overflow);
                warp_append(s_la[wid], nla, P.maxLat, la1, 2 * jl + 1, overflow);
            }
        }
        __syncwarp();
        if (P.lj_on) {
            const int n = min(nlj, capLJ);
            warp_rank_store(s_lj[wid], n, B.lj + g, nb, 0, h0);
            if (lane == 0) B.ljc[g] = n;
            if (nlj > capLJ) overflow = true;
        }
        if (P.is_assembly) {
            const int n1 = min(nlo, P.maxLong), n2 = min(nla, P.maxLat);
            warp_rank_store(s_lo[wid], n1, B.lon + g, nb, 1, h0);
            warp_rank_store(s_la[wid], n2, B.lat + g, nb, 2, h0);
            if (lane == 0) {
                B.lonc[g] = n1;
                B.latc[g] = n2;
            }
        }
        if (__any_sync(0xffffffffu, overflow) && lane == 0) atomicOr(B.err, kErrOverflow);
        __syncwarp();
    }
}

inline int nblk(int n, int t) { return (n + t - 1) / t; }

}  // namespace

float bin_beads(const KParams &P, const DevBuffers &B, const CellBuffers &C, float reach, cudaStream_t s) {
    // cells slightly larger than the reach, so that rounding of x / edge can
    // never put two beads closer than the reach two cells apart
    const float inv = 1.0f / (reach * 1.001f + 1e-3f);
    cudaMemsetAsync(C.cnt, 0, sizeof(int) * C.nbuckets, s);
    k_cell_count<<<nblk(P.nb, 256), 256, 0, s>>>(P, B.frame_in, B.traj, C.tbase, C.tmask, inv, C.key, C.cnt);
    k_cell_scan<<<P.nt, 1024, 0, s>>>(C.tbase, C.cnt, C.start, C.cursor);
    k_cell_fill<<<nblk(P.nb, 256), 256, 0, s>>>(P.nb, B.traj, B.off, C.key, C.cursor, C.cell_bead);
    return inv;
}

void launch_rebuild_cells(const KParams &P, const DevBuffers &B, const CellBuffers &C, const int2 *work, int nwork,
                          cudaStream_t s) {
    const float reach = fmaxf(P.lj_on ? P.ljcut : 0.f, P.is_assembly ? kPairReach : 0.f);
    const float inv = bin_beads(P, B, C, reach, s);
    k_cell_lists<<<nwork, kListWarps * 32, 0, s>>>(P, B, work, C.tbase, C.tmask, C.start, C.cnt, C.cell_bead, inv);
}

}  // namespace mtg
