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
//   4. k_cell_lists : per bead, candidates from the 27 cells' buckets (each
//      bucket visited once) read from a bucket-ordered copy of the
//      positions, the reference's list tests, then an insertion sort so each
//      list is in ascending j (orientation 0 before 1 for the lateral list),
//      exactly the order of the reference's j loops
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
    for (int i = lo; i < hi; i++) {
        start[b0 + i] = run;
        cursor[b0 + i] = run;
        run += cnt[b0 + i];
    }
}

// Bucket-ordered bead lists; positions are relative to the trajectory's
// first bead, so slots of trajectory t start at off[t].
__global__ void k_cell_fill(int nb, const int *traj, const int *off, const int *key, const int *flags, int *cursor,
                            int *cell_bead, const float4 *pos, float4 *cell_pos) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const int slot = off[traj[g]] + atomicAdd(&cursor[key[g]], 1);
    cell_bead[slot] = g;
    float4 p = pos[g];
    // bucket-ordered copy of the positions, bead index (and the extra flag) in w
    p.w = __int_as_float(g | ((flags[g] & kFlagExtra) ? kCellExtraBit : 0));
    cell_pos[slot] = p;
}

// Ascending bead index within every bucket (the atomic fill leaves them in
// arrival order), so that sums over a bucket are reproducible.  Grid
// (trajectory, bucket chunk), one thread per bucket; buckets hold a few beads.
__global__ void k_cell_sort(const int *off, const int *tbase, const int *tmask, const int *start, const int *cnt,
                            int *cell_bead, float4 *cell_pos) {
    const int t = blockIdx.x, base = off[t], tb = tbase[t], nbk = tmask[t] + 1;
    const int b = blockIdx.y * blockDim.x + threadIdx.x;
    if (b >= nbk) return;
    const int n = cnt[tb + b];
    if (n < 2) return;
    int *cb = cell_bead + base + start[tb + b];
    float4 *cp = cell_pos + base + start[tb + b];
    for (int i = 1; i < n; i++) {
        const int v = cb[i];
        const float4 pv = cp[i];
        int j = i - 1;
        while (j >= 0 && cb[j] > v) {
            cb[j + 1] = cb[j];
            cp[j + 1] = cp[j];
            j--;
        }
        cb[j + 1] = v;
        cp[j + 1] = pv;
    }
}

__device__ __forceinline__ void isort(int *a, int n) {
    for (int i = 1; i < n; i++) {
        const int v = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > v) {
            a[j + 1] = a[j];
            j--;
        }
        a[j + 1] = v;
    }
}

// In-place insertion sort of a k-major list (rare path: > kLocalLJ entries).
__device__ void isort_strided(int *a, int n, int stride) {
    for (int i = 1; i < n; i++) {
        const int v = a[(size_t)i * stride];
        int j = i - 1;
        while (j >= 0 && a[(size_t)j * stride] > v) {
            a[(size_t)(j + 1) * stride] = a[(size_t)j * stride];
            j--;
        }
        a[(size_t)(j + 1) * stride] = v;
    }
}

constexpr int kLocalLJ = 16;   // LJ hits sorted in shared memory; more are sorted in place

// Insertion sort of one thread's column of a [rows][kTile] shared array.
__device__ __forceinline__ void isort_col(int (*a)[kTile], int n, int t) {
    for (int i = 1; i < n; i++) {
        const int v = a[i][t];
        int j = i - 1;
        while (j >= 0 && a[j][t] > v) {
            a[j + 1][t] = a[j][t];
            j--;
        }
        a[j + 1][t] = v;
    }
}

// Thread per bead: candidates are read from the bucket-ordered position copy
// (one contiguous 16 B load each); the rare assembly candidates (< 6.6 nm)
// also read the neighbour's site planes.
template <bool PAIRS>
__global__ void __launch_bounds__(kTile, 6) k_cell_lists(KParams P, DevBuffers B, const int2 *work, const int *tbase,
                                                         const int *tmask, const int *start, const int *cnt,
                                                         const float4 *cell_pos, float inv_cell) {
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int g = w.y + threadIdx.x;
    if (g >= end) return;
    const int nb = P.nb;
    const float4 *fr = B.frame_in;
    const int flags = B.flags[g];
    const bool extra_i = (flags & kFlagExtra) != 0;
    const bool do_lj = P.lj_on && !extra_i;
    const bool do_pairs = PAIRS && P.is_assembly && !extra_i;
    if (!do_lj && !do_pairs) {
        if (P.lj_on) B.ljc[g] = 0;
        if (PAIRS && P.is_assembly) {
            B.lonc[g] = 0;
            B.latc[g] = 0;
        }
        return;
    }
    const float4 pi = fr[g];
    const int il = g - base;
    const int h0 = B.harm[g * P.maxH];
    const int hpart = h0 < 0 ? -h0 : h0;
    const int cx = cell_coord(pi.x, inv_cell), cy = cell_coord(pi.y, inv_cell), cz = cell_coord(pi.z, inv_cell);
    const int tb = tbase[traj];
    const uint32_t mask = (uint32_t)tmask[traj];

    // this thread's LJ hits: a column of shared memory (its own bank), so the
    // buffer and its sort never leave the SM
    __shared__ int s_lj[kLocalLJ][kTile];
    int lo_buf[kCellMaxLong], la_buf[kCellMaxLat];
    int nlj = 0, nlo = 0, nla = 0;
    bool overflow = false;
    // the ranges of the 27 cells' buckets, all requested at once and kept in
    // shared memory for the rolled cell loop, and a mask of the cells whose
    // bucket an earlier cell already has
    __shared__ int s_st[27][kTile], s_ct[27][kTile];
    uint32_t dup = 0;
    {
        int bk[27];
#pragma unroll
        for (int c = 0; c < 27; c++)
            bk[c] = tb + (int)(cell_hash(cx + c % 3 - 1, cy + (c / 3) % 3 - 1, cz + c / 9 - 1) & mask);
#pragma unroll
        for (int c = 0; c < 27; c++) {
            s_st[c][threadIdx.x] = start[bk[c]];
            s_ct[c][threadIdx.x] = cnt[bk[c]];
        }
#pragma unroll
        for (int c = 1; c < 27; c++) {
            bool seen = false;
#pragma unroll
            for (int v = 0; v < c; v++) seen |= (bk[v] == bk[c]);
            dup |= (seen ? 1u : 0u) << c;
        }
    }
    // drop the buckets an earlier cell already has, then walk the remaining
    // candidates in cell order four at a time across cell boundaries, so a
    // sparse neighbourhood still has four loads in flight
    for (int c = 0; c < 27; c++)
        if ((dup >> c) & 1u) s_ct[c][threadIdx.x] = 0;
    int c = 0, off = 0;
    while (c < 27 && s_ct[c][threadIdx.x] == 0) c++;
    while (c < 27) {
        int sl[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            sl[u] = -1;
            if (c < 27) {
                sl[u] = base + s_st[c][threadIdx.x] + off;
                if (++off == s_ct[c][threadIdx.x]) {
                    off = 0;
                    do {
                        c++;
                    } while (c < 27 && s_ct[c][threadIdx.x] == 0);
                }
            }
        }
        float4 qq[4];   // four candidates in flight
#pragma unroll
        for (int u = 0; u < 4; u++) qq[u] = sl[u] >= 0 ? cell_pos[sl[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (sl[u] < 0) break;
            const float4 q = qq[u];
            const int jg = __float_as_int(q.w) & kCellIndexMask;
            const int jl = jg - base;
            const float cd = centre_dist(pi, q);
            if (do_lj && jl != il && cd < P.ljcut) {
                if (nlj >= P.maxLJ) {
                    overflow = true;
                } else if (nlj < kLocalLJ) {
                    s_lj[nlj][threadIdx.x] = jl;
                } else {
                    if (nlj == kLocalLJ)  // spill the local part first
                        for (int k = 0; k < kLocalLJ; k++) B.lj[k * nb + g] = s_lj[k][threadIdx.x];
                    B.lj[nlj * nb + g] = jl;
                }
                nlj++;
            }
            if (do_pairs && cd < kPairReach && jl != hpart) {
                const float4 pj = fr[jg];   // the exact state (q carries the index in w)
                const float rmon = h0 < 0 ? -2.0f : 2.0f;
                const int fj = B.flags[jg];
                if (((flags ^ fj) & kFlagBeta) != 0) {
                    const float4 ui = fr[nb + g], uj = fr[nb + jg];
                    const float3 wi = make_float3(ui.x * rmon, ui.y * rmon, ui.z * rmon);
                    if (norm3_rn(site_delta(pi, pj, wi, make_float3(-uj.x * rmon, -uj.y * rmon, -uj.z * rmon))) <
                        2.5f) {
                        if (nlo < P.maxLong)
                            lo_buf[nlo] = jl;
                        else
                            overflow = true;
                        nlo++;
                    }
                }
                if (jl != il) {
                    const float4 li1 = fr[2 * nb + g], li2 = fr[3 * nb + g];
                    const float4 l1 = fr[2 * nb + jg], l2 = fr[3 * nb + jg];
                    if (norm3_rn(site_delta(pi, pj, f3(li1), f3(l2))) < 2.5f) {
                        if (nla < P.maxLat)
                            la_buf[nla] = 2 * jl;       // orientation 0 -> -j
                        else
                            overflow = true;
                        nla++;
                    }
                    if (norm3_rn(site_delta(pi, pj, f3(li2), f3(l1))) < 2.5f) {
                        if (nla < P.maxLat)
                            la_buf[nla] = 2 * jl + 1;   // orientation 1 -> +j
                        else
                            overflow = true;
                        nla++;
                    }
                }
            }
        }
    }
    if (P.lj_on) {
        const int n = min(nlj, P.maxLJ);
        if (n <= kLocalLJ) {
            isort_col(s_lj, n, threadIdx.x);
            for (int k = 0; k < n; k++) B.lj[k * nb + g] = s_lj[k][threadIdx.x];
        } else {
            isort_strided(B.lj + g, n, nb);
        }
        B.ljc[g] = n;
    }
    if (PAIRS && P.is_assembly) {
        const int n1 = min(nlo, P.maxLong), n2 = min(nla, P.maxLat);
        isort(lo_buf, n1);
        isort(la_buf, n2);
        for (int k = 0; k < n1; k++) B.lon[k * nb + g] = h0 < 0 ? lo_buf[k] : -lo_buf[k];
        for (int k = 0; k < n2; k++) {
            const int j = la_buf[k] >> 1;
            const int code = j != 0 ? j : kZeroCode;
            B.lat[k * nb + g] = (la_buf[k] & 1) ? code : -code;
        }
        B.lonc[g] = n1;
        B.latc[g] = n2;
    }
    if (overflow) atomicOr(B.err, kErrOverflow);
}

// Longitudinal and lateral lists (pairs_kernel, src/compute_cuda.cu:527-674)
// from the bead's LJ list: every assembly candidate (centre distance below
// kPairReach) is in the LJ list when the LJ cutoff is longer, and the LJ list
// is in ascending j, so the lists come out in the reference's order without a
// sort.  Runs after k_cell_lists<false>.
__global__ void __launch_bounds__(kTile) k_pairs_from_lj(KParams P, DevBuffers B) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.nb) return;
    const int nb = P.nb;
    const int flags = B.flags[g];
    if (flags & kFlagExtra) {
        B.lonc[g] = 0;
        B.latc[g] = 0;
        return;
    }
    const float4 *fr = B.frame_in;
    const int base = B.off[B.traj[g]], il = g - base;
    const float4 pi = fr[g], ui = fr[nb + g], li1 = fr[2 * nb + g], li2 = fr[3 * nb + g];
    const int h0 = B.harm[g * P.maxH];
    const int hpart = h0 < 0 ? -h0 : h0;
    const float rmon = h0 < 0 ? -2.0f : 2.0f;
    const float3 wi = make_float3(ui.x * rmon, ui.y * rmon, ui.z * rmon);
    const int n = min(B.ljc[g], P.maxLJ);
    int nlo = 0, nla = 0;
    bool overflow = false;
    for (int k0 = 0; k0 < n; k0 += 4) {
        int jj[4];
        float4 q[4];
#pragma unroll
        for (int u = 0; u < 4; u++) jj[u] = k0 + u < n ? B.lj[(k0 + u) * nb + g] : -1;
#pragma unroll
        for (int u = 0; u < 4; u++) q[u] = jj[u] >= 0 ? fr[base + jj[u]] : pi;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int jl = jj[u];
            if (jl < 0 || jl == hpart || !(centre_dist(pi, q[u]) < kPairReach)) continue;
            const int jg = base + jl;
            const float4 pj = q[u];
            const int fj = B.flags[jg];
            if (((flags ^ fj) & kFlagBeta) != 0) {
                const float4 uj = fr[nb + jg];
                if (norm3_rn(site_delta(pi, pj, wi, make_float3(-uj.x * rmon, -uj.y * rmon, -uj.z * rmon))) < 2.5f) {
                    if (nlo < P.maxLong)
                        B.lon[nlo * nb + g] = h0 < 0 ? jl : -jl;
                    else
                        overflow = true;
                    nlo++;
                }
            }
            if (jl != il) {
                const float4 l1 = fr[2 * nb + jg], l2 = fr[3 * nb + jg];
                const int code = jl != 0 ? jl : kZeroCode;
                if (norm3_rn(site_delta(pi, pj, f3(li1), f3(l2))) < 2.5f) {
                    if (nla < P.maxLat)
                        B.lat[nla * nb + g] = -code;   // orientation 0 -> -j
                    else
                        overflow = true;
                    nla++;
                }
                if (norm3_rn(site_delta(pi, pj, f3(li2), f3(l1))) < 2.5f) {
                    if (nla < P.maxLat)
                        B.lat[nla * nb + g] = code;    // orientation 1 -> +j
                    else
                        overflow = true;
                    nla++;
                }
            }
        }
    }
    B.lonc[g] = min(nlo, P.maxLong);
    B.latc[g] = min(nla, P.maxLat);
    if (overflow) atomicOr(B.err, kErrOverflow);
}

inline int nblk(int n, int t) { return (n + t - 1) / t; }

}  // namespace

float bin_beads(const KParams &P, const DevBuffers &B, const CellBuffers &C, float reach, bool ordered,
                cudaStream_t s) {
    // cells slightly larger than the reach, so that rounding of x / edge can
    // never put two beads closer than the reach two cells apart
    const float inv = 1.0f / (reach * 1.001f + 1e-3f);
    cudaMemsetAsync(C.cnt, 0, sizeof(int) * C.nbuckets, s);
    k_cell_count<<<nblk(P.nb, 256), 256, 0, s>>>(P, B.frame_in, B.traj, C.tbase, C.tmask, inv, C.key, C.cnt);
    k_cell_scan<<<P.nt, 1024, 0, s>>>(C.tbase, C.cnt, C.start, C.cursor);
    k_cell_fill<<<nblk(P.nb, 256), 256, 0, s>>>(P.nb, B.traj, B.off, C.key, B.flags, C.cursor, C.cell_bead,
                                                 B.frame_in, C.cell_pos);
    if (ordered)
        k_cell_sort<<<dim3(P.nt, (C.max_buckets + 127) / 128), 128, 0, s>>>(B.off, C.tbase, C.tmask, C.start, C.cnt,
                                                                            C.cell_bead, C.cell_pos);
    return inv;
}

void launch_rebuild_cells(const KParams &P, const DevBuffers &B, const CellBuffers &C, const int2 *work, int nwork,
                          cudaStream_t s) {
    const float reach = fmaxf(P.lj_on ? P.ljcut : 0.f, P.is_assembly ? kPairReach : 0.f);
    const float inv = bin_beads(P, B, C, reach, false, s);   // the lists are sorted afterwards
    if (P.is_assembly && P.lj_on && P.ljcut >= kPairReach) {
        // LJ lists from the cells, then the assembly lists from the LJ lists
        k_cell_lists<false><<<nwork, kTile, 0, s>>>(P, B, work, C.tbase, C.tmask, C.start, C.cnt, C.cell_pos, inv);
        k_pairs_from_lj<<<nblk(P.nb, kTile), kTile, 0, s>>>(P, B);
    } else {
        k_cell_lists<true><<<nwork, kTile, 0, s>>>(P, B, work, C.tbase, C.tmask, C.start, C.cnt, C.cell_pos, inv);
    }
}

}  // namespace mtg
