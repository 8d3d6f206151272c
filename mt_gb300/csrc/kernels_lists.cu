// kernels_lists.cu - neighbour-list rebuild (LJ list and assembly-mode
// longitudinal/lateral partner lists) for every trajectory of the batch.
//
// One CTA per (trajectory, chunk of kTile beads).  The trajectory's beads are
// streamed through shared memory in tiles of kTile in ascending index order,
// so every thread appends its partners in ascending j exactly as the
// reference's brute-force loops do (LJ_kernel, src/compute_cuda.cu:913-940;
// pairs_kernel, :527-674).  A tile is skipped when the bounding boxes of the
// chunk and the tile are further apart than the largest cutoff.
#include "mtg_internal.cuh"

namespace mtg {

__device__ __forceinline__ void block_box(float3 p, bool valid, float *sbox /*[6]*/, float *scratch /*[2*6*warps]*/) {
    float v[6] = {valid ? p.x : 3.0e38f, valid ? p.y : 3.0e38f, valid ? p.z : 3.0e38f,
                  valid ? p.x : -3.0e38f, valid ? p.y : -3.0e38f, valid ? p.z : -3.0e38f};
    for (int o = 16; o > 0; o >>= 1) {
        for (int c = 0; c < 3; c++) v[c] = fminf(v[c], __shfl_xor_sync(0xffffffffu, v[c], o));
        for (int c = 3; c < 6; c++) v[c] = fmaxf(v[c], __shfl_xor_sync(0xffffffffu, v[c], o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int c = 0; c < 6; c++) scratch[6 * wid + c] = v[c];
    __syncthreads();
    if (threadIdx.x < 6) {
        float r = scratch[threadIdx.x];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            const float q = scratch[6 * w + threadIdx.x];
            r = threadIdx.x < 3 ? fminf(r, q) : fmaxf(r, q);
        }
        sbox[threadIdx.x] = r;
    }
    __syncthreads();
}

__device__ __forceinline__ float box_gap(const float *a, const float *b) {
    const float gx = fmaxf(0.f, fmaxf(a[0] - b[3], b[0] - a[3]));
    const float gy = fmaxf(0.f, fmaxf(a[1] - b[4], b[1] - a[4]));
    const float gz = fmaxf(0.f, fmaxf(a[2] - b[5], b[2] - a[5]));
    return sqrtf(gx * gx + gy * gy + gz * gz);
}

__global__ void __launch_bounds__(kTile) k_rebuild(KParams P, DevBuffers B, const int2 *work) {
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int g = w.y + threadIdx.x;
    const bool valid = g < end;
    const int nb = P.nb;
    const float4 *fr = B.frame_in;

    __shared__ float4 s_pos[kTile], s_uz[kTile], s_l1[kTile], s_l2[kTile];
    __shared__ int s_flags[kTile];
    __shared__ float s_box_i[6], s_box_j[6], s_scr[6 * (kTile / 32)];

    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f), ui = pi, li1 = pi, li2 = pi;
    int flags = kFlagExtra, h0 = -1;
    if (valid) {
        pi = fr[g];
        ui = fr[nb + g];
        li1 = fr[2 * nb + g];
        li2 = fr[3 * nb + g];
        flags = B.flags[g];
        h0 = B.harm[g * P.maxH];
    }
    const ListSite I = list_site(P, pi, ui, li1, li2, flags, g - base, h0);
    const bool do_lj = valid && I.do_lj, do_pairs = valid && I.do_pairs;
    const float reach = fmaxf(P.lj_on ? P.ljcut : 0.f, P.is_assembly ? kPairPrefilter : 0.f);

    block_box(f3(pi), valid, s_box_i, s_scr);

    int nlj = 0, nlo = 0, nla = 0;
    bool overflow = false;
    for (int j0 = base; j0 < end; j0 += kTile) {
        const int jg = j0 + threadIdx.x;
        const bool jv = jg < end;
        float4 pj = make_float4(0.f, 0.f, 0.f, 0.f);
        if (jv) {
            pj = fr[jg];
            s_pos[threadIdx.x] = pj;
            if (P.is_assembly) {
                s_uz[threadIdx.x] = fr[nb + jg];
                s_l1[threadIdx.x] = fr[2 * nb + jg];
                s_l2[threadIdx.x] = fr[3 * nb + jg];
                s_flags[threadIdx.x] = B.flags[jg];
            }
        }
        block_box(f3(pj), jv, s_box_j, s_scr);  // includes the barrier for the tile stores
        const bool skip = box_gap(s_box_i, s_box_j) >= reach + 0.05f;  // margin over rounding
        if (!skip && (do_lj || do_pairs)) {
            const int n = min(kTile, end - j0);
            for (int t = 0; t < n; t++) {
                const int jl = j0 + t - base;
                const unsigned bits = list_bits(P, I, jl, s_pos[t], s_uz[t], s_l1[t], s_l2[t], s_flags[t]);
                list_append(P, B, g, I, bits, jl, nlj, nlo, nla, overflow);
            }
        }
        __syncthreads();
    }
    if (valid) {
        if (P.lj_on) B.ljc[g] = min(nlj, P.maxLJ);
        if (P.is_assembly) {
            B.lonc[g] = min(nlo, P.maxLong);
            B.latc[g] = min(nla, P.maxLat);
        }
        if (overflow) atomicOr(B.err, kErrOverflow);
    }
}

void launch_rebuild(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s) {
    k_rebuild<<<nwork, kTile, 0, s>>>(P, B, work);
}

}  // namespace mtg
