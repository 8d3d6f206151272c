// kernels_tea.cu - TEA hydrodynamics (Geyer & Winter 2009): the all-pairs
// epsilon / C_i pass, the FP64 epsilon -> beta reduction, and the all-pairs
// RPY mobility product fused with the position update.
//
// Both O(N^2) kernels run one CTA per (trajectory, chunk of kTeaChunk beads)
// and stream the trajectory through shared memory in tiles; each bead i is
// served by `tea_slices` threads that take interleaved j of every tile, so
// small batches still fill the GPU, and the partial sums meet in shared
// memory.  Every thread reads the tile by broadcast.  They are bound by the
// FP32 pipe (about 45 FLOP per ordered pair).
#include "mtg_internal.cuh"

namespace mtg {

// Normalised RPY block D_ij/D_ii (integrateTea_RPY, src/bdhitea_kernel.cu:38-58):
// T = cii I + crr u u^T with ra = r/a; ra > 2: crr = 0.75/ra (1 - 2/ra^2),
// cii = 0.75/ra (1 + 2/(3 ra^2)); otherwise crr = 3 ra/32, cii = 1 - 9 ra/32.
// RPY coefficients from the squared distance (branch-free): cii, and
// crr / r^2 so that T g = cii g + (crr / r^2) d (d . g) with d = r_j - r_i.
__device__ __forceinline__ void rpy_pair(float r2, float a, float inv_a, float &cii, float &crr_r2, float &rinv) {
    r2 = fmaxf(r2, 1e-6f);                  // coincident beads stay finite (masked by the caller)
    rinv = rsqrtf(r2);
    const float ra = r2 * rinv * inv_a;
    const float ira = a * rinv, ira2 = ira * ira;
    const float far_rr = 0.75f * ira * (1.0f - 2.0f * ira2);
    const float far_ii = 0.75f * ira * (1.0f + (2.0f / 3.0f) * ira2);
    const bool far = ra > 2.0f;
    crr_r2 = (far ? far_rr : (3.0f / 32.0f) * ra) * rinv * rinv;
    cii = far ? far_ii : 1.0f - (9.0f / 32.0f) * ra;
}

// Work split of the all-pairs TEA kernels: a CTA holds kTeaI beads i, each
// served by `slices` threads that cover interleaved j of every tile; the
// partial sums meet in shared memory.  slices = blockDim.x / kTeaI.
constexpr int kTeaI = kTeaChunk;
constexpr int kTeaTile = 256;

// integrateTea_epsilon_unlisted (src/bdhitea_kernel.cu:84-101): per bead i,
// sum over non-extra j != i of the row sums of squared entries (-> tea_ci)
// and of all nine entries (-> tea_eps).  With T = cii I + crr u u^T the row
// sums of squares are cii^2 + (2 cii + crr) crr u_c^2 and the sum of all
// entries is 3 cii + crr (u_x + u_y + u_z)^2.  Two beads i per thread, like
// k_tea_step; extra j enter the tile flagged and are skipped.
template <int SLICES>
__global__ void __launch_bounds__(kTeaI / 2 * SLICES) k_tea_eps(KParams P, DevBuffers B, const int2 *work,
                                                                 const int *gate, int run_if) {
    if (gate && *gate != run_if) return;
    constexpr int kHalf = kTeaI / 2;
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int il = threadIdx.x % kHalf, sl = threadIdx.x / kHalf;
    __shared__ float4 s_pos[kTeaTile];
    __shared__ float4 s_red[kTeaI * SLICES];
    int gi[2];
    bool act[2];
    float4 pi[2];
    float sx[2] = {0.f, 0.f}, sy[2] = {0.f, 0.f}, sz[2] = {0.f, 0.f}, sw[2] = {0.f, 0.f};
#pragma unroll
    for (int h = 0; h < 2; h++) {
        gi[h] = w.y + il + h * kHalf;
        act[h] = false;
        pi[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gi[h] < end) {
            pi[h] = B.frame_in[gi[h]];
            act[h] = (B.flags[gi[h]] & kFlagExtra) == 0;
        }
    }
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    const float c075a = 0.75f * a, c05a3 = 0.5f * a * a * a, c15a3 = 1.5f * a * a * a, four_a2 = 4.0f * a * a;
    const bool any_act = act[0] || act[1];
    for (int j0 = base; j0 < end; j0 += kTeaTile) {
        for (int k = threadIdx.x; k < kTeaTile; k += kHalf * SLICES) {
            const int jg = j0 + k;
            if (jg < end) {
                float4 q = B.frame_in[jg];
                q.w = (B.flags[jg] & kFlagExtra) ? 1.0f : 0.0f;
                s_pos[k] = q;
            }
        }
        __syncthreads();
        if (any_act) {
            const int n = min(kTeaTile, end - j0);
#pragma unroll 2
            for (int t = sl; t < n; t += SLICES) {
                const float4 q = s_pos[t];
                if (q.w != 0.0f) continue;   // extra j
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    if (j0 + t == gi[h]) continue;
                    const float dx = q.x - pi[h].x, dy = q.y - pi[h].y, dz = q.z - pi[h].z;
                    const float r2 = fmaxf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), 1e-6f);
                    const float rinv = rsqrtf(r2);
                    const float qq = rinv * rinv;
                    float cii = rinv * fmaf(c05a3, qq, c075a);
                    float crr = rinv * fmaf(-c15a3, qq, c075a);
                    if (r2 <= four_a2) {
                        const float ra = r2 * rinv * inv_a;
                        cii = 1.0f - (9.0f / 32.0f) * ra;
                        crr = (3.0f / 32.0f) * ra;
                    }
                    const float A = cii * cii, Bc = fmaf(2.0f, cii, crr) * crr * qq;
                    sx[h] = fmaf(Bc, dx * dx, sx[h] + A);
                    sy[h] = fmaf(Bc, dy * dy, sy[h] + A);
                    sz[h] = fmaf(Bc, dz * dz, sz[h] + A);
                    const float us = dx + dy + dz;
                    sw[h] = fmaf(crr * qq, us * us, fmaf(3.0f, cii, sw[h]));
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int h = 0; h < 2; h++) s_red[(sl * 2 + h) * kHalf + il] = make_float4(sx[h], sy[h], sz[h], sw[h]);
    __syncthreads();
    if (sl != 0) return;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        if (gi[h] >= end) continue;
        float4 acc = s_red[h * kHalf + il];
        for (int k = 1; k < SLICES; k++) {
            const float4 v = s_red[(k * 2 + h) * kHalf + il];
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
        }
        if (!act[h]) acc = make_float4(0.f, 0.f, 0.f, 0.f);
        B.tea_ci[gi[h]] = make_float4(acc.x, acc.y, acc.z, 0.f);
        B.tea_eps[gi[h]] = acc.w;
    }
}

// updateTea's reduction (src/bdhitea.cu:75-116), in FP64 on the device: one
// CTA per trajectory sums the bead epsilons and counts the non-extra beads N',
// eps = sum / (3N'(3N'-3)), clamped to 1; a = (3N'-1) eps^2 - (3N'-2) eps;
// beta = (1 - sqrt(1 - a)) / a, or 0.5 when |a| < 1e-7.  The reference's
// exits become the kErrTeaEps bit.
__global__ void __launch_bounds__(256) k_tea_beta(KParams P, DevBuffers B, int capricious, float epsmax,
                                                  const int *gate, int run_if) {
    if (gate && *gate != run_if) return;
    const int t = blockIdx.x;
    const int base = B.off[t], end = B.off[t + 1];
    double s = 0.0;
    int cnt = 0;
    for (int g = base + threadIdx.x; g < end; g += blockDim.x) {
        s += (double)B.tea_eps[g];
        cnt += (B.flags[g] & kFlagExtra) ? 0 : 1;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    }
    __shared__ double ss[8];
    __shared__ int sc[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        ss[wid] = s;
        sc[wid] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double e = 0.0;
        int n = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            e += ss[k];
            n += sc[k];
        }
        e /= 3.0 * n * (3.0 * n - 3.0);
        int bad = 0;
        if (e > 1.0) {
            if (capricious) bad = 1;
            e = 1.0;
        }
        if (e > (double)epsmax) bad = 1;
        const double a = (3.0 * n - 1.0) * e * e - (3.0 * n - 2.0) * e;
        float beta;
        if (fabs(a) < 1e-7) {
            beta = 0.5f;
            if (capricious && P.tea_a > 0.0f) bad = 1;
        } else {
            beta = (float)((1.0 - sqrt(1.0 - a)) / a);
        }
        B.tea_beta[t] = beta;
        B.tea_eps_t[t] = e;
        if (bad) atomicOr(B.err, kErrTeaEps);
    }
}

// One pair's contribution T_ij g to f, with d = r_j - r_i and r2 = |d|^2 > 0.
// Far field (r > 2a, the common case): cii = 0.75 a/r (1 + 2a^2/(3r^2)),
// crr/r^2 = 0.75 a/r^3 (1 - 2a^2/r^2), written in q = 1/r^2; the overlap
// branch (r <= 2a) is rare and taken under a warp-divergent branch.
__device__ __forceinline__ void tea_pair(float dx, float dy, float dz, float gx, float gy, float gz, float a,
                                         float inv_a, float c075a, float c05a3, float c15a3, float four_a2,
                                         float &fx, float &fy, float &fz) {
    const float r2 = fmaxf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), 1e-6f);
    const float rinv = rsqrtf(r2);
    const float q = rinv * rinv;
    float cii = rinv * fmaf(c05a3, q, c075a);
    float crr_r2 = rinv * q * fmaf(-c15a3, q, c075a);
    if (r2 <= four_a2) {
        const float ra = r2 * rinv * inv_a;
        cii = 1.0f - (9.0f / 32.0f) * ra;
        crr_r2 = (3.0f / 32.0f) * ra * q;
    }
    const float s = crr_r2 * fmaf(dx, gx, fmaf(dy, gy, dz * gz));
    fx = fmaf(cii, gx, fmaf(s, dx, fx));
    fy = fmaf(cii, gy, fmaf(s, dy, fy));
    fz = fmaf(cii, gz, fmaf(s, dz, fz));
}

// Two pairs at once (beads i0, i1 against one j) in packed FP32x2
// arithmetic (each lane an IEEE single-precision fma/add/mul, as the scalar
// path): the same formula as tea_pair.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ void tea_pair2(float2 dx, float2 dy, float2 dz, float2 gx, float2 gy, float2 gz, float a,
                                          float inv_a, float2 c075a, float2 c05a3, float2 nc15a3, float four_a2,
                                          float2 &fx, float2 &fy, float2 &fz) {
    float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    r2.x = fmaxf(r2.x, 1e-6f);
    r2.y = fmaxf(r2.y, 1e-6f);
    const float2 rinv = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
    const float2 q = __fmul2_rn(rinv, rinv);
    float2 cii = __fmul2_rn(rinv, __ffma2_rn(c05a3, q, c075a));
    float2 crr_r2 = __fmul2_rn(__fmul2_rn(rinv, q), __ffma2_rn(nc15a3, q, c075a));
    if (r2.x <= four_a2) {
        const float ra = r2.x * rinv.x * inv_a;
        cii.x = 1.0f - (9.0f / 32.0f) * ra;
        crr_r2.x = (3.0f / 32.0f) * ra * q.x;
    }
    if (r2.y <= four_a2) {
        const float ra = r2.y * rinv.y * inv_a;
        cii.y = 1.0f - (9.0f / 32.0f) * ra;
        crr_r2.y = (3.0f / 32.0f) * ra * q.y;
    }
    const float2 s = __fmul2_rn(crr_r2, __ffma2_rn(dx, gx, __ffma2_rn(dy, gy, __fmul2_rn(dz, gz))));
    fx = __ffma2_rn(cii, gx, __ffma2_rn(s, dx, fx));
    fy = __ffma2_rn(cii, gy, __ffma2_rn(s, dy, fy));
    fz = __ffma2_rn(cii, gz, __ffma2_rn(s, dz, fz));
}

// integrateTea_kernel_unlisted + integrateTea_force (src/bdhitea_kernel.cu:104-213):
// f_i = F_i + C_i o R_i + sum_{j != i, non-extra} T_ij (F_j + beta C_i o R_j),
// x_i += dt/gammaR f_i; angles by Euler-Maruyama from stream i + nb, which is
// drawn for every bead.  Reads the current frame, writes the next one.
// Each thread serves two beads i (il and il + kTeaI/2) against the tile's j,
// so every shared-memory load feeds two pairs; extra beads enter the tile
// with zero F and R and contribute nothing.
template <int SLICES, bool FEFF>
__global__ void __launch_bounds__(kTeaI / 2 * SLICES) k_tea_step(KParams P, DevBuffers B, const int2 *work,
                                                                  float4 *feff, const int *gate) {
    if (FEFF && gate && *gate != 0) return;
    constexpr int kHalf = kTeaI / 2;
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int il = threadIdx.x % kHalf, sl = threadIdx.x / kHalf;
    const int nb = P.nb;
    __shared__ float4 s_pos[kTeaTile], s_f[kTeaTile], s_r[kTeaTile];
    __shared__ float4 s_red[kTeaI * SLICES];

    int gi[2];
    bool act[2];
    float4 pi[2];
    float fx[2], fy[2], fz[2], cbx[2], cby[2], cbz[2];
    const float beta = B.tea_beta[traj], b2 = beta * beta;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        gi[h] = w.y + il + h * kHalf;
        pi[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        fx[h] = fy[h] = fz[h] = 0.f;
        cbx[h] = cby[h] = cbz[h] = 0.f;
        act[h] = false;
        if (gi[h] < end) {
            pi[h] = B.frame_in[gi[h]];
            act[h] = (B.flags[gi[h]] & kFlagExtra) == 0;
            const float4 ci = B.tea_ci[gi[h]];
            const float cx = 1.0f / sqrtf(1.0f + b2 * ci.x);
            const float cy = 1.0f / sqrtf(1.0f + b2 * ci.y);
            const float cz = 1.0f / sqrtf(1.0f + b2 * ci.z);
            if (sl == 0) {
                const float4 Fi = B.force[gi[h]], Ri = B.tea_r[gi[h]];
                fx[h] = Fi.x + Ri.x * cx;
                fy[h] = Fi.y + Ri.y * cy;
                fz[h] = Fi.z + Ri.z * cz;
            }
            cbx[h] = cx * beta;
            cby[h] = cy * beta;
            cbz[h] = cz * beta;
        }
    }
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    const float c075a = 0.75f * a, c05a3 = 0.5f * a * a * a, c15a3 = 1.5f * a * a * a, four_a2 = 4.0f * a * a;
    const bool any_act = act[0] || act[1];
    for (int j0 = base; j0 < end; j0 += kTeaTile) {
        for (int k = threadIdx.x; k < kTeaTile; k += kHalf * SLICES) {
            const int jg = j0 + k;
            if (jg < end) {
                s_pos[k] = B.frame_in[jg];
                const bool ex = (B.flags[jg] & kFlagExtra) != 0;
                s_f[k] = ex ? make_float4(0.f, 0.f, 0.f, 0.f) : B.force[jg];
                s_r[k] = ex ? make_float4(0.f, 0.f, 0.f, 0.f) : B.tea_r[jg];
            }
        }
        __syncthreads();
        if (any_act) {
            const int n = min(kTeaTile, end - j0);
            // the CTA's own beads (the self pairs) can only sit in this tile range
            const bool self_tile = (w.y < j0 + n) && (w.y + kTeaI > j0);
            if (!self_tile) {
                // packed over the two beads: lane x = bead il, lane y = bead il + 32
                const float2 nx = make_float2(-pi[0].x, -pi[1].x), ny = make_float2(-pi[0].y, -pi[1].y),
                             nz = make_float2(-pi[0].z, -pi[1].z);
                const float2 cb2x = make_float2(cbx[0], cbx[1]), cb2y = make_float2(cby[0], cby[1]),
                             cb2z = make_float2(cbz[0], cbz[1]);
                float2 ax = make_float2(fx[0], fx[1]), ay = make_float2(fy[0], fy[1]), az = make_float2(fz[0], fz[1]);
                const float2 v075a = f2(c075a), v05a3 = f2(c05a3), vn15a3 = f2(-c15a3);
#pragma unroll 4
                for (int t = sl; t < n; t += SLICES) {
                    const float4 q = s_pos[t], Fj = s_f[t], Rj = s_r[t];
                    tea_pair2(__fadd2_rn(f2(q.x), nx), __fadd2_rn(f2(q.y), ny), __fadd2_rn(f2(q.z), nz),
                              __ffma2_rn(f2(Rj.x), cb2x, f2(Fj.x)), __ffma2_rn(f2(Rj.y), cb2y, f2(Fj.y)),
                              __ffma2_rn(f2(Rj.z), cb2z, f2(Fj.z)), a, inv_a, v075a, v05a3, vn15a3, four_a2, ax, ay,
                              az);
                }
                fx[0] = ax.x;
                fx[1] = ax.y;
                fy[0] = ay.x;
                fy[1] = ay.y;
                fz[0] = az.x;
                fz[1] = az.y;
            } else {
                for (int t = sl; t < n; t += SLICES) {
                    const float4 q = s_pos[t], Fj = s_f[t], Rj = s_r[t];
#pragma unroll
                    for (int h = 0; h < 2; h++)
                        if (j0 + t != gi[h])
                            tea_pair(q.x - pi[h].x, q.y - pi[h].y, q.z - pi[h].z, fmaf(Rj.x, cbx[h], Fj.x),
                                     fmaf(Rj.y, cby[h], Fj.y), fmaf(Rj.z, cbz[h], Fj.z), a, inv_a, c075a, c05a3,
                                     c15a3, four_a2, fx[h], fy[h], fz[h]);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int h = 0; h < 2; h++) s_red[(sl * 2 + h) * kHalf + il] = make_float4(fx[h], fy[h], fz[h], 0.f);
    __syncthreads();
    if (sl != 0) return;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int g = gi[h];
        if (g >= end) continue;
        float sx = fx[h], sy = fy[h], sz = fz[h];
        for (int k = 1; k < SLICES; k++) {
            const float4 v = s_red[(k * 2 + h) * kHalf + il];
            sx += v.x;
            sy += v.y;
            sz += v.z;
        }
        if (FEFF) {
            feff[g] = make_float4(sx, sy, sz, 0.f);
            continue;
        }
        const int flags = B.flags[g];
        Frame Fr;
        Fr.p0 = pi[h];
        Fr.p1 = B.frame_in[nb + g];
        Fr.p2 = B.frame_in[2 * nb + g];
        Fr.p3 = B.frame_in[3 * nb + g];
        uint4 s2 = B.seeds[nb + g];
        const float4 ga = gauss4(s2);
        B.seeds[nb + g] = s2;
        if (!(flags & (kFlagExtra | kFlagFixed))) {
            const float4 fa = B.force[nb + g];  // (ffi, ftheta, fpsi)
            const float x = Fr.p0.x + P.kr * sx, y = Fr.p0.y + P.kr * sy, z = Fr.p0.z + P.kr * sz;
            const float fi = Fr.p0.w + (P.kfi * fa.x + P.nfi * ga.x);
            const float psi = Fr.p1.w + (P.kfi * fa.z + P.nfi * ga.y);
            const float th = Fr.p2.w + (P.kth * fa.y + P.varTheta * ga.z);
            Fr = make_frame(P, x, y, z, fi, th, psi);
        }
        store_frame(B.frame_out, nb, g, Fr);
    }
}

void launch_tea_eps_gated(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, const int *gate,
                          int run_if, cudaStream_t s) {
    const int t = kTeaI / 2 * P.tea_slices;
    switch (P.tea_slices) {
        case 1: k_tea_eps<1><<<nwork, t, 0, s>>>(P, B, work, gate, run_if); break;
        case 2: k_tea_eps<2><<<nwork, t, 0, s>>>(P, B, work, gate, run_if); break;
        case 4: k_tea_eps<4><<<nwork, t, 0, s>>>(P, B, work, gate, run_if); break;
        default: k_tea_eps<8><<<nwork, t, 0, s>>>(P, B, work, gate, run_if); break;
    }
}
void launch_tea_eps(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s) {
    launch_tea_eps_gated(P, B, work, nwork, nullptr, 0, s);
}
void launch_tea_beta_gated(const KParams &P, const DevBuffers &B, int capricious, float epsmax, const int *gate,
                           int run_if, cudaStream_t s) {
    k_tea_beta<<<P.nt, 256, 0, s>>>(P, B, capricious, epsmax, gate, run_if);
}
void launch_tea_beta(const KParams &P, const DevBuffers &B, int capricious, float epsmax, cudaStream_t s) {
    launch_tea_beta_gated(P, B, capricious, epsmax, nullptr, 0, s);
}
template <bool FEFF>
static void tea_step_dispatch(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, float4 *feff,
                              const int *gate, cudaStream_t s) {
    const int t = kTeaI / 2 * P.tea_slices;
    switch (P.tea_slices) {
        case 1: k_tea_step<1, FEFF><<<nwork, t, 0, s>>>(P, B, work, feff, gate); break;
        case 2: k_tea_step<2, FEFF><<<nwork, t, 0, s>>>(P, B, work, feff, gate); break;
        case 4: k_tea_step<4, FEFF><<<nwork, t, 0, s>>>(P, B, work, feff, gate); break;
        default: k_tea_step<8, FEFF><<<nwork, t, 0, s>>>(P, B, work, feff, gate); break;
    }
}
void launch_tea_step(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s) {
    tea_step_dispatch<false>(P, B, work, nwork, nullptr, nullptr, s);
}
void launch_tea_feff(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, float4 *feff,
                     const int *gate, cudaStream_t s) {
    tea_step_dispatch<true>(P, B, work, nwork, feff, gate, s);
}

}  // namespace mtg
