// kernels_tea.cu - TEA hydrodynamics (Geyer & Winter 2009): the all-pairs
// epsilon / C_i pass, the FP64 epsilon -> beta reduction, and the all-pairs
// RPY mobility product fused with the position update.
//
// Both O(N^2) kernels run one CTA per (trajectory, chunk of kTeaChunk beads)
// and stream the trajectory through shared memory in tiles; each bead i is
// served by `tea_slices` threads that take interleaved j of every tile, so
// small batches still fill the GPU, and the partial sums meet in shared
// memory.  Every thread reads the tile by broadcast, two beads j per load,
// and works on them in packed FP32x2 arithmetic.  They are bound by the FP32
// pipe (about 45 FLOP per ordered pair).
#include "mtg_internal.cuh"

namespace mtg {

// 1/sqrt(x) as the single hardware approximation instruction (a few ulp);
// pair distances are never subnormal, so the flush-to-zero form gives the
// same value for them without a subnormal fix-up.
__device__ __forceinline__ float rsqrt_hw(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Normalised RPY block D_ij/D_ii (integrateTea_RPY, src/bdhitea_kernel.cu:38-58):
// T = cii I + crr u u^T with ra = r/a; ra > 2: crr = 0.75/ra (1 - 2/ra^2),
// cii = 0.75/ra (1 + 2/(3 ra^2)); otherwise crr = 3 ra/32, cii = 1 - 9 ra/32.
// RPY coefficients from the squared distance (branch-free): cii, and
// crr / r^2 so that T g = cii g + (crr / r^2) d (d . g) with d = r_j - r_i.
__device__ __forceinline__ void rpy_pair(float r2, float a, float inv_a, float &cii, float &crr_r2, float &rinv) {
    r2 = fmaxf(r2, 1e-6f);                  // coincident beads stay finite (masked by the caller)
    rinv = rsqrt_hw(r2);
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

// Shared-memory tile of the all-pairs kernels as a structure of arrays: one
// 8-byte load gives the values of two consecutive beads j, which are the two
// lanes of the packed FP32x2 arithmetic.  Beads past the trajectory's end and
// extra beads get a far-away position (and zero F and R): every term they
// give is zero or below the rounding of the sums, and every tile is full.
struct TeaTile {
    float x[kTeaTile], y[kTeaTile], z[kTeaTile];
    float fx[kTeaTile], fy[kTeaTile], fz[kTeaTile];
    float rx[kTeaTile], ry[kTeaTile], rz[kTeaTile];
};
constexpr float kFarAway = 1.0e18f;

template <bool WITH_FR>
__device__ __forceinline__ void tea_tile_load(TeaTile &T, const DevBuffers &B, int j0, int end) {
    for (int k = threadIdx.x; k < kTeaTile; k += blockDim.x) {
        const int jg = j0 + k;
        float4 p = make_float4(kFarAway, kFarAway, kFarAway, 0.f), F = make_float4(0.f, 0.f, 0.f, 0.f), R = F;
        if (jg < end && !(B.flags[jg] & kFlagExtra)) {
            p = B.frame_in[jg];
            if (WITH_FR) {
                F = B.force[jg];
                R = B.tea_r[jg];
            }
        }
        T.x[k] = p.x;
        T.y[k] = p.y;
        T.z[k] = p.z;
        if (WITH_FR) {
            T.fx[k] = F.x;
            T.fy[k] = F.y;
            T.fz[k] = F.z;
            T.rx[k] = R.x;
            T.ry[k] = R.y;
            T.rz[k] = R.z;
        }
    }
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 ld2(const float *a, int m) { return reinterpret_cast<const float2 *>(a)[m]; }

// The epsilon-pass terms of one pair from its coefficients: the row sums of
// squares minus cii^2 (Bc d_c^2 with Bc = (2 cii + crr) crr / r^2), cii^2,
// and the sum of all nine entries 3 cii + crr/r^2 (d_x + d_y + d_z)^2.
struct EpsTerms {
    float bx, by, bz, a2, w;
};
__device__ __forceinline__ EpsTerms eps_terms(float dx, float dy, float dz, float cii, float crr, float q) {
    const float bc = fmaf(2.0f, cii, crr) * crr * q;
    const float us = dx + dy + dz;
    return {bc * dx * dx, bc * dy * dy, bc * dz * dz, cii * cii, fmaf(crr * q, us * us, 3.0f * cii)};
}

// integrateTea_epsilon_unlisted (src/bdhitea_kernel.cu:84-101): per bead i,
// sum over non-extra j != i of the row sums of squared entries (-> tea_ci)
// and of all nine entries (-> tea_eps).  With T = cii I + crr u u^T the row
// sums of squares are cii^2 + (2 cii + crr) crr u_c^2 and the sum of all
// entries is 3 cii + crr (u_x + u_y + u_z)^2.  Two beads i per thread and,
// away from the CTA's own beads, packed over pairs of j with the far-field
// coefficients (cii = 0.75 a/r + 0.5 a^3/r^3, crr = 0.75 a/r - 1.5 a^3/r^3);
// overlapping pairs (r <= 2a) are corrected afterwards, as in k_tea_step.
template <int SLICES>
__global__ void __launch_bounds__(kTeaI / 2 * SLICES) k_tea_eps(KParams P, DevBuffers B, const int2 *work,
                                                                 const int *gate, int run_if) {
    if (gate && *gate != run_if) return;
    constexpr int kHalf = kTeaI / 2;
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int il = threadIdx.x % kHalf, sl = threadIdx.x / kHalf;
    __shared__ TeaTile T;
    __shared__ float4 s_red[kTeaI * SLICES];
    int gi[2];
    bool act[2];
    float4 pi[2];
    float2 nx[2], ny[2], nz[2], sx[2], sy[2], sz[2], sa[2], sw[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        gi[h] = w.y + il + h * kHalf;
        act[h] = false;
        pi[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gi[h] < end) {
            pi[h] = B.frame_in[gi[h]];
            act[h] = (B.flags[gi[h]] & kFlagExtra) == 0;
        }
        nx[h] = f2(-pi[h].x);
        ny[h] = f2(-pi[h].y);
        nz[h] = f2(-pi[h].z);
        sx[h] = sy[h] = sz[h] = sa[h] = sw[h] = f2(0.f);
    }
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    const float c075a = 0.75f * a, c05a3 = 0.5f * a * a * a, c15a3 = 1.5f * a * a * a, four_a2 = 4.0f * a * a;
    const float2 v075a = f2(c075a), v05a3 = f2(c05a3), vn15a3 = f2(-c15a3), two = f2(2.0f), three = f2(3.0f);
    const bool any_act = act[0] || act[1];
    for (int j0 = base; j0 < end; j0 += kTeaTile) {
        tea_tile_load<false>(T, B, j0, end);
        __syncthreads();
        if (any_act) {
            const bool self_tile = (w.y < j0 + kTeaTile) && (w.y + kTeaI > j0);
            if (!self_tile) {
                float rmin[2] = {3.4e38f, 3.4e38f};
#pragma unroll 2
                for (int m = sl; m < kTeaTile / 2; m += SLICES) {
                    const float2 xj = ld2(T.x, m), yj = ld2(T.y, m), zj = ld2(T.z, m);
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const float2 dx = __fadd2_rn(xj, nx[h]), dy = __fadd2_rn(yj, ny[h]),
                                     dz = __fadd2_rn(zj, nz[h]);
                        const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                        rmin[h] = fminf(rmin[h], fminf(r2.x, r2.y));
                        const float2 rinv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
                        const float2 q = __fmul2_rn(rinv, rinv);
                        const float2 t = __fmul2_rn(q, rinv);
                        const float2 ar = __fmul2_rn(v075a, rinv);
                        const float2 cii = __ffma2_rn(v05a3, t, ar);
                        const float2 crr = __ffma2_rn(vn15a3, t, ar);
                        const float2 crq = __fmul2_rn(crr, q);
                        const float2 bc = __fmul2_rn(__ffma2_rn(two, cii, crr), crq);
                        sa[h] = __ffma2_rn(cii, cii, sa[h]);
                        sx[h] = __ffma2_rn(__fmul2_rn(bc, dx), dx, sx[h]);
                        sy[h] = __ffma2_rn(__fmul2_rn(bc, dy), dy, sy[h]);
                        sz[h] = __ffma2_rn(__fmul2_rn(bc, dz), dz, sz[h]);
                        const float2 us = __fadd2_rn(__fadd2_rn(dx, dy), dz);
                        sw[h] = __ffma2_rn(__fmul2_rn(crq, us), us, __ffma2_rn(three, cii, sw[h]));
                    }
                }
                // overlapping pairs (r <= 2a): replace the far-field terms by the near ones
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    if (!(rmin[h] <= four_a2)) continue;
                    for (int m = sl; m < kTeaTile / 2; m += SLICES) {
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            const int t = 2 * m + e;
                            const float dx = T.x[t] + nx[h].x, dy = T.y[t] + ny[h].x, dz = T.z[t] + nz[h].x;
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            if (!(r2 <= four_a2)) continue;
                            const float rinv = rsqrt_hw(r2), q = rinv * rinv, tq = q * rinv, ar = c075a * rinv;
                            const EpsTerms f = eps_terms(dx, dy, dz, fmaf(c05a3, tq, ar), fmaf(-c15a3, tq, ar), q);
                            const float ra = r2 * rinv * inv_a;
                            const EpsTerms n =
                                eps_terms(dx, dy, dz, 1.0f - (9.0f / 32.0f) * ra, (3.0f / 32.0f) * ra, q);
                            sx[h].x += n.bx - f.bx;
                            sy[h].x += n.by - f.by;
                            sz[h].x += n.bz - f.bz;
                            sa[h].x += n.a2 - f.a2;
                            sw[h].x += n.w - f.w;
                        }
                    }
                }
            } else {
                for (int t = sl; t < kTeaTile; t += SLICES) {
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (j0 + t == gi[h]) continue;
                        const float dx = T.x[t] - pi[h].x, dy = T.y[t] - pi[h].y, dz = T.z[t] - pi[h].z;
                        const float r2 = fmaxf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), 1e-6f);
                        const float rinv = rsqrt_hw(r2);
                        const float q = rinv * rinv;
                        float cii = rinv * fmaf(c05a3, q, c075a);
                        float crr = rinv * fmaf(-c15a3, q, c075a);
                        if (r2 <= four_a2) {
                            const float ra = r2 * rinv * inv_a;
                            cii = 1.0f - (9.0f / 32.0f) * ra;
                            crr = (3.0f / 32.0f) * ra;
                        }
                        const EpsTerms n = eps_terms(dx, dy, dz, cii, crr, q);
                        sx[h].x += n.bx;
                        sy[h].x += n.by;
                        sz[h].x += n.bz;
                        sa[h].x += n.a2;
                        sw[h].x += n.w;
                    }
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const float A = sa[h].x + sa[h].y;
        s_red[(sl * 2 + h) * kHalf + il] =
            make_float4(sx[h].x + sx[h].y + A, sy[h].x + sy[h].y + A, sz[h].x + sz[h].y + A, sw[h].x + sw[h].y);
    }
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
    const float rinv = rsqrt_hw(r2);
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

// Far-field pair term for two beads j (the lanes) against one bead i, with
// d = r_j - r_i, g = F_j + beta C_i o R_j and, in q = 1/r^2, t = q/r:
// cii = 0.75 a/r + 0.5 a^3 t, crr/r^2 = t (0.75 a - 1.5 a^3 q); the running
// minimum of r^2 flags the rare overlapping pairs (r <= 2a) for correction.
__device__ __forceinline__ void tea_far2(float2 dx, float2 dy, float2 dz, float2 gx, float2 gy, float2 gz,
                                         float2 c075a, float2 c05a3, float2 nc15a3, float2 &ax, float2 &ay,
                                         float2 &az, float &rmin) {
    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    rmin = fminf(rmin, fminf(r2.x, r2.y));
    const float2 rinv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
    const float2 q = __fmul2_rn(rinv, rinv);
    const float2 t = __fmul2_rn(q, rinv);
    const float2 cii = __ffma2_rn(c05a3, t, __fmul2_rn(c075a, rinv));
    const float2 crr_r2 = __fmul2_rn(t, __ffma2_rn(nc15a3, q, c075a));
    const float2 s = __fmul2_rn(crr_r2, __ffma2_rn(dx, gx, __ffma2_rn(dy, gy, __fmul2_rn(dz, gz))));
    ax = __ffma2_rn(cii, gx, __ffma2_rn(s, dx, ax));
    ay = __ffma2_rn(cii, gy, __ffma2_rn(s, dy, ay));
    az = __ffma2_rn(cii, gz, __ffma2_rn(s, dz, az));
}

// One lane of tea_far2 in scalar arithmetic (the same operations in the same
// order, so the value is the one the packed lane added).
__device__ __forceinline__ float3 tea_far1(float dx, float dy, float dz, float gx, float gy, float gz, float c075a,
                                           float c05a3, float nc15a3) {
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float rinv = rsqrt_hw(r2);
    const float q = rinv * rinv, t = q * rinv;
    const float cii = fmaf(c05a3, t, c075a * rinv);
    const float crr_r2 = t * fmaf(nc15a3, q, c075a);
    const float s = crr_r2 * fmaf(dx, gx, fmaf(dy, gy, dz * gz));
    return make_float3(fmaf(cii, gx, s * dx), fmaf(cii, gy, s * dy), fmaf(cii, gz, s * dz));
}

// integrateTea_kernel_unlisted + integrateTea_force (src/bdhitea_kernel.cu:104-213):
// f_i = F_i + C_i o R_i + sum_{j != i, non-extra} T_ij (F_j + beta C_i o R_j),
// x_i += dt/gammaR f_i; angles by Euler-Maruyama from stream i + nb, which is
// drawn for every bead.  Reads the current frame, writes the next one.
// Each thread serves two beads i (il and il + kTeaI/2); slice sl takes the
// j-pairs sl, sl + SLICES, ... of every tile.  Tiles that do not hold the
// CTA's own beads run packed over pairs of j with the far-field formula and
// correct the few overlapping pairs afterwards; the tile with the self pairs
// runs the scalar formula with both branches.
template <int SLICES, bool FEFF>
__global__ void __launch_bounds__(kTeaI / 2 * SLICES) k_tea_step(KParams P, DevBuffers B, const int2 *work,
                                                                  float4 *feff, const int *gate) {
    if (FEFF && gate && *gate != 0) return;
    constexpr int kHalf = kTeaI / 2;
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int il = threadIdx.x % kHalf, sl = threadIdx.x / kHalf;
    const int nb = P.nb;
    __shared__ TeaTile T;
    __shared__ float4 s_red[kTeaI * SLICES];

    int gi[2];
    bool act[2];
    float4 pi[2];
    float2 ax[2], ay[2], az[2], nx[2], ny[2], nz[2], cbx[2], cby[2], cbz[2];
    const float beta = B.tea_beta[traj], b2 = beta * beta;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        gi[h] = w.y + il + h * kHalf;
        pi[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        ax[h] = ay[h] = az[h] = f2(0.f);
        float cx = 0.f, cy = 0.f, cz = 0.f;
        act[h] = false;
        if (gi[h] < end) {
            pi[h] = B.frame_in[gi[h]];
            act[h] = (B.flags[gi[h]] & kFlagExtra) == 0;
            const float4 ci = B.tea_ci[gi[h]];
            cx = 1.0f / sqrtf(1.0f + b2 * ci.x);
            cy = 1.0f / sqrtf(1.0f + b2 * ci.y);
            cz = 1.0f / sqrtf(1.0f + b2 * ci.z);
            if (sl == 0) {
                const float4 Fi = B.force[gi[h]], Ri = B.tea_r[gi[h]];
                ax[h].x = Fi.x + Ri.x * cx;
                ay[h].x = Fi.y + Ri.y * cy;
                az[h].x = Fi.z + Ri.z * cz;
            }
        }
        nx[h] = f2(-pi[h].x);
        ny[h] = f2(-pi[h].y);
        nz[h] = f2(-pi[h].z);
        cbx[h] = f2(cx * beta);
        cby[h] = f2(cy * beta);
        cbz[h] = f2(cz * beta);
    }
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    const float c075a = 0.75f * a, c05a3 = 0.5f * a * a * a, c15a3 = 1.5f * a * a * a, four_a2 = 4.0f * a * a;
    const float2 v075a = f2(c075a), v05a3 = f2(c05a3), vn15a3 = f2(-c15a3);
    const bool any_act = act[0] || act[1];
    for (int j0 = base; j0 < end; j0 += kTeaTile) {
        tea_tile_load<true>(T, B, j0, end);
        __syncthreads();
        if (any_act) {
            const bool self_tile = (w.y < j0 + kTeaTile) && (w.y + kTeaI > j0);
            if (!self_tile) {
                float rmin[2] = {3.4e38f, 3.4e38f};
#pragma unroll 2
                for (int m = sl; m < kTeaTile / 2; m += SLICES) {
                    const float2 xj = ld2(T.x, m), yj = ld2(T.y, m), zj = ld2(T.z, m);
                    const float2 fxj = ld2(T.fx, m), fyj = ld2(T.fy, m), fzj = ld2(T.fz, m);
                    const float2 rxj = ld2(T.rx, m), ryj = ld2(T.ry, m), rzj = ld2(T.rz, m);
#pragma unroll
                    for (int h = 0; h < 2; h++)
                        tea_far2(__fadd2_rn(xj, nx[h]), __fadd2_rn(yj, ny[h]), __fadd2_rn(zj, nz[h]),
                                 __ffma2_rn(rxj, cbx[h], fxj), __ffma2_rn(ryj, cby[h], fyj),
                                 __ffma2_rn(rzj, cbz[h], fzj), v075a, v05a3, vn15a3, ax[h], ay[h], az[h], rmin[h]);
                }
                // overlapping pairs (r <= 2a): replace the far-field term by the near one
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    if (!(rmin[h] <= four_a2)) continue;
                    for (int m = sl; m < kTeaTile / 2; m += SLICES) {
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            const int t = 2 * m + e;
                            const float dx = T.x[t] + nx[h].x, dy = T.y[t] + ny[h].x, dz = T.z[t] + nz[h].x;
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            if (!(r2 <= four_a2)) continue;
                            const float gx = fmaf(T.rx[t], cbx[h].x, T.fx[t]), gy = fmaf(T.ry[t], cby[h].x, T.fy[t]),
                                        gz = fmaf(T.rz[t], cbz[h].x, T.fz[t]);
                            const float3 far = tea_far1(dx, dy, dz, gx, gy, gz, c075a, c05a3, -c15a3);
                            float nfx = 0.f, nfy = 0.f, nfz = 0.f;
                            tea_pair(dx, dy, dz, gx, gy, gz, a, inv_a, c075a, c05a3, c15a3, four_a2, nfx, nfy, nfz);
                            ax[h].x += nfx - far.x;
                            ay[h].x += nfy - far.y;
                            az[h].x += nfz - far.z;
                        }
                    }
                }
            } else {
                for (int t = sl; t < kTeaTile; t += SLICES) {
#pragma unroll
                    for (int h = 0; h < 2; h++)
                        if (j0 + t != gi[h])
                            tea_pair(T.x[t] - pi[h].x, T.y[t] - pi[h].y, T.z[t] - pi[h].z,
                                     fmaf(T.rx[t], cbx[h].x, T.fx[t]), fmaf(T.ry[t], cby[h].x, T.fy[t]),
                                     fmaf(T.rz[t], cbz[h].x, T.fz[t]), a, inv_a, c075a, c05a3, c15a3, four_a2,
                                     ax[h].x, ay[h].x, az[h].x);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int h = 0; h < 2; h++)
        s_red[(sl * 2 + h) * kHalf + il] = make_float4(ax[h].x + ax[h].y, ay[h].x + ay[h].y, az[h].x + az[h].y, 0.f);
    __syncthreads();
    if (sl != 0) return;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int g = gi[h];
        if (g >= end) continue;
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int k = 0; k < SLICES; k++) {
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
