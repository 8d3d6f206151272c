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
// and of all nine entries (-> tea_eps).
__global__ void __launch_bounds__(512) k_tea_eps(KParams P, DevBuffers B, const int2 *work) {
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int slices = blockDim.x / kTeaI;
    const int il = threadIdx.x % kTeaI, sl = threadIdx.x / kTeaI;
    const int g = w.y + il;
    const bool valid = g < end;
    __shared__ float4 s_pos[kTeaTile];
    __shared__ float4 s_red[512];
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    bool extra_i = true;
    if (valid) {
        pi = B.frame_in[g];
        extra_i = (B.flags[g] & kFlagExtra) != 0;
    }
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
    for (int j0 = base; j0 < end; j0 += kTeaTile) {
        for (int k = threadIdx.x; k < kTeaTile; k += blockDim.x) {
            const int jg = j0 + k;
            if (jg < end) {
                float4 q = B.frame_in[jg];
                q.w = (B.flags[jg] & kFlagExtra) ? 0.0f : 1.0f;
                s_pos[k] = q;
            }
        }
        __syncthreads();
        if (valid && !extra_i) {
            const int n = min(kTeaTile, end - j0);
#pragma unroll 4
            for (int t = sl; t < n; t += slices) {
                const float4 q = s_pos[t];
                const float m = (j0 + t == g) ? 0.0f : q.w;
                const float dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
                float cii, crr_r2, rinv;
                rpy_pair(dx * dx + dy * dy + dz * dz, a, inv_a, cii, crr_r2, rinv);
                cii *= m;
                crr_r2 *= m;
                const float xx = fmaf(dx * dx, crr_r2, cii), yy = fmaf(dy * dy, crr_r2, cii),
                            zz = fmaf(dz * dz, crr_r2, cii);
                const float xy = dx * dy * crr_r2, xz = dx * dz * crr_r2, yz = dy * dz * crr_r2;
                sw += (xx + yy + zz) + 2.0f * (xy + xz + yz);
                sx += xx * xx + xy * xy + xz * xz;
                sy += xy * xy + yy * yy + yz * yz;
                sz += xz * xz + yz * yz + zz * zz;
            }
        }
        __syncthreads();
    }
    s_red[threadIdx.x] = make_float4(sx, sy, sz, sw);
    __syncthreads();
    if (sl == 0 && valid) {
        float4 acc = s_red[il];
        for (int k = 1; k < slices; k++) {
            const float4 v = s_red[k * kTeaI + il];
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
        }
        B.tea_ci[g] = make_float4(acc.x, acc.y, acc.z, 0.f);
        B.tea_eps[g] = acc.w;
    }
}

// updateTea's reduction (src/bdhitea.cu:75-116), in FP64 on the device: one
// CTA per trajectory sums the bead epsilons and counts the non-extra beads N',
// eps = sum / (3N'(3N'-3)), clamped to 1; a = (3N'-1) eps^2 - (3N'-2) eps;
// beta = (1 - sqrt(1 - a)) / a, or 0.5 when |a| < 1e-7.  The reference's
// exits become the kErrTeaEps bit.
__global__ void __launch_bounds__(256) k_tea_beta(KParams P, DevBuffers B, int capricious, float epsmax) {
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

// integrateTea_kernel_unlisted + integrateTea_force (src/bdhitea_kernel.cu:104-213):
// f_i = F_i + C_i o R_i + sum_{j != i, non-extra} T_ij (F_j + beta C_i o R_j),
// x_i += dt/gammaR f_i; angles by Euler-Maruyama from stream i + nb, which is
// drawn for every bead.  Reads the current frame, writes the next one.
__global__ void __launch_bounds__(512) k_tea_step(KParams P, DevBuffers B, const int2 *work) {
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int slices = blockDim.x / kTeaI;
    const int il = threadIdx.x % kTeaI, sl = threadIdx.x / kTeaI;
    const int g = w.y + il;
    const bool valid = g < end;
    const int nb = P.nb;
    __shared__ float4 s_pos[kTeaTile], s_f[kTeaTile], s_r[kTeaTile];
    __shared__ float4 s_red[512];

    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    int flags = kFlagExtra;
    float fx = 0.f, fy = 0.f, fz = 0.f, cbx = 0.f, cby = 0.f, cbz = 0.f;
    if (valid) {
        pi = B.frame_in[g];
        flags = B.flags[g];
        const float beta = B.tea_beta[traj], b2 = beta * beta;
        const float4 ci = B.tea_ci[g];
        const float cx = 1.0f / sqrtf(1.0f + b2 * ci.x);
        const float cy = 1.0f / sqrtf(1.0f + b2 * ci.y);
        const float cz = 1.0f / sqrtf(1.0f + b2 * ci.z);
        if (sl == 0) {
            const float4 Fi = B.force[g], Ri = B.tea_r[g];
            fx = Fi.x + Ri.x * cx;
            fy = Fi.y + Ri.y * cy;
            fz = Fi.z + Ri.z * cz;
        }
        cbx = cx * beta;
        cby = cy * beta;
        cbz = cz * beta;
    }
    const bool extra_i = (flags & kFlagExtra) != 0;
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    for (int j0 = base; j0 < end; j0 += kTeaTile) {
        for (int k = threadIdx.x; k < kTeaTile; k += blockDim.x) {
            const int jg = j0 + k;
            if (jg < end) {
                float4 q = B.frame_in[jg];
                q.w = (B.flags[jg] & kFlagExtra) ? 0.0f : 1.0f;
                s_pos[k] = q;
                s_f[k] = B.force[jg];
                s_r[k] = B.tea_r[jg];
            }
        }
        __syncthreads();
        if (valid && !extra_i) {
            const int n = min(kTeaTile, end - j0);
#pragma unroll 4
            for (int t = sl; t < n; t += slices) {
                const float4 q = s_pos[t];
                const float m = (j0 + t == g) ? 0.0f : q.w;
                const float4 Fj = s_f[t], Rj = s_r[t];
                const float dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
                float cii, crr_r2, rinv;
                rpy_pair(dx * dx + dy * dy + dz * dz, a, inv_a, cii, crr_r2, rinv);
                cii *= m;
                const float gx = fmaf(Rj.x, cbx, Fj.x), gy = fmaf(Rj.y, cby, Fj.y), gz = fmaf(Rj.z, cbz, Fj.z);
                const float s = m * crr_r2 * (dx * gx + dy * gy + dz * gz);
                fx = fmaf(cii, gx, fmaf(s, dx, fx));
                fy = fmaf(cii, gy, fmaf(s, dy, fy));
                fz = fmaf(cii, gz, fmaf(s, dz, fz));
            }
        }
        __syncthreads();
    }
    s_red[threadIdx.x] = make_float4(fx, fy, fz, 0.f);
    __syncthreads();
    if (sl != 0 || !valid) return;
    for (int k = 1; k < slices; k++) {
        const float4 v = s_red[k * kTeaI + il];
        fx += v.x;
        fy += v.y;
        fz += v.z;
    }
    Frame Fr;
    Fr.p0 = pi;
    Fr.p1 = B.frame_in[nb + g];
    Fr.p2 = B.frame_in[2 * nb + g];
    Fr.p3 = B.frame_in[3 * nb + g];
    uint4 s2 = B.seeds[nb + g];
    const float4 ga = gauss4(s2);
    B.seeds[nb + g] = s2;
    if (!(flags & (kFlagExtra | kFlagFixed))) {
        const float4 fa = B.force[nb + g];  // (ffi, ftheta, fpsi)
        const float x = pi.x + P.kr * fx, y = pi.y + P.kr * fy, z = pi.z + P.kr * fz;
        const float fi = pi.w + (P.kfi * fa.x + P.nfi * ga.x);
        const float psi = Fr.p1.w + (P.kfi * fa.z + P.nfi * ga.y);
        const float th = Fr.p2.w + (P.kth * fa.y + P.varTheta * ga.z);
        Fr = make_frame(P, x, y, z, fi, th, psi);
    }
    store_frame(B.frame_out, nb, g, Fr);
}

void launch_tea_eps(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s) {
    k_tea_eps<<<nwork, kTeaI * P.tea_slices, 0, s>>>(P, B, work);
}
void launch_tea_beta(const KParams &P, const DevBuffers &B, int capricious, float epsmax, cudaStream_t s) {
    k_tea_beta<<<P.nt, 256, 0, s>>>(P, B, capricious, epsmax);
}
void launch_tea_step(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s) {
    k_tea_step<<<nwork, kTeaI * P.tea_slices, 0, s>>>(P, B, work);
}

}  // namespace mtg
