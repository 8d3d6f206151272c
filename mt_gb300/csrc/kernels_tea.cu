// kernels_tea.cu - TEA hydrodynamics (Geyer & Winter 2009): the all-pairs
// epsilon / C_i pass, the FP64 epsilon -> beta reduction, and the all-pairs
// RPY mobility product fused with the position update.
//
// Both O(N^2) kernels run one CTA per (trajectory, chunk of kTile beads) and
// stream the trajectory through shared memory in tiles; every thread keeps
// its bead i in registers and reads the tile by broadcast.  They are bound by
// the FP32 pipe (about 45 FLOP per ordered pair).
#include "mtg_internal.cuh"

namespace mtg {

// Normalised RPY block D_ij/D_ii (integrateTea_RPY, src/bdhitea_kernel.cu:38-58)
// as (cii, crr): T = cii I + crr u u^T, from the squared distance r2.
__device__ __forceinline__ void rpy_coeffs(float r2, float inv_a, float a, float &cii, float &crr, float &rinv) {
    rinv = rsqrtf(r2);
    const float r = r2 * rinv;
    const float ra = r * inv_a;
    if (ra > 2.0f) {
        const float ira = a * rinv;         // 1 / ra
        const float ira2 = ira * ira;
        crr = 0.75f * ira * (1.0f - 2.0f * ira2);
        cii = 0.75f * ira * (1.0f + (2.0f / 3.0f) * ira2);
    } else {
        crr = (3.0f / 32.0f) * ra;
        cii = 1.0f - (9.0f / 32.0f) * ra;
    }
}

// integrateTea_epsilon_unlisted (src/bdhitea_kernel.cu:84-101): per bead i,
// sum over non-extra j != i of the row sums of squared entries (-> tea_ci)
// and of all nine entries (-> tea_eps).
__global__ void __launch_bounds__(kTile) k_tea_eps(KParams P, DevBuffers B, const int2 *work) {
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int g = w.y + threadIdx.x;
    const bool valid = g < end;
    __shared__ float4 s_pos[kTile];
    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    bool extra_i = true;
    if (valid) {
        pi = B.frame_in[g];
        extra_i = (B.flags[g] & kFlagExtra) != 0;
    }
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
    for (int j0 = base; j0 < end; j0 += kTile) {
        const int jg = j0 + threadIdx.x;
        if (jg < end) {
            float4 q = B.frame_in[jg];
            q.w = (B.flags[jg] & kFlagExtra) ? 1.0f : 0.0f;
            s_pos[threadIdx.x] = q;
        }
        __syncthreads();
        if (valid && !extra_i) {
            const int n = min(kTile, end - j0);
            for (int t = 0; t < n; t++) {
                const float4 q = s_pos[t];
                if (j0 + t == g || q.w != 0.0f) continue;
                const float dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
                float cii, crr, rinv;
                rpy_coeffs(dx * dx + dy * dy + dz * dz, inv_a, a, cii, crr, rinv);
                const float ux = dx * rinv, uy = dy * rinv, uz = dz * rinv;
                const float xx = ux * ux * crr + cii, yy = uy * uy * crr + cii, zz = uz * uz * crr + cii;
                const float xy = ux * uy * crr, xz = ux * uz * crr, yz = uy * uz * crr;
                sw += xx + yy + zz + 2.0f * (xy + xz + yz);
                sx += xx * xx + xy * xy + xz * xz;
                sy += xy * xy + yy * yy + yz * yz;
                sz += xz * xz + yz * yz + zz * zz;
            }
        }
        __syncthreads();
    }
    if (valid) {
        B.tea_ci[g] = make_float4(sx, sy, sz, 0.f);
        B.tea_eps[g] = sw;
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
__global__ void __launch_bounds__(kTile) k_tea_step(KParams P, DevBuffers B, const int2 *work) {
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int g = w.y + threadIdx.x;
    const bool valid = g < end;
    const int nb = P.nb;
    __shared__ float4 s_pos[kTile], s_f[kTile], s_r[kTile];

    float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
    int flags = kFlagExtra;
    float fx = 0.f, fy = 0.f, fz = 0.f, cbx = 0.f, cby = 0.f, cbz = 0.f;
    if (valid) {
        pi = B.frame_in[g];
        flags = B.flags[g];
        const float beta = B.tea_beta[traj], b2 = beta * beta;
        const float4 ci = B.tea_ci[g], Fi = B.force[g], Ri = B.tea_r[g];
        const float cx = 1.0f / sqrtf(1.0f + b2 * ci.x);
        const float cy = 1.0f / sqrtf(1.0f + b2 * ci.y);
        const float cz = 1.0f / sqrtf(1.0f + b2 * ci.z);
        fx = Fi.x + Ri.x * cx;
        fy = Fi.y + Ri.y * cy;
        fz = Fi.z + Ri.z * cz;
        cbx = cx * beta;
        cby = cy * beta;
        cbz = cz * beta;
    }
    const bool extra_i = (flags & kFlagExtra) != 0;
    const float a = P.tea_a, inv_a = 1.0f / P.tea_a;
    for (int j0 = base; j0 < end; j0 += kTile) {
        const int jg = j0 + threadIdx.x;
        if (jg < end) {
            float4 q = B.frame_in[jg];
            q.w = (B.flags[jg] & kFlagExtra) ? 1.0f : 0.0f;
            s_pos[threadIdx.x] = q;
            s_f[threadIdx.x] = B.force[jg];
            s_r[threadIdx.x] = B.tea_r[jg];
        }
        __syncthreads();
        if (valid && !extra_i) {
            const int n = min(kTile, end - j0);
#pragma unroll 4
            for (int t = 0; t < n; t++) {
                const float4 q = s_pos[t];
                if (j0 + t == g || q.w != 0.0f) continue;
                const float4 Fj = s_f[t], Rj = s_r[t];
                const float dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
                float cii, crr, rinv;
                rpy_coeffs(dx * dx + dy * dy + dz * dz, inv_a, a, cii, crr, rinv);
                const float ux = dx * rinv, uy = dy * rinv, uz = dz * rinv;
                const float gx = Fj.x + Rj.x * cbx, gy = Fj.y + Rj.y * cby, gz = Fj.z + Rj.z * cbz;
                const float ug = crr * (ux * gx + uy * gy + uz * gz);
                fx += cii * gx + ug * ux;
                fy += cii * gy + ug * uy;
                fz += cii * gz + ug * uz;
            }
        }
        __syncthreads();
    }
    if (!valid) return;
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
    k_tea_eps<<<nwork, kTile, 0, s>>>(P, B, work);
}
void launch_tea_beta(const KParams &P, const DevBuffers &B, int capricious, float epsmax, cudaStream_t s) {
    k_tea_beta<<<P.nt, 256, 0, s>>>(P, B, capricious, epsmax);
}
void launch_tea_step(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s) {
    k_tea_step<<<nwork, kTile, 0, s>>>(P, B, work);
}

}  // namespace mtg
