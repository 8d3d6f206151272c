// kernels_step.cu - per-bead forces, the fused force + Euler-Maruyama step,
// energies, and the state <-> Coord conversions.
//
// One thread per bead.  A bead's neighbours are read from the current frame
// buffer (16 B gathers of precomputed lab-frame site vectors, L2-resident for
// the batch sizes of interest); the moving bead writes its new state and new
// site vectors to the other buffer, so forces and integration fuse into one
// launch per step without a race.
#include "mtg_internal.cuh"

namespace mtg {

struct Acc {
    float fx, fy, fz, ffi, fpsi, fth, tx, ty, tz;
};

// Adds a pair term with radial factor dUdr = U'(r)/r along d = site_j - site_i
// and its torque dUdr * (w_i x d) about the bead centre.
__device__ __forceinline__ void acc_pair(Acc &A, float dUdr, float3 d, float3 wi) {
    A.fx += dUdr * d.x;
    A.fy += dUdr * d.y;
    A.fz += dUdr * d.z;
    A.tx += dUdr * (wi.y * d.z - wi.z * d.y);
    A.ty += dUdr * (wi.z * d.x - wi.x * d.z);
    A.tz += dUdr * (wi.x * d.y - wi.y * d.x);
}

// Bending terms of a harmonic/longitudinal partner (src/compute_cuda.cu:142-180,
// :265-298): sign by the site side, theta0 chosen by the caller.
__device__ __forceinline__ void acc_bend(const KParams &P, Acc &A, float rmon, float dpsi, float dfi, float dth,
                                         float th0) {
    if (rmon > 0.0f) {
        A.fpsi += P.B_psi * sinf(dpsi - P.psi_0);
        A.ffi += P.B_fi * sinf(dfi - P.fi_0);
        A.fth += P.B_theta * sinf(dth - th0);
    } else {
        A.fpsi -= P.B_psi * sinf(-dpsi - P.psi_0);
        A.ffi -= P.B_fi * sinf(-dfi - P.fi_0);
        A.fth -= P.B_theta * sinf(-dth - th0);
    }
}

// Where a bead's neighbours' frames and flags are read: plane k of local bead
// j at fr[k * stride + base + j], its flags at fl[base + j].  The per-step
// kernels read the global frame buffer (stride nb, base = the trajectory's
// first bead); the persistent kernel reads its trajectory's copy in shared
// memory (stride = trajectory size, base 0).  Same arithmetic either way.
struct NbrView {
    const float4 *fr;
    const int *fl;
    int stride, base;
};
__device__ __forceinline__ NbrView global_view(const KParams &P, const DevBuffers &B, int traj) {
    return {B.frame_in, B.flags, P.nb, B.off[traj]};
}

// Generalised force on bead g (compute_kernel, src/compute_cuda.cu:32-525):
// harmonic + bending, Morse longitudinal + bending, Morse lateral with seam
// coefficient, barriers, LJ inside 6 nm, walls.  out = (fx, fy, fz, ffi,
// ftheta, fpsi).
__device__ __forceinline__ void bead_forces(const KParams &P, const DevBuffers &B, const NbrView &V, int g, int traj,
                                            int flags, const Frame &Fi, float out[6]) {
    const int nb = P.nb;          // list layout (k-major over all beads)
    const int ps = V.stride;      // plane stride of the neighbour frames
    const int base = V.base;
    const float4 *fr = V.fr;
    Acc A = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const float3 uzi = f3(Fi.p1);
    const bool off_tub = (flags & kFlagOnTubule) == 0;

    // Every list count and the first entries of every list are requested
    // before any is used (entries past a count are in bounds and ignored):
    // the dependent chain index -> neighbour state starts for all lists at once.
    const int hc = (flags >> kHarmShift) & 7;
    const int nl = P.maxLong > 0 ? B.lonc[g] : 0;
    const int nt = P.maxLat > 0 ? B.latc[g] : 0;
    const int nlj = P.lj_on ? B.ljc[g] : 0;
    const int e_h0 = B.harm[g * P.maxH];
    const int e_l0 = P.maxLong > 0 ? B.lon[g] : 0;
    const int e_t0 = P.maxLat > 0 ? B.lat[g] : 0;
    int jj0[4];
#pragma unroll
    for (int u = 0; u < 4; u++) jj0[u] = (P.lj_on && u < P.maxLJ) ? B.lj[u * nb + g] : 0;

    // harmonic bond inside the dimer (:69-182)
    for (int k = 0; k < hc; k++) {
        const int e = k == 0 ? e_h0 : B.harm[g * P.maxH + k];
        const float rmon = e < 0 ? 2.0f : -2.0f;
        const int pj = base + (e < 0 ? -e : e);
        const float4 rj = fr[pj], uj = fr[ps + pj];
        const float3 wi = make_float3(uzi.x * rmon, uzi.y * rmon, uzi.z * rmon);
        const float3 wj = make_float3(-uj.x * rmon, -uj.y * rmon, -uj.z * rmon);
        const float3 d = site_delta(Fi.p0, rj, wi, wj);
        const float dr = norm3_rn(d);
        acc_pair(A, P.C, d, wi);
        if (dr < 1.0f) {
            const float thj = fr[2 * ps + pj].w;
            acc_bend(P, A, rmon, uj.w - Fi.p1.w, rj.w - Fi.p0.w, thj - Fi.p2.w,
                     (flags & kFlagGtp) ? P.th0_gtp : P.th0_gdp);
        }
    }
    // Morse longitudinal (:187-301)
    for (int k = 0; k < nl; k++) {
        const int e = k == 0 ? e_l0 : B.lon[k * nb + g];
        const float rmon = e < 0 ? 2.0f : -2.0f;
        const int pj = base + (e < 0 ? -e : e);
        const float4 rj = fr[pj], uj = fr[ps + pj];
        const float3 wi = make_float3(uzi.x * rmon, uzi.y * rmon, uzi.z * rmon);
        const float3 wj = make_float3(-uj.x * rmon, -uj.y * rmon, -uj.z * rmon);
        const float3 d = site_delta(Fi.p0, rj, wi, wj);
        const float dr = norm3_rn(d);
        float dUdr = dr == 0.0f ? 0.0f : dmorse(P.D_long, P.A_long, dr) / dr;
        int fj = -1;
        if (P.barrier) {
            fj = V.fl[pj];
            if (off_tub && (fj & kFlagOnTubule) == 0 && dr != 0.0f) dUdr += dbarr(P.a_bl, P.r_bl, P.w_bl, dr) / dr;
        }
        acc_pair(A, dUdr, d, wi);
        if (dr < 1.0f) {
            // theta0 of the bead nearer the plus end (:282-283)
            int glast = flags;
            if (!(Fi.p0.z > rj.z)) glast = fj >= 0 ? fj : V.fl[pj];
            const float thj = fr[2 * ps + pj].w;
            acc_bend(P, A, rmon, uj.w - Fi.p1.w, rj.w - Fi.p0.w, thj - Fi.p2.w,
                     (glast & kFlagGtp) ? P.th0_gtp : P.th0_gdp);
        }
    }
    // Morse lateral (:303-467)
    for (int k = 0; k < nt; k++) {
        const int e = k == 0 ? e_t0 : B.lat[k * nb + g];
        const bool neg = e <= 0;
        int j = e < 0 ? -e : e;
        if (j == kZeroCode) j = 0;
        const int pj = base + j;
        const float4 rj = fr[pj];
        const float4 sj = neg ? fr[3 * ps + pj] : fr[2 * ps + pj];
        const float3 wi = neg ? f3(Fi.p2) : f3(Fi.p3);
        const float3 d = site_delta(Fi.p0, rj, wi, f3(sj));
        const float dr = norm3_rn(d);
        const int fj = V.fl[pj];
        const float D = ((flags ^ fj) & kFlagBeta) ? P.D_lat_seam : P.D_lat;
        float dUdr = dr == 0.0f ? 0.0f : dmorse(D, P.A_lat, dr) / dr;
        if (P.barrier && off_tub && (fj & kFlagOnTubule) == 0 && dr != 0.0f)
            dUdr += dbarr(P.a_bt, P.r_bt, P.w_bt, dr) / dr;
        acc_pair(A, dUdr, d, wi);
    }
    // LJ r^-6 repulsion with the hard 6 nm force cutoff (:470-495)
    if (P.lj_on) {
        // four neighbours per round: their indices, then their positions, are
        // all in flight before the first is used
        for (int k0 = 0; k0 < nlj; k0 += 4) {
            int jj[4];
            float4 rj[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                jj[u] = k0 + u < nlj ? (k0 == 0 ? jj0[u] : B.lj[(k0 + u) * nb + g]) : -1;
#pragma unroll
            for (int u = 0; u < 4; u++) rj[u] = jj[u] >= 0 ? fr[base + jj[u]] : Fi.p0;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (jj[u] < 0) continue;
                const float dx = Fi.p0.x - rj[u].x, dy = Fi.p0.y - rj[u].y, dz = Fi.p0.z - rj[u].z;
                const float dr = sqrtf(dx * dx + dy * dy + dz * dz);
                if (dr < 6.0f) {
                    const float dr2 = dr * dr, dr4 = dr2 * dr2;
                    const float s = P.lj_pref * (6.0f / (dr4 * dr4));
                    A.fx += s * dx;
                    A.fy += s * dy;
                    A.fz += s * dz;
                }
            }
        }
    }
    // cylindrical walls (:497-517)
    if (P.is_wall) {
        const float z = Fi.p0.z, top = B.zs[traj] + P.lb;
        if (z < P.lb)
            A.fz += P.rep_eps * fabsf(z - P.lb);
        else if (z > top)
            A.fz += -P.rep_eps * fabsf(z - top);
        const float rad2 = Fi.p0.x * Fi.p0.x + Fi.p0.y * Fi.p0.y;
        if (rad2 > P.rep_r * P.rep_r) {
            const float rad = sqrtf(rad2);
            const float coeff = -P.rep_eps * (rad - P.rep_r);
            A.fx += Fi.p0.x / rad * coeff;
            A.fy += Fi.p0.y / rad * coeff;
        }
    }
    // generalised forces = bending terms + torque projected on the Euler axes:
    // psi about z, theta about Rz(psi) y, fi about R x.
    float sp, cp, st, ct;
    sincosf(Fi.p1.w, &sp, &cp);
    sincosf(Fi.p2.w, &st, &ct);
    out[0] = A.fx;
    out[1] = A.fy;
    out[2] = A.fz;
    out[3] = A.ffi + (cp * ct * A.tx + sp * ct * A.ty - st * A.tz);
    out[4] = A.fth + (-sp * A.tx + cp * A.ty);
    out[5] = A.fpsi + A.tz;
}

__device__ __forceinline__ Frame load_frame(const float4 *planes, int nb, int g) {
    Frame F;
    F.p0 = planes[g];
    F.p1 = planes[nb + g];
    F.p2 = planes[2 * nb + g];
    F.p3 = planes[3 * nb + g];
    return F;
}

// Euler-Maruyama update of one moving bead (integrate_kernel,
// src/compute_cuda.cu:955-963): xyz from normals gx, angles from ga.
// Explicitly rounded, like make_frame, so that every kernel gets the same bits.
__device__ __forceinline__ float em_rn(float x, float k, float f, float v, float g) {
    return __fadd_rn(x, __fadd_rn(__fmul_rn(k, f), __fmul_rn(v, g)));
}
__device__ __forceinline__ Frame em_update(const KParams &P, const Frame &Fi, const float f[6], float4 gx,
                                           float4 ga) {
    const float x = em_rn(Fi.p0.x, P.kr, f[0], P.varR, gx.x);
    const float y = em_rn(Fi.p0.y, P.kr, f[1], P.varR, gx.y);
    const float z = em_rn(Fi.p0.z, P.kr, f[2], P.varR, gx.z);
    const float fi = em_rn(Fi.p0.w, P.kfi, f[3], P.nfi, ga.x);
    const float psi = em_rn(Fi.p1.w, P.kfi, f[5], P.nfi, ga.y);
    const float th = em_rn(Fi.p2.w, P.kth, f[4], P.varTheta, ga.z);
    return make_frame(P, x, y, z, fi, th, psi);
}

template <bool KEEP_FORCES>
__global__ void __launch_bounds__(256) k_step_plain(KParams P, DevBuffers B) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.nb) return;
    const int nb = P.nb;
    const int flags = B.flags[g];
    Frame Fi = load_frame(B.frame_in, nb, g);
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (!(flags & kFlagExtra)) {
        const bool moving = !(flags & kFlagFixed);
        if (moving || KEEP_FORCES) {
            const int traj = B.traj[g];
            bead_forces(P, B, global_view(P, B, traj), g, traj, flags, Fi, f);
        }
        if (moving) {
            uint4 s1 = B.seeds[g], s2 = B.seeds[nb + g];
            const float4 gx = gauss4(s1), ga = gauss4(s2);
            B.seeds[g] = s1;
            B.seeds[nb + g] = s2;
            Fi = em_update(P, Fi, f, gx, ga);
        }
    }
    store_frame(B.frame_out, nb, g, Fi);
    if (KEEP_FORCES) {
        B.force[g] = make_float4(f[0], f[1], f[2], 0.f);
        B.force[nb + g] = make_float4(f[3], f[4], f[5], 0.f);
    }
}

// ------------------------------------------------------- persistent period
// A whole run of plain steps between two pair-list rebuilds in one launch:
// one CTA per trajectory keeps the trajectory's frames (the four planes) and
// flags in shared memory across the steps, so every neighbour gather of the
// force loop is a shared-memory load; the pair lists and noise streams stay
// in global memory (L2).  Each step is a force phase over the CTA's beads, a
// barrier, the Euler-Maruyama update of every moving bead into shared
// memory, and a barrier; trajectories never interact, so no grid-wide
// synchronisation is needed.  The arithmetic is bead_forces / em_update, as in
// k_step_plain: the result equals that of nsteps launches of k_step_plain bit
// for bit.  At the end the frames go to the buffer the engine's step parity
// expects (frame_out for an odd number of steps, frame_in otherwise).
template <bool KEEP_FORCES>
__global__ void __launch_bounds__(kPeriodThreads, 2) k_step_period(KParams P, DevBuffers B, int nsteps, int nmax,
                                                                   int rebuild) {
    extern __shared__ float4 s_dyn[];
    const int traj = blockIdx.x;
    const int base = B.off[traj], n = B.off[traj + 1] - base;
    const int nb = P.nb, nt = blockDim.x;
    float4 *sf = s_dyn;                                       // plane k of bead j at sf[k * n + j]
    int *sfl = reinterpret_cast<int *>(s_dyn + 4 * (size_t)nmax);
    for (int j = threadIdx.x; j < n; j += nt) {
        const int g = base + j;
        sf[j] = B.frame_in[g];
        sf[n + j] = B.frame_in[nb + g];
        sf[2 * n + j] = B.frame_in[2 * nb + g];
        sf[3 * n + j] = B.frame_in[3 * nb + g];
        sfl[j] = B.flags[g];
    }
    __syncthreads();
    if (rebuild) {
        // the pair lists of this state first, from the frames in shared
        // memory: every bead against the trajectory in ascending j, the
        // decisions of k_rebuild (the same lists)
        // beads farther apart than every cutoff (plus a margin over the
        // rounding of the distance) are skipped before the full decisions
        const float reach = fmaxf(P.lj_on ? P.ljcut : 0.f, P.is_assembly ? kPairPrefilter : 0.f) + 0.05f;
        const float reach2 = reach * reach;
        for (int il = threadIdx.x; il < n; il += nt) {
            const int g = base + il;
            const ListSite I = list_site(P, sf[il], sf[n + il], sf[2 * n + il], sf[3 * n + il], sfl[il], il,
                                         B.harm[g * P.maxH]);
            int nlj = 0, nlo = 0, nla = 0;
            bool overflow = false;
            if (I.do_lj || I.do_pairs)
                for (int jl = 0; jl < n; jl++) {
                    const float4 q = sf[jl];
                    const float dx = q.x - I.p.x, dy = q.y - I.p.y, dz = q.z - I.p.z;
                    if (dx * dx + dy * dy + dz * dz > reach2) continue;
                    const unsigned bits = list_bits(P, I, jl, q, sf[n + jl], sf[2 * n + jl], sf[3 * n + jl], sfl[jl]);
                    list_append(P, B, g, I, bits, jl, nlj, nlo, nla, overflow);
                }
            if (P.lj_on) B.ljc[g] = min(nlj, P.maxLJ);
            if (P.is_assembly) {
                B.lonc[g] = min(nlo, P.maxLong);
                B.latc[g] = min(nla, P.maxLat);
            }
            if (overflow) atomicOr(B.err, kErrOverflow);
        }
        __syncthreads();
    }
    const NbrView V = {sf, sfl, n, 0};
    float f[kPeriodBeads][6];
    for (int step = 0; step < nsteps; step++) {
#pragma unroll
        for (int q = 0; q < kPeriodBeads; q++) {
            const int j = threadIdx.x + q * nt;
#pragma unroll
            for (int c = 0; c < 6; c++) f[q][c] = 0.f;
            if (j < n) {
                const int fl = sfl[j];
                if (!(fl & kFlagExtra) && (KEEP_FORCES || !(fl & kFlagFixed))) {
                    Frame Fi;
                    Fi.p0 = sf[j];
                    Fi.p1 = sf[n + j];
                    Fi.p2 = sf[2 * n + j];
                    Fi.p3 = sf[3 * n + j];
                    bead_forces(P, B, V, base + j, traj, fl, Fi, f[q]);
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kPeriodBeads; q++) {
            const int j = threadIdx.x + q * nt;
            if (j >= n) continue;
            const int fl = sfl[j], g = base + j;
            if (!(fl & (kFlagExtra | kFlagFixed))) {
                Frame Fi;
                Fi.p0 = sf[j];
                Fi.p1 = sf[n + j];
                Fi.p2 = sf[2 * n + j];
                Fi.p3 = sf[3 * n + j];
                uint4 s1 = B.seeds[g], s2 = B.seeds[nb + g];
                const float4 gx = gauss4(s1), ga = gauss4(s2);
                B.seeds[g] = s1;
                B.seeds[nb + g] = s2;
                Fi = em_update(P, Fi, f[q], gx, ga);
                sf[j] = Fi.p0;
                sf[n + j] = Fi.p1;
                sf[2 * n + j] = Fi.p2;
                sf[3 * n + j] = Fi.p3;
            }
            if (KEEP_FORCES && step == nsteps - 1) {
                B.force[g] = make_float4(f[q][0], f[q][1], f[q][2], 0.f);
                B.force[nb + g] = make_float4(f[q][3], f[q][4], f[q][5], 0.f);
            }
        }
        __syncthreads();
    }
    float4 *out = (nsteps & 1) ? B.frame_out : B.frame_in;
    for (int j = threadIdx.x; j < n; j += nt) {
        const int g = base + j;
        out[g] = sf[j];
        out[nb + g] = sf[n + j];
        out[2 * nb + g] = sf[2 * n + j];
        out[3 * nb + g] = sf[3 * n + j];
    }
}

// Forces only (for output and the TEA path).  With TEA_PREPARE it also draws
// the random force of every bead from stream g scaled by sqrt(2 kB T gammaR /
// dt) (integrateTea_prepare, src/bdhitea_kernel.cu:16-36).
template <bool TEA_PREPARE>
__global__ void __launch_bounds__(256) k_forces(KParams P, DevBuffers B) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.nb) return;
    const int nb = P.nb;
    const int flags = B.flags[g];
    float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (!(flags & kFlagExtra)) {
        const Frame Fi = load_frame(B.frame_in, nb, g);
        const int traj = B.traj[g];
        bead_forces(P, B, global_view(P, B, traj), g, traj, flags, Fi, f);
    }
    B.force[g] = make_float4(f[0], f[1], f[2], 0.f);
    B.force[nb + g] = make_float4(f[3], f[4], f[5], 0.f);
    if (TEA_PREPARE) {
        uint4 s = B.seeds[g];
        float4 r = gauss4(s);
        B.seeds[g] = s;
        r.x *= P.tea_var;
        r.y *= P.tea_var;
        r.z *= P.tea_var;
        B.tea_r[g] = r;
    }
}

// ------------------------------------------------------------- energies
// energy_kernel (src/compute_cuda.cu:676-911): per-bead FP32 terms, halved;
// block partial sums in FP64 over one trajectory chunk.
__global__ void __launch_bounds__(kTile) k_energy(KParams P, DevBuffers B, const int2 *work, double *per_bead,
                                                  double *partials) {
    const int2 w = work[blockIdx.x];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    const int g = w.y + threadIdx.x;
    const int nb = P.nb;
    const float4 *fr = B.frame_in;
    float U[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (g < end) {
        const int flags = B.flags[g];
        if (!(flags & kFlagExtra)) {
            const Frame Fi = load_frame(fr, nb, g);
            const float3 uzi = f3(Fi.p1);
            const bool off_tub = (flags & kFlagOnTubule) == 0;
            const int hc = (flags >> kHarmShift) & 7;
            for (int k = 0; k < hc; k++) {
                const int e = B.harm[g * P.maxH + k];
                const float rmon = e < 0 ? 2.0f : -2.0f;
                const int pj = base + (e < 0 ? -e : e);
                const float4 rj = fr[pj], uj = fr[nb + pj];
                const float3 d = site_delta(Fi.p0, rj, make_float3(uzi.x * rmon, uzi.y * rmon, uzi.z * rmon),
                                            make_float3(-uj.x * rmon, -uj.y * rmon, -uj.z * rmon));
                const float dr = norm3_rn(d);
                U[0] += (P.C / 2.0f) * dr * dr;
                if (dr < 1.0f) {
                    // psi_ij, fi_ij, theta_ji (src/compute_cuda.cu:751-756)
                    const float th0 = (flags & kFlagGtp) ? P.th0_gtp : P.th0_gdp;
                    U[3] += P.B_psi * (1.0f - cosf((Fi.p1.w - uj.w) - P.psi_0));
                    U[4] += P.B_fi * (1.0f - cosf((Fi.p0.w - rj.w) - P.fi_0));
                    U[5] += P.B_theta * (1.0f - cosf((fr[2 * nb + pj].w - Fi.p2.w) - th0));
                }
            }
            const int nl = B.lonc[g];
            for (int k = 0; k < nl; k++) {
                const int e = B.lon[k * nb + g];
                const float rmon = e < 0 ? 2.0f : -2.0f;
                const int pj = base + (e < 0 ? -e : e);
                const float4 rj = fr[pj], uj = fr[nb + pj];
                const float3 d = site_delta(Fi.p0, rj, make_float3(uzi.x * rmon, uzi.y * rmon, uzi.z * rmon),
                                            make_float3(-uj.x * rmon, -uj.y * rmon, -uj.z * rmon));
                const float dr = norm3_rn(d);
                U[1] += morse_en(P.D_long, P.A_long, dr);
                const int fj = B.flags[pj];
                if (P.barrier && off_tub && (fj & kFlagOnTubule) == 0) U[1] += barr(P.a_bl, P.r_bl, P.w_bl, dr);
                if (dr < 1.0f) {
                    const int glast = (Fi.p0.z > rj.z) ? flags : fj;
                    const float th0 = (glast & kFlagGtp) ? P.th0_gtp : P.th0_gdp;
                    U[3] += P.B_psi * (1.0f - cosf((Fi.p1.w - uj.w) - P.psi_0));
                    U[4] += P.B_fi * (1.0f - cosf((Fi.p0.w - rj.w) - P.fi_0));
                    U[5] += P.B_theta * (1.0f - cosf((Fi.p2.w - fr[2 * nb + pj].w) - th0));
                }
            }
            const int nt = B.latc[g];
            for (int k = 0; k < nt; k++) {
                const int e = B.lat[k * nb + g];
                const bool neg = e <= 0;
                int j = e < 0 ? -e : e;
                if (j == kZeroCode) j = 0;
                const int pj = base + j;
                const float4 rj = fr[pj];
                const float4 sj = neg ? fr[3 * nb + pj] : fr[2 * nb + pj];
                const float3 d = site_delta(Fi.p0, rj, neg ? f3(Fi.p2) : f3(Fi.p3), f3(sj));
                const float dr = norm3_rn(d);
                const int fj = B.flags[pj];
                U[2] += morse_en(((flags ^ fj) & kFlagBeta) ? P.D_lat_seam : P.D_lat, P.A_lat, dr);
                if (P.barrier && off_tub && (fj & kFlagOnTubule) == 0) U[2] += barr(P.a_bt, P.r_bt, P.w_bt, dr);
            }
            if (P.lj_on) {
                const int n = B.ljc[g];
                for (int k = 0; k < n; k++) {
                    const float4 rj = fr[base + B.lj[k * nb + g]];
                    const float dx = Fi.p0.x - rj.x, dy = Fi.p0.y - rj.y, dz = Fi.p0.z - rj.z;
                    const float dr2 = dx * dx + dy * dy + dz * dz;
                    if (sqrtf(dr2) < 6.0f) U[6] += P.lj_pref / (dr2 * dr2 * dr2);
                }
            }
        }
        if (per_bead) {
            for (int c = 0; c < 7; c++) per_bead[7 * (size_t)g + c] = (double)(U[c] / 2.0f);
        }
    }
    // FP64 block reduction: warp shuffles, then one warp over the warp sums.
    __shared__ double red[kTile / 32][7];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int c = 0; c < 7; c++) {
        double v = (double)(U[c] / 2.0f);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wid][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        double v = 0.0;
        for (int w2 = 0; w2 < kTile / 32; w2++) v += red[w2][threadIdx.x];
        partials[7 * (size_t)blockIdx.x + threadIdx.x] = v;
    }
}

// Per-trajectory totals: fixed-order sum of the trajectory's block partials.
__global__ void k_energy_totals(int nt, const double *partials, const int *work_first, double *per_traj,
                                int *err) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int w = work_first[t]; w < work_first[t + 1]; w++)
        for (int c = 0; c < 7; c++) s[c] += partials[7 * (size_t)w + c];
    for (int c = 0; c < 7; c++) per_traj[7 * (size_t)t + c] = s[c];
    // the terms the reference checks (src/updater.cpp:27)
    if (!isfinite(s[0]) || !isfinite(s[1]) || !isfinite(s[2]) || !isfinite(s[6])) atomicOr(err, kErrNonFinite);
}

// ----------------------------------------------------------- conversions
__global__ void k_frames_from_coords(KParams P, const float *c7, float4 *planes) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.nb) return;
    const float *c = c7 + 7 * (size_t)g;
    store_frame(planes, P.nb, g, make_frame(P, c[0], c[1], c[2], c[3], c[4], c[5]));
}

__global__ void k_coords_from_frames(int nb, const float4 *planes, float *c7) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const float4 a = planes[g];
    float *c = c7 + 7 * (size_t)g;
    c[0] = a.x;
    c[1] = a.y;
    c[2] = a.z;
    c[3] = a.w;
    c[4] = planes[2 * nb + g].w;
    c[5] = planes[nb + g].w;
    c[6] = 0.f;
}

__global__ void k_forces_to_coords(int nb, const float4 *force, float *c7) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    const float4 a = force[g], b = force[nb + g];
    float *c = c7 + 7 * (size_t)g;
    c[0] = a.x;
    c[1] = a.y;
    c[2] = a.z;
    c[3] = b.x;
    c[4] = b.y;
    c[5] = b.z;
    c[6] = 0.f;
}

__global__ void k_set_flags(int nb, const uint8_t *extra, const int *gtp, const int *ontub, int *flags) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nb) return;
    int f = flags[g];
    if (extra) f = extra[g] ? (f | kFlagExtra) : (f & ~kFlagExtra);
    if (gtp) f = gtp[g] == 1 ? (f | kFlagGtp) : (f & ~kFlagGtp);
    if (ontub) f = ontub[g] != 0 ? (f | kFlagOnTubule) : (f & ~kFlagOnTubule);
    flags[g] = f;
}

// --------------------------------------------------------------- launchers
static inline int blocks(int n, int t) { return (n + t - 1) / t; }

void launch_frames_from_coords(const KParams &P, const float *c7, float4 *frame, cudaStream_t s) {
    k_frames_from_coords<<<blocks(P.nb, 256), 256, 0, s>>>(P, c7, frame);
}
void launch_coords_from_frames(const KParams &P, const float4 *frame, float *c7, cudaStream_t s) {
    k_coords_from_frames<<<blocks(P.nb, 256), 256, 0, s>>>(P.nb, frame, c7);
}
void launch_forces_to_coords(const KParams &P, const float4 *force, float *c7, cudaStream_t s) {
    k_forces_to_coords<<<blocks(P.nb, 256), 256, 0, s>>>(P.nb, force, c7);
}
void launch_step_plain(const KParams &P, const DevBuffers &B, bool keep_forces, cudaStream_t s) {
    const int t = P.step_block > 0 ? P.step_block : 128;
    if (keep_forces)
        k_step_plain<true><<<blocks(P.nb, t), t, 0, s>>>(P, B);
    else
        k_step_plain<false><<<blocks(P.nb, t), t, 0, s>>>(P, B);
}
size_t period_smem_bytes(int nmax) { return (size_t)nmax * (4 * sizeof(float4) + sizeof(int)); }
bool period_fits(int nmax) {
    return nmax > 0 && nmax <= kPeriodThreads * kPeriodBeads && period_smem_bytes(nmax) <= kPeriodMaxSmem;
}
int period_prepare(int nmax) {
    const int bytes = (int)period_smem_bytes(nmax);
    if (cudaFuncSetAttribute(k_step_period<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_step_period<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
        return -1;
    return 0;
}
bool period_rebuilds(int nmax) { return nmax <= kPeriodRebuildMax; }
void launch_step_period(const KParams &P, const DevBuffers &B, bool keep_forces, int nsteps, int nmax, bool rebuild,
                        cudaStream_t s) {
    int t = ((nmax + 31) / 32) * 32;
    if (t > kPeriodThreads) t = kPeriodThreads;
    const size_t bytes = period_smem_bytes(nmax);
    if (keep_forces)
        k_step_period<true><<<P.nt, t, bytes, s>>>(P, B, nsteps, nmax, rebuild ? 1 : 0);
    else
        k_step_period<false><<<P.nt, t, bytes, s>>>(P, B, nsteps, nmax, rebuild ? 1 : 0);
}

void launch_forces(const KParams &P, const DevBuffers &B, bool tea_prepare, cudaStream_t s) {
    if (tea_prepare)
        k_forces<true><<<blocks(P.nb, 128), 128, 0, s>>>(P, B);
    else
        k_forces<false><<<blocks(P.nb, 128), 128, 0, s>>>(P, B);
}
void launch_energy(const KParams &P, const DevBuffers &B, double *per_bead, double *partials, const int2 *work,
                   int nwork, cudaStream_t s) {
    k_energy<<<nwork, kTile, 0, s>>>(P, B, work, per_bead, partials);
}
void launch_energy_totals(const KParams &P, const double *partials, const int *work_first, double *per_traj,
                          int *err, cudaStream_t s) {
    k_energy_totals<<<blocks(P.nt, 128), 128, 0, s>>>(P.nt, partials, work_first, per_traj, err);
}
void launch_set_flags(int nb, const uint8_t *extra, const int *gtp, const int *ontub, int *flags, cudaStream_t s) {
    k_set_flags<<<blocks(nb, 256), 256, 0, s>>>(nb, extra, gtp, ontub, flags);
}

}  // namespace mtg
