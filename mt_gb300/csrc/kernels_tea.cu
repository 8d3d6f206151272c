// kernels_tea.cu - TEA hydrodynamics (Geyer & Winter 2009): the all-pairs
// epsilon / C_i pass, the FP64 epsilon -> beta reduction, and the all-pairs
// RPY mobility product fused with the position update.
//
// Both O(N^2) kernels run one CTA per (trajectory, chunk of kTeaChunk beads)
// and stream the trajectory through shared memory in tiles of kTeaTile
// beads j.  A thread serves kTeaNI beads i (lanes il, il + 32, ...) as packed
// FP32x2 pairs; `tea_slices` threads share each bead i and take interleaved
// j of every tile, so small batches still fill the GPU, and the partial sums
// meet in shared memory.  The tile holds every value of bead j twice (both
// lanes of a packed operand, two operands per 16-byte word), so broadcast
// loads feed the packed pairs of beads i directly.  Away from the CTA's own
// beads the far-field formula runs for every pair; the few overlapping pairs
// (r <= 2a) are found through running minima of r^2, one per quarter of a
// thread's j values, and only a quarter that holds one is rescanned with the
// near-field formula.  With tea_jparts > 1 the work items of the last waves
// are split over parts of their j range (see tea_item).  In the tile that holds
// the CTA's own beads the self pairs get r^2 = 1e30: their terms are then
// far below the rounding of the sums, and the correction skips them.
// Sums are kept in units of 0.75 a (T' = T / (0.75 a)).  The kernels are
// bound by the FP32 pipe (about 45 FLOP per ordered pair).
#include "mtg_internal.cuh"

namespace mtg {

constexpr int kTeaNI = 4;                   // beads i per thread
constexpr int kTeaPairsI = kTeaNI / 2;      // packed pairs of them
constexpr int kTeaLanes = 32;               // threads per slice
constexpr int kTeaSeg = 4;                  // segments of a thread's j values, each with its own r^2 minimum
constexpr int kTeaI = kTeaChunk;            // beads i per CTA
static_assert(kTeaI == kTeaLanes * kTeaNI, "chunk = lanes x beads per thread");
constexpr int kTeaTile = 128;               // beads j per tile
constexpr float kFarAway = 1.0e18f;         // position of padding and extra beads j

// Tile of the all-pairs kernels, every value duplicated into both lanes of
// a packed pair and two pairs per 16-byte word, so that a bead j takes five
// shared-memory loads (two without F and R).  Beads past the trajectory's end
// and extra beads sit far away with zero F and R: every term they give is
// zero or below the rounding of the sums.
struct TeaTile {
    float4 xy[kTeaTile];   // x x y y
    float4 zf[kTeaTile];   // z z Fx Fx
    float4 fyz[kTeaTile];  // Fy Fy Fz Fz
    float4 rxy[kTeaTile];  // Rx Rx Ry Ry
    float2 rz[kTeaTile];   // Rz Rz
};
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

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
        T.xy[k] = make_float4(p.x, p.x, p.y, p.y);
        T.zf[k] = make_float4(p.z, p.z, F.x, F.x);
        if (WITH_FR) {
            T.fyz[k] = make_float4(F.y, F.y, F.z, F.z);
            T.rxy[k] = make_float4(R.x, R.x, R.y, R.y);
            T.rz[k] = f2(R.z);
        }
    }
}

// Scaled RPY coefficients (integrateTea_RPY, src/bdhitea_kernel.cu:38-58:
// T = cii I + crr u u^T, ra = r/a; ra > 2: cii = 0.75/ra (1 + 2/(3 ra^2)),
// crr = 0.75/ra (1 - 2/ra^2); otherwise cii = 1 - 9 ra/32, crr = 3 ra/32),
// divided by 0.75 a.  With rinv = 1/r, q = rinv^2, t = q rinv the far field
// is cii' = rinv + (2/3) a^2 t and crr' = rinv - 2 a^2 t.
struct TeaConst {
    float kap, two_a2, four_a2, inv_a, inv_c075a, c075a;
};
__device__ __forceinline__ TeaConst tea_const(float a) {
    return {(2.0f / 3.0f) * a * a, 2.0f * a * a, 4.0f * a * a, 1.0f / a, 1.0f / (0.75f * a), 0.75f * a};
}
// near branch (r <= 2a): scaled cii', crr'
__device__ __forceinline__ void rpy_near(const TeaConst &K, float r2, float rinv, float &cii, float &crr) {
    const float ra = r2 * rinv * K.inv_a;
    cii = (1.0f - (9.0f / 32.0f) * ra) * K.inv_c075a;
    crr = (3.0f / 32.0f) * ra * K.inv_c075a;
}

// ------------------------------------------------------------ epsilon pass
// Scaled epsilon terms of one pair from cii', crr', q: the row sums of
// squares minus cii'^2 (Bc d_c^2 with Bc = (2 cii' + crr') crr' q), cii'^2, and
// the sum of all nine entries 3 cii' + crr' q (d_x + d_y + d_z)^2.
struct EpsTerms {
    float bx, by, bz, a2, w;
};
__device__ __forceinline__ EpsTerms eps_terms(float dx, float dy, float dz, float cii, float crr, float q) {
    const float crq = crr * q;
    const float bc = fmaf(2.0f, cii, crr) * crq;
    const float us = dx + dy + dz;
    return {bc * dx * dx, bc * dy * dy, bc * dz * dz, cii * cii, fmaf(crq * us, us, 3.0f * cii)};
}

// Range of beads j of part `part` of `parts` of a trajectory [base, end):
// whole tiles, the parts as equal as the tile count allows.
__device__ __forceinline__ void tea_jrange(int base, int end, int part, int parts, int &jb, int &je) {
    const int ntiles = (end - base + kTeaTile - 1) / kTeaTile;
    const int per = (ntiles + parts - 1) / parts;
    jb = min(end, base + part * per * kTeaTile);
    je = min(end, base + (part + 1) * per * kTeaTile);
}

// Work item and j part of this CTA.  The first P.tea_nhead items run whole;
// with SPLIT every later item runs as P.tea_jparts CTAs over parts of its j
// range, so that the last waves of a launch are made of short CTAs.
template <bool SPLIT>
__device__ __forceinline__ void tea_item(const KParams &P, int &item, int &part, int &parts) {
    item = (int)blockIdx.x;
    part = 0;
    parts = 1;
    if (SPLIT && item >= P.tea_nhead) {
        const int k = item - P.tea_nhead;
        item = P.tea_nhead + k / P.tea_jparts;
        part = k % P.tea_jparts;
        parts = P.tea_jparts;
    }
}
// Bead of a finish kernel (one CTA of kTeaChunk threads per split item), or -1.
__device__ __forceinline__ int tea_tail_bead(const KParams &P, const DevBuffers &B, const int2 *work) {
    const int2 w = work[P.tea_nhead + blockIdx.x];
    const int g = w.y + (int)threadIdx.x;
    return g < B.off[w.x + 1] ? g : -1;
}

// Stores the epsilon-pass result of bead g from its scaled sums
// (x, y, z: row sums of squares; w: sum of all entries).
__device__ __forceinline__ void eps_store(const KParams &P, const DevBuffers &B, int g, bool active, float4 acc,
                                          const TeaConst &K) {
    const float c2 = K.c075a * K.c075a;
    if (!active) acc = make_float4(0.f, 0.f, 0.f, 0.f);
    B.tea_ci[g] = make_float4(acc.x * c2, acc.y * c2, acc.z * c2, 0.f);
    B.tea_eps[g] = acc.w * K.c075a;
}

// The packed pass of one tile of the epsilon pass (self pairs pushed to
// r^2 = 1e30 when SELF), running minimum of r^2 per bead pair.
template <int SLICES, bool SELF>
__device__ __forceinline__ void tea_eps_tile(const TeaTile &T, int sl, int self_t, const float2 (&nx)[kTeaPairsI],
                                             const float2 (&ny)[kTeaPairsI], const float2 (&nz)[kTeaPairsI],
                                             float2 vkap, float2 vn2a2, float2 two, float2 three,
                                             float2 (&sx)[kTeaPairsI], float2 (&sy)[kTeaPairsI],
                                             float2 (&sz)[kTeaPairsI], float2 (&sa)[kTeaPairsI],
                                             float2 (&sw)[kTeaPairsI], float (&rmin)[kTeaPairsI][kTeaSeg]) {
    constexpr int kLen = kTeaTile / SLICES / kTeaSeg;
#pragma unroll
    for (int sg = 0; sg < kTeaSeg; sg++) {
#pragma unroll 2
        for (int k = 0; k < kLen; k++) {
            const int t = sl + (sg * kLen + k) * SLICES;
            const float4 a = T.xy[t];
            const float2 xj = lo2(a), yj = hi2(a), zj = lo2(T.zf[t]);
#pragma unroll
            for (int p = 0; p < kTeaPairsI; p++) {
                const float2 dx = __fadd2_rn(xj, nx[p]), dy = __fadd2_rn(yj, ny[p]), dz = __fadd2_rn(zj, nz[p]);
                float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                if (SELF) {
                    if (t == self_t + kTeaLanes * 2 * p) r2.x = 1e30f;
                    if (t == self_t + kTeaLanes * (2 * p + 1)) r2.y = 1e30f;
                }
                rmin[p][sg] = fmin3(rmin[p][sg], r2.x, r2.y);
                const float2 rinv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
                const float2 q = __fmul2_rn(rinv, rinv);
                const float2 tq = __fmul2_rn(q, rinv);
                const float2 cii = __ffma2_rn(vkap, tq, rinv);
                const float2 crr = __ffma2_rn(vn2a2, tq, rinv);
                const float2 crq = __fmul2_rn(crr, q);
                const float2 bc = __fmul2_rn(__ffma2_rn(two, cii, crr), crq);
                sa[p] = __ffma2_rn(cii, cii, sa[p]);
                sx[p] = __ffma2_rn(__fmul2_rn(bc, dx), dx, sx[p]);
                sy[p] = __ffma2_rn(__fmul2_rn(bc, dy), dy, sy[p]);
                sz[p] = __ffma2_rn(__fmul2_rn(bc, dz), dz, sz[p]);
                const float2 us = __fadd2_rn(__fadd2_rn(dx, dy), dz);
                sw[p] = __ffma2_rn(__fmul2_rn(crq, us), us, __ffma2_rn(three, cii, sw[p]));
            }
        }
    }
}

// integrateTea_epsilon_unlisted (src/bdhitea_kernel.cu:84-101): per bead i,
// sum over non-extra j != i of the row sums of squared entries (-> tea_ci)
// and of all nine entries (-> tea_eps).  With T = cii I + crr u u^T the row
// sums of squares are cii^2 + (2 cii + crr) crr u_c^2 and the sum of all
// entries is 3 cii + crr (u_x + u_y + u_z)^2.
template <int SLICES, bool SPLIT>
__global__ void __launch_bounds__(kTeaLanes *SLICES, 20 / SLICES) k_tea_eps(KParams P, DevBuffers B, const int2 *work,
                                                                const int *gate, int run_if) {
    if (gate && *gate != run_if) return;
    int item, part, parts;
    tea_item<SPLIT>(P, item, part, parts);
    const int2 w = work[item];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    int jb, je;
    tea_jrange(base, end, part, parts, jb, je);
    const int il = threadIdx.x % kTeaLanes, sl = threadIdx.x / kTeaLanes;
    __shared__ TeaTile T;
    __shared__ float4 s_red[kTeaI * SLICES];
    int gi[kTeaNI];
    bool act[kTeaNI];
    float4 pi[kTeaNI];
    float2 nx[kTeaPairsI], ny[kTeaPairsI], nz[kTeaPairsI];
    float2 sx[kTeaPairsI], sy[kTeaPairsI], sz[kTeaPairsI], sa[kTeaPairsI], sw[kTeaPairsI];
    bool any_act = false;
#pragma unroll
    for (int h = 0; h < kTeaNI; h++) {
        gi[h] = w.y + il + h * kTeaLanes;
        act[h] = false;
        pi[h] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gi[h] < end) {
            pi[h] = B.frame_in[gi[h]];
            act[h] = (B.flags[gi[h]] & kFlagExtra) == 0;
        }
        any_act |= act[h];
    }
#pragma unroll
    for (int p = 0; p < kTeaPairsI; p++) {
        nx[p] = make_float2(-pi[2 * p].x, -pi[2 * p + 1].x);
        ny[p] = make_float2(-pi[2 * p].y, -pi[2 * p + 1].y);
        nz[p] = make_float2(-pi[2 * p].z, -pi[2 * p + 1].z);
        sx[p] = sy[p] = sz[p] = sa[p] = sw[p] = f2(0.f);
    }
    const TeaConst K = tea_const(P.tea_a);
    const float2 vkap = f2(K.kap), vn2a2 = f2(-K.two_a2), two = f2(2.0f), three = f2(3.0f);
    for (int j0 = jb; j0 < je; j0 += kTeaTile) {
        tea_tile_load<false>(T, B, j0, end);
        __syncthreads();
        if (any_act) {
            // self pairs: as in k_tea_step
            const bool self_tile = (w.y < j0 + kTeaTile) && (w.y + kTeaI > j0);
            const int self_t = self_tile ? w.y - j0 + il : -(1 << 30);
            float rmin[kTeaPairsI][kTeaSeg];
#pragma unroll
            for (int p = 0; p < kTeaPairsI; p++)
#pragma unroll
                for (int sg = 0; sg < kTeaSeg; sg++) rmin[p][sg] = 3.4e38f;
            if (self_tile)
                tea_eps_tile<SLICES, true>(T, sl, self_t, nx, ny, nz, vkap, vn2a2, two, three, sx, sy, sz, sa, sw,
                                           rmin);
            else
                tea_eps_tile<SLICES, false>(T, sl, self_t, nx, ny, nz, vkap, vn2a2, two, three, sx, sy, sz, sa, sw,
                                            rmin);
            // overlapping pairs (r <= 2a): replace the far-field terms by the near ones
#pragma unroll
            for (int p = 0; p < kTeaPairsI; p++) {
                unsigned segs = 0;
#pragma unroll
                for (int sg = 0; sg < kTeaSeg; sg++) segs |= (rmin[p][sg] <= K.four_a2 ? 1u : 0u) << sg;
                constexpr int kLen = kTeaTile / SLICES / kTeaSeg;
                while (segs) {  // the segments that hold an overlapping pair
                    const int sg = __ffs(segs) - 1;
                    segs &= segs - 1;
                    for (int k = 0; k < kLen; k++) {
                        const int t = sl + (sg * kLen + k) * SLICES;
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            if (t == self_t + kTeaLanes * (2 * p + e)) continue;
                            const float ax = e ? nx[p].y : nx[p].x, ay = e ? ny[p].y : ny[p].x,
                                        az = e ? nz[p].y : nz[p].x;
                            const float dx = T.xy[t].x + ax, dy = T.xy[t].z + ay, dz = T.zf[t].x + az;
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            if (!(r2 <= K.four_a2)) continue;
                            const float rinv = rsqrt_hw(r2), q = rinv * rinv, tq = q * rinv;
                            const EpsTerms f = eps_terms(dx, dy, dz, fmaf(K.kap, tq, rinv), fmaf(-K.two_a2, tq, rinv), q);
                            float cn, rn;
                            rpy_near(K, r2, rinv, cn, rn);
                            const EpsTerms n = eps_terms(dx, dy, dz, cn, rn, q);
                            if (e) {
                                sx[p].y += n.bx - f.bx;
                                sy[p].y += n.by - f.by;
                                sz[p].y += n.bz - f.bz;
                                sa[p].y += n.a2 - f.a2;
                                sw[p].y += n.w - f.w;
                            } else {
                                sx[p].x += n.bx - f.bx;
                                sy[p].x += n.by - f.by;
                                sz[p].x += n.bz - f.bz;
                                sa[p].x += n.a2 - f.a2;
                                sw[p].x += n.w - f.w;
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int h = 0; h < kTeaNI; h++) {
        const int p = h >> 1;
        const bool hi = h & 1;
        const float A = hi ? sa[p].y : sa[p].x;
        s_red[(sl * kTeaNI + h) * kTeaLanes + il] =
            make_float4((hi ? sx[p].y : sx[p].x) + A, (hi ? sy[p].y : sy[p].x) + A, (hi ? sz[p].y : sz[p].x) + A,
                        hi ? sw[p].y : sw[p].x);
    }
    __syncthreads();
    if (sl != 0) return;
#pragma unroll
    for (int h = 0; h < kTeaNI; h++) {
        if (gi[h] >= end) continue;
        float4 acc = s_red[h * kTeaLanes + il];
        for (int k = 1; k < SLICES; k++) {
            const float4 v = s_red[(k * kTeaNI + h) * kTeaLanes + il];
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
        }
        if (SPLIT && parts > 1)
            B.tea_part[(size_t)part * P.nb + gi[h]] = acc;
        else
            eps_store(P, B, gi[h], act[h], acc, K);
    }
}

// Sums of the parts of a split epsilon pass.
__global__ void k_tea_eps_finish(KParams P, DevBuffers B, const int2 *work, const int *gate, int run_if) {
    if (gate && *gate != run_if) return;
    const int g = tea_tail_bead(P, B, work);
    if (g < 0) return;
    float4 acc = B.tea_part[g];
    for (int k = 1; k < P.tea_jparts; k++) {
        const float4 v = B.tea_part[(size_t)k * P.nb + g];
        acc.x += v.x;
        acc.y += v.y;
        acc.z += v.z;
        acc.w += v.w;
    }
    eps_store(P, B, g, (B.flags[g] & kFlagExtra) == 0, acc, tea_const(P.tea_a));
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

// ------------------------------------------------------- mobility product
// Scaled far-field term of one pair in scalar arithmetic, the operations of
// one lane of the packed loop in the same order.
__device__ __forceinline__ float3 tea_far1(const TeaConst &K, float dx, float dy, float dz, float gx, float gy,
                                           float gz) {
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float rinv = rsqrt_hw(r2), q = rinv * rinv, tq = q * rinv;
    const float cii = fmaf(K.kap, tq, rinv);
    const float cr = tq * fmaf(-K.two_a2, q, 1.0f);
    const float s = cr * fmaf(dx, gx, fmaf(dy, gy, dz * gz));
    return make_float3(fmaf(cii, gx, s * dx), fmaf(cii, gy, s * dy), fmaf(cii, gz, s * dz));
}
// Scaled term of one pair with both branches (r2 > 0).
__device__ __forceinline__ float3 tea_pair1(const TeaConst &K, float dx, float dy, float dz, float gx, float gy,
                                            float gz) {
    const float r2 = fmaxf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), 1e-6f);
    const float rinv = rsqrt_hw(r2), q = rinv * rinv, tq = q * rinv;
    float cii = fmaf(K.kap, tq, rinv);
    float cr = tq * fmaf(-K.two_a2, q, 1.0f);
    if (r2 <= K.four_a2) {
        float crr;
        rpy_near(K, r2, rinv, cii, crr);
        cr = crr * q;
    }
    const float s = cr * fmaf(dx, gx, fmaf(dy, gy, dz * gz));
    return make_float3(fmaf(cii, gx, s * dx), fmaf(cii, gy, s * dy), fmaf(cii, gz, s * dz));
}

// The packed pass of one tile: far-field terms of every pair (self pairs
// pushed to r^2 = 1e30 when SELF), running minimum of r^2 per bead pair.
template <int SLICES, bool SELF>
__device__ __forceinline__ void tea_step_tile(const TeaTile &T, int sl, int self_t, const float2 (&nx)[kTeaPairsI],
                                              const float2 (&ny)[kTeaPairsI], const float2 (&nz)[kTeaPairsI],
                                              const float2 (&cbx)[kTeaPairsI], const float2 (&cby)[kTeaPairsI],
                                              const float2 (&cbz)[kTeaPairsI], float2 vkap, float2 vn2a2,
                                              float2 one, float2 (&ax)[kTeaPairsI], float2 (&ay)[kTeaPairsI],
                                              float2 (&az)[kTeaPairsI], float (&rmin)[kTeaPairsI][kTeaSeg]) {
    constexpr int kLen = kTeaTile / SLICES / kTeaSeg;
#pragma unroll
    for (int sg = 0; sg < kTeaSeg; sg++) {
#pragma unroll(kLen <= 8 ? kLen : 2)
        for (int k = 0; k < kLen; k++) {
            const int t = sl + (sg * kLen + k) * SLICES;
            const float4 a = T.xy[t], b = T.zf[t], c = T.fyz[t], d = T.rxy[t];
            const float2 xj = lo2(a), yj = hi2(a), zj = lo2(b);
            const float2 fxj = hi2(b), fyj = lo2(c), fzj = hi2(c);
            const float2 rxj = lo2(d), ryj = hi2(d), rzj = T.rz[t];
#pragma unroll
            for (int p = 0; p < kTeaPairsI; p++) {
                const float2 dx = __fadd2_rn(xj, nx[p]), dy = __fadd2_rn(yj, ny[p]), dz = __fadd2_rn(zj, nz[p]);
                const float2 gx = __ffma2_rn(rxj, cbx[p], fxj), gy = __ffma2_rn(ryj, cby[p], fyj),
                             gz = __ffma2_rn(rzj, cbz[p], fzj);
                float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                if (SELF) {
                    if (t == self_t + kTeaLanes * 2 * p) r2.x = 1e30f;
                    if (t == self_t + kTeaLanes * (2 * p + 1)) r2.y = 1e30f;
                }
                rmin[p][sg] = fmin3(rmin[p][sg], r2.x, r2.y);
                const float2 rinv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
                const float2 q = __fmul2_rn(rinv, rinv);
                const float2 tq = __fmul2_rn(q, rinv);
                const float2 cii = __ffma2_rn(vkap, tq, rinv);
                const float2 cr = __fmul2_rn(tq, __ffma2_rn(vn2a2, q, one));
                const float2 s = __fmul2_rn(cr, __ffma2_rn(dx, gx, __ffma2_rn(dy, gy, __fmul2_rn(dz, gz))));
                ax[p] = __ffma2_rn(cii, gx, __ffma2_rn(s, dx, ax[p]));
                ay[p] = __ffma2_rn(cii, gy, __ffma2_rn(s, dy, ay[p]));
                az[p] = __ffma2_rn(cii, gz, __ffma2_rn(s, dz, az[p]));
            }
        }
    }
}

// The update of bead g from its scaled mobility sums (sx, sy, sz): back to
// units of D_ii, plus the bead's own term F_i + C_i o R_i; FEFF stores f_i.
template <bool FEFF>
__device__ __forceinline__ void tea_bead_update(const KParams &P, const DevBuffers &B, int g, float sx, float sy,
                                                float sz, float b2, const TeaConst &K, float4 *feff) {
    const int nb = P.nb;
    const float4 ci = B.tea_ci[g], Fi = B.force[g], Ri = B.tea_r[g];
    sx = fmaf(K.c075a, sx, Fi.x + Ri.x * (1.0f / sqrtf(1.0f + b2 * ci.x)));
    sy = fmaf(K.c075a, sy, Fi.y + Ri.y * (1.0f / sqrtf(1.0f + b2 * ci.y)));
    sz = fmaf(K.c075a, sz, Fi.z + Ri.z * (1.0f / sqrtf(1.0f + b2 * ci.z)));
    if (FEFF) {
        feff[g] = make_float4(sx, sy, sz, 0.f);
        return;
    }
    const int flags = B.flags[g];
    Frame Fr;
    Fr.p0 = B.frame_in[g];
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

// integrateTea_kernel_unlisted + integrateTea_force (src/bdhitea_kernel.cu:104-213):
// f_i = F_i + C_i o R_i + sum_{j != i, non-extra} T_ij (F_j + beta C_i o R_j),
// x_i += dt/gammaR f_i; angles by Euler-Maruyama from stream i + nb, which is
// drawn for every bead.  Reads the current frame, writes the next one.  With
// FEFF the kernel stores f_i instead and moves nothing.
template <int SLICES, bool FEFF, bool SPLIT>
__global__ void __launch_bounds__(kTeaLanes *SLICES, 20 / SLICES) k_tea_step(KParams P, DevBuffers B, const int2 *work,
                                                                 float4 *feff, const int *gate) {
    if (FEFF && gate && *gate != 0) return;
    if (!FEFF && gate && *gate == 0) return;   // the gated update runs after a fall-back only
    int item, part, parts;
    tea_item<SPLIT>(P, item, part, parts);
    const int2 w = work[item];
    const int traj = w.x, base = B.off[traj], end = B.off[traj + 1];
    int jb, je;
    tea_jrange(base, end, part, parts, jb, je);
    const int il = threadIdx.x % kTeaLanes, sl = threadIdx.x / kTeaLanes;
    const int nb = P.nb;
    __shared__ TeaTile T;
    __shared__ float4 s_red[kTeaI * SLICES];

    // per packed pair p of beads i (2p, 2p+1): -position, beta C_i, sums
    float2 nx[kTeaPairsI], ny[kTeaPairsI], nz[kTeaPairsI], cbx[kTeaPairsI], cby[kTeaPairsI], cbz[kTeaPairsI];
    float2 ax[kTeaPairsI], ay[kTeaPairsI], az[kTeaPairsI];
    bool any_act = false;
    const float beta = B.tea_beta[traj], b2 = beta * beta;
#pragma unroll
    for (int h = 0; h < kTeaNI; h++) {
        const int g = w.y + il + h * kTeaLanes;
        float4 p = make_float4(0.f, 0.f, 0.f, 0.f), c = p;
        if (g < end) {
            p = B.frame_in[g];
            any_act |= (B.flags[g] & kFlagExtra) == 0;
            const float4 ci = B.tea_ci[g];
            c = make_float4(beta / sqrtf(1.0f + b2 * ci.x), beta / sqrtf(1.0f + b2 * ci.y),
                            beta / sqrtf(1.0f + b2 * ci.z), 0.f);
        }
        float2 *v[6] = {&nx[h >> 1], &ny[h >> 1], &nz[h >> 1], &cbx[h >> 1], &cby[h >> 1], &cbz[h >> 1]};
        const float val[6] = {-p.x, -p.y, -p.z, c.x, c.y, c.z};
#pragma unroll
        for (int k = 0; k < 6; k++) {
            if (h & 1)
                v[k]->y = val[k];
            else
                v[k]->x = val[k];
        }
    }
#pragma unroll
    for (int p = 0; p < kTeaPairsI; p++) ax[p] = ay[p] = az[p] = f2(0.f);
    const TeaConst K = tea_const(P.tea_a);
    const float2 vkap = f2(K.kap), vn2a2 = f2(-K.two_a2), one = f2(1.0f);
    for (int j0 = jb; j0 < je; j0 += kTeaTile) {
        tea_tile_load<true>(T, B, j0, end);
        __syncthreads();
        if (any_act) {
            // the tile that holds this CTA's beads: bead h of this thread sits
            // at tile index self_t + 32 h, and its self pair gets r^2 = 1e30
            // (a far-away term that is below the rounding of the sums)
            const bool self_tile = (w.y < j0 + kTeaTile) && (w.y + kTeaI > j0);
            const int self_t = self_tile ? w.y - j0 + il : -(1 << 30);
            float rmin[kTeaPairsI][kTeaSeg];
#pragma unroll
            for (int p = 0; p < kTeaPairsI; p++)
#pragma unroll
                for (int sg = 0; sg < kTeaSeg; sg++) rmin[p][sg] = 3.4e38f;
            if (self_tile)
                tea_step_tile<SLICES, true>(T, sl, self_t, nx, ny, nz, cbx, cby, cbz, vkap, vn2a2, one, ax, ay, az,
                                            rmin);
            else
                tea_step_tile<SLICES, false>(T, sl, self_t, nx, ny, nz, cbx, cby, cbz, vkap, vn2a2, one, ax, ay, az,
                                             rmin);
            // overlapping pairs (r <= 2a): replace the far-field term by the near one
#pragma unroll
            for (int p = 0; p < kTeaPairsI; p++) {
                unsigned segs = 0;
#pragma unroll
                for (int sg = 0; sg < kTeaSeg; sg++) segs |= (rmin[p][sg] <= K.four_a2 ? 1u : 0u) << sg;
                constexpr int kLen = kTeaTile / SLICES / kTeaSeg;
                while (segs) {  // the segments that hold an overlapping pair
                    const int sg = __ffs(segs) - 1;
                    segs &= segs - 1;
                    for (int k = 0; k < kLen; k++) {
                        const int t = sl + (sg * kLen + k) * SLICES;
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            if (t == self_t + kTeaLanes * (2 * p + e)) continue;
                            const float dx = T.xy[t].x + (e ? nx[p].y : nx[p].x),
                                        dy = T.xy[t].z + (e ? ny[p].y : ny[p].x),
                                        dz = T.zf[t].x + (e ? nz[p].y : nz[p].x);
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            if (!(r2 <= K.four_a2)) continue;
                            const float gx = fmaf(T.rxy[t].x, e ? cbx[p].y : cbx[p].x, T.zf[t].z),
                                        gy = fmaf(T.rxy[t].z, e ? cby[p].y : cby[p].x, T.fyz[t].x),
                                        gz = fmaf(T.rz[t].x, e ? cbz[p].y : cbz[p].x, T.fyz[t].z);
                            const float3 fa = tea_far1(K, dx, dy, dz, gx, gy, gz);
                            const float3 nr = tea_pair1(K, dx, dy, dz, gx, gy, gz);
                            if (e) {
                                ax[p].y += nr.x - fa.x;
                                ay[p].y += nr.y - fa.y;
                                az[p].y += nr.z - fa.z;
                            } else {
                                ax[p].x += nr.x - fa.x;
                                ay[p].x += nr.y - fa.y;
                                az[p].x += nr.z - fa.z;
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int h = 0; h < kTeaNI; h++) {
        const int p = h >> 1;
        const bool hi = h & 1;
        s_red[(sl * kTeaNI + h) * kTeaLanes + il] =
            make_float4(hi ? ax[p].y : ax[p].x, hi ? ay[p].y : ay[p].x, hi ? az[p].y : az[p].x, 0.f);
    }
    __syncthreads();
    if (sl != 0) return;
#pragma unroll
    for (int h = 0; h < kTeaNI; h++) {
        const int g = w.y + il + h * kTeaLanes;
        if (g >= end) continue;
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int k = 0; k < SLICES; k++) {
            const float4 v = s_red[(k * kTeaNI + h) * kTeaLanes + il];
            sx += v.x;
            sy += v.y;
            sz += v.z;
        }
        if (SPLIT && parts > 1)
            B.tea_part[(size_t)part * nb + g] = make_float4(sx, sy, sz, 0.f);
        else
            tea_bead_update<FEFF>(P, B, g, sx, sy, sz, b2, K, feff);
    }
}

// Sums of the parts of a split mobility product, then the bead's update.
template <bool FEFF>
__global__ void k_tea_step_finish(KParams P, DevBuffers B, const int2 *work, float4 *feff, const int *gate) {
    if (FEFF && gate && *gate != 0) return;
    if (!FEFF && gate && *gate == 0) return;
    const int g = tea_tail_bead(P, B, work);
    if (g < 0) return;
    float4 acc = B.tea_part[g];
    for (int k = 1; k < P.tea_jparts; k++) {
        const float4 v = B.tea_part[(size_t)k * P.nb + g];
        acc.x += v.x;
        acc.y += v.y;
        acc.z += v.z;
    }
    const float beta = B.tea_beta[B.traj[g]];
    tea_bead_update<FEFF>(P, B, g, acc.x, acc.y, acc.z, beta * beta, tea_const(P.tea_a), feff);
}

// CTAs of kernel k that fit on the device at once.
template <typename Kern>
static int tea_slots(Kern k, int threads) {
    int dev = 0, sms = 1, occ = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, threads, 0);
    return (occ > 0 ? occ : 1) * sms;
}
// Items run whole: all but the last one to two waves' worth; grid of the launch.
static int tea_split_grid(KParams &Q, int nwork, int slots) {
    const int full = nwork / slots;
    Q.tea_nhead = full >= 2 ? (full - 1) * slots : 0;
    return Q.tea_nhead + (nwork - Q.tea_nhead) * Q.tea_jparts;
}

template <int SL>
static void tea_eps_launch(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, const int *gate,
                           int run_if, cudaStream_t s) {
    const int t = kTeaLanes * SL;
    KParams Q = P;
    if (P.tea_jparts > 1) {
        const int grid = tea_split_grid(Q, nwork, tea_slots(k_tea_eps<SL, true>, t));
        k_tea_eps<SL, true><<<grid, t, 0, s>>>(Q, B, work, gate, run_if);
        if (nwork > Q.tea_nhead) k_tea_eps_finish<<<nwork - Q.tea_nhead, kTeaChunk, 0, s>>>(Q, B, work, gate, run_if);
        return;
    }
    Q.tea_nhead = nwork;
    k_tea_eps<SL, false><<<nwork, t, 0, s>>>(Q, B, work, gate, run_if);
}
void launch_tea_eps_gated(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, const int *gate,
                          int run_if, cudaStream_t s) {
    switch (P.tea_slices) {
        case 1: tea_eps_launch<1>(P, B, work, nwork, gate, run_if, s); break;
        case 2: tea_eps_launch<2>(P, B, work, nwork, gate, run_if, s); break;
        case 4: tea_eps_launch<4>(P, B, work, nwork, gate, run_if, s); break;
        default: tea_eps_launch<8>(P, B, work, nwork, gate, run_if, s); break;
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
template <int SL, bool FEFF>
static void tea_step_launch(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, float4 *feff,
                            const int *gate, cudaStream_t s) {
    const int t = kTeaLanes * SL;
    KParams Q = P;
    if (P.tea_jparts > 1) {
        const int grid = tea_split_grid(Q, nwork, tea_slots(k_tea_step<SL, FEFF, true>, t));
        k_tea_step<SL, FEFF, true><<<grid, t, 0, s>>>(Q, B, work, feff, gate);
        if (nwork > Q.tea_nhead) k_tea_step_finish<FEFF><<<nwork - Q.tea_nhead, kTeaChunk, 0, s>>>(Q, B, work, feff, gate);
        return;
    }
    Q.tea_nhead = nwork;
    k_tea_step<SL, FEFF, false><<<nwork, t, 0, s>>>(Q, B, work, feff, gate);
}
template <bool FEFF>
static void tea_step_dispatch(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, float4 *feff,
                              const int *gate, cudaStream_t s) {
    switch (P.tea_slices) {
        case 1: tea_step_launch<1, FEFF>(P, B, work, nwork, feff, gate, s); break;
        case 2: tea_step_launch<2, FEFF>(P, B, work, nwork, feff, gate, s); break;
        case 4: tea_step_launch<4, FEFF>(P, B, work, nwork, feff, gate, s); break;
        default: tea_step_launch<8, FEFF>(P, B, work, nwork, feff, gate, s); break;
    }
}
void launch_tea_step(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s) {
    tea_step_dispatch<false>(P, B, work, nwork, nullptr, nullptr, s);
}
void launch_tea_step_gated(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, const int *gate,
                           cudaStream_t s) {
    tea_step_dispatch<false>(P, B, work, nwork, nullptr, gate, s);
}
void launch_tea_feff(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, float4 *feff,
                     const int *gate, cudaStream_t s) {
    tea_step_dispatch<true>(P, B, work, nwork, feff, gate, s);
}

// ---------------------------------------------- far field of learned TEA
// The learned mode's approximation of sum_j T_ij (F_j + beta C_i o R_j) on a
// k-d tree per trajectory (tea_ff.cu): pairs of beads in near leaves are
// summed exactly (the packed pair loop of k_tea_step, source beads in the two
// lanes), and every far node J acts on a target node N through proxies: J's
// sources are spread onto the 8 points of a Chebyshev grid in its bounding box
// (P2M, trilinear Lagrange weights at nodes +-h/sqrt(2)), the RPY far field
// of those 8 charges is evaluated at the 8 grid points of N (M2L), brought
// down to the leaves under N (L2L) and interpolated to their beads (L2P).
// Because C_i weights R_j per component and per target, the proxies carry F
// and R separately and the targets receive A = T Q_F and B_k = T e_k Q_R,k
// (k = x, y, z); a bead adds A + sum_k beta C_ik B_k.

// Tile of kFFTileLeaves source leaves (kFFPairSlots bead pairs each), in the
// layout of FFBuffers::pack: the two lanes of a packed pair are two source
// beads.  Filled from pack by asynchronous 16-byte copies.
constexpr int kFFTileLeaves = 4;   // 128 beads; tiles of 8 leaves measured slower (0.288 against 0.246 ms)
constexpr int kFFTileSlots = kFFPairSlots * kFFTileLeaves;
struct FFTile {
    float4 xy[kFFTileSlots];   // xa xb ya yb
    float4 zf[kFFTileSlots];   // za zb Fxa Fxb
    float4 fyz[kFFTileSlots];  // Fya Fyb Fza Fzb
    float4 rxy[kFFTileSlots];  // Rxa Rxb Rya Ryb
    float2 rz[kFFTileSlots];   // Rza Rzb
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Near-list entries a step CTA keeps in shared memory (longer lists are read
// from global memory).
constexpr int kFFNearSmem = 256;

// Issues the copies of near-list entries e0 .. min(e0 + kFFTileLeaves, e1) - 1
// (entries relative to the list's start) into tile T: each leaf is kFFPackF4
// contiguous float4 of pack.
__device__ __forceinline__ void ff_tile_issue(FFTile &T, const FFBuffers &F, const int *near, int e0, int e1) {
    constexpr int kPer = kFFPackF4;
    for (int c = threadIdx.x; c < kFFTileLeaves * kPer; c += blockDim.x) {
        const int q = c / kPer, w = c % kPer;
        const int e = e0 + q;
        if (e >= e1) continue;   // past the list: the tile pass skips the slot
        const int J = near[e];
        const float4 *src = F.pack + (size_t)J * kPer + w;
        float4 *dst;
        if (w < 4 * kFFPairSlots) {
            const int a = w / kFFPairSlots, k = q * kFFPairSlots + w % kFFPairSlots;
            dst = a == 0 ? &T.xy[k] : a == 1 ? &T.zf[k] : a == 2 ? &T.fyz[k] : &T.rxy[k];
        } else {
            dst = reinterpret_cast<float4 *>(&T.rz[q * kFFPairSlots + 2 * (w - 4 * kFFPairSlots)]);
        }
        cp_async16(dst, src);
    }
}

// Trilinear Lagrange weights of the 8 proxies (bit 0: x, bit 1: y, bit 2: z;
// a clear bit is the node at -h/sqrt(2), a set bit the one at +h/sqrt(2)) at
// position x of a box (c, h); the fast division's 2-ulp error is far below
// the interpolation's own.
__device__ __forceinline__ void ff_weights(float3 x, float4 c, float4 h, float w[8]) {
    const float tx = __fdividef(x.x - c.x, h.x * kFFNode), ty = __fdividef(x.y - c.y, h.y * kFFNode),
                tz = __fdividef(x.z - c.z, h.z * kFFNode);
    const float lx[2] = {0.5f * (1.0f - tx), 0.5f * (1.0f + tx)};
    const float ly[2] = {0.5f * (1.0f - ty), 0.5f * (1.0f + ty)};
    const float lz[2] = {0.5f * (1.0f - tz), 0.5f * (1.0f + tz)};
#pragma unroll
    for (int m = 0; m < 8; m++) w[m] = lx[m & 1] * ly[(m >> 1) & 1] * lz[(m >> 2) & 1];
}
__device__ __forceinline__ float3 ff_proxy(float4 c, float4 h, int m) {
    return make_float3(c.x + ((m & 1) ? kFFNode : -kFFNode) * h.x, c.y + ((m & 2) ? kFFNode : -kFFNode) * h.y,
                       c.z + ((m & 4) ? kFFNode : -kFFNode) * h.z);
}

__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sum over the 32 lanes of a warp of 32 values per lane, scattered: lane l
// ends with the sum of value l (recursive halving: at offset o a lane keeps
// the half of its values selected by bit o of its index and receives its
// partner's partial sums of that half; 31 shuffles instead of 160).
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16, n = 32; o > 0; o >>= 1, n >>= 1) {
        const bool up = lane & o;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            if (i >= n / 2) break;
            const float send = up ? v[i] : v[i + n / 2];
            const float keep = up ? v[i + n / 2] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
    return v[0];
}

constexpr int kP2MWarps = 4;   // warps of a P2M block, one node each

// Writes the 48 charge sums of a warp (acc[6m + v], summed per lane) as the
// node's proxy charges: (QF.xyz, QR.x) at float4 16N + m, (QR.y, QR.z) at
// 16N + 8 + m.
__device__ __forceinline__ void ff_store_charges(const FFBuffers &F, int N, float (&acc)[48]) {
    const int lane = threadIdx.x & 31;
    float lo[32], hi[32];
#pragma unroll
    for (int i = 0; i < 32; i++) lo[i] = acc[i];
#pragma unroll
    for (int i = 0; i < 16; i++) hi[i] = acc[32 + i];
#pragma unroll
    for (int i = 16; i < 32; i++) hi[i] = 0.f;
    const float s_lo = warp_reduce_scatter32(lo);   // value lane
    const float s_hi = warp_reduce_scatter32(hi);   // value 32 + lane (lanes < 16)
    float *q = reinterpret_cast<float *>(F.q);
    auto put = [&](int idx, float val) {
        const int m = idx / 6, c = idx % 6;
        q[(size_t)4 * (16 * N + (c < 4 ? m : 8 + m)) + (c < 4 ? c : c - 4)] = val;
    };
    put(lane, s_lo);
    if (lane < 16) put(32 + lane, s_hi);
}

// Writes lane k's bead (or an empty slot: far away, zero F and R) into leaf
// N's pack: lanes 2p and 2p + 1 swap their values and write bead pair p as
// whole 16-byte words (the even lane the position words, the odd lane the
// force and random-force words, the even lane Rz with its neighbour pair's).
// Called by all 32 lanes of the warp.
__device__ __forceinline__ void ff_pack_warp(const FFBuffers &F, int N, float3 x, float4 Fv, float4 R) {
    const int lane = threadIdx.x & 31, p = lane >> 1;
    const bool odd = lane & 1;
    const float v[9] = {x.x, x.y, x.z, Fv.x, Fv.y, Fv.z, R.x, R.y, R.z};
    float o[9];
#pragma unroll
    for (int i = 0; i < 9; i++) o[i] = __shfl_xor_sync(0xffffffffu, v[i], 1);
    // (a, b) = (even lane's bead, odd lane's bead)
    float a[9], b[9];
#pragma unroll
    for (int i = 0; i < 9; i++) {
        a[i] = odd ? o[i] : v[i];
        b[i] = odd ? v[i] : o[i];
    }
    float4 *pk = F.pack + (size_t)N * kFFPackF4;
    if (!odd) {
        pk[p] = make_float4(a[0], b[0], a[1], b[1]);                      // xa xb ya yb
        pk[kFFPairSlots + p] = make_float4(a[2], b[2], a[3], b[3]);       // za zb Fxa Fxb
    } else {
        pk[2 * kFFPairSlots + p] = make_float4(a[4], b[4], a[5], b[5]);   // Fya Fyb Fza Fzb
        pk[3 * kFFPairSlots + p] = make_float4(a[6], b[6], a[7], b[7]);   // Rxa Rxb Rya Ryb
    }
    // Rz of pairs p (lanes 4w, 4w+1) and p + 1 (lanes 4w+2, 4w+3) in one word
    const float rz2a = __shfl_down_sync(0xffffffffu, a[8], 2), rz2b = __shfl_down_sync(0xffffffffu, b[8], 2);
    if ((lane & 3) == 0) pk[4 * kFFPairSlots + (p >> 1)] = make_float4(a[8], b[8], rz2a, rz2b);
}

// P2M of the leaves, one warp per leaf (lane k: bead k): the bounding box,
// the proxy charges Q_m = sum_j w_m(x_j) (F_j, R_j), and the leaf's beads in
// the step kernel's tile layout (leaf nleaf: the padding leaf's pack).
__global__ void __launch_bounds__(32 * kP2MWarps) k_ff_p2m(KParams P, DevBuffers B, FFBuffers F, const int *gate) {
    if (gate && *gate != 0) return;
    const int N = blockIdx.x * kP2MWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (N > F.nleaf) return;
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 away = make_float3(kFarAway, kFarAway, kFarAway);
    if (N == F.nleaf) {
        ff_pack_warp(F, N, away, zero, zero);
        return;
    }
    const int b0 = F.leaf_start[N], n = F.leaf_start[N + 1] - b0;
    float3 x = make_float3(0.f, 0.f, 0.f);
    float4 Fv = zero, R = zero;
    if (lane < n) {
        const int g = F.leaf_bead[b0 + lane];
        x = f3(B.frame_in[g]);
        Fv = B.force[g];
        R = B.tea_r[g];
    }
    const float3 lo = make_float3(warp_min(lane < n ? x.x : 3.4e38f), warp_min(lane < n ? x.y : 3.4e38f),
                                  warp_min(lane < n ? x.z : 3.4e38f));
    const float3 hi = make_float3(warp_max(lane < n ? x.x : -3.4e38f), warp_max(lane < n ? x.y : -3.4e38f),
                                  warp_max(lane < n ? x.z : -3.4e38f));
    const float4 c = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.f);
    const float4 h = make_float4(fmaxf(0.5f * (hi.x - lo.x), 1e-3f), fmaxf(0.5f * (hi.y - lo.y), 1e-3f),
                                 fmaxf(0.5f * (hi.z - lo.z), 1e-3f), 0.f);
    ff_pack_warp(F, N, lane < n ? x : away, Fv, R);
    float w[8];
    ff_weights(x, c, h, w);
    const float val[6] = {Fv.x, Fv.y, Fv.z, R.x, R.y, R.z};
    float acc[48];
#pragma unroll
    for (int m = 0; m < 8; m++)
#pragma unroll
        for (int v = 0; v < 6; v++) acc[6 * m + v] = lane < n ? w[m] * val[v] : 0.f;
    ff_store_charges(F, N, acc);
    if (lane == 0) {
        F.box[2 * N] = c;
        F.box[2 * N + 1] = h;
    }
}

// P2M of the inner nodes, one warp per node, from the node's leaves: the
// bounding box is the union of theirs, and since trilinear interpolation on
// a leaf's proxies reproduces every trilinear function, the node's weights
// at the leaf proxies carry the leaf charges over exactly:
// Q^N_m = sum_leaves sum_k w^N_m(y_k) Q^leaf_k.
__global__ void __launch_bounds__(32 * kP2MWarps) k_ff_p2m_inner(KParams P, FFBuffers F, const int *gate) {
    if (gate && *gate != 0) return;
    const int k = blockIdx.x * kP2MWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (k >= F.ninner) return;
    const int N = F.inner[k];
    const int l0 = F.node_leaves[2 * N], l1 = F.node_leaves[2 * N + 1];
    float3 lo = make_float3(3.4e38f, 3.4e38f, 3.4e38f), hi = make_float3(-3.4e38f, -3.4e38f, -3.4e38f);
    for (int l = l0 + lane; l < l1; l += 32) {
        const float4 c = F.box[2 * l], h = F.box[2 * l + 1];
        lo = make_float3(fminf(lo.x, c.x - h.x), fminf(lo.y, c.y - h.y), fminf(lo.z, c.z - h.z));
        hi = make_float3(fmaxf(hi.x, c.x + h.x), fmaxf(hi.y, c.y + h.y), fmaxf(hi.z, c.z + h.z));
    }
    lo = make_float3(warp_min(lo.x), warp_min(lo.y), warp_min(lo.z));
    hi = make_float3(warp_max(hi.x), warp_max(hi.y), warp_max(hi.z));
    const float4 c = make_float4(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z), 0.f);
    const float4 h = make_float4(fmaxf(0.5f * (hi.x - lo.x), 1e-3f), fmaxf(0.5f * (hi.y - lo.y), 1e-3f),
                                 fmaxf(0.5f * (hi.z - lo.z), 1e-3f), 0.f);
    float acc[48];
#pragma unroll
    for (int i = 0; i < 48; i++) acc[i] = 0.f;
    // lane t takes proxy t % 8 of every fourth leaf
    for (int e = l0 * 8 + lane; e < l1 * 8; e += 32) {
        const int l = e >> 3, m = e & 7;
        const float3 y = ff_proxy(F.box[2 * l], F.box[2 * l + 1], m);
        const float4 qa = F.q[16 * l + m], qb = F.q[16 * l + 8 + m];
        const float val[6] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y};
        float w[8];
        ff_weights(y, c, h, w);
#pragma unroll
        for (int mm = 0; mm < 8; mm++)
#pragma unroll
            for (int v = 0; v < 6; v++) acc[6 * mm + v] = fmaf(w[mm], val[v], acc[6 * mm + v]);
    }
    ff_store_charges(F, N, acc);
    if (lane == 0) {
        F.box[2 * N] = c;
        F.box[2 * N + 1] = h;
    }
}

// M2L: 4 x kM2LSlices lanes per target node; lane t serves the target
// proxies t % 4 and t % 4 + 4 (the same x and y, opposite z) as one packed
// pair over every kM2LSlices-th far node, and the slices meet by shuffles in
// a fixed order.
constexpr int kM2LWarps = 4;
// 8 slices (a warp per target); 4 and 2 (two and four targets per warp)
// measured the same and slower
constexpr int kM2LSlices = 8, kM2LLanes = 4 * kM2LSlices;
__global__ void __launch_bounds__(32 * kM2LWarps) k_ff_m2l(KParams P, FFBuffers F, const int *gate) {
    if (gate && *gate != 0) return;
    const int lane = threadIdx.x & 31;
    const int wk = (blockIdx.x * kM2LWarps + (threadIdx.x >> 5)) * (32 / kM2LLanes) + lane / kM2LLanes;
    const bool active = wk < F.ntgt;
    const int L = active ? F.tgt[wk] : 0, t = lane % kM2LLanes, np = t & 3, sl = t >> 2;
    const TeaConst K = tea_const(P.tea_a);
    const float4 cL = F.box[2 * L], hL = F.box[2 * L + 1];
    const float3 x0 = ff_proxy(cL, hL, np), x1 = ff_proxy(cL, hL, np + 4);
    const float2 nxx = f2(-x0.x), nxy = f2(-x0.y), nxz = make_float2(-x0.z, -x1.z);
    const float2 vkap = f2(K.kap), vn2a2 = f2(-K.two_a2), one = f2(1.0f);
    float2 acc[12];
#pragma unroll
    for (int c = 0; c < 12; c++) acc[c] = f2(0.f);
    for (int k = F.far_start[L] + sl; active && k < F.far_start[L + 1]; k += kM2LSlices) {
        const int J = F.far[k];
        const float4 cJ = F.box[2 * J], hJ = F.box[2 * J + 1];
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const float3 y = ff_proxy(cJ, hJ, m);
            const float2 dx = __fadd2_rn(f2(y.x), nxx), dy = __fadd2_rn(f2(y.y), nxy), dz = __fadd2_rn(f2(y.z), nxz);
            const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
            const float2 rinv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
            const float2 q2 = __fmul2_rn(rinv, rinv), tq = __fmul2_rn(q2, rinv);
            const float2 cii = __ffma2_rn(vkap, tq, rinv);
            const float2 cr = __fmul2_rn(tq, __ffma2_rn(vn2a2, q2, one));
            const float4 qa = F.q[16 * J + m], qb = F.q[16 * J + 8 + m];
            const float2 qfx = f2(qa.x), qfy = f2(qa.y), qfz = f2(qa.z);
            const float2 sF = __fmul2_rn(cr, __ffma2_rn(dx, qfx, __ffma2_rn(dy, qfy, __fmul2_rn(dz, qfz))));
            acc[0] = __ffma2_rn(cii, qfx, __ffma2_rn(sF, dx, acc[0]));
            acc[1] = __ffma2_rn(cii, qfy, __ffma2_rn(sF, dy, acc[1]));
            acc[2] = __ffma2_rn(cii, qfz, __ffma2_rn(sF, dz, acc[2]));
            const float2 rx = f2(qa.w), ry = f2(qb.x), rz = f2(qb.y);
            const float2 s0 = __fmul2_rn(__fmul2_rn(cr, dx), rx), s1 = __fmul2_rn(__fmul2_rn(cr, dy), ry),
                         s2 = __fmul2_rn(__fmul2_rn(cr, dz), rz);
            acc[3] = __ffma2_rn(cii, rx, __ffma2_rn(s0, dx, acc[3]));
            acc[4] = __ffma2_rn(s0, dy, acc[4]);
            acc[5] = __ffma2_rn(s0, dz, acc[5]);
            acc[6] = __ffma2_rn(s1, dx, acc[6]);
            acc[7] = __ffma2_rn(cii, ry, __ffma2_rn(s1, dy, acc[7]));
            acc[8] = __ffma2_rn(s1, dz, acc[8]);
            acc[9] = __ffma2_rn(s2, dx, acc[9]);
            acc[10] = __ffma2_rn(s2, dy, acc[10]);
            acc[11] = __ffma2_rn(cii, rz, __ffma2_rn(s2, dz, acc[11]));
        }
    }
#pragma unroll
    for (int o = 4; o < kM2LLanes; o <<= 1)
#pragma unroll
        for (int c = 0; c < 12; c++) {
            acc[c].x += __shfl_xor_sync(0xffffffffu, acc[c].x, o);
            acc[c].y += __shfl_xor_sync(0xffffffffu, acc[c].y, o);
        }
    if (active && sl == 0) {
        float *phi = reinterpret_cast<float *>(F.phi) + (size_t)96 * L;
#pragma unroll
        for (int c = 0; c < 12; c++) {
            phi[12 * np + c] = acc[c].x;
            phi[12 * (np + 4) + c] = acc[c].y;
        }
    }
}

// Targets of one thread of the far-field step: TPT beads of the leaf, each
// with its negated position, its weights beta C_i (both duplicated into the
// two lanes of a packed pair), its packed sums, its own pair slot and lane.
template <int TPT>
struct FFTargets {
    float2 nx[TPT], ny[TPT], nz[TPT], cbx[TPT], cby[TPT], cbz[TPT];
    float2 ax[TPT], ay[TPT], az[TPT];
    int self_p[TPT], self_h[TPT];
};

// The packed pass of one tile: the thread's targets against the tile's bead
// pairs; with SELF a target's own slot is pushed to r^2 = 1e30, with TRACK
// the running minimum of r^2 per segment of the thread's pairs is kept.
// A thread takes the pair slots sl, sl + SLICES, ... of every leaf of the
// tile, leaf after leaf (so the order of its sums does not depend on the tile
// size); the padding leaves of a list's last tile (q >= nleaves) are skipped.
template <int SLICES, int TPT, bool SELF, bool TRACK>
__device__ __forceinline__ void ff_step_tile(const FFTile &T, int sl, int nleaves, FFTargets<TPT> &X, float2 vkap,
                                             float2 vn2a2, float2 one, float (&rmin)[kFFTileLeaves]) {
    constexpr int kLen = kFFPairSlots / SLICES;
#pragma unroll
    for (int q = 0; q < kFFTileLeaves; q++) {
        if (q >= nleaves) break;
#pragma unroll(kLen <= 4 ? kLen : 4)
        for (int k = 0; k < kLen; k++) {
            const int t = q * kFFPairSlots + sl + k * SLICES;
            const float4 a = T.xy[t], b = T.zf[t], c = T.fyz[t], d = T.rxy[t];
            const float2 rz = T.rz[t];
#pragma unroll
            for (int h = 0; h < TPT; h++) {
                const float2 dx = __fadd2_rn(lo2(a), X.nx[h]), dy = __fadd2_rn(hi2(a), X.ny[h]),
                             dz = __fadd2_rn(lo2(b), X.nz[h]);
                const float2 gx = __ffma2_rn(lo2(d), X.cbx[h], hi2(b)), gy = __ffma2_rn(hi2(d), X.cby[h], lo2(c)),
                             gz = __ffma2_rn(rz, X.cbz[h], hi2(c));
                float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
                if (SELF && t == X.self_p[h]) {
                    if (X.self_h[h])
                        r2.y = 1e30f;
                    else
                        r2.x = 1e30f;
                }
                if (TRACK) rmin[q] = fmin3(rmin[q], r2.x, r2.y);
                const float2 rinv = make_float2(rsqrt_hw(r2.x), rsqrt_hw(r2.y));
                const float2 q2 = __fmul2_rn(rinv, rinv);
                const float2 tq = __fmul2_rn(q2, rinv);
                const float2 cii = __ffma2_rn(vkap, tq, rinv);
                const float2 cr = __fmul2_rn(tq, __ffma2_rn(vn2a2, q2, one));
                const float2 s = __fmul2_rn(cr, __ffma2_rn(dx, gx, __ffma2_rn(dy, gy, __fmul2_rn(dz, gz))));
                X.ax[h] = __ffma2_rn(cii, gx, __ffma2_rn(s, dx, X.ax[h]));
                X.ay[h] = __ffma2_rn(cii, gy, __ffma2_rn(s, dy, X.ay[h]));
                X.az[h] = __ffma2_rn(cii, gz, __ffma2_rn(s, dz, X.az[h]));
            }
        }
    }
}

// Near pairs: one CTA of (32 / TPT) x SLICES threads per target leaf; thread
// lane il serves the leaf's beads il + h 32 / TPT (h < TPT), the SLICES
// groups of lanes take interleaved bead pairs of every tile of near leaves
// (kFFTileLeaves leaves per tile, copied asynchronously one tile ahead), the
// two lanes of each packed operation being two source beads.  Overlapping
// pairs (r <= 2a) get the near formula: with LISTCORR by walking the bead's
// LJ list once (while the first tile is in flight), otherwise by rescanning
// the tile segments whose running minimum of r^2 flags one, as in
// k_tea_step.  The bead's sum goes to FFBuffers::nearsum (k_ff_far adds the
// far field and moves it).
template <int SLICES, int TPT, bool LISTCORR>
__global__ void __launch_bounds__(32 / TPT * SLICES, 32 * TPT / SLICES) k_ff_near(KParams P, DevBuffers B,
                                                                                FFBuffers F, const int *gate) {
    if (gate && *gate != 0) return;
    constexpr int kLanes = 32 / TPT;
    const int L = blockIdx.x;
    const int il = threadIdx.x % kLanes, sl = threadIdx.x / kLanes;
    const int s0 = F.leaf_start[L], n = F.leaf_start[L + 1] - s0;
    const int traj = F.leaf_traj[L];
    __shared__ FFTile T2[2];
    __shared__ float4 s_red[SLICES * 32];
    __shared__ float4 s_x[32], s_cb[32];       // the leaf's beads: position, beta C_i
    __shared__ int s_near[kFFNearSmem];
    const float beta = B.tea_beta[traj], b2 = beta * beta;
    if (threadIdx.x < 32) {
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f), cb = x;
        if (threadIdx.x < n) {
            const int g = F.leaf_bead[s0 + threadIdx.x];
            x = B.frame_in[g];
            const float4 ci = B.tea_ci[g];
            cb = make_float4(beta / sqrtf(1.0f + b2 * ci.x), beta / sqrtf(1.0f + b2 * ci.y),
                             beta / sqrtf(1.0f + b2 * ci.z), 0.f);
        }
        s_x[threadIdx.x] = x;
        s_cb[threadIdx.x] = cb;
    }
    // near leaves in tiles of kFFTileLeaves, double-buffered: the copies of
    // tile k + 1 are in flight while tile k is summed
    const int e_beg = F.near_start[L], nnear = F.near_start[L + 1] - e_beg;
    const int *near = F.near + e_beg;
    const bool near_smem = nnear <= kFFNearSmem;
    if (near_smem)
        for (int k = threadIdx.x; k < nnear; k += blockDim.x) s_near[k] = near[k];
    __syncthreads();
    if (near_smem) near = s_near;
    const TeaConst K = tea_const(P.tea_a);
    const float2 vkap = f2(K.kap), vn2a2 = f2(-K.two_a2), one = f2(1.0f);
    const int ntiles = (nnear + kFFTileLeaves - 1) / kFFTileLeaves;
    ff_tile_issue(T2[0], F, near, 0, nnear);
    cp_async_commit();
    FFTargets<TPT> X;
    float3 corr[TPT];
#pragma unroll
    for (int h = 0; h < TPT; h++) {
        const int bi = il + h * kLanes;
        const float4 x = s_x[bi], cb = s_cb[bi];
        X.nx[h] = f2(-x.x);
        X.ny[h] = f2(-x.y);
        X.nz[h] = f2(-x.z);
        X.cbx[h] = f2(cb.x);
        X.cby[h] = f2(cb.y);
        X.cbz[h] = f2(cb.z);
        X.ax[h] = X.ay[h] = X.az[h] = f2(0.f);
        corr[h] = make_float3(0.f, 0.f, 0.f);
        if (LISTCORR && bi < n) {
            // overlapping pairs (r <= 2a): every one is within the LJ list
            // cutoff (checked by the launcher), so the far-field term of the
            // tile pass is replaced by the near one while walking the bead's
            // list, the SLICES threads of a bead taking interleaved entries;
            // done while the first tile is in flight
            const int g = F.leaf_bead[s0 + bi];
            const int base = B.off[traj], nb = P.nb;
            const int cnt = B.ljc[g];
            for (int q = sl; q < cnt; q += SLICES) {
                const int pj = base + B.lj[q * nb + g];
                const float4 xj = B.frame_in[pj];
                const float dx = xj.x - x.x, dy = xj.y - x.y, dz = xj.z - x.z;
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                if (!(r2 <= K.four_a2) || (B.flags[pj] & kFlagExtra)) continue;
                const float4 Fj = B.force[pj], Rj = B.tea_r[pj];
                const float gx = fmaf(Rj.x, cb.x, Fj.x), gy = fmaf(Rj.y, cb.y, Fj.y), gz = fmaf(Rj.z, cb.z, Fj.z);
                const float3 fa = tea_far1(K, dx, dy, dz, gx, gy, gz);
                const float3 nr = tea_pair1(K, dx, dy, dz, gx, gy, gz);
                corr[h].x += nr.x - fa.x;
                corr[h].y += nr.y - fa.y;
                corr[h].z += nr.z - fa.z;
            }
        }
    }
    for (int it = 0; it < ntiles; it++) {
        if (it + 1 < ntiles) ff_tile_issue(T2[(it + 1) & 1], F, near, (it + 1) * kFFTileLeaves, nnear);
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
        const FFTile &T = T2[it & 1];
        int self_q = -1;
#pragma unroll
        for (int q = 0; q < kFFTileLeaves; q++) {
            const int e = it * kFFTileLeaves + q;
            if (e < nnear && near[e] == L) self_q = q;
        }
        float rmin[kFFTileLeaves];
#pragma unroll
        for (int q = 0; q < kFFTileLeaves; q++) rmin[q] = 3.4e38f;
        const bool self = self_q >= 0;
#pragma unroll
        for (int h = 0; h < TPT; h++) {
            const int bi = il + h * kLanes;
            X.self_p[h] = self_q * kFFPairSlots + (bi >> 1);
            X.self_h[h] = bi & 1;
        }
        const int nleaves = min(kFFTileLeaves, nnear - it * kFFTileLeaves);
        if (self)
            ff_step_tile<SLICES, TPT, true, !LISTCORR>(T, sl, nleaves, X, vkap, vn2a2, one, rmin);
        else
            ff_step_tile<SLICES, TPT, false, !LISTCORR>(T, sl, nleaves, X, vkap, vn2a2, one, rmin);
        if (!LISTCORR) {
            constexpr int kLen = kFFPairSlots / SLICES;
            unsigned segs = 0;
#pragma unroll
            for (int q = 0; q < kFFTileLeaves; q++) segs |= (rmin[q] <= K.four_a2 ? 1u : 0u) << q;
            while (segs) {  // the tile leaves that hold an overlapping pair
                const int sg = __ffs(segs) - 1;
                segs &= segs - 1;
                for (int k = 0; k < kLen; k++) {
                    const int t = sg * kFFPairSlots + sl + k * SLICES;
                    const float4 a = T.xy[t], b = T.zf[t], c = T.fyz[t], d = T.rxy[t];
                    const float2 rz = T.rz[t];
#pragma unroll
                    for (int h = 0; h < TPT; h++)
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            if (self && t == X.self_p[h] && e == X.self_h[h]) continue;
                            const float dx = (e ? a.y : a.x) + X.nx[h].x, dy = (e ? a.w : a.z) + X.ny[h].x,
                                        dz = (e ? b.y : b.x) + X.nz[h].x;
                            const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            if (!(r2 <= K.four_a2)) continue;
                            const float gx = fmaf(e ? d.y : d.x, X.cbx[h].x, e ? b.w : b.z),
                                        gy = fmaf(e ? d.w : d.z, X.cby[h].x, e ? c.y : c.x),
                                        gz = fmaf(e ? rz.y : rz.x, X.cbz[h].x, e ? c.w : c.z);
                            const float3 fa = tea_far1(K, dx, dy, dz, gx, gy, gz);
                            const float3 nr = tea_pair1(K, dx, dy, dz, gx, gy, gz);
                            corr[h].x += nr.x - fa.x;
                            corr[h].y += nr.y - fa.y;
                            corr[h].z += nr.z - fa.z;
                        }
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int h = 0; h < TPT; h++) {
        const int bi = il + h * kLanes;
        s_red[sl * 32 + bi] = make_float4(X.ax[h].x + X.ax[h].y + corr[h].x, X.ay[h].x + X.ay[h].y + corr[h].y,
                                          X.az[h].x + X.az[h].y + corr[h].z, 0.f);
    }
    __syncthreads();
    if (threadIdx.x < n) {
        float4 v = s_red[threadIdx.x];
        for (int k = 1; k < SLICES; k++) {
            const float4 u = s_red[k * 32 + threadIdx.x];
            v.x += u.x;
            v.y += u.y;
            v.z += u.z;
        }
        F.nearsum[s0 + threadIdx.x] = v;
    }
}

// Far field and update: one warp per leaf.  The far fields of the leaf and
// of each ancestor with a far list are brought to the leaf's 8 proxies (L2L:
// one (ancestor, proxy) per lane, exact because interpolating on the leaf
// reproduces any trilinear field), summed in ancestor order, interpolated to
// each bead (L2P), added to its near sum, and the bead moves (FEFF: its
// effective force goes to feff instead).
template <bool FEFF>
__global__ void __launch_bounds__(32) k_ff_far(KParams P, DevBuffers B, FFBuffers F, float4 *feff, const int *gate) {
    if (gate && *gate != 0) return;
    const int L = blockIdx.x, lane = threadIdx.x;
    const int s0 = F.leaf_start[L], n = F.leaf_start[L + 1] - s0;
    // per ancestor: box (2) and potentials (24), then its far field at the
    // leaf's proxies; sized for the tree's longest ancestor list (max_anc)
    extern __shared__ float4 s_dyn[];
    float4 *s_far = s_dyn;
    float *s_l2l = reinterpret_cast<float *>(s_dyn + 26 * F.max_anc);
    __shared__ float s_pl[8 * 12];             // the far field at the leaf's proxies
    __shared__ float4 s_lbox[2];
    const int a0 = F.anc_start[L], na = min(F.anc_start[L + 1] - a0, F.max_anc);
    for (int k = lane; k < 26 * na; k += 32) {
        const int N = F.anc[a0 + k / 26], w = k % 26;
        s_far[k] = w < 2 ? F.box[2 * N + w] : F.phi[24 * N + w - 2];
    }
    if (lane < 2) s_lbox[lane] = F.box[2 * L + lane];
    __syncwarp();
    for (int t = lane; t < 8 * na; t += 32) {
        const int A = t >> 3, pn = t & 7;
        const float4 *fr = s_far + 26 * A;
        const float *ph = reinterpret_cast<const float *>(fr + 2);
        float w[8];
        ff_weights(ff_proxy(s_lbox[0], s_lbox[1], pn), fr[0], fr[1], w);
#pragma unroll
        for (int c = 0; c < 12; c++) {
            float v = 0.f;
#pragma unroll
            for (int m = 0; m < 8; m++) v = fmaf(w[m], ph[12 * m + c], v);
            s_l2l[96 * A + 12 * pn + c] = v;
        }
    }
    __syncwarp();
    for (int t = lane; t < 96; t += 32) {
        float v = 0.f;
        for (int A = 0; A < na; A++) v += s_l2l[96 * A + t];
        s_pl[t] = v;
    }
    __syncwarp();
    if (lane >= n) return;
    const int g = F.leaf_bead[s0 + lane];
    const int traj = F.leaf_traj[L];
    const float beta = B.tea_beta[traj], b2 = beta * beta;
    const float3 xi = f3(B.frame_in[g]);
    const float4 ci = B.tea_ci[g];
    const float3 cbi = make_float3(beta / sqrtf(1.0f + b2 * ci.x), beta / sqrtf(1.0f + b2 * ci.y),
                                   beta / sqrtf(1.0f + b2 * ci.z));
    const float4 ns = F.nearsum[s0 + lane];
    float sx = ns.x, sy = ns.y, sz = ns.z;
    if (na > 0) {   // L2P from the leaf's proxies
        float w[8];
        ff_weights(xi, s_lbox[0], s_lbox[1], w);
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const float *p = s_pl + 12 * m;   // A.xyz, B_x.xyz, B_y.xyz, B_z.xyz
            // A + beta C_x B_x + beta C_y B_y + beta C_z B_z
            const float ux = p[0] + cbi.x * p[3] + cbi.y * p[6] + cbi.z * p[9];
            const float uy = p[1] + cbi.x * p[4] + cbi.y * p[7] + cbi.z * p[10];
            const float uz = p[2] + cbi.x * p[5] + cbi.y * p[8] + cbi.z * p[11];
            sx = fmaf(w[m], ux, sx);
            sy = fmaf(w[m], uy, sy);
            sz = fmaf(w[m], uz, sz);
        }
    }
    tea_bead_update<FEFF>(P, B, g, sx, sy, sz, b2, tea_const(P.tea_a), feff);
}

// Beads in no leaf (extra beads): the update draws their angular noise and
// keeps their frame, as the all-pairs update does.
template <bool FEFF>
__global__ void k_ff_rest(KParams P, DevBuffers B, FFBuffers F, float4 *feff, const int *gate) {
    if (gate && *gate != 0) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= F.nrest) return;
    const int g = F.rest[k];
    const float beta = B.tea_beta[B.traj[g]];
    tea_bead_update<FEFF>(P, B, g, 0.f, 0.f, 0.f, beta * beta, tea_const(P.tea_a), feff);
}

void launch_ff_p2m_leaves(const KParams &P, const DevBuffers &B, const FFBuffers &F, const int *gate,
                          cudaStream_t s) {
    if (F.nleaf == 0) return;
    k_ff_p2m<<<(F.nleaf + kP2MWarps) / kP2MWarps, 32 * kP2MWarps, 0, s>>>(P, B, F, gate);
}
void launch_ff_m2l(const KParams &P, const FFBuffers &F, const int *gate, cudaStream_t s) {
    if (F.nleaf == 0) return;
    if (F.ninner > 0)
        k_ff_p2m_inner<<<(F.ninner + kP2MWarps - 1) / kP2MWarps, 32 * kP2MWarps, 0, s>>>(P, F, gate);
    constexpr int per_block = kM2LWarps * (32 / kM2LLanes);
    if (F.ntgt > 0) k_ff_m2l<<<(F.ntgt + per_block - 1) / per_block, 32 * kM2LWarps, 0, s>>>(P, F, gate);
}
void launch_ff_proxies(const KParams &P, const DevBuffers &B, const FFBuffers &F, const int *gate, cudaStream_t s) {
    launch_ff_p2m_leaves(P, B, F, gate, s);
    launch_ff_m2l(P, F, gate, s);
}

// Overlapping pairs can be taken from the LJ list when it holds every pair
// within 2a (plus 2 nm for the motion since its rebuild).
static bool ff_list_corr(const KParams &P) { return P.lj_on && P.ljcut >= 2.0f * P.tea_a + 2.0f; }

// target beads per thread of the near-pair kernel (two, with 16 lanes per
// slice, measured slower)
constexpr int kFFTPT = 1;
template <int SL>
static void ff_near_launch(const KParams &P, const DevBuffers &B, const FFBuffers &F, const int *gate,
                           cudaStream_t s) {
    constexpr int threads = 32 / kFFTPT * SL;
    if (F.nleaf == 0) return;
    if (ff_list_corr(P))
        k_ff_near<SL, kFFTPT, true><<<F.nleaf, threads, 0, s>>>(P, B, F, gate);
    else
        k_ff_near<SL, kFFTPT, false><<<F.nleaf, threads, 0, s>>>(P, B, F, gate);
}
void launch_ff_near(const KParams &P, const DevBuffers &B, const FFBuffers &F, const int *gate, cudaStream_t s) {
    switch (P.tea_slices) {
        case 1:
        case 2: ff_near_launch<2>(P, B, F, gate, s); break;
        case 4: ff_near_launch<4>(P, B, F, gate, s); break;
        default: ff_near_launch<8>(P, B, F, gate, s); break;
    }
}
void launch_ff_far(const KParams &P, const DevBuffers &B, const FFBuffers &F, bool feff_only, float4 *feff,
                   const int *gate, cudaStream_t s) {
    if (F.nleaf > 0) {
        const size_t smem = (size_t)F.max_anc * (26 * sizeof(float4) + 96 * sizeof(float));
        if (feff_only)
            k_ff_far<true><<<F.nleaf, 32, smem, s>>>(P, B, F, feff, gate);
        else
            k_ff_far<false><<<F.nleaf, 32, smem, s>>>(P, B, F, feff, gate);
    }
    if (F.nrest > 0) {
        if (feff_only)
            k_ff_rest<true><<<(F.nrest + 127) / 128, 128, 0, s>>>(P, B, F, feff, gate);
        else
            k_ff_rest<false><<<(F.nrest + 127) / 128, 128, 0, s>>>(P, B, F, feff, gate);
    }
}
void launch_ff_step(const KParams &P, const DevBuffers &B, const FFBuffers &F, bool feff_only, float4 *feff,
                    const int *gate, cudaStream_t s) {
    launch_ff_near(P, B, F, gate, s);
    launch_ff_far(P, B, F, feff_only, feff, gate, s);
}

}  // namespace mtg
