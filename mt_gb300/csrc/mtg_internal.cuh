// mtg_internal.cuh - shared device helpers, kernel parameters and the engine
// object of the GB300 engine.  Not part of the public ABI (include/mtg.h).
//
// HBM layout (nb beads over nt trajectories, CSR offsets):
//   frame[2]   : two buffers of 4 planes x nb float4 (double-buffered state)
//                plane 0 = (x, y, z, fi)
//                plane 1 = (R e_z, psi)       axial site direction
//                plane 2 = (R p1, theta)      lateral site p1 in the lab frame
//                plane 3 = (R p2, 0)          lateral site p2 in the lab frame
//                R = Rz(psi) Ry(theta) Rx(fi) is the bead's orientation; the
//                planes are written by the kernel that moves the bead, so a
//                neighbour's sites cost one 16 B gather instead of six sin/cos.
//   flags[nb]  : bit 0 extra, 1 fixed, 2 mon_type, 3 gtp==1, 4 on_tubule!=0,
//                bits 8..10 harmonic count
//   harm[nb*maxH] : harmonic partners, local index, reference sign encoding
//   lists      : counts [nb] + entries k-major [cap][nb] (coalesced per k)
//   seeds[2nb] : HybridTaus uint4 states; stream g = xyz noise of bead g,
//                stream g+nb = its angle noise
//   force[2nb] : last generalised forces, (fx, fy, fz, 0), (ffi, ftheta, fpsi, 0)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mtg {

constexpr int kFlagExtra = 1 << 0;
constexpr int kFlagFixed = 1 << 1;
constexpr int kFlagBeta = 1 << 2;
constexpr int kFlagGtp = 1 << 3;
constexpr int kFlagOnTubule = 1 << 4;
constexpr int kHarmShift = 8;
constexpr int kZeroCode = 999999;   // lateral encoding of bead 0 (src/mt.h:35)

constexpr int kErrOverflow = 1;     // bit in the device error word
constexpr int kErrTeaEps = 2;
constexpr int kErrNonFinite = 4;
constexpr int kErrTimeout = 8;     // a bounded wait on the tensor cores ran out

// Scalars every kernel reads (passed by value: constant bank).
struct KParams {
    int nb, nt;
    // Euler-Maruyama coefficients (integrate_kernel, src/compute_cuda.cu:955-963)
    float kr, kfi, kth, varR, nfi, varTheta;
    // harmonic + bending
    float C, B_psi, B_fi, B_theta, psi_0, fi_0, th0_gtp, th0_gdp;
    // Morse
    float A_long, D_long, A_lat, D_lat, D_lat_seam;
    // barriers
    int barrier;
    float a_bl, r_bl, w_bl, a_bt, r_bt, w_bt;
    // LJ
    int lj_on;
    float lj_pref, ljcut;
    // walls
    int is_wall;
    float rep_r, rep_eps, lb;
    int is_assembly;
    // lateral binding sites p1, p2 (src/mt.h:44-50)
    float p1x, p1y, p1z, p2x, p2y, p2z;
    int maxH, maxLong, maxLat, maxLJ;
    // TEA
    float tea_a, tea_var;
    int tea_slices;        // threads per bead i in the all-pairs TEA kernels (1, 2, 4 or 8)
    int tea_jparts;        // parts of a split work item's j range (1..kTeaMaxParts), summed by a second kernel
    int tea_nhead;         // work items run whole before the split tail (set by the TEA launchers)
    int step_block;        // threads per CTA of the fused plain step (64, 128 or 256)
};

// Device buffers of one engine.
struct DevBuffers {
    const int *off;        // [nt+1]
    const int *traj;       // [nb]
    const int *flags;      // [nb]
    const int *harm;       // [nb*maxH]
    const float *zs;       // [nt]
    float4 *frame_in;      // 4 planes
    float4 *frame_out;     // 4 planes
    float4 *force;         // 2 planes (may be null where unused)
    uint4 *seeds;          // [2nb]
    int *ljc, *lj, *lonc, *lon, *latc, *lat;
    int *err;
    // TEA
    float4 *tea_r;         // random forces of all beads (xyz scaled, w raw)
    float4 *tea_ci;        // row sums of squared normalised RPY entries
    float *tea_eps;        // per-bead epsilon sums
    float *tea_beta;       // [nt]
    double *tea_eps_t;     // [nt]
    float4 *tea_part;      // [kTeaMaxParts][nb] partial sums of the split all-pairs kernels
};

// ------------------------------------------------------------------ RNG
// HybridTaus (src/HybridTaus.cu:63-82): three Tausworthe steps and one LCG.
__device__ __forceinline__ uint32_t taus_step(uint32_t &z, int s1, int s2, int s3, uint32_t m) {
    const uint32_t b = ((z << s1) ^ z) >> s2;
    z = ((z & m) << s3) ^ b;
    return z;
}
__device__ __forceinline__ uint32_t hybrid_taus(uint4 &s) {
    const uint32_t a = taus_step(s.x, 13, 19, 12, 4294967294u);
    const uint32_t b = taus_step(s.y, 2, 25, 4, 4294967288u);
    const uint32_t c = taus_step(s.z, 3, 11, 17, 4294967280u);
    s.w = 1664525u * s.w + 1013904223u;
    return a ^ b ^ c ^ s.w;
}
// uintToFloat (src/HybridTaus.cu:53-61): 23 mantissa bits -> [0,1), 0 -> 1e-8.
__device__ __forceinline__ float uint_to_unit(uint32_t u) {
    const float f = __uint_as_float(0x3f800000u | (0x007fffffu & u)) - 1.0f;
    return f == 0.0f ? 1.0e-8f : f;
}
// rforce (src/HybridTaus.cu:84-98): four N(0,1) deviates by Box-Muller.  The
// sine and cosine are the hardware approximations the reference calls
// (__sinf/__cosf), and the logarithm is the one its -use_fast_math build
// (CMakeLists.txt:62) turns logf into.
__device__ __forceinline__ float4 gauss4(uint4 &s) {
    float4 g;
    float u1 = uint_to_unit(hybrid_taus(s));
    float u2 = uint_to_unit(hybrid_taus(s));
    float r = sqrtf(-2.0f * __logf(u1));
    float sn, cs;
    __sincosf(6.28318548f * u2, &sn, &cs);
    g.x = r * sn;
    g.y = r * cs;
    u1 = uint_to_unit(hybrid_taus(s));
    u2 = uint_to_unit(hybrid_taus(s));
    r = sqrtf(-2.0f * __logf(u1));
    __sincosf(6.28318548f * u2, &sn, &cs);
    g.z = r * sn;
    g.w = r * cs;
    return g;
}

// --------------------------------------------------------------- frames
struct Frame {
    float4 p0, p1, p2, p3;
};

__device__ __forceinline__ float3 f3(const float4 &v) { return make_float3(v.x, v.y, v.z); }

// Builds the four planes of a bead from its state.  Every product and sum
// is an explicitly rounded intrinsic, so no multiply-add is contracted: the
// result does not depend on the kernel this is inlined into (the per-step and
// the persistent plain step agree bit for bit).
__device__ __forceinline__ float dot3_rn(float a0, float b0, float a1, float b1, float a2, float b2) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}
__device__ __forceinline__ Frame make_frame(const KParams &P, float x, float y, float z, float fi, float theta,
                                            float psi) {
    float sf, cf, st, ct, sp, cp;
    sincosf(fi, &sf, &cf);
    sincosf(theta, &st, &ct);
    sincosf(psi, &sp, &cp);
    const float cpst = __fmul_rn(cp, st), spst = __fmul_rn(sp, st);
    const float m00 = __fmul_rn(cp, ct), m01 = __fsub_rn(__fmul_rn(cpst, sf), __fmul_rn(sp, cf)),
                m02 = __fadd_rn(__fmul_rn(cpst, cf), __fmul_rn(sp, sf));
    const float m10 = __fmul_rn(sp, ct), m11 = __fadd_rn(__fmul_rn(spst, sf), __fmul_rn(cp, cf)),
                m12 = __fsub_rn(__fmul_rn(spst, cf), __fmul_rn(cp, sf));
    const float m20 = -st, m21 = __fmul_rn(ct, sf), m22 = __fmul_rn(ct, cf);
    Frame F;
    F.p0 = make_float4(x, y, z, fi);
    F.p1 = make_float4(m02, m12, m22, psi);
    F.p2 = make_float4(dot3_rn(m00, P.p1x, m01, P.p1y, m02, P.p1z), dot3_rn(m10, P.p1x, m11, P.p1y, m12, P.p1z),
                       dot3_rn(m20, P.p1x, m21, P.p1y, m22, P.p1z), theta);
    F.p3 = make_float4(dot3_rn(m00, P.p2x, m01, P.p2y, m02, P.p2z), dot3_rn(m10, P.p2x, m11, P.p2y, m12, P.p2z),
                       dot3_rn(m20, P.p2x, m21, P.p2y, m22, P.p2z), 0.0f);
    return F;
}

__device__ __forceinline__ void store_frame(float4 *planes, int nb, int g, const Frame &F) {
    planes[g] = F.p0;
    planes[nb + g] = F.p1;
    planes[2 * nb + g] = F.p2;
    planes[3 * nb + g] = F.p3;
}

// ------------------------------------------------------------ potentials
// Morse derivative / energy and Gaussian barrier (src/compute_cuda.cu:16-30).
__device__ __forceinline__ float dmorse(float D, float a, float x) {
    const float e = expf(-a * x);
    return 2.0f * a * D * (1.0f - e) * e;
}
__device__ __forceinline__ float morse_en(float D, float a, float x) {
    const float e = expf(-a * x);
    return D * (1.0f - e) * (1.0f - e) - D;
}
__device__ __forceinline__ float dbarr(float a, float r, float w, float x) {
    return -a * expf(-(x - r) * (x - r) / (2.0f * w * w)) * (x - r) / (w * w);
}
__device__ __forceinline__ float barr(float a, float r, float w, float x) {
    return a * expf(-(x - r) * (x - r) / (2.0f * w * w));
}

// Centre distance in a fixed, contraction-free order shared with the CPU
// oracle, so that LJ list membership is bit-identical for identical inputs.
__device__ __forceinline__ float centre_dist(float4 a, float4 b) {
    const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}

// Site-to-site vector d = (r_j + w_j) - (r_i + w_i), position difference first.
__device__ __forceinline__ float3 site_delta(float4 ri, float4 rj, float3 wi, float3 wj) {
    return make_float3(__fsub_rn(__fadd_rn(__fsub_rn(rj.x, ri.x), wj.x), wi.x),
                       __fsub_rn(__fadd_rn(__fsub_rn(rj.y, ri.y), wj.y), wi.y),
                       __fsub_rn(__fadd_rn(__fsub_rn(rj.z, ri.z), wj.z), wi.z));
}
__device__ __forceinline__ float norm3_rn(float3 d) {
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d.x, d.x), __fmul_rn(d.y, d.y)), __fmul_rn(d.z, d.z)));
}

// --------------------------------------------------------- list decisions
// Site offsets are at most |p1| ~ 2 nm from the centre, so a site distance
// below 2.5 nm needs a centre distance below 2.5 + 2 + 2 = 6.5 nm; 6.6 nm
// leaves room for rounding.
constexpr float kPairPrefilter = 6.6f;

// Bead i's side of the pair-list decisions (LJ_kernel,
// src/compute_cuda.cu:913-940; pairs_kernel, :527-674).
struct ListSite {
    float4 p, l1, l2;
    float3 wi;        // R_MON * e_z, R_MON = -r_mon without a harmonic partner
    float rmon;
    int flags, il, hpart, h0;
    bool do_lj, do_pairs;
};
__device__ __forceinline__ ListSite list_site(const KParams &P, float4 p, float4 uz, float4 l1, float4 l2, int flags,
                                              int il, int h0) {
    ListSite I;
    I.p = p;
    I.l1 = l1;
    I.l2 = l2;
    // pairs_kernel reads harmonic[max*i] even without a partner (-1 fill):
    // < 0 -> R_MON = -r_mon and |.| is excluded (src/compute_cuda.cu:548,565,599)
    I.rmon = h0 < 0 ? -2.0f : 2.0f;
    I.hpart = h0 < 0 ? -h0 : h0;
    I.h0 = h0;
    I.wi = make_float3(uz.x * I.rmon, uz.y * I.rmon, uz.z * I.rmon);
    I.flags = flags;
    I.il = il;
    const bool extra = (flags & kFlagExtra) != 0;
    I.do_lj = P.lj_on && !extra;
    I.do_pairs = P.is_assembly && !extra;
    return I;
}
// The lists bead j (index jl in its trajectory) enters for bead i: bit 0 LJ,
// bit 1 longitudinal, bit 2 lateral with i's site p1 against j's p2 (code
// -j), bit 3 lateral with i's p2 against j's p1 (code +j); appended in that
// order for ascending j, as the reference's loops do.
__device__ __forceinline__ unsigned list_bits(const KParams &P, const ListSite &I, int jl, float4 q, float4 uj,
                                              float4 l1j, float4 l2j, int fj) {
    unsigned bits = 0;
    const float cd = centre_dist(I.p, q);
    if (I.do_lj && jl != I.il && cd < P.ljcut) bits |= 1u;
    if (I.do_pairs && cd < kPairPrefilter && jl != I.hpart) {
        if (((I.flags ^ fj) & kFlagBeta) != 0) {
            const float3 d = site_delta(I.p, q, I.wi, make_float3(-uj.x * I.rmon, -uj.y * I.rmon, -uj.z * I.rmon));
            if (norm3_rn(d) < 2.5f) bits |= 2u;
        }
        if (jl != I.il) {
            if (norm3_rn(site_delta(I.p, q, f3(I.l1), f3(l2j))) < 2.5f) bits |= 4u;
            if (norm3_rn(site_delta(I.p, q, f3(I.l2), f3(l1j))) < 2.5f) bits |= 8u;
        }
    }
    return bits;
}
// Appends bead j's entries to bead g's lists (k-major, capacity-checked).
__device__ __forceinline__ void list_append(const KParams &P, const DevBuffers &B, int g, const ListSite &I,
                                            unsigned bits, int jl, int &nlj, int &nlo, int &nla, bool &overflow) {
    const int nb = P.nb;
    if (bits & 1u) {
        if (nlj < P.maxLJ)
            B.lj[nlj * nb + g] = jl;
        else
            overflow = true;
        nlj++;
    }
    if (bits & 2u) {
        if (nlo < P.maxLong)
            B.lon[nlo * nb + g] = I.h0 < 0 ? jl : -jl;
        else
            overflow = true;
        nlo++;
    }
    const int code = jl != 0 ? jl : kZeroCode;
    // orientation 0: i site p1, j site p2 -> -j; orientation 1: p2 / p1 -> +j
    if (bits & 4u) {
        if (nla < P.maxLat)
            B.lat[nla * nb + g] = -code;
        else
            overflow = true;
        nla++;
    }
    if (bits & 8u) {
        if (nla < P.maxLat)
            B.lat[nla * nb + g] = code;
        else
            overflow = true;
        nla++;
    }
}

// 1/sqrt(x) as the single hardware approximation instruction (a few ulp);
// pair distances are never subnormal, so the flush-to-zero form gives the
// same value for them without a subnormal fix-up.
__device__ __forceinline__ float rsqrt_hw(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// min(a, b, c) as one three-input instruction (sm_100 and later).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float y;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(a), "f"(b), "f"(c));
    return y;
}

// Spatial-hash buffers of the cell-list rebuild (kernels_cells.cu).
struct CellBuffers {
    int nbuckets;          // sum over trajectories of their table sizes
    int max_buckets;       // largest table of one trajectory
    const int *tbase;      // [nt+1] first bucket of each trajectory's table
    const int *tmask;      // [nt] table size - 1 (power of two)
    int *key;              // [nb] bucket of each bead
    int *cnt, *start, *cursor;  // [nbuckets]
    int *cell_bead;        // [nb] beads in bucket order (ascending index within a bucket)
    float4 *cell_pos;      // [nb] their positions; w = bead index | kCellExtraBit for extra beads
};
constexpr int kCellIndexMask = 0x7fffffff;
constexpr int kCellExtraBit = (int)0x80000000u;
constexpr int kCellMaxLong = 16;   // largest list capacities the cell rebuild buffers locally
constexpr int kCellMaxLat = 32;

// Cell of a coordinate for cells of edge 1/inv (NaN and far-away values clamp).
__device__ __forceinline__ int cell_coord(float x, float inv) {
    float c = floorf(x * inv);
    c = fminf(fmaxf(c, -1048576.0f), 1048576.0f);  // NaN -> -2^20 (fmaxf drops NaN)
    return (int)c;
}
__device__ __forceinline__ uint32_t cell_hash(int cx, int cy, int cz) {
    return ((uint32_t)cx * 73856093u) ^ ((uint32_t)cy * 19349663u) ^ ((uint32_t)cz * 83492791u);
}

// ------------------------------------------------------ host entry points
// (kernel launchers, defined in the .cu files)
void launch_frames_from_coords(const KParams &P, const float *coords7, float4 *frame, cudaStream_t s);
void launch_coords_from_frames(const KParams &P, const float4 *frame, float *coords7, cudaStream_t s);
void launch_forces_to_coords(const KParams &P, const float4 *force, float *coords7, cudaStream_t s);
void launch_rebuild(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s);
void launch_rebuild_cells(const KParams &P, const DevBuffers &B, const CellBuffers &C, const int2 *work, int nwork,
                          cudaStream_t s);
// Bins the current positions into the per-trajectory spatial hash with cells
// just larger than `reach`; returns 1/edge for the consumers' cell lookups.
// `ordered` sorts every bucket by bead index (for sums that must not depend
// on the arrival order of the atomic fill).
float bin_beads(const KParams &P, const DevBuffers &B, const CellBuffers &C, float reach, bool ordered,
                cudaStream_t s);
void launch_step_plain(const KParams &P, const DevBuffers &B, bool keep_forces, cudaStream_t s);
void launch_forces(const KParams &P, const DevBuffers &B, bool tea_prepare, cudaStream_t s);
// Persistent run of nsteps plain steps (no rebuild inside), one CTA per
// trajectory with its frames in shared memory; nmax = the largest trajectory.
constexpr int kPeriodThreads = 256;
constexpr int kPeriodBeads = 8;                   // beads per thread: trajectories up to 2048 beads
constexpr size_t kPeriodMaxSmem = 227 * 1024;     // bytes of dynamic shared memory a CTA may hold
size_t period_smem_bytes(int nmax);
bool period_fits(int nmax);
int period_prepare(int nmax);                     // opts the kernel into its shared memory (outside captures)
// trajectories this small rebuild their pair lists inside the persistent
// kernel (every bead against the whole trajectory) instead of by launch_lists
constexpr int kPeriodRebuildMax = 512;
bool period_rebuilds(int nmax);
void launch_step_period(const KParams &P, const DevBuffers &B, bool keep_forces, int nsteps, int nmax, bool rebuild,
                        cudaStream_t s);
void launch_energy(const KParams &P, const DevBuffers &B, double *per_bead, double *partials,
                   const int2 *work, int nwork, cudaStream_t s);
void launch_energy_totals(const KParams &P, const double *partials, const int *work_first, double *per_traj,
                          int *err, cudaStream_t s);
// TEA kernels run over their own work list: chunks of kTeaChunk beads.
constexpr int kTeaChunk = 128;
constexpr int kTeaMaxParts = 4;
void launch_tea_eps(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s);
void launch_tea_beta(const KParams &P, const DevBuffers &B, int capricious, float epsmax, cudaStream_t s);
void launch_tea_step(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, cudaStream_t s);
// gated variants: run only while *gate == run_if
void launch_tea_eps_gated(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, const int *gate,
                          int run_if, cudaStream_t s);
void launch_tea_beta_gated(const KParams &P, const DevBuffers &B, int capricious, float epsmax, const int *gate,
                           int run_if, cudaStream_t s);
// effective TEA force (no update) into feff, while *gate == 0
void launch_tea_feff(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, float4 *feff,
                     const int *gate, cudaStream_t s);
void launch_set_flags(int nb, const uint8_t *extra, const int *gtp, const int *on_tubule, int *flags,
                      cudaStream_t s);

constexpr int kTile = 128;   // beads per CTA tile of the O(N^2) kernels

// ---------------------------------------------- far field of learned TEA
// A k-d tree over each trajectory's beads (tea_ff.cu) with leaves of at most
// kFFLeaf beads; every node is a contiguous range of the leaf bead order.
// Leaf pairs that are not well separated are summed bead by bead (near
// lists of the leaves); well-separated node pairs, at the coarsest level
// where they are, interact through proxies: the 8 points
// c + h (+-kFFNode, +-kFFNode, +-kFFNode) of a node's bounding box (centre c,
// half extent h; tensor-product Chebyshev nodes of degree 2) carry the
// node's sources (F, R) as interpolation charges and receive the far field
// of the nodes far from it, interpolated to each bead of the node.
constexpr int kFFLeaf = 32;
constexpr float kFFNode = 0.70710678f;
constexpr int kFFMaxAnc = 16;          // nodes with far fields on a leaf's path to the root (tree depth bound)
struct FFBuffers {
    int nleaf, nnode, ntgt, ninner, nrest;
    int max_anc;             // the longest ancestor list of a leaf (at most kFFMaxAnc)
    const int *leaf_start;   // [nleaf+1] into leaf_bead
    const int *leaf_bead;    // beads of every leaf, leaf after leaf (every node a contiguous range)
    const int *leaf_traj;    // [nleaf]
    const int *near_start;   // [nleaf+1] into near: source leaves summed pair by pair
    const int *near;
    const int *node_range;   // [2*nnode] begin, end in leaf_bead; nodes 0 .. nleaf-1 are the leaves, larger nodes first after them
    const int *node_leaves;  // [2*nnode] first leaf, last leaf + 1 of each node
    const int *far_start;    // [nnode+1] into far: source nodes taken through their proxies
    const int *far;
    const int *tgt;          // [ntgt] nodes with a non-empty far list
    const int *inner;        // [ninner] internal nodes that are far sources or targets, larger first
    const int *anc_start;    // [nleaf+1] into anc: the leaf and its ancestors with a far list
    const int *anc;
    const int *rest;         // [nrest] beads in no leaf (extra beads)
    float4 *box;             // [2*nnode] centre, half extent (w unused)
    float4 *q;               // [16*nnode] proxy m: (QF.xyz, QR.x) at 16N+m, (QR.y, QR.z, 0, 0) at 16N+8+m
    float4 *phi;             // [24*nnode] target proxy n: (A.xyz, B0.x), (B0.yz, B1.xy), (B1.z, B2.xyz) at 24N+3n
    float4 *pack;            // [(nleaf+1)*kFFPackF4] each leaf's beads in the tile layout of the step kernel
                             // (leaf nleaf: padding, far away with zero F and R), written every step by P2M
    float4 *nearsum;         // [leaf beads] each bead's near-pair sum, in leaf bead order
};
// float4 per leaf of FFBuffers::pack, for the bead pairs (2p, 2p+1):
// xa xb ya yb | za zb Fxa Fxb | Fya Fyb Fza Fzb | Rxa Rxb Rya Ryb (kFFLeaf / 2
// each), then Rza Rzb of two pairs per float4 (kFFLeaf / 4)
constexpr int kFFPairSlots = kFFLeaf / 2;
constexpr int kFFPackF4 = 4 * kFFPairSlots + kFFPairSlots / 2;
// All of the kernels below run while *gate == 0.
// leaf proxies (P2M of the leaves, and their packed beads)
void launch_ff_p2m_leaves(const KParams &P, const DevBuffers &B, const FFBuffers &F, const int *gate,
                          cudaStream_t s);
// inner-node proxies and far-field potentials at target proxies (M2L); needs the leaf proxies
void launch_ff_m2l(const KParams &P, const FFBuffers &F, const int *gate, cudaStream_t s);
// both of the above
void launch_ff_proxies(const KParams &P, const DevBuffers &B, const FFBuffers &F, const int *gate, cudaStream_t s);
// near-pair sums; needs the leaf proxies' packed beads
void launch_ff_near(const KParams &P, const DevBuffers &B, const FFBuffers &F, const int *gate, cudaStream_t s);
// far field + update (FEFF: effective forces into feff, no update); needs the near sums and M2L
void launch_ff_far(const KParams &P, const DevBuffers &B, const FFBuffers &F, bool feff_only, float4 *feff,
                   const int *gate, cudaStream_t s);
// near + far
void launch_ff_step(const KParams &P, const DevBuffers &B, const FFBuffers &F, bool feff_only, float4 *feff,
                    const int *gate, cudaStream_t s);
// the exact mobility product + update, only while *gate == 1 (after a fall-back to exact TEA)
void launch_tea_step_gated(const KParams &P, const DevBuffers &B, const int2 *work, int nwork, const int *gate,
                           cudaStream_t s);

}  // namespace mtg
