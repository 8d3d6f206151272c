// surrogate.cu - learned TEA: per-bead descriptors, the surrogate network's
// C ABI (create, train, predict, gradients), and the learned mode of the TEA
// step with its exact re-check and fallback.
//
// Descriptor (32 features per bead, neighbours j != i of the same
// trajectory, extra beads excluded, r < 20 nm), in three radial shells
// [0,5), [5,10), [10,20) nm, ten features each:
//   count, sum 1/r, sum 1/r^2, sum 1/r^3,
//   sum u_x^2/r, sum u_y^2/r, sum u_z^2/r, sum u_x u_y/r, sum u_x u_z/r, sum u_y u_z/r
// (u = (r_j - r_i)/r), then log N' (non-extra beads of the trajectory) and
// the bead's distance from the trajectory centroid / 100 nm.
// Targets: C_i (3 components, integrateTea_kernel_unlisted,
// src/bdhitea_kernel.cu:160-163) and the trajectory's beta (src/bdhitea.cu:101-110).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "mtg_engine.cuh"
#include "mtg_mlp.cuh"

using namespace mtg;

namespace {

constexpr float kDescCut = 20.0f;
constexpr int kF = mlp::kIn;

// centroid and non-extra count of every trajectory: (cx, cy, cz, N')
__global__ void k_traj_stats(KParams P, DevBuffers B, float4 *stats) {
    const int t = blockIdx.x;
    const int base = B.off[t], end = B.off[t + 1];
    double sx = 0, sy = 0, sz = 0;
    int cnt = 0;
    for (int g = base + threadIdx.x; g < end; g += blockDim.x) {
        if (B.flags[g] & kFlagExtra) continue;
        const float4 p = B.frame_in[g];
        sx += p.x;
        sy += p.y;
        sz += p.z;
        cnt++;
    }
    for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
        sz += __shfl_xor_sync(0xffffffffu, sz, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    __shared__ double s[4][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][wid] = sx;
        s[1][wid] = sy;
        s[2][wid] = sz;
        s[3][wid] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0, n = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            a += s[0][w];
            b += s[1][w];
            c += s[2][w];
            n += s[3][w];
        }
        const double inv = n > 0 ? 1.0 / n : 0.0;
        stats[t] = make_float4((float)(a * inv), (float)(b * inv), (float)(c * inv), (float)n);
    }
}

// Shell accumulation of one neighbour: the ten features of its shell.
__device__ __forceinline__ void desc_add(float (&s)[10], float rinv, float ux, float uy, float uz) {
    const float r2i = rinv * rinv;
    s[0] += 1.0f;
    s[1] += rinv;
    s[2] += r2i;
    s[3] += r2i * rinv;
    s[4] += ux * ux * rinv;
    s[5] += uy * uy * rinv;
    s[6] += uz * uz * rinv;
    s[7] += ux * uy * rinv;
    s[8] += ux * uz * rinv;
    s[9] += uy * uz * rinv;
}

// One thread per bead, taken in bucket order: the threads of a warp sit in
// one or two cells and walk the same 27-cell neighbourhood, so candidate
// loads are broadcasts and the loops mostly uniform.  Cells are 20 nm; the
// candidates of a bucket are visited in ascending bead index.
__global__ void __launch_bounds__(kTile) k_descriptors(KParams P, DevBuffers B, CellBuffers C, const int2 *work,
                                                       float inv_cell, const float4 *stats, float *desc,
                                                       const int *gate) {
    if (gate && *gate) return;
    const int2 w = work[blockIdx.x];
    const int traj = w.x, end = B.off[traj + 1];
    const int base = B.off[traj];
    const int slot = w.y + threadIdx.x;
    __shared__ int s_bk[27][kTile];
    if (slot >= end) return;
    const float4 pi = C.cell_pos[slot];
    const int word = __float_as_int(pi.w), g = word & kCellIndexMask;
    float s0[10], s1[10], s2[10];
#pragma unroll
    for (int k = 0; k < 10; k++) s0[k] = s1[k] = s2[k] = 0.f;
    float f30 = 0.f, f31 = 0.f;
    if (!(word & kCellExtraBit)) {
        const int cx = cell_coord(pi.x, inv_cell), cy = cell_coord(pi.y, inv_cell), cz = cell_coord(pi.z, inv_cell);
        const int tb = C.tbase[traj];
        const uint32_t mask = (uint32_t)C.tmask[traj];
        // the 27 buckets (kept in shared memory for the rolled cell loop) and
        // a mask of the cells whose bucket an earlier cell already has
        int bk[27];
#pragma unroll
        for (int c = 0; c < 27; c++) {
            bk[c] = tb + (int)(cell_hash(cx + c % 3 - 1, cy + (c / 3) % 3 - 1, cz + c / 9 - 1) & mask);
            s_bk[c][threadIdx.x] = bk[c];
        }
        uint32_t dup = 0;
#pragma unroll
        for (int c = 1; c < 27; c++) {
            bool seen = false;
#pragma unroll
            for (int v = 0; v < c; v++) seen |= (bk[v] == bk[c]);
            dup |= (seen ? 1u : 0u) << c;
        }
        int st_next = C.start[bk[0]], ct_next = C.cnt[bk[0]];
        for (int c = 0; c < 27; c++) {
            const int st_c = st_next, ct_c = ct_next;
            if (c + 1 < 27) {   // the next cell's range is fetched while this one runs
                const int b = s_bk[c + 1][threadIdx.x];
                st_next = C.start[b];
                ct_next = C.cnt[b];
            }
            if (((dup >> c) & 1u) || ct_c == 0) continue;
            const int s1e = base + st_c + ct_c;
            for (int s = base + st_c; s < s1e; s += 4) {
                float4 q[4];   // four candidates in flight
#pragma unroll
                for (int u = 0; u < 4; u++)
                    q[u] = s + u < s1e ? C.cell_pos[s + u] : make_float4(0.f, 0.f, 0.f, __int_as_float(kCellExtraBit));
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int wj = __float_as_int(q[u].w);
                    const float ex = q[u].x - pi.x, ey = q[u].y - pi.y, ez = q[u].z - pi.z;
                    const float r2 = ex * ex + ey * ey + ez * ez;
                    if (!(r2 < kDescCut * kDescCut) || !(r2 > 0.f) || (wj & kCellExtraBit) || wj == g) continue;
                    const float rinv = rsqrt_hw(r2), r = r2 * rinv;
                    const float ux = ex * rinv, uy = ey * rinv, uz = ez * rinv;
                    if (r < 5.0f)
                        desc_add(s0, rinv, ux, uy, uz);
                    else if (r < 10.0f)
                        desc_add(s1, rinv, ux, uy, uz);
                    else
                        desc_add(s2, rinv, ux, uy, uz);
                }
            }
        }
        const float4 ts = stats[traj];
        f30 = logf(fmaxf(ts.w, 1.0f));
        const float dx = pi.x - ts.x, dy = pi.y - ts.y, dz = pi.z - ts.z;
        f31 = sqrtf(dx * dx + dy * dy + dz * dz) * 0.01f;
    }
    float4 *o = reinterpret_cast<float4 *>(desc + (size_t)g * kF);
    o[0] = make_float4(s0[0], s0[1], s0[2], s0[3]);
    o[1] = make_float4(s0[4], s0[5], s0[6], s0[7]);
    o[2] = make_float4(s0[8], s0[9], s1[0], s1[1]);
    o[3] = make_float4(s1[2], s1[3], s1[4], s1[5]);
    o[4] = make_float4(s1[6], s1[7], s1[8], s1[9]);
    o[5] = make_float4(s2[0], s2[1], s2[2], s2[3]);
    o[6] = make_float4(s2[4], s2[5], s2[6], s2[7]);
    o[7] = make_float4(s2[8], s2[9], f30, f31);
}

// Exact targets from the current epsilon pass: C_i and beta.
__global__ void k_tea_targets(KParams P, DevBuffers B, float *targets) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.nb) return;
    const float beta = B.tea_beta[B.traj[g]], b2 = beta * beta;
    const float4 ci = B.tea_ci[g];
    float *t = targets + (size_t)g * mlp::kOut;
    t[0] = 1.0f / sqrtf(1.0f + b2 * ci.x);
    t[1] = 1.0f / sqrtf(1.0f + b2 * ci.y);
    t[2] = 1.0f / sqrtf(1.0f + b2 * ci.z);
    t[3] = beta;
}

// Surrogate outputs -> the TEA state the mobility kernel reads: beta of a
// trajectory = mean of its non-extra beads' predictions; tea_ci = the row
// sums that reproduce the predicted C_i, (1/C_i^2 - 1)/beta^2.
__global__ void k_surr_beta(KParams P, DevBuffers B, const float *pred, const float *ynorm, const int *gate) {
    if (gate && *gate) return;
    const int t = blockIdx.x;
    const int base = B.off[t], end = B.off[t + 1];
    double s = 0.0;
    int cnt = 0;
    for (int g = base + threadIdx.x; g < end; g += blockDim.x) {
        if (B.flags[g] & kFlagExtra) continue;
        s += (double)(pred[(size_t)g * mlp::kOut + 3] * ynorm[mlp::kOut + 3] + ynorm[3]);
        cnt++;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
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
        double a = 0;
        int n = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            a += ss[w];
            n += sc[w];
        }
        float beta = n > 0 ? (float)(a / n) : 0.5f;
        beta = fminf(fmaxf(beta, 1e-4f), 0.5f);
        B.tea_beta[t] = beta;
    }
}

__global__ void k_surr_ci(KParams P, DevBuffers B, const float *pred, const float *ynorm, const int *gate) {
    if (gate && *gate) return;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.nb) return;
    const float beta = B.tea_beta[B.traj[g]], ib2 = 1.0f / (beta * beta);
    float c[3];
    for (int k = 0; k < 3; k++) {
        const float v = pred[(size_t)g * mlp::kOut + k] * ynorm[mlp::kOut + k] + ynorm[k];
        c[k] = fminf(fmaxf(v, 0.05f), 1.0f);
    }
    B.tea_ci[g] = make_float4((1.0f / (c[0] * c[0]) - 1.0f) * ib2, (1.0f / (c[1] * c[1]) - 1.0f) * ib2,
                              (1.0f / (c[2] * c[2]) - 1.0f) * ib2, 0.f);
}

// Mobility error of a re-check: sum |f_s - f_e|^2 and |f_e|^2 over active
// beads (FP64 block partials, then one block); sets *gate when
// sqrt(num/den) exceeds max_err.
__global__ void k_mob_partial(int nb, const int *flags, const float4 *fs, const float4 *fe, double *part,
                              const int *gate) {
    if (gate && *gate) return;
    double a = 0.0, b = 0.0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < nb; g += gridDim.x * blockDim.x) {
        if (flags[g] & kFlagExtra) continue;
        const float4 s = fs[g], e = fe[g];
        const double dx = (double)s.x - e.x, dy = (double)s.y - e.y, dz = (double)s.z - e.z;
        a += dx * dx + dy * dy + dz * dz;
        b += (double)e.x * e.x + (double)e.y * e.y + (double)e.z * e.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __shared__ double sa[8], sb[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sa[wid] = a;
        sb[wid] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0, y = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            x += sa[w];
            y += sb[w];
        }
        part[2 * blockIdx.x] = x;
        part[2 * blockIdx.x + 1] = y;
    }
}

__global__ void k_mob_final(const double *part, int nparts, float max_err, double *err_out, int *gate,
                            int *nchecks) {
    if (gate[0]) return;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < nparts; i++) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    const double e = b > 0 ? sqrt(a / b) : 0.0;
    *err_out = e;
    *nchecks += 1;
    if (!(e <= (double)max_err)) {  // NaN falls back too
        gate[0] = 1;
        gate[2] = 1;
    }
}

// At the fall-back: the exact C_i and beta of the re-check replace the
// surrogate's at once (gate[2] marks a fall-back not yet applied).
__global__ void k_fallback_copy(int nb, int nt, const int *gate, const float4 *ci2, const float *beta2, float4 *ci,
                                float *beta) {
    if (gate[2] == 0) return;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < nb) ci[g] = ci2[g];
    if (g < nt) beta[g] = beta2[g];
}
__global__ void k_fallback_clear(int *gate) { gate[2] = 0; }

constexpr int kMobBlocks = 256;

}  // namespace

// ------------------------------------------------------------ the network
struct mtg_surrogate {
    int device = 0;
    cudaStream_t stream = nullptr;
    mlp::Weights W{};
    float *norm = nullptr;     // [2*kIn] input mean, inverse std
    float *ynorm = nullptr;    // [2*kOut] output mean, std
    float h_norm[2 * mlp::kIn] = {0};
    float h_ynorm[2 * mlp::kOut] = {0};
    __nv_bfloat16 *bf = nullptr;  // all BF16 copies
    int *err = nullptr;            // device error word of the tensor-core inference
    int adam_step = 0;
    uint32_t spin = mlp::tc_default_spin();   // polls of the inference's waits for its MMAs
};

namespace {

thread_local char g_surr_err[256] = "no error";

int sfail(int code, const char *msg) {
    std::snprintf(g_surr_err, sizeof g_surr_err, "%s", msg);
    return mtg_internal_fail(code, msg);
}

#define SCK(call)                                                                  \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) return sfail(MTG_E_CUDA, cudaGetErrorString(e_));   \
    } while (0)

int upload_norms(mtg_surrogate *s) {
    SCK(cudaMemcpyAsync(s->norm, s->h_norm, sizeof(s->h_norm), cudaMemcpyHostToDevice, s->stream));
    SCK(cudaMemcpyAsync(s->ynorm, s->h_ynorm, sizeof(s->h_ynorm), cudaMemcpyHostToDevice, s->stream));
    return MTG_OK;
}

}  // namespace

extern "C" {

int mtg_surrogate_create(int device, int seed, mtg_surrogate **out) {
    if (!out) return sfail(MTG_E_CONFIG, "out is NULL");
    *out = nullptr;
    SCK(cudaSetDevice(device));
    SCK(mlp::prepare_tc());
    auto *s = new mtg_surrogate();
    s->device = device;
    SCK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    const size_t P = mlp::kParams;
    SCK(cudaMalloc(&s->W.master, 3 * P * sizeof(float)));
    s->W.m = s->W.master + P;
    s->W.v = s->W.m + P;
    s->W.b = s->W.master + mlp::kOffB;
    const size_t nbf = (size_t)mlp::kHid * mlp::kIn + 2 * 2 * mlp::kHid * mlp::kHid + 2 * mlp::kOut * mlp::kHid;
    SCK(cudaMalloc(&s->bf, nbf * sizeof(__nv_bfloat16)));
    s->W.w1 = s->bf;
    s->W.w2 = s->W.w1 + mlp::kHid * mlp::kIn;
    s->W.w3 = s->W.w2 + mlp::kHid * mlp::kHid;
    s->W.w4 = s->W.w3 + mlp::kHid * mlp::kHid;
    s->W.w2t = s->W.w4 + mlp::kOut * mlp::kHid;
    s->W.w3t = s->W.w2t + mlp::kHid * mlp::kHid;
    s->W.w4t = s->W.w3t + mlp::kHid * mlp::kHid;
    SCK(cudaMalloc(&s->norm, sizeof(s->h_norm)));
    SCK(cudaMalloc(&s->ynorm, sizeof(s->h_ynorm)));
    SCK(cudaMalloc(&s->err, sizeof(int)));
    SCK(cudaMemsetAsync(s->err, 0, sizeof(int), s->stream));
    // Glorot-uniform weights, zero biases, identity normalisation
    std::vector<float> h(P, 0.f);
    std::mt19937 rng((uint32_t)seed);
    auto fill = [&](int off, int fan_out, int fan_in) {
        const float lim = std::sqrt(6.0f / (float)(fan_in + fan_out));
        std::uniform_real_distribution<float> u(-lim, lim);
        for (int i = 0; i < fan_out * fan_in; i++) h[off + i] = u(rng);
    };
    fill(mlp::kOffW1, mlp::kHid, mlp::kIn);
    fill(mlp::kOffW2, mlp::kHid, mlp::kHid);
    fill(mlp::kOffW3, mlp::kHid, mlp::kHid);
    fill(mlp::kOffW4, mlp::kOut, mlp::kHid);
    for (int k = 0; k < mlp::kIn; k++) s->h_norm[mlp::kIn + k] = 1.0f;
    for (int k = 0; k < mlp::kOut; k++) s->h_ynorm[mlp::kOut + k] = 1.0f;
    SCK(cudaMemcpyAsync(s->W.master, h.data(), P * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    SCK(cudaMemsetAsync(s->W.m, 0, 2 * P * sizeof(float), s->stream));
    SCK(mlp::launch_refresh(s->W, s->stream));
    int rc = upload_norms(s);
    if (rc) return rc;
    SCK(cudaStreamSynchronize(s->stream));
    *out = s;
    return MTG_OK;
}

int mtg_surrogate_destroy(mtg_surrogate *s) {
    if (!s) return MTG_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->W.master);
    cudaFree(s->bf);
    cudaFree(s->norm);
    cudaFree(s->ynorm);
    cudaFree(s->err);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return MTG_OK;
}

int mtg_surrogate_get_params(mtg_surrogate *s, float *params, float *norm) {
    if (!s) return sfail(MTG_E_CONFIG, "surrogate is NULL");
    SCK(cudaSetDevice(s->device));
    if (params)
        SCK(cudaMemcpyAsync(params, s->W.master, sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaStreamSynchronize(s->stream));
    if (norm) {
        std::memcpy(norm, s->h_norm, sizeof(s->h_norm));
        std::memcpy(norm + 2 * mlp::kIn, s->h_ynorm, sizeof(s->h_ynorm));
    }
    return MTG_OK;
}

int mtg_surrogate_set_params(mtg_surrogate *s, const float *params, const float *norm) {
    if (!s) return sfail(MTG_E_CONFIG, "surrogate is NULL");
    SCK(cudaSetDevice(s->device));
    if (params) {
        SCK(cudaMemcpyAsync(s->W.master, params, sizeof(float) * mlp::kParams, cudaMemcpyHostToDevice, s->stream));
        SCK(mlp::launch_refresh(s->W, s->stream));
    }
    if (norm) {
        std::memcpy(s->h_norm, norm, sizeof(s->h_norm));
        std::memcpy(s->h_ynorm, norm + 2 * mlp::kIn, sizeof(s->h_ynorm));
        int rc = upload_norms(s);
        if (rc) return rc;
    }
    SCK(cudaStreamSynchronize(s->stream));
    return MTG_OK;
}

int mtg_surrogate_predict(mtg_surrogate *s, const float *X, int n, float *Y) {
    if (!s || !X || !Y || n < 0) return sfail(MTG_E_CONFIG, "bad arguments");
    SCK(cudaSetDevice(s->device));
    float *dX = nullptr, *dY = nullptr;
    SCK(cudaMalloc(&dX, sizeof(float) * (size_t)n * mlp::kIn + 16));
    SCK(cudaMalloc(&dY, sizeof(float) * (size_t)n * mlp::kOut + 16));
    SCK(cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * mlp::kIn, cudaMemcpyHostToDevice, s->stream));
    SCK(mlp::launch_infer_tc(s->W, dX, n, s->norm, dY, s->err, s->stream, s->spin));
    int herr = 0;
    SCK(cudaMemcpyAsync(Y, dY, sizeof(float) * (size_t)n * mlp::kOut, cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaMemcpyAsync(&herr, s->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaStreamSynchronize(s->stream));
    cudaFree(dX);
    cudaFree(dY);
    if (herr) {
        cudaMemsetAsync(s->err, 0, sizeof(int), s->stream);
        return sfail(MTG_E_TIMEOUT, "a bounded wait for the tensor cores ran out");
    }
    // back to target units
    for (int i = 0; i < n; i++)
        for (int k = 0; k < mlp::kOut; k++)
            Y[(size_t)i * mlp::kOut + k] = Y[(size_t)i * mlp::kOut + k] * s->h_ynorm[mlp::kOut + k] + s->h_ynorm[k];
    return MTG_OK;
}

// Loss and parameter gradient of one batch (no update): T in target units,
// loss = mean over samples and outputs of the squared normalised error.
int mtg_surrogate_loss_grad(mtg_surrogate *s, const float *X, const float *T, int n, double *loss, float *grad) {
    if (!s || !X || !T || n <= 0) return sfail(MTG_E_CONFIG, "bad arguments");
    SCK(cudaSetDevice(s->device));
    const int parts = mlp::backward_parts(n);
    std::vector<float> Tn((size_t)n * mlp::kOut);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < mlp::kOut; k++)
            Tn[(size_t)i * mlp::kOut + k] = (T[(size_t)i * mlp::kOut + k] - s->h_ynorm[k]) / s->h_ynorm[mlp::kOut + k];
    float *dX, *dT, *dY, *dZ, *dG, *dL;
    SCK(cudaMalloc(&dX, sizeof(float) * (size_t)n * mlp::kIn));
    SCK(cudaMalloc(&dT, sizeof(float) * (size_t)n * mlp::kOut));
    SCK(cudaMalloc(&dY, sizeof(float) * (size_t)n * mlp::kOut));
    SCK(cudaMalloc(&dZ, sizeof(float) * (size_t)n * 3 * mlp::kHid));
    SCK(cudaMalloc(&dG, sizeof(float) * (size_t)parts * mlp::kParams));
    SCK(cudaMalloc(&dL, sizeof(float) * parts));
    SCK(cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * mlp::kIn, cudaMemcpyHostToDevice, s->stream));
    SCK(cudaMemcpyAsync(dT, Tn.data(), sizeof(float) * Tn.size(), cudaMemcpyHostToDevice, s->stream));
    SCK(mlp::launch_forward_tc(s->W, dX, nullptr, n, s->norm, dY, dZ, s->err, s->stream));
    SCK(mlp::launch_backward_tc(s->W, dX, nullptr, s->norm, dT, n, dY, dZ, dG, dL, s->err, s->stream));
    std::vector<float> G((size_t)parts * mlp::kParams), L(parts);
    int herr = 0;
    SCK(cudaMemcpyAsync(G.data(), dG, sizeof(float) * G.size(), cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaMemcpyAsync(L.data(), dL, sizeof(float) * parts, cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaMemcpyAsync(&herr, s->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaStreamSynchronize(s->stream));
    if (herr) {
        for (float *p : {dX, dT, dY, dZ, dG, dL}) cudaFree(p);
        cudaMemsetAsync(s->err, 0, sizeof(int), s->stream);
        return sfail(MTG_E_TIMEOUT, "a bounded wait for the tensor cores ran out");
    }
    for (float *p : {dX, dT, dY, dZ, dG, dL}) cudaFree(p);
    double l = 0.0;
    for (float v : L) l += v;
    if (loss) *loss = l / ((double)n * mlp::kOut);
    if (grad)
        for (int i = 0; i < mlp::kParams; i++) {
            double g = 0.0;
            for (int p = 0; p < parts; p++) g += G[(size_t)p * mlp::kParams + i];
            grad[i] = (float)g;
        }
    return MTG_OK;
}

// Trains on n samples (X raw features, T targets in their units) with Adam:
// the normalisation (per-feature mean/std of X and T) is fitted first;
// loss_per_epoch [epochs] receives the mean normalised squared error.
int mtg_surrogate_train(mtg_surrogate *s, const float *X, const float *T, int n, int epochs, int batch, float lr,
                        int seed, float *loss_per_epoch) {
    if (!s || !X || !T || n <= 0 || epochs <= 0 || batch <= 0) return sfail(MTG_E_CONFIG, "bad arguments");
    if (batch % 32 != 0) return sfail(MTG_E_CONFIG, "batch must be a multiple of 32");
    SCK(cudaSetDevice(s->device));
    // normalisation: per-column mean and standard deviation, two row-major passes
    auto moments = [n](const float *A, int cols, std::vector<double> &mean, std::vector<double> &sd) {
        mean.assign(cols, 0.0);
        sd.assign(cols, 0.0);
        for (size_t i = 0; i < (size_t)n; i++)
            for (int k = 0; k < cols; k++) mean[k] += A[i * cols + k];
        for (int k = 0; k < cols; k++) mean[k] /= n;
        for (size_t i = 0; i < (size_t)n; i++)
            for (int k = 0; k < cols; k++) {
                const double d = A[i * cols + k] - mean[k];
                sd[k] += d * d;
            }
        for (int k = 0; k < cols; k++) sd[k] = std::sqrt(sd[k] / n);
    };
    std::vector<double> mean, sd;
    moments(X, mlp::kIn, mean, sd);
    for (int k = 0; k < mlp::kIn; k++) {
        s->h_norm[k] = (float)mean[k];
        s->h_norm[mlp::kIn + k] = sd[k] > 1e-12 ? (float)(1.0 / sd[k]) : 1.0f;
    }
    moments(T, mlp::kOut, mean, sd);
    std::vector<float> Tn((size_t)n * mlp::kOut);
    for (int k = 0; k < mlp::kOut; k++) {
        s->h_ynorm[k] = (float)mean[k];
        s->h_ynorm[mlp::kOut + k] = sd[k] > 1e-12 ? (float)sd[k] : 1.0f;
    }
    for (size_t i = 0; i < (size_t)n; i++)
        for (int k = 0; k < mlp::kOut; k++)
            Tn[i * mlp::kOut + k] = (float)((T[i * mlp::kOut + k] - mean[k]) / s->h_ynorm[mlp::kOut + k]);
    int rc = upload_norms(s);
    if (rc) return rc;
    const int parts = mlp::backward_parts(batch);
    const int nbatches = n / batch;
    if (nbatches == 0) return sfail(MTG_E_CONFIG, "fewer samples than one batch");
    // scratch of the run, released on every return (cudaFree waits for the
    // device, so no kernel still reads it)
    struct Scratch {
        float *X = nullptr, *T = nullptr, *Y = nullptr, *Z = nullptr, *G = nullptr, *L = nullptr, *Lsum = nullptr;
        int *idx = nullptr;
        cudaEvent_t copied[2] = {nullptr, nullptr};
        ~Scratch() {
            for (float *p : {X, T, Y, Z, G, L, Lsum})
                if (p) cudaFree(p);
            if (idx) cudaFree(idx);
            for (cudaEvent_t ev : copied)
                if (ev) cudaEventDestroy(ev);
        }
    } S;
    SCK(cudaMalloc(&S.X, sizeof(float) * (size_t)n * mlp::kIn));
    SCK(cudaMalloc(&S.T, sizeof(float) * (size_t)n * mlp::kOut));
    SCK(cudaMalloc(&S.Y, sizeof(float) * (size_t)batch * mlp::kOut));
    SCK(cudaMalloc(&S.Z, sizeof(float) * (size_t)batch * 3 * mlp::kHid));
    SCK(cudaMalloc(&S.G, sizeof(float) * (size_t)parts * mlp::kParams));
    SCK(cudaMalloc(&S.L, sizeof(float) * (size_t)parts * nbatches));
    SCK(cudaMalloc(&S.Lsum, sizeof(float) * epochs));
    SCK(cudaMalloc(&S.idx, sizeof(int) * (size_t)n));
    float *dX = S.X, *dT = S.T, *dY = S.Y, *dZ = S.Z, *dG = S.G, *dL = S.L, *dLsum = S.Lsum;
    int *dIdx = S.idx;
    cudaEvent_t *copied = S.copied;
    SCK(cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * mlp::kIn, cudaMemcpyHostToDevice, s->stream));
    SCK(cudaMemcpyAsync(dT, Tn.data(), sizeof(float) * Tn.size(), cudaMemcpyHostToDevice, s->stream));
    // The host shuffles epoch ep + 1 while the device runs epoch ep: two host
    // permutations, the one being refilled last read by the copy of two
    // epochs ago (waited for through its event); dIdx itself is rewritten in
    // stream order after the previous epoch's kernels.
    std::vector<int> perm[2] = {std::vector<int>(n), std::vector<int>(n)};
    std::iota(perm[1].begin(), perm[1].end(), 0);
    SCK(cudaEventCreateWithFlags(&copied[0], cudaEventDisableTiming));
    SCK(cudaEventCreateWithFlags(&copied[1], cudaEventDisableTiming));
    std::mt19937 rng((uint32_t)seed);
    for (int ep = 0; ep < epochs; ep++) {
        const int k = ep & 1;
        if (ep >= 2) SCK(cudaEventSynchronize(copied[k]));
        perm[k] = perm[k ^ 1];
        std::shuffle(perm[k].begin(), perm[k].end(), rng);
        SCK(cudaMemcpyAsync(dIdx, perm[k].data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s->stream));
        SCK(cudaEventRecord(copied[k], s->stream));
        for (int b = 0; b < nbatches; b++) {
            const int *idx = dIdx + (size_t)b * batch;
            SCK(mlp::launch_forward_tc(s->W, dX, idx, batch, s->norm, dY, dZ, s->err, s->stream));
            SCK(mlp::launch_backward_tc(s->W, dX, idx, s->norm, dT, batch, dY, dZ, dG, dL + (size_t)b * parts, s->err,
                                        s->stream));
            SCK(mlp::launch_adam(s->W, dG, parts, lr, ++s->adam_step, s->stream));
        }
        SCK(mlp::launch_loss_sum(dL, parts * nbatches, dLsum + ep, s->stream));
    }
    std::vector<float> ls(epochs);
    int herr = 0;
    SCK(cudaMemcpyAsync(ls.data(), dLsum, sizeof(float) * epochs, cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaMemcpyAsync(&herr, s->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    SCK(cudaStreamSynchronize(s->stream));
    if (herr) {
        cudaMemsetAsync(s->err, 0, sizeof(int), s->stream);
        return sfail(MTG_E_TIMEOUT, "a bounded wait for the tensor cores ran out");
    }
    if (loss_per_epoch)
        for (int ep = 0; ep < epochs; ep++) loss_per_epoch[ep] = ls[ep] / ((float)nbatches * batch * mlp::kOut);
    return MTG_OK;
}

// --------------------------------------------------- engine integration
// Descriptors of the current state and, with TEA on, the exact targets
// (an epsilon pass is run first).  X [nb*32], T [nb*4] (either may be NULL).
int mtg_tea_training_data(mtg_engine *e, float *X, float *T) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (!e->have_state) return mtg_internal_fail(MTG_E_STATE, "no state uploaded");
    if (T && !e->p.hdi_on) return mtg_internal_fail(MTG_E_STATE, "targets need an engine created with hdi_on");
    SCK(cudaSetDevice(e->device));
    int rc = mtg_surrogate_buffers(e);
    if (rc) return rc;
    const DevBuffers B = e->bufs();
    k_traj_stats<<<e->nt, 256, 0, e->stream>>>(e->kp, B, e->surr_stats);
    const float inv = bin_beads(e->kp, B, e->cells(), kDescCut, true, e->stream);
    k_descriptors<<<e->nwork, kTile, 0, e->stream>>>(e->kp, B, e->cells(), e->work, inv, e->surr_stats, e->surr_desc,
                                                     nullptr);
    if (T) {
        launch_tea_eps(e->kp, B, e->tea_work, e->tea_nwork, e->stream);
        launch_tea_beta(e->kp, B, e->p.tea_capricious, e->p.tea_epsmax, e->stream);
        k_tea_targets<<<(e->nb + 255) / 256, 256, 0, e->stream>>>(e->kp, B, e->surr_pred);
    }
    SCK(cudaGetLastError());
    if (X) SCK(cudaMemcpyAsync(X, e->surr_desc, sizeof(float) * (size_t)e->nb * kF, cudaMemcpyDeviceToHost, e->stream));
    if (T)
        SCK(cudaMemcpyAsync(T, e->surr_pred, sizeof(float) * (size_t)e->nb * mlp::kOut, cudaMemcpyDeviceToHost,
                            e->stream));
    SCK(cudaStreamSynchronize(e->stream));
    return MTG_OK;
}

}  // extern "C"

// Allocates the engine's surrogate buffers on first use (outside captures).
int mtg_surrogate_buffers(mtg_engine *e) {
    if (e->surr_desc) return MTG_OK;
    const size_t nb = e->nb;
    SCK(cudaMalloc(&e->surr_desc, sizeof(float) * nb * kF));
    SCK(cudaMalloc(&e->surr_pred, sizeof(float) * nb * mlp::kOut));
    SCK(cudaMalloc(&e->surr_stats, sizeof(float4) * e->nt));
    SCK(cudaMalloc(&e->surr_gate, sizeof(int) * 3));
    SCK(cudaMalloc(&e->surr_err, sizeof(double)));
    SCK(cudaMalloc(&e->surr_part, sizeof(double) * 2 * kMobBlocks));
    SCK(cudaMemsetAsync(e->surr_gate, 0, sizeof(int) * 3, e->stream));
    SCK(cudaMemsetAsync(e->surr_err, 0, sizeof(double), e->stream));
    if (e->p.hdi_on) {
        SCK(cudaMalloc(&e->tea_ci2, sizeof(float4) * nb));
        SCK(cudaMalloc(&e->tea_eps2, sizeof(float) * nb));
        SCK(cudaMalloc(&e->tea_beta2, sizeof(float) * e->nt));
        SCK(cudaMalloc(&e->tea_eps_t2, sizeof(double) * e->nt));
        SCK(cudaMalloc(&e->feff_a, sizeof(float4) * nb));
        SCK(cudaMalloc(&e->feff_b, sizeof(float4) * nb));
    }
    return MTG_OK;
}

// Learned-mode work at an epsilon step: descriptors, network, TEA state.
void enqueue_surrogate_eps(mtg_engine *e) {
    const DevBuffers B = e->bufs();
    const int *gate = e->surr_gate;
    k_traj_stats<<<e->nt, 256, 0, e->stream>>>(e->kp, B, e->surr_stats);
    const float inv = bin_beads(e->kp, B, e->cells(), kDescCut, true, e->stream);
    k_descriptors<<<e->nwork, kTile, 0, e->stream>>>(e->kp, B, e->cells(), e->work, inv, e->surr_stats, e->surr_desc,
                                                     gate);
    mlp::launch_infer_tc(e->surr->W, e->surr_desc, e->nb, e->surr->norm, e->surr_pred, e->err, e->stream,
                         e->surr->spin);
    k_surr_beta<<<e->nt, 256, 0, e->stream>>>(e->kp, B, e->surr_pred, e->surr->ynorm, gate);
    k_surr_ci<<<(e->nb + 255) / 256, 256, 0, e->stream>>>(e->kp, B, e->surr_pred, e->surr->ynorm, gate);
    // after a fallback the exact pass runs instead (gated on the flag)
    launch_tea_eps_gated(e->kp, B, e->tea_work, e->tea_nwork, gate, 1, e->stream);
    launch_tea_beta_gated(e->kp, B, e->p.tea_capricious, e->p.tea_epsmax, gate, 1, e->stream);
}

// Exact re-check: exact C_i and beta into the second set of TEA buffers,
// the effective forces under both from identical F and R, their RMS
// difference; the gate flips to exact TEA when it exceeds the threshold.
void enqueue_surrogate_recheck(mtg_engine *e) {
    DevBuffers Bs = e->bufs();
    DevBuffers Be = Bs;
    Be.tea_ci = e->tea_ci2;
    Be.tea_eps = e->tea_eps2;
    Be.tea_beta = e->tea_beta2;
    Be.tea_eps_t = e->tea_eps_t2;
    const int *gate = e->surr_gate;
    launch_tea_eps_gated(e->kp, Be, e->tea_work, e->tea_nwork, gate, 0, e->stream);
    launch_tea_beta_gated(e->kp, Be, e->p.tea_capricious, e->p.tea_epsmax, gate, 0, e->stream);
    launch_tea_feff(e->kp, Be, e->tea_work, e->tea_nwork, e->feff_a, gate, e->stream);
    if (e->ff_on)   // the learned mode's product is the far-field one
        launch_ff_step(e->kp, Bs, e->ffb, true, e->feff_b, gate, e->stream);
    else
        launch_tea_feff(e->kp, Bs, e->tea_work, e->tea_nwork, e->feff_b, gate, e->stream);
    k_mob_partial<<<kMobBlocks, 256, 0, e->stream>>>(e->nb, e->flags, e->feff_b, e->feff_a, e->surr_part, gate);
    k_mob_final<<<1, 1, 0, e->stream>>>(e->surr_part, kMobBlocks, e->surr_max_err, e->surr_err, e->surr_gate,
                                        e->surr_gate + 1);
    const int n = e->nb > e->nt ? e->nb : e->nt;
    k_fallback_copy<<<(n + 255) / 256, 256, 0, e->stream>>>(e->nb, e->nt, e->surr_gate, e->tea_ci2, e->tea_beta2,
                                                            e->tea_ci, e->tea_beta);
    k_fallback_clear<<<1, 1, 0, e->stream>>>(e->surr_gate);
}

extern "C" {

int mtg_set_surrogate(mtg_engine *e, mtg_surrogate *s, int recheck_every, float max_err) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (s && !e->p.hdi_on) return mtg_internal_fail(MTG_E_STATE, "the learned mode replaces TEA: create with hdi_on");
    if (s && s->device != e->device) return mtg_internal_fail(MTG_E_CONFIG, "surrogate and engine on different GPUs");
    if (recheck_every < 0) return mtg_internal_fail(MTG_E_CONFIG, "recheck_every must be >= 0");
    SCK(cudaSetDevice(e->device));
    int rc = mtg_surrogate_buffers(e);
    if (rc) return rc;
    e->surr = s;
    e->surr_recheck = recheck_every;
    e->surr_max_err = max_err;
    SCK(cudaMemsetAsync(e->surr_gate, 0, sizeof(int) * 3, e->stream));
    SCK(cudaMemsetAsync(e->surr_err, 0, sizeof(double), e->stream));
    SCK(cudaStreamSynchronize(e->stream));
    mtg_internal_reset_graphs(e);
    return MTG_OK;
}

int mtg_surrogate_set_wait_limit(mtg_surrogate *s, int polls) {
    if (!s) return sfail(MTG_E_CONFIG, "surrogate is NULL");
    s->spin = polls < 0 ? mlp::tc_default_spin() : (uint32_t)polls;
    return MTG_OK;
}

int mtg_surrogate_status(mtg_engine *e, int *fell_back, int *rechecks, double *last_error) {
    if (!e) return mtg_internal_fail(MTG_E_CONFIG, "engine is NULL");
    if (!e->surr_gate) {
        if (fell_back) *fell_back = 0;
        if (rechecks) *rechecks = 0;
        if (last_error) *last_error = 0.0;
        return MTG_OK;
    }
    SCK(cudaSetDevice(e->device));
    int g[2];
    double err = 0.0;
    SCK(cudaMemcpyAsync(g, e->surr_gate, sizeof g, cudaMemcpyDeviceToHost, e->stream));
    SCK(cudaMemcpyAsync(&err, e->surr_err, sizeof err, cudaMemcpyDeviceToHost, e->stream));
    SCK(cudaStreamSynchronize(e->stream));
    if (fell_back) *fell_back = g[0];
    if (rechecks) *rechecks = g[1];
    if (last_error) *last_error = err;
    return MTG_OK;
}

}  // extern "C"
