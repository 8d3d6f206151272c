// kernels_mlp.cu - the TEA surrogate network: a 32-128-128-128-4 perceptron
// with SiLU activations, BF16 weights and activations, FP32 accumulation on
// the tensor cores, trained with Adam on FP32 master weights.
//
// One CTA handles kRows samples; each of its warps owns 16 rows and keeps
// them through all layers, so layers need no CTA barrier.  Weights live in
// shared memory, K-contiguous and padded by 8 elements per row so that the
// fragment loads of the m16n8k16 MMA are bank-conflict free.
//
//   k_mlp_forward   : inference, or training forward that also stores the
//                     pre-activations z1..z3 and the output
//   k_mlp_backward  : output gradient of the MSE loss, activation gradients
//                     back to layer 1, per-CTA partial weight/bias gradients
//   k_mlp_adam      : reduces the partials, Adam step on the FP32 masters,
//                     refreshes both BF16 copies (forward and transposed)
#include <cuda_bf16.h>
#include <stdint.h>

#include "mtg_mlp.cuh"

namespace mtg {
namespace mlp {

namespace {

constexpr int kRows = 32;    // samples per CTA (a 4096-sample batch spreads over 128 CTAs)
constexpr int kWarps = kRows / 16;
constexpr int kPadIn = kIn + 8;    // 40
constexpr int kPadH = kHid + 8;    // 136
constexpr int kPadRows = kRows + 8;

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment (16x16, row-major, leading dimension lda elements) at (r0, k0).
__device__ __forceinline__ void load_a(uint32_t (&a)[4], const __nv_bfloat16 *s, int lda, int r0, int k0, int lane) {
    const int r = r0 + (lane >> 2), c = k0 + (lane & 3) * 2;
    a[0] = *reinterpret_cast<const uint32_t *>(s + r * lda + c);
    a[1] = *reinterpret_cast<const uint32_t *>(s + (r + 8) * lda + c);
    a[2] = *reinterpret_cast<const uint32_t *>(s + r * lda + c + 8);
    a[3] = *reinterpret_cast<const uint32_t *>(s + (r + 8) * lda + c + 8);
}
// B fragment (16x8, stored N-major: element (k, n) at s[n * ldb + k]) at (k0, n0).
__device__ __forceinline__ void load_b(uint32_t (&b)[2], const __nv_bfloat16 *s, int ldb, int k0, int n0, int lane) {
    const int n = n0 + (lane >> 2), k = k0 + (lane & 3) * 2;
    b[0] = *reinterpret_cast<const uint32_t *>(s + n * ldb + k);
    b[1] = *reinterpret_cast<const uint32_t *>(s + n * ldb + k + 8);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// rows of this warp: acc[n-tile][4] for N = NT*8 columns, K = KT*16
template <int NT, int KT>
__device__ __forceinline__ void warp_gemm(float (&acc)[NT][4], const __nv_bfloat16 *sA, int lda, int r0,
                                          const __nv_bfloat16 *sB, int ldb, int lane) {
#pragma unroll
    for (int n = 0; n < NT; n++) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
#pragma unroll
    for (int k = 0; k < KT; k++) {
        uint32_t a[4];
        load_a(a, sA, lda, r0, k * 16, lane);
#pragma unroll
        for (int n = 0; n < NT; n++) {
            uint32_t b[2];
            load_b(b, sB, ldb, k * 16, n * 8, lane);
            mma16816(acc[n], a, b);
        }
    }
}

// Copies a [rows][cols] BF16 matrix (row-major, cols a multiple of 8) into
// shared memory rows of ld elements, 16 bytes per thread and step.
__device__ __forceinline__ void stage_rows(__nv_bfloat16 *dst, int ld, const __nv_bfloat16 *src, int rows, int cols) {
    const int vpr = cols / 8;
    for (int i = threadIdx.x; i < rows * vpr; i += blockDim.x) {
        const int r = i / vpr, c = (i % vpr) * 8;
        *reinterpret_cast<uint4 *>(dst + r * ld + c) = *reinterpret_cast<const uint4 *>(src + (size_t)r * cols + c);
    }
}

}  // namespace

// ---------------------------------------------------------------- forward
// X: [n][kIn] f32 (normalised features) gathered through idx (or identity);
// Y: [n][kOut] f32 outputs.  When train != 0, Z: [n][3][kHid] f32
// pre-activations of the hidden layers are stored (row order of the batch).
__global__ void __launch_bounds__(kRows * 2) k_mlp_forward(const Weights W, const float *X, const int *idx, int n,
                                                           const float *norm, float *Y, float *Z) {
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16 *sW1 = reinterpret_cast<__nv_bfloat16 *>(smem);            // [kHid][kPadIn]
    __nv_bfloat16 *sW2 = sW1 + kHid * kPadIn;                                 // [kHid][kPadH]
    __nv_bfloat16 *sW3 = sW2 + kHid * kPadH;                                  // [kHid][kPadH]
    __nv_bfloat16 *sW4 = sW3 + kHid * kPadH;                                  // [8][kPadH]
    __nv_bfloat16 *sX = sW4 + 8 * kPadH;                                      // [kRows][kPadIn]
    __nv_bfloat16 *sH = sX + kRows * kPadIn;                                  // [kRows][kPadH]
    float *sb = reinterpret_cast<float *>(sH + kRows * kPadH);               // biases: 3*kHid + 8
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int row0 = blockIdx.x * kRows;
    // weights (BF16, N-major) and biases
    stage_rows(sW1, kPadIn, W.w1, kHid, kIn);
    stage_rows(sW2, kPadH, W.w2, kHid, kHid);
    stage_rows(sW3, kPadH, W.w3, kHid, kHid);
    for (int i = tid; i < 8 * kHid; i += blockDim.x)
        sW4[(i / kHid) * kPadH + i % kHid] = (i / kHid) < kOut ? W.w4[i] : __float2bfloat16(0.f);
    for (int i = tid; i < 3 * kHid; i += blockDim.x) sb[i] = W.b[i];
    for (int i = tid; i < 8; i += blockDim.x) sb[3 * kHid + i] = i < kOut ? W.b[3 * kHid + i] : 0.f;
    // inputs
    for (int i = tid; i < kRows * kIn; i += blockDim.x) {
        const int r = i / kIn, c = i % kIn, gr = row0 + r;
        float v = 0.f;
        if (gr < n) {
            v = X[(size_t)(idx ? idx[gr] : gr) * kIn + c];
            if (norm) v = (v - norm[c]) * norm[kIn + c];
        }
        sX[r * kPadIn + c] = __float2bfloat16(v);
    }
    __syncthreads();
    if (warp >= kWarps) return;
    const int r0 = warp * 16;
    const int ra = r0 + (lane >> 2), cb = (lane & 3) * 2;
    float acc[kHid / 8][4];
    // layer 1 (K = 32)
    warp_gemm<kHid / 8, kIn / 16>(acc, sX, kPadIn, r0, sW1, kPadIn, lane);
    for (int layer = 0; layer < 3; layer++) {
        if (layer > 0) {
            __syncwarp();
            if (layer == 1)
                warp_gemm<kHid / 8, kHid / 16>(acc, sH, kPadH, r0, sW2, kPadH, lane);
            else
                warp_gemm<kHid / 8, kHid / 16>(acc, sH, kPadH, r0, sW3, kPadH, lane);
            __syncwarp();
        }
#pragma unroll
        for (int t = 0; t < kHid / 8; t++) {
            const int c = t * 8 + cb;
            const float z0 = acc[t][0] + sb[layer * kHid + c], z1 = acc[t][1] + sb[layer * kHid + c + 1];
            const float z2 = acc[t][2] + sb[layer * kHid + c], z3 = acc[t][3] + sb[layer * kHid + c + 1];
            if (Z) {
                const int g0 = row0 + ra, g1 = row0 + ra + 8;
                if (g0 < n) {
                    Z[((size_t)g0 * 3 + layer) * kHid + c] = z0;
                    Z[((size_t)g0 * 3 + layer) * kHid + c + 1] = z1;
                }
                if (g1 < n) {
                    Z[((size_t)g1 * 3 + layer) * kHid + c] = z2;
                    Z[((size_t)g1 * 3 + layer) * kHid + c + 1] = z3;
                }
            }
            *reinterpret_cast<uint32_t *>(sH + ra * kPadH + c) = pack2(silu(z0), silu(z1));
            *reinterpret_cast<uint32_t *>(sH + (ra + 8) * kPadH + c) = pack2(silu(z2), silu(z3));
        }
    }
    __syncwarp();
    // output layer (N = 8, first kOut used)
    float out[1][4];
    warp_gemm<1, kHid / 16>(out, sH, kPadH, r0, sW4, kPadH, lane);
    const int g0 = row0 + ra, g1 = row0 + ra + 8;
    if (cb < kOut) {
        if (g0 < n) {
            Y[(size_t)g0 * kOut + cb] = out[0][0] + sb[3 * kHid + cb];
            if (cb + 1 < kOut) Y[(size_t)g0 * kOut + cb + 1] = out[0][1] + sb[3 * kHid + cb + 1];
        }
        if (g1 < n) {
            Y[(size_t)g1 * kOut + cb] = out[0][2] + sb[3 * kHid + cb];
            if (cb + 1 < kOut) Y[(size_t)g1 * kOut + cb + 1] = out[0][3] + sb[3 * kHid + cb + 1];
        }
    }
}

// --------------------------------------------------------------- backward
// Loss = mean over the batch and the kOut outputs of (Y - T)^2.  Per CTA:
// activation gradients for its 128 rows and partial weight gradients
// G[cta] = sum over its rows (layout of the FP32 masters).
__global__ void __launch_bounds__(kRows * 2) k_mlp_backward(const Weights W, const float *X, const int *idx,
                                                            const float *norm, const float *T, int n, const float *Y,
                                                            const float *Z, float *G, float *loss_part) {
    extern __shared__ __align__(16) unsigned char smem[];
    // transposed weights for the activation gradients: element (k = out, n = in)
    __nv_bfloat16 *sW2t = reinterpret_cast<__nv_bfloat16 *>(smem);    // [kHid in][kPadH]
    __nv_bfloat16 *sW3t = sW2t + kHid * kPadH;                        // [kHid in][kPadH]
    __nv_bfloat16 *sW4t = sW3t + kHid * kPadH;                        // [kHid in][24] (k = out, 16 used)
    __nv_bfloat16 *sD = sW4t + kHid * 24;                             // [kRows][kPadH] dZ of the current layer
    __nv_bfloat16 *sDt = sD + kRows * kPadH;                          // [kHid][kPadRows] dZ transposed
    __nv_bfloat16 *sHt = sDt + kHid * kPadRows;                       // [kHid][kPadRows] activations transposed
    float *sred = reinterpret_cast<float *>(sHt + kHid * kPadRows);   // [kWarps] loss partial
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int row0 = blockIdx.x * kRows;
    const float scale = 2.0f / ((float)n * kOut);
    stage_rows(sW2t, kPadH, W.w2t, kHid, kHid);
    stage_rows(sW3t, kPadH, W.w3t, kHid, kHid);
    for (int i = tid; i < kHid * 24; i += blockDim.x) {
        const int in = i / 24, o = i % 24;
        sW4t[i] = o < kOut ? W.w4t[in * kOut + o] : __float2bfloat16(0.f);
    }
    __syncthreads();
    const int r0 = warp * 16;
    const int ra = r0 + (lane >> 2), cb = (lane & 3) * 2;
    const int g0 = row0 + ra, g1 = row0 + ra + 8;
    // this CTA's partial gradients, in the parameter layout
    float *Gc = G + (size_t)blockIdx.x * kParams;
    float *Gw[4] = {Gc + kOffW1, Gc + kOffW2, Gc + kOffW3, Gc + kOffW4};
    float *Gb = Gc + kOffB;
    // ---- dY (rows of this warp), stored as an A operand with K = 16 (kOut used)
    float lsum = 0.f;
    if (warp < kWarps) {
        for (int i = lane; i < 16 * 16; i += 32) {
            const int r = r0 + i / 16, c = i % 16, g = row0 + r;
            float d = 0.f;
            if (c < kOut && g < n) {
                const float e = Y[(size_t)g * kOut + c] - T[(size_t)(idx ? idx[g] : g) * kOut + c];
                lsum += e * e;
                d = scale * e;
            }
            sD[r * kPadH + c] = __float2bfloat16(d);
            sDt[c * kPadRows + r] = __float2bfloat16(d);
        }
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if (lane == 0 && warp < kWarps) sred[warp] = lsum;
    // ---- layers 3..1: dH = dZ_next W_next^T, dZ = dH * silu'(z)
    for (int layer = 2; layer >= 0; layer--) {
        __syncthreads();
        // activation of the layer below (input of W_{layer+1}) transposed, for dW
        // layer 2 -> h3 (input of W4), etc.: h_{layer} = silu(z_layer)
        for (int i = tid; i < kRows * kHid; i += blockDim.x) {
            const int r = i / kHid, c = i % kHid, g = row0 + r;
            const float z = g < n ? Z[((size_t)g * 3 + layer) * kHid + c] : 0.f;
            sHt[c * kPadRows + r] = __float2bfloat16(g < n ? silu(z) : 0.f);
        }
        __syncthreads();
        // weight gradient of the layer above: dW_{layer+1}[out][in] = sum_rows dZ_next[row][out] h[row][in]
        {
            const int nout = layer == 2 ? kOut : kHid;
            float *gw = Gw[layer + 1];
            float *gb = Gb + (layer + 1) * kHid;
            // warps split the output rows of dW in 16-row slices: A = dZ_next^T [out][rows], B = h^T [in][rows]
            const int slices = (nout + 15) / 16;
            for (int sidx = warp; sidx < slices; sidx += kWarps) {
                float acc[kHid / 8][4];
                warp_gemm<kHid / 8, kRows / 16>(acc, sDt, kPadRows, sidx * 16, sHt, kPadRows, lane);
#pragma unroll
                for (int t = 0; t < kHid / 8; t++) {
                    const int o0 = sidx * 16 + (lane >> 2), o1 = o0 + 8, c = t * 8 + cb;
                    if (o0 < nout) {
                        gw[o0 * kHid + c] = acc[t][0];
                        gw[o0 * kHid + c + 1] = acc[t][1];
                    }
                    if (o1 < nout) {
                        gw[o1 * kHid + c] = acc[t][2];
                        gw[o1 * kHid + c + 1] = acc[t][3];
                    }
                }
            }
            // bias gradient: column sums of dZ_next
            for (int o = tid; o < nout; o += blockDim.x) {
                float sacc = 0.f;
                for (int r = 0; r < kRows; r++) sacc += __bfloat162float(sDt[o * kPadRows + r]);
                gb[o] = sacc;
            }
        }
        __syncthreads();
        // dH_layer = dZ_next W_next^T  (rows of this warp), then dZ_layer
        if (warp < kWarps) {
            float acc[kHid / 8][4];
            if (layer == 2)
                warp_gemm<kHid / 8, 1>(acc, sD, kPadH, r0, sW4t, 24, lane);
            else if (layer == 1)
                warp_gemm<kHid / 8, kHid / 16>(acc, sD, kPadH, r0, sW3t, kPadH, lane);
            else
                warp_gemm<kHid / 8, kHid / 16>(acc, sD, kPadH, r0, sW2t, kPadH, lane);
            __syncwarp();
#pragma unroll
            for (int t = 0; t < kHid / 8; t++) {
                const int c = t * 8 + cb;
                float z[4] = {0.f, 0.f, 0.f, 0.f};
                if (g0 < n) {
                    z[0] = Z[((size_t)g0 * 3 + layer) * kHid + c];
                    z[1] = Z[((size_t)g0 * 3 + layer) * kHid + c + 1];
                }
                if (g1 < n) {
                    z[2] = Z[((size_t)g1 * 3 + layer) * kHid + c];
                    z[3] = Z[((size_t)g1 * 3 + layer) * kHid + c + 1];
                }
                const float d0 = acc[t][0] * dsilu(z[0]), d1 = acc[t][1] * dsilu(z[1]);
                const float d2 = acc[t][2] * dsilu(z[2]), d3 = acc[t][3] * dsilu(z[3]);
                *reinterpret_cast<uint32_t *>(sD + ra * kPadH + c) = pack2(d0, d1);
                *reinterpret_cast<uint32_t *>(sD + (ra + 8) * kPadH + c) = pack2(d2, d3);
                sDt[c * kPadRows + ra] = __float2bfloat16(d0);
                sDt[(c + 1) * kPadRows + ra] = __float2bfloat16(d1);
                sDt[c * kPadRows + ra + 8] = __float2bfloat16(d2);
                sDt[(c + 1) * kPadRows + ra + 8] = __float2bfloat16(d3);
            }
        }
    }
    __syncthreads();
    // dW1 = dZ1^T X: A = dZ1^T [kHid][rows], B = X^T [kIn][rows]
    for (int i = tid; i < kRows * kIn; i += blockDim.x) {
        const int r = i / kIn, c = i % kIn, g = row0 + r;
        float v = 0.f;
        if (g < n) {
            v = X[(size_t)(idx ? idx[g] : g) * kIn + c];
            if (norm) v = (v - norm[c]) * norm[kIn + c];
        }
        sHt[c * kPadRows + r] = __float2bfloat16(v);
    }
    __syncthreads();
    for (int sidx = warp; sidx < kHid / 16; sidx += kWarps) {
        float acc[kIn / 8][4];
        warp_gemm<kIn / 8, kRows / 16>(acc, sDt, kPadRows, sidx * 16, sHt, kPadRows, lane);
#pragma unroll
        for (int t = 0; t < kIn / 8; t++) {
            const int o0 = sidx * 16 + (lane >> 2), c = t * 8 + cb;
            Gw[0][o0 * kIn + c] = acc[t][0];
            Gw[0][o0 * kIn + c + 1] = acc[t][1];
            Gw[0][(o0 + 8) * kIn + c] = acc[t][2];
            Gw[0][(o0 + 8) * kIn + c + 1] = acc[t][3];
        }
    }
    for (int o = tid; o < kHid; o += blockDim.x) {
        float sacc = 0.f;
        for (int r = 0; r < kRows; r++) sacc += __bfloat162float(sDt[o * kPadRows + r]);
        Gb[o] = sacc;
    }
    __syncthreads();
    if (tid == 0) {
        float l = 0.f;
        for (int w = 0; w < kWarps; w++) l += sred[w];
        loss_part[blockIdx.x] = l;
    }
}

// ------------------------------------------------------------------- Adam
// Sums the per-CTA partial gradients, applies Adam to the FP32 masters and
// writes the BF16 forward ([out][in]) and transposed ([in][out]) copies.
__global__ void k_mlp_adam(Weights W, const float *G, int nparts, float lr, float b1, float b2, float eps, int step) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    float g = 0.f;
    for (int p = 0; p < nparts; p++) g += G[(size_t)p * kParams + i];
    float m = W.m[i] = b1 * W.m[i] + (1.0f - b1) * g;
    float v = W.v[i] = b2 * W.v[i] + (1.0f - b2) * g * g;
    const float mh = m / (1.0f - powf(b1, (float)step)), vh = v / (1.0f - powf(b2, (float)step));
    const float w = W.master[i] - lr * mh / (sqrtf(vh) + eps);
    W.master[i] = w;
    refresh_one(W, i, w);
}

__global__ void k_mlp_refresh(Weights W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) refresh_one(W, i, W.master[i]);
}

__global__ void k_mlp_loss_sum(const float *part, int nparts, float *out) {
    float s = 0.f;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += w[k];
        *out = t;
    }
}

size_t forward_smem() {
    return sizeof(__nv_bfloat16) * (kHid * kPadIn + 2 * kHid * kPadH + 8 * kPadH + kRows * kPadIn + kRows * kPadH) +
           sizeof(float) * (3 * kHid + 8);
}
size_t backward_smem() {
    return sizeof(__nv_bfloat16) * (2 * kHid * kPadH + kHid * 24 + kRows * kPadH + 2 * kHid * kPadRows) +
           sizeof(float) * kWarps;
}

int rows_per_cta() { return kRows; }

cudaError_t prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)forward_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)backward_smem());
    return e;
}

cudaError_t launch_forward(const Weights &W, const float *X, const int *idx, int n, const float *norm, float *Y,
                           float *Z, cudaStream_t s) {
    const int blocks = (n + kRows - 1) / kRows;
    if (blocks == 0) return cudaSuccess;
    k_mlp_forward<<<blocks, kWarps * 32, forward_smem(), s>>>(W, X, idx, n, norm, Y, Z);
    return cudaGetLastError();
}

cudaError_t launch_backward(const Weights &W, const float *X, const int *idx, const float *norm, const float *T, int n,
                            const float *Y, const float *Z, float *G, float *loss_part, cudaStream_t s) {
    const int blocks = (n + kRows - 1) / kRows;
    k_mlp_backward<<<blocks, kWarps * 32, backward_smem(), s>>>(W, X, idx, norm, T, n, Y, Z, G, loss_part);
    return cudaGetLastError();
}

cudaError_t launch_adam(const Weights &W, const float *G, int nparts, float lr, int step, cudaStream_t s) {
    k_mlp_adam<<<(kParams + 255) / 256, 256, 0, s>>>(W, G, nparts, lr, 0.9f, 0.999f, 1e-8f, step);
    return cudaGetLastError();
}

cudaError_t launch_refresh(const Weights &W, cudaStream_t s) {
    k_mlp_refresh<<<(kParams + 255) / 256, 256, 0, s>>>(W);
    return cudaGetLastError();
}

cudaError_t launch_loss_sum(const float *part, int nparts, float *out, cudaStream_t s) {
    k_mlp_loss_sum<<<1, 256, 0, s>>>(part, nparts, out);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace mtg
