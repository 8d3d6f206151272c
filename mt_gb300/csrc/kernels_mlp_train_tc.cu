// kernels_mlp_train_tc.cu - backward pass of the TEA surrogate network on the
// fifth-generation tensor cores (training; the forward pass with stored
// pre-activations is k_mlp_fwd_tc<true> in kernels_mlp_tc.cu).
//
// One persistent CTA per SM (four warps) walks 128-row tiles of the batch.
// Per tile, with dZ_l = dH_l o silu'(z_l) and H_l = silu(z_l):
//   dH3 = dY W4,  dW4^T += H3^T dY
//   dH2 = dZ3 W3, dW3 += dZ3^T H2, db3 += dZ3^T 1
//   dH1 = dZ2 W2, dW2 += dZ2^T H1, db2 += dZ2^T 1
//                 dW1 += dZ1^T X,  db1 += dZ1^T 1
// all as tcgen05.mma kind::f16 (M = 128) with the weight and bias gradients
// accumulating in tensor memory over the CTA's tiles (496 of 512 columns);
// the activation gradients pass through 128 TMEM columns and come back to the
// threads (one row each) for the SiLU derivative.  The operands sit in shared
// memory in the canonical no-swizzle K-major layout; the transposed copies
// (dZ^T, H^T, X^T, dY^T) are written by the threads.  At the end each CTA
// writes its partial gradients in the parameter layout; the Adam kernel sums
// them.  Loss = mean over the batch and the outputs of (Y - T)^2.
#include <cuda_bf16.h>
#include <stdint.h>

#include "mtg_tc.cuh"

namespace mtg {
namespace mlp {

namespace {

using namespace tc;

constexpr int kBwdCols = 512;
// TMEM columns of the accumulators
constexpr uint32_t kColDH = 0, kColW2 = 128, kColW3 = 256, kColW1 = 384, kColW4 = 416, kColB1 = 432,
                   kColB2 = 448, kColB3 = 464;

struct __align__(128) TcBwdSmem {
    __nv_bfloat16 w2t[kHid * kHid];         // B of dH1 = dZ2 W2: [N = in][K = out]
    __nv_bfloat16 w3t[kHid * kHid];         // B of dH2 = dZ3 W3
    __nv_bfloat16 w4t[kHid * kOutPad];      // B of dH3 = dY W4: [N = in][K = out, 4 of 16 used]
    __nv_bfloat16 dz[kTcRows * kHid];       // A of dH: [M = rows][K = out]
    __nv_bfloat16 dzt[kHid * kTcRows];      // A of dW and db: [M = out][K = rows]
    __nv_bfloat16 ht[kHid * kTcRows];       // B of dW: [N = in][K = rows]; A of dW4^T: [M = in][K = rows]
    __nv_bfloat16 dy[kTcRows * kOutPad];    // A of dH3: [M = rows][K = 16]
    __nv_bfloat16 dyt[kOutPad * kTcRows];   // B of dW4^T: [N = 16][K = rows]
    __nv_bfloat16 xt[kIn * kTcRows];        // B of dW1: [N = in][K = rows]
    __nv_bfloat16 ones[kOutPad * kTcRows];  // B of the bias sums: row 0 ones, the rest zero
    float nrm[2 * kIn];
    float red[kTcThreads / 32];
    float db4[kTcThreads / 32][kOutPad];   // per warp, summed in a fixed order
    uint64_t mbar;
    uint32_t tmem_base;
};

__device__ __forceinline__ void put_bf16(__nv_bfloat16 *base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(base) + off) = __float2bfloat16(v);
}

// sigmoid and SiLU derivative through the hardware tanh (as the forward pass)
__device__ __forceinline__ float sig_tanh(float z) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return fmaf(0.5f, t, 0.5f);
}
__device__ __forceinline__ float dsilu_tanh(float z) {
    const float s = sig_tanh(z);
    return s * fmaf(z, 1.0f - s, 1.0f);
}

// D = A B^T over K (multiples of 16) with the given shapes' descriptors
__device__ __forceinline__ void issue(uint32_t d, uint32_t a, uint32_t b, int K, uint32_t idesc, bool accumulate) {
    const uint32_t sbo = (uint32_t)(K / 8) * 128u;
    for (int ks = 0; ks < K / 16; ks++)
        mma_bf16(d, smem_desc(a + ks * 256u, 128u, sbo), smem_desc(b + ks * 256u, 128u, sbo), idesc,
                 (accumulate || ks > 0) ? 1u : 0u);
}

// reads columns [c0, c0 + 32) of this thread's TMEM lane
__device__ __forceinline__ void tmem_row32(uint32_t lane_base, uint32_t c0, float (&out)[32]) {
    uint32_t v[32];
    tmem_ld_x32(lane_base + c0, v);
    tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 32; i++) out[i] = __uint_as_float(v[i]);
}

}  // namespace

__global__ void __launch_bounds__(kTcThreads, 1) k_mlp_backward_tc(const Weights W, const float *X, const int *idx,
                                                                   const float *norm, const float *T, int n,
                                                                   const float *Y, const float *Z, float *G,
                                                                   float *loss_part, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcBwdSmem &S = *reinterpret_cast<TcBwdSmem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    stage_weights(S.w2t, W.w2t, kHid, kHid, kHid);
    stage_weights(S.w3t, W.w3t, kHid, kHid, kHid);
    // W4^T as [in][16]: element (in, out) = W4[out][in] = w4t[in * kOut + out]
    for (int i = tid; i < kHid * kOutPad; i += blockDim.x) {
        const int in = i / kOutPad, o = i % kOutPad;
        put_bf16(S.w4t, core_off(in, o, kOutPad), o < kOut ? __bfloat162float(W.w4t[in * kOut + o]) : 0.f);
    }
    for (int i = tid; i < kOutPad * kTcRows; i += blockDim.x) {
        const int r = i / kTcRows, k = i % kTcRows;
        put_bf16(S.ones, core_off(r, k, kTcRows), r == 0 ? 1.f : 0.f);
        put_bf16(S.dyt, core_off(r, k, kTcRows), 0.f);   // rows >= kOut stay zero
    }
    for (int i = tid; i < 2 * kIn; i += blockDim.x) S.nrm[i] = norm ? norm[i] : (i < kIn ? 0.f : 1.f);
    if (tid < (kTcThreads / 32) * kOutPad) S.db4[tid / kOutPad][tid % kOutPad] = 0.f;
    const uint32_t mbar = smem_u32(&S.mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(kBwdCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t a_dz = smem_u32(S.dz), a_dzt = smem_u32(S.dzt), a_ht = smem_u32(S.ht), a_dy = smem_u32(S.dy);
    const uint32_t b_w2t = smem_u32(S.w2t), b_w3t = smem_u32(S.w3t), b_w4t = smem_u32(S.w4t);
    const uint32_t b_dyt = smem_u32(S.dyt), b_xt = smem_u32(S.xt), b_ones = smem_u32(S.ones);
    const float scale = 2.0f / ((float)n * kOut);
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    uint32_t phase = 0;
    float lsum = 0.f;
    bool ok = true;
    const int r = tid;   // this thread's row of the tile = its TMEM lane

    // one synchronisation point: operands written, MMAs issued by thread 0,
    // committed, and their completion awaited by every thread
    auto run = [&](auto &&issue_all) -> bool {
        fence_async_smem();
        fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            fence_after_sync();
            issue_all();
            mma_commit(mbar);
        }
        const bool done = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
        phase ^= 1u;
        fence_after_sync();
        return done;
    };
    // dZ of this thread's row from dH in TMEM and z of the layer; writes dz
    // (unless last) and dzt
    // 32 pre-activations of this thread's row, all requested before any is used
    auto load_z32 = [&](int layer, int gr, int c0, float (&z)[32]) {
        const float4 *zr = reinterpret_cast<const float4 *>(Z + ((size_t)gr * 3 + layer) * kHid + c0);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const float4 v = gr < n ? __ldg(zr + q) : make_float4(0.f, 0.f, 0.f, 0.f);
            z[4 * q] = v.x;
            z[4 * q + 1] = v.y;
            z[4 * q + 2] = v.z;
            z[4 * q + 3] = v.w;
        }
    };
    auto dz_rows = [&](int layer, int gr, bool write_dz) {
        for (int c0 = 0; c0 < kHid; c0 += 32) {
            float dh[32], z[32];
            load_z32(layer, gr, c0, z);
            tmem_row32(lane_base, kColDH + (uint32_t)c0, dh);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                float d[8];
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int c = c0 + q * 8 + j;
                    d[j] = gr < n ? dh[q * 8 + j] * dsilu_tanh(z[q * 8 + j]) : 0.f;
                    put_bf16(S.dzt, core_off(c, r, kTcRows), d[j]);
                }
                if (write_dz) {
                    uint4 o;
                    o.x = pack_bf16(d[0], d[1]);
                    o.y = pack_bf16(d[2], d[3]);
                    o.z = pack_bf16(d[4], d[5]);
                    o.w = pack_bf16(d[6], d[7]);
                    *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(S.dz) + core_off(r, c0 + q * 8, kHid)) = o;
                }
            }
        }
    };
    // H^T of this thread's row: silu(z) of the layer
    auto ht_rows = [&](int layer, int gr) {
        for (int c0 = 0; c0 < kHid; c0 += 32) {
            float z[32];
            load_z32(layer, gr, c0, z);
#pragma unroll
            for (int j = 0; j < 32; j++)
                put_bf16(S.ht, core_off(c0 + j, r, kTcRows), gr < n ? silu_tanh(z[j]) : 0.f);
        }
    };

    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, it++) {
        const int row0 = tile * kTcRows, gr = row0 + r;
        const bool first = it == 0;
        // output gradient dY, loss, db4, H3
        {
            float d[kOut] = {0.f, 0.f, 0.f, 0.f};
            if (gr < n) {
                const int src = idx ? idx[gr] : gr;
#pragma unroll
                for (int c = 0; c < kOut; c++) {
                    const float e = Y[(size_t)gr * kOut + c] - T[(size_t)src * kOut + c];
                    lsum += e * e;
                    d[c] = scale * e;
                }
            }
            uint4 o0, o1;
            o0.x = pack_bf16(d[0], d[1]);
            o0.y = pack_bf16(d[2], d[3]);
            o0.z = o0.w = 0u;
            o1.x = o1.y = o1.z = o1.w = 0u;
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(S.dy) + core_off(r, 0, kOutPad)) = o0;
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(S.dy) + core_off(r, 8, kOutPad)) = o1;
#pragma unroll
            for (int c = 0; c < kOut; c++) {
                put_bf16(S.dyt, core_off(c, r, kTcRows), d[c]);
                float s = d[c];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) S.db4[warp][c] += s;
            }
            ht_rows(2, gr);
        }
        ok = run([&] {
            issue(tmem + kColDH, a_dy, b_w4t, kOutPad, instr_desc(kTcRows, kHid), false);
            issue(tmem + kColW4, a_ht, b_dyt, kTcRows, instr_desc(kHid, kOutPad), !first);
        });
        if (!ok) break;
        dz_rows(2, gr, true);
        ht_rows(1, gr);
        ok = run([&] {
            issue(tmem + kColDH, a_dz, b_w3t, kHid, instr_desc(kTcRows, kHid), false);
            issue(tmem + kColW3, a_dzt, a_ht, kTcRows, instr_desc(kHid, kHid), !first);
            issue(tmem + kColB3, a_dzt, b_ones, kTcRows, instr_desc(kHid, kOutPad), !first);
        });
        if (!ok) break;
        dz_rows(1, gr, true);
        ht_rows(0, gr);
        ok = run([&] {
            issue(tmem + kColDH, a_dz, b_w2t, kHid, instr_desc(kTcRows, kHid), false);
            issue(tmem + kColW2, a_dzt, a_ht, kTcRows, instr_desc(kHid, kHid), !first);
            issue(tmem + kColB2, a_dzt, b_ones, kTcRows, instr_desc(kHid, kOutPad), !first);
        });
        if (!ok) break;
        dz_rows(0, gr, false);
        {
            const int src = gr < n ? (idx ? idx[gr] : gr) : 0;
            const float4 *xr = reinterpret_cast<const float4 *>(X + (size_t)src * kIn);
            float x[kIn];
#pragma unroll
            for (int q = 0; q < kIn / 4; q++) {
                const float4 v = __ldg(xr + q);
                x[4 * q] = v.x;
                x[4 * q + 1] = v.y;
                x[4 * q + 2] = v.z;
                x[4 * q + 3] = v.w;
            }
#pragma unroll
            for (int c = 0; c < kIn; c++) {
                const float v = gr < n ? (x[c] - S.nrm[c]) * S.nrm[kIn + c] : 0.f;
                put_bf16(S.xt, core_off(c, r, kTcRows), v);
            }
        }
        ok = run([&] {
            issue(tmem + kColW1, a_dzt, b_xt, kTcRows, instr_desc(kHid, kIn), !first);
            issue(tmem + kColB1, a_dzt, b_ones, kTcRows, instr_desc(kHid, kOutPad), !first);
        });
    }
    if (!ok) {
        if (tid == 0) {
            atomicOr(err, kErrTimeout);
            mbar_wait(mbar, phase ^ 1u);   // bounded wait for MMAs still in flight
        }
    } else {
        // partial gradients of this CTA in the parameter layout: lane = output
        // unit (dW1, dW2, dW3, db1..db3) or input unit (dW4^T)
        float *Gc = G + (size_t)blockIdx.x * kParams;
        const int o = tid;
        for (int c0 = 0; c0 < kHid; c0 += 32) {
            float v[32];
            tmem_row32(lane_base, kColW2 + (uint32_t)c0, v);
            for (int j = 0; j < 32; j += 4)
                *reinterpret_cast<float4 *>(Gc + kOffW2 + o * kHid + c0 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            tmem_row32(lane_base, kColW3 + (uint32_t)c0, v);
            for (int j = 0; j < 32; j += 4)
                *reinterpret_cast<float4 *>(Gc + kOffW3 + o * kHid + c0 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
        }
        {
            float v[32];
            tmem_row32(lane_base, kColW1, v);
            for (int j = 0; j < 32; j += 4)
                *reinterpret_cast<float4 *>(Gc + kOffW1 + o * kIn + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            uint32_t u[16];
            tmem_ld_x16(lane_base + kColW4, u);
            tmem_wait_ld();
            for (int c = 0; c < kOut; c++) Gc[kOffW4 + c * kHid + o] = __uint_as_float(u[c]);
            const uint32_t cols[3] = {kColB1, kColB2, kColB3};
            for (int l = 0; l < 3; l++) {
                tmem_ld_x16(lane_base + cols[l], u);
                tmem_wait_ld();
                Gc[kOffB + l * kHid + o] = __uint_as_float(u[0]);
            }
        }
        __syncthreads();
        if (tid < kOut) {
            float b = 0.f;
            for (int w = 0; w < kTcThreads / 32; w++) b += S.db4[w][tid];
            Gc[kOffB + 3 * kHid + tid] = b;
        }
        for (int s = 16; s > 0; s >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, s);
        if (lane == 0) S.red[warp] = lsum;
        __syncthreads();
        if (tid == 0) {
            float l = 0.f;
            for (int w = 0; w < kTcThreads / 32; w++) l += S.red[w];
            loss_part[blockIdx.x] = l;
        }
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBwdCols) : "memory");
}

size_t backward_tc_smem() { return sizeof(TcBwdSmem) + 128; }

cudaError_t prepare_backward_tc() {
    return cudaFuncSetAttribute(k_mlp_backward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)backward_tc_smem());
}

int backward_parts(int n) {
    const int tiles = (n + kTcRows - 1) / kTcRows;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return tiles < sms ? tiles : sms;
}

cudaError_t launch_backward_tc(const Weights &W, const float *X, const int *idx, const float *norm, const float *T,
                               int n, const float *Y, const float *Z, float *G, float *loss_part, int *err,
                               cudaStream_t s) {
    const int grid = backward_parts(n);
    if (grid == 0) return cudaSuccess;
    k_mlp_backward_tc<<<grid, kTcThreads, backward_tc_smem(), s>>>(W, X, idx, norm, T, n, Y, Z, G, loss_part, err);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace mtg
