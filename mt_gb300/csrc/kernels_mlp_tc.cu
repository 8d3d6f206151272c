// kernels_mlp_tc.cu - inference of the TEA surrogate network on the
// fifth-generation tensor cores: tcgen05.mma with both operands in shared
// memory and the FP32 accumulator in tensor memory (TMEM).
//
// One persistent CTA per SM (4 warps, 128 threads) keeps the BF16 weights in
// shared memory and walks 128-row tiles of the batch.  Per layer one thread
// issues the K/16 MMAs (M = 128, N = 128, or 16 for the output layer) into
// 128 TMEM columns and commits them to an mbarrier; the four warps read
// their 32 TMEM lanes (one row per thread) back with tcgen05.ld, add the
// bias, apply SiLU, round to BF16 and write the next layer's A operand.
// Shared-memory operands use the canonical no-swizzle K-major layout: 8x8
// core matrices of 128 contiguous bytes, K-adjacent cores 128 B apart (LBO),
// row-group-adjacent cores K/8 * 128 B apart (SBO).
//
// Every mbarrier wait is bounded; a wait that runs out sets kErrTimeout in
// the caller's error word, the CTA leaves the tile loop, frees its TMEM and
// returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "mtg_internal.cuh"
#include "mtg_mlp.cuh"

namespace mtg {
namespace mlp {

namespace {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 128;
constexpr int kOutPad = 16;          // N of the output layer (4 used)
constexpr int kTmemCols = 128;
constexpr uint32_t kSpinLimit = 1u << 20;

struct __align__(128) TcSmem {
    __nv_bfloat16 w1[kHid * kIn];
    __nv_bfloat16 w2[kHid * kHid];
    __nv_bfloat16 w3[kHid * kHid];
    __nv_bfloat16 w4[kOutPad * kHid];
    __nv_bfloat16 x[kTcRows * kIn];
    __nv_bfloat16 h[kTcRows * kHid];
    float bias[3 * kHid + kOutPad];
    float nrm[2 * kIn];
    uint64_t mbar;
    uint32_t tmem_base;
};

// byte offset of element (r, k) of an R x K K-major tile in the core-matrix layout
__device__ __forceinline__ uint32_t core_off(int r, int k, int K) {
    return (uint32_t)((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start, LBO, SBO (all >> 4), version 1 (bits
// 46-47), no swizzle (bits 61-63 = 0), base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait for the given phase of the mbarrier; true when it completed.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
    for (uint32_t i = 0; i < kSpinLimit; i++)
        if (mbar_try_wait(mbar, phase)) return true;
    return false;
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld_x32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_ld_x16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// SiLU through the hardware tanh: z sigmoid(z) = z/2 (1 + tanh(z/2)).
__device__ __forceinline__ float silu_tanh(float z) {
    const float hz = 0.5f * z;
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(hz));
    return fmaf(hz, t, hz);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// global [N][K] BF16 (K-major) -> core-matrix layout, rows >= rows_valid zero
__device__ void stage_weights(__nv_bfloat16 *dst, const __nv_bfloat16 *src, int N, int K, int rows_valid) {
    const int chunks = N * (K / 8);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int n = c / (K / 8), k = (c % (K / 8)) * 8;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (n < rows_valid) v = *reinterpret_cast<const uint4 *>(src + (size_t)n * K + k);
        *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(dst) + core_off(n, k, K)) = v;
    }
}

// Issues the K/16 MMAs of one layer: D[128 x N] (TMEM) = A[128 x K] B[N x K]^T.
__device__ __forceinline__ void issue_layer(uint32_t tmem, uint32_t a, uint32_t b, int K, uint32_t idesc) {
    const uint32_t sbo = (uint32_t)(K / 8) * 128u;
    for (int ks = 0; ks < K / 16; ks++)
        mma_bf16(tmem, smem_desc(a + ks * 256u, 128u, sbo), smem_desc(b + ks * 256u, 128u, sbo), idesc,
                 ks > 0 ? 1u : 0u);
}

}  // namespace

// Y[n][kOut] = network(normalise(X)) for n rows; err gets kErrTimeout if a
// wait for the tensor cores runs out.
__global__ void __launch_bounds__(kTcThreads, 1) k_mlp_infer_tc(const Weights W, const float *X, int n,
                                                                const float *norm, float *Y, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    stage_weights(S.w1, W.w1, kHid, kIn, kHid);
    stage_weights(S.w2, W.w2, kHid, kHid, kHid);
    stage_weights(S.w3, W.w3, kHid, kHid, kHid);
    stage_weights(S.w4, W.w4, kOutPad, kHid, kOut);
    for (int i = tid; i < 3 * kHid + kOutPad; i += blockDim.x) S.bias[i] = i < 3 * kHid + kOut ? W.b[i] : 0.f;
    for (int i = tid; i < 2 * kIn; i += blockDim.x) S.nrm[i] = norm ? norm[i] : (i < kIn ? 0.f : 1.f);
    const uint32_t mbar = smem_u32(&S.mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);   // this warp's TMEM lanes
    const uint32_t ax = smem_u32(S.x), ah = smem_u32(S.h);
    const uint32_t bw[4] = {smem_u32(S.w1), smem_u32(S.w2), smem_u32(S.w3), smem_u32(S.w4)};
    uint32_t phase = 0;
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    // inputs: 128 rows x 32 features = 8 float4 per thread, coalesced; the
    // next tile's are loaded while the current one runs
    constexpr int kXv = kTcRows * (kIn / 4) / kTcThreads;
    float4 xv[kXv];
    auto load_x = [&](int tile) {
#pragma unroll
        for (int u = 0; u < kXv; u++) {
            const int i = tid + u * kTcThreads, r = i / (kIn / 4), c = (i % (kIn / 4)) * 4;
            const int gr = tile * kTcRows + r;
            xv[u] = (tile < ntiles && gr < n) ? *reinterpret_cast<const float4 *>(X + (size_t)gr * kIn + c)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    load_x(blockIdx.x);
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int row0 = tile * kTcRows;
#pragma unroll
        for (int u = 0; u < kXv; u++) {
            const int i = tid + u * kTcThreads, r = i / (kIn / 4), c = (i % (kIn / 4)) * 4;
            float4 v = xv[u];
            if (row0 + r < n) {
                v.x = (v.x - S.nrm[c]) * S.nrm[kIn + c];
                v.y = (v.y - S.nrm[c + 1]) * S.nrm[kIn + c + 1];
                v.z = (v.z - S.nrm[c + 2]) * S.nrm[kIn + c + 2];
                v.w = (v.w - S.nrm[c + 3]) * S.nrm[kIn + c + 3];
            }
            *reinterpret_cast<uint2 *>(reinterpret_cast<char *>(S.x) + core_off(r, c, kIn)) =
                make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
        }
        load_x(tile + gridDim.x);
        bool ok = true;
        for (int layer = 0; layer < 4 && ok; layer++) {
            fence_async_smem();
            fence_before_sync();
            __syncthreads();
            if (tid == 0) {
                fence_after_sync();
                if (layer == 0)
                    issue_layer(tmem, ax, bw[0], kIn, instr_desc(kTcRows, kHid));
                else
                    issue_layer(tmem, ah, bw[layer], kHid, instr_desc(kTcRows, layer == 3 ? kOutPad : kHid));
                mma_commit(mbar);
            }
            ok = __syncthreads_and(mbar_wait(mbar, phase)) != 0;
            phase ^= 1u;
            if (!ok) break;
            fence_after_sync();
            const int r = tid;   // this thread's row = its TMEM lane
            if (layer < 3) {
                const float *bias = S.bias + layer * kHid;
#pragma unroll 1
                for (int c0 = 0; c0 < kHid; c0 += 32) {
                    uint32_t v[32];
                    tmem_ld_x32(lane_base + (uint32_t)c0, v);
                    tmem_wait_ld();
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        uint4 o;
                        const int k = c0 + q * 8;
                        o.x = pack_bf16(silu_tanh(__uint_as_float(v[q * 8 + 0]) + bias[k + 0]),
                                        silu_tanh(__uint_as_float(v[q * 8 + 1]) + bias[k + 1]));
                        o.y = pack_bf16(silu_tanh(__uint_as_float(v[q * 8 + 2]) + bias[k + 2]),
                                        silu_tanh(__uint_as_float(v[q * 8 + 3]) + bias[k + 3]));
                        o.z = pack_bf16(silu_tanh(__uint_as_float(v[q * 8 + 4]) + bias[k + 4]),
                                        silu_tanh(__uint_as_float(v[q * 8 + 5]) + bias[k + 5]));
                        o.w = pack_bf16(silu_tanh(__uint_as_float(v[q * 8 + 6]) + bias[k + 6]),
                                        silu_tanh(__uint_as_float(v[q * 8 + 7]) + bias[k + 7]));
                        *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(S.h) + core_off(r, k, kHid)) = o;
                    }
                }
            } else {
                uint32_t v[16];
                tmem_ld_x16(lane_base, v);
                tmem_wait_ld();
                if (row0 + r < n) {
                    const float *bias = S.bias + 3 * kHid;
                    *reinterpret_cast<float4 *>(Y + (size_t)(row0 + r) * kOut) =
                        make_float4(__uint_as_float(v[0]) + bias[0], __uint_as_float(v[1]) + bias[1],
                                    __uint_as_float(v[2]) + bias[2], __uint_as_float(v[3]) + bias[3]);
                }
            }
        }
        if (!ok) {
            if (tid == 0) {
                atomicOr(err, kErrTimeout);
                // the MMAs already issued may still run: give them a bounded
                // time to finish before the TMEM goes back
                mbar_wait(mbar, phase ^ 1u);
            }
            break;
        }
        fence_before_sync();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

size_t infer_tc_smem() { return sizeof(TcSmem) + 128; }

cudaError_t prepare_tc() {
    return cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_tc_smem());
}

cudaError_t launch_infer_tc(const Weights &W, const float *X, int n, const float *norm, float *Y, int *err,
                            cudaStream_t s) {
    const int tiles = (n + kTcRows - 1) / kTcRows;
    if (tiles == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = tiles < sms ? tiles : sms;
    k_mlp_infer_tc<<<grid, kTcThreads, infer_tc_smem(), s>>>(W, X, n, norm, Y, err);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace mtg
