// mtg_tc.cuh - building blocks of the fifth-generation tensor-core kernels
// of the surrogate network (kernels_mlp_tc.cu, kernels_mlp_train_tc.cu):
// shared-memory matrix and instruction descriptors of tcgen05.mma kind::f16,
// the MMA, commit and bounded mbarrier wait, TMEM loads, fences, SiLU.
//
// Shared-memory operands use the canonical no-swizzle K-major layout: 8x8
// core matrices of 128 contiguous bytes, K-adjacent cores 128 B apart (LBO),
// row-group-adjacent cores K/8 * 128 B apart (SBO).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "mtg_internal.cuh"
#include "mtg_mlp.cuh"

namespace mtg {
namespace mlp {
namespace tc {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 128;
constexpr int kOutPad = 16;          // N of the output layer (4 used)
constexpr int kTmemCols = 128;
constexpr uint32_t kSpinLimit = 1u << 20;


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

// Bounded wait for the given phase of the mbarrier (at most `limit` polls);
// true when it completed.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, uint32_t limit = kSpinLimit) {
    for (uint32_t i = 0; i < limit; i++)
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
__device__ __forceinline__ void stage_weights(__nv_bfloat16 *dst, const __nv_bfloat16 *src, int N, int K, int rows_valid) {
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


}  // namespace tc
}  // namespace mlp
}  // namespace mtg
