// kernels_mlp_tc.cu - inference of the TEA surrogate network on the
// fifth-generation tensor cores: tcgen05.mma with both operands in shared
// memory and the FP32 accumulator in tensor memory (TMEM).
//
// One persistent CTA per SM keeps the BF16 weights in shared memory and runs
// two groups of 4 warps, each on its own 128-row tiles of the batch with its
// own input/activation buffers, mbarrier and 128 TMEM columns, so that one
// group's MMAs run while the other reads back, activates and rounds.  Per
// layer one thread of the group issues the K/16 MMAs (M = 128, N = 128, or 16
// for the output layer) and commits them to the group's mbarrier; the
// group's warps read their 32 TMEM lanes (one row per thread) back with
// tcgen05.ld, add the bias, apply SiLU, round to BF16 and write the next
// layer's A operand.  Groups synchronise on named barriers 1 and 2.
// Shared-memory operands use the canonical no-swizzle K-major layout: 8x8
// core matrices of 128 contiguous bytes, K-adjacent cores 128 B apart (LBO),
// row-group-adjacent cores K/8 * 128 B apart (SBO).
//
// Every mbarrier wait is bounded; a wait that runs out sets kErrTimeout in
// the caller's error word, the CTA leaves the tile loop, frees its TMEM and
// returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "mtg_tc.cuh"

namespace mtg {
namespace mlp {

namespace {

using namespace tc;

constexpr int kGroups = 2;                       // tiles in flight per CTA
constexpr int kFwdThreads = kGroups * kTcThreads;
constexpr int kFwdCols = kGroups * kTmemCols;     // TMEM columns of the CTA

struct __align__(128) TcSmem {
    __nv_bfloat16 w1[kHid * kIn];
    __nv_bfloat16 w2[kHid * kHid];
    __nv_bfloat16 w3[kHid * kHid];
    __nv_bfloat16 w4[kOutPad * kHid];
    __nv_bfloat16 x[kGroups][kTcRows * kIn];
    __nv_bfloat16 h[kGroups][kTcRows * kHid];
    float bias[3 * kHid + kOutPad];
    float nrm[2 * kIn];
    uint64_t mbar[kGroups];
    uint32_t tmem_base;
};

// barrier of the 128 threads of group g (named barrier 1 + g)
__device__ __forceinline__ void group_sync(int g) { asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory"); }
// group barrier that also ANDs v over the group's threads
__device__ __forceinline__ bool group_and(int g, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + g)
        : "memory");
    return r != 0;
}

}  // namespace

// Y[n][kOut] = network(normalise(X)) for n rows; err gets kErrTimeout if a
// wait for the tensor cores runs out.  TRAIN: row i of the batch is sample
// idx[i] of X (idx may be NULL), and the pre-activations z1..z3 are stored
// to Z [n][3][kHid] for the backward pass.
template <bool TRAIN>
__global__ void __launch_bounds__(kFwdThreads, 1) k_mlp_fwd_tc(const Weights W, const float *X, const int *idx, int n,
                                                               const float *norm, float *Y, float *Z, int *err,
                                                               uint32_t spin) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TcSmem &S = *reinterpret_cast<TcSmem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int g = warp / 4, gtid = tid % kTcThreads;   // group, thread in the group (= tile row)
    stage_weights(S.w1, W.w1, kHid, kIn, kHid);
    stage_weights(S.w2, W.w2, kHid, kHid, kHid);
    stage_weights(S.w3, W.w3, kHid, kHid, kHid);
    stage_weights(S.w4, W.w4, kOutPad, kHid, kOut);
    for (int i = tid; i < 3 * kHid + kOutPad; i += blockDim.x) S.bias[i] = i < 3 * kHid + kOut ? W.b[i] : 0.f;
    for (int i = tid; i < 2 * kIn; i += blockDim.x) S.nrm[i] = norm ? norm[i] : (i < kIn ? 0.f : 1.f);
    if (tid == 0) {
        for (int k = 0; k < kGroups; k++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&S.mbar[k])), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(kFwdCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t mbar = smem_u32(&S.mbar[g]);
    const uint32_t tmem = S.tmem_base + (uint32_t)(g * kTmemCols);          // this group's columns
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);   // this warp's TMEM lanes
    const uint32_t ax = smem_u32(S.x[g]), ah = smem_u32(S.h[g]);
    const uint32_t bw[4] = {smem_u32(S.w1), smem_u32(S.w2), smem_u32(S.w3), smem_u32(S.w4)};
    __nv_bfloat16 *const xs = S.x[g], *const hs = S.h[g];
    uint32_t phase = 0;
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    // group 0 of every CTA takes the first gridDim.x tiles, so a batch of at
    // most one tile per SM still spreads over the SMs
    const int first = blockIdx.x + g * gridDim.x, stride = gridDim.x * kGroups;
    // inputs: 128 rows x 32 features = 8 float4 per thread, coalesced; the
    // next tile's are loaded while the current one runs
    constexpr int kXv = kTcRows * (kIn / 4) / kTcThreads;
    float4 xv[kXv];
    auto load_x = [&](int tile) {
#pragma unroll
        for (int u = 0; u < kXv; u++) {
            const int i = gtid + u * kTcThreads, r = i / (kIn / 4), c = (i % (kIn / 4)) * 4;
            const int gr = tile * kTcRows + r;
            const int src = (TRAIN && idx && tile < ntiles && gr < n) ? idx[gr] : gr;
            xv[u] = (tile < ntiles && gr < n) ? *reinterpret_cast<const float4 *>(X + (size_t)src * kIn + c)
                                              : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    load_x(first);
    for (int tile = first; tile < ntiles; tile += stride) {
        const int row0 = tile * kTcRows;
#pragma unroll
        for (int u = 0; u < kXv; u++) {
            const int i = gtid + u * kTcThreads, r = i / (kIn / 4), c = (i % (kIn / 4)) * 4;
            float4 v = xv[u];
            if (row0 + r < n) {
                v.x = (v.x - S.nrm[c]) * S.nrm[kIn + c];
                v.y = (v.y - S.nrm[c + 1]) * S.nrm[kIn + c + 1];
                v.z = (v.z - S.nrm[c + 2]) * S.nrm[kIn + c + 2];
                v.w = (v.w - S.nrm[c + 3]) * S.nrm[kIn + c + 3];
            }
            *reinterpret_cast<uint2 *>(reinterpret_cast<char *>(xs) + core_off(r, c, kIn)) =
                make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
        }
        load_x(tile + stride);
        bool ok = true;
        for (int layer = 0; layer < 4 && ok; layer++) {
            fence_async_smem();
            fence_before_sync();
            group_sync(g);
            if (gtid == 0) {
                fence_after_sync();
                if (layer == 0)
                    issue_layer(tmem, ax, bw[0], kIn, instr_desc(kTcRows, kHid));
                else
                    issue_layer(tmem, ah, bw[layer], kHid, instr_desc(kTcRows, layer == 3 ? kOutPad : kHid));
                mma_commit(mbar);
            }
            ok = group_and(g, mbar_wait(mbar, phase, spin));   // the tile loop's wait: `spin` polls
            phase ^= 1u;
            if (!ok) break;
            fence_after_sync();
            const int r = gtid;   // this thread's row = its TMEM lane
            if (layer < 3) {
                const float *bias = S.bias + layer * kHid;
#pragma unroll 1
                for (int c0 = 0; c0 < kHid; c0 += 32) {
                    uint32_t v[32];
                    tmem_ld_x32(lane_base + (uint32_t)c0, v);
                    tmem_wait_ld();
                    if (TRAIN && row0 + r < n) {   // pre-activations for the backward pass
                        float4 *zr = reinterpret_cast<float4 *>(Z + ((size_t)(row0 + r) * 3 + layer) * kHid + c0);
#pragma unroll
                        for (int q = 0; q < 8; q++)
                            zr[q] = make_float4(__uint_as_float(v[4 * q]) + bias[c0 + 4 * q],
                                                __uint_as_float(v[4 * q + 1]) + bias[c0 + 4 * q + 1],
                                                __uint_as_float(v[4 * q + 2]) + bias[c0 + 4 * q + 2],
                                                __uint_as_float(v[4 * q + 3]) + bias[c0 + 4 * q + 3]);
                    }
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
                        *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(hs) + core_off(r, k, kHid)) = o;
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
            if (gtid == 0) {
                atomicOr(err, kErrTimeout);
                // the MMAs already issued may still run: give them a bounded
                // time (the full default limit, whatever `spin` is) to finish
                // before the TMEM goes back
                mbar_wait(mbar, phase ^ 1u, kSpinLimit);
            }
            break;
        }
        fence_before_sync();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.tmem_base), "r"(kFwdCols)
                     : "memory");
}

size_t infer_tc_smem() { return sizeof(TcSmem) + 128; }

uint32_t tc_default_spin() { return kSpinLimit; }

cudaError_t prepare_tc() {
    cudaError_t e =
        cudaFuncSetAttribute(k_mlp_fwd_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_tc_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_fwd_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)infer_tc_smem());
    if (e == cudaSuccess) e = prepare_backward_tc();
    return e;
}

int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

cudaError_t launch_infer_tc(const Weights &W, const float *X, int n, const float *norm, float *Y, int *err,
                            cudaStream_t s, uint32_t spin) {
    const int tiles = (n + kTcRows - 1) / kTcRows;
    if (tiles == 0) return cudaSuccess;
    const int sms = sm_count(), grid = tiles < sms ? tiles : sms;
    k_mlp_fwd_tc<false><<<grid, kFwdThreads, infer_tc_smem(), s>>>(W, X, nullptr, n, norm, Y, nullptr, err, spin);
    return cudaGetLastError();
}

cudaError_t launch_forward_tc(const Weights &W, const float *X, const int *idx, int n, const float *norm, float *Y,
                              float *Z, int *err, cudaStream_t s) {
    const int tiles = (n + kTcRows - 1) / kTcRows;
    if (tiles == 0) return cudaSuccess;
    const int sms = sm_count(), grid = tiles < sms ? tiles : sms;
    k_mlp_fwd_tc<true><<<grid, kFwdThreads, infer_tc_smem(), s>>>(W, X, idx, n, norm, Y, Z, err, kSpinLimit);
    return cudaGetLastError();
}

}  // namespace mlp
}  // namespace mtg
