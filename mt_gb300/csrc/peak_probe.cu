// peak_probe.cu - measured FP32 FMA throughput of the current GPU, the
// denominator of the roofline of the FP32-pipe-bound TEA kernels.
#include <cuda_runtime.h>

#include "../../include/mtg.h"

namespace {

// 8 independent FMA chains per thread, 2 FLOP each per iteration.
__global__ void __launch_bounds__(256) k_fma_chain(float *out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 12345.678f) out[0] = s;  // keeps the chains live
}

// The same with packed FP32x2 FMAs (2 FLOP x 2 lanes per instruction).
__global__ void __launch_bounds__(256) k_fma2_chain(float *out, int iters, float a, float b) {
    float2 x0 = make_float2(threadIdx.x * 1e-3f, 1), x1 = make_float2(2, 3), x2 = make_float2(4, 5),
           x3 = make_float2(6, 7);
    const float2 va = make_float2(a, a), vb = make_float2(b, b);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            x0 = __ffma2_rn(x0, va, vb); x1 = __ffma2_rn(x1, va, vb);
            x2 = __ffma2_rn(x2, va, vb); x3 = __ffma2_rn(x3, va, vb);
        }
    }
    const float s = ((x0.x + x0.y) + (x1.x + x1.y)) + ((x2.x + x2.y) + (x3.x + x3.y));
    if (s == 12345.678f) out[0] = s;
}

}  // namespace

extern "C" int mtg_measure_fp32_tflops(int device, double *tflops) {
    if (!tflops) return MTG_E_CONFIG;
    if (cudaSetDevice(device) != cudaSuccess) return MTG_E_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return MTG_E_CUDA;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_fma_chain<<<blocks, threads>>>(out, 64, 0.999f, 1e-3f);  // warm-up
    k_fma2_chain<<<blocks, threads>>>(out, 64, 0.999f, 1e-3f);
    double best = 0.0;
    for (int rep = 0; rep < 10; rep++) {
        cudaEventRecord(a);
        if (rep & 1)
            k_fma2_chain<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
        else
            k_fma_chain<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double flop = 2.0 * 8 * 16 * (double)iters * blocks * threads;  // same FLOP count in both chains
        if (ms > 0) best = flop / (ms * 1e-3) / 1e12 > best ? flop / (ms * 1e-3) / 1e12 : best;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return MTG_E_CUDA;
    *tflops = best;
    return MTG_OK;
}

// Architecture of the device code the library loads on `device`
// (cudaFuncGetAttributes of one of its kernels: binaryVersion = major * 10 +
// minor of the SASS that runs, ptxVersion of its PTX; 103 for sm_103a).
extern "C" int mtg_device_code_version(int device, int *binary_version, int *ptx_version) {
    if (!binary_version) return MTG_E_CONFIG;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (cudaSetDevice(device) != cudaSuccess) return MTG_E_CUDA;
    cudaFuncAttributes fa{};
    const cudaError_t err = cudaFuncGetAttributes(&fa, k_fma_chain);
    if (prev >= 0) cudaSetDevice(prev);
    if (err != cudaSuccess) return MTG_E_CUDA;
    *binary_version = fa.binaryVersion;
    if (ptx_version) *ptx_version = fa.ptxVersion;
    return MTG_OK;
}
