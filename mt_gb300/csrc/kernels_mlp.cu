// kernels_mlp.cu - parameter updates of the TEA surrogate network (a
// 32-128-128-128-4 perceptron with SiLU activations, BF16 weights and
// activations, FP32 accumulation on the tensor cores; the forward and
// backward passes are in kernels_mlp_tc.cu and kernels_mlp_train_tc.cu):
// Adam on FP32 master weights, the BF16 copies, the loss sum.
//
//   k_mlp_adam      : reduces the per-CTA partial gradients, Adam step on
//                     the FP32 masters, refreshes both BF16 copies (forward
//                     [out][in] and transposed [in][out])
#include <cuda_bf16.h>
#include <stdint.h>

#include "mtg_mlp.cuh"

namespace mtg {
namespace mlp {

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
