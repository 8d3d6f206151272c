// mtg_mlp.cuh - shapes, parameter layout and launchers of the TEA surrogate
// network: Adam and the BF16 copies (kernels_mlp.cu), the tensor-core forward
// pass (kernels_mlp_tc.cu) and backward pass (kernels_mlp_train_tc.cu).
//
// Parameter vector (FP32 masters, Adam moments and gradients share it):
//   w1 [kHid][kIn] | w2 [kHid][kHid] | w3 [kHid][kHid] | w4 [kOut][kHid] |
//   b1 [kHid] | b2 [kHid] | b3 [kHid] | b4 [kOut]
// Weights are stored output-major ([out][in]); the BF16 copies exist in that
// layout (forward) and transposed ([in][out], backward).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mtg {
namespace mlp {

constexpr int kIn = 32, kHid = 128, kOut = 4;
constexpr int kOffW1 = 0;
constexpr int kOffW2 = kOffW1 + kHid * kIn;
constexpr int kOffW3 = kOffW2 + kHid * kHid;
constexpr int kOffW4 = kOffW3 + kHid * kHid;
constexpr int kOffB = kOffW4 + kOut * kHid;
constexpr int kParams = kOffB + 3 * kHid + kOut;

struct Weights {
    float *master, *m, *v;                 // [kParams]
    const float *b;                        // = master + kOffB
    __nv_bfloat16 *w1, *w2, *w3, *w4;      // forward copies, [out][in]
    __nv_bfloat16 *w2t, *w3t, *w4t;        // transposed copies, [in][out]
};

__device__ __forceinline__ void refresh_one(const Weights &W, int i, float w) {
    const __nv_bfloat16 h = __float2bfloat16(w);
    if (i < kOffW2) {
        W.w1[i - kOffW1] = h;
    } else if (i < kOffW3) {
        const int k = i - kOffW2, o = k / kHid, in = k % kHid;
        W.w2[k] = h;
        W.w2t[in * kHid + o] = h;
    } else if (i < kOffW4) {
        const int k = i - kOffW3, o = k / kHid, in = k % kHid;
        W.w3[k] = h;
        W.w3t[in * kHid + o] = h;
    } else if (i < kOffB) {
        const int k = i - kOffW4, o = k / kHid, in = k % kHid;
        W.w4[k] = h;
        W.w4t[in * kOut + o] = h;
    }
}

cudaError_t launch_adam(const Weights &W, const float *G, int nparts, float lr, int step, cudaStream_t s);
cudaError_t launch_refresh(const Weights &W, cudaStream_t s);
cudaError_t launch_loss_sum(const float *part, int nparts, float *out, cudaStream_t s);

// Inference on the tcgen05 tensor cores (kernels_mlp_tc.cu): Y = network of
// the normalised X, n rows; a wait that runs out sets kErrTimeout in *err.
// spin: polls of each wait for a layer's MMAs (0: none, the wait gives up at
// once); tc_default_spin() is the limit every other wait uses.
cudaError_t prepare_tc();
uint32_t tc_default_spin();
cudaError_t launch_infer_tc(const Weights &W, const float *X, int n, const float *norm, float *Y, int *err,
                            cudaStream_t s, uint32_t spin = tc_default_spin());
// Training on the tcgen05 tensor cores: the forward pass with the
// pre-activations Z [n][3][kHid] (rows of X gathered through idx, may be
// NULL), and the backward pass (kernels_mlp_train_tc.cu) writing per-CTA
// partial gradients G [backward_parts(n)][kParams] and loss sums.
cudaError_t launch_forward_tc(const Weights &W, const float *X, const int *idx, int n, const float *norm, float *Y,
                              float *Z, int *err, cudaStream_t s);
cudaError_t prepare_backward_tc();
int backward_parts(int n);
cudaError_t launch_backward_tc(const Weights &W, const float *X, const int *idx, const float *norm, const float *T,
                               int n, const float *Y, const float *Z, float *G, float *loss_part, int *err,
                               cudaStream_t s);

}  // namespace mlp
}  // namespace mtg
