// mlp.cu — the radiance cache's optimiser step.
//
//   k_mlp_adam    Adam on the FP32 master weights, BF16 copies for the next pass
//   k_mlp_sum_parts  the training kernel's per-CTA gradient slots summed in slot order
//
// The network's products (inference, and the training step's forward pass,
// backward pass and weight gradients) run on the tcgen05 tensor cores in
// mlp_tc.cu.
#include <cuda_bf16.h>
#include <cmath>
#include <cuda_runtime.h>

#include "mlp.cuh"
#include "pt_device.h"

namespace bsm {

// The gradient of parameter i from its per-CTA slots, summed in a fixed order (so the sum, and every step
// trained on it, is the same from run to run): kGradLanes consecutive lanes take parameter i, lane j adds the
// slots j, j + kGradLanes, ... in order, and the lanes' sums are combined pairwise in lane order.  Every lane
// of the group returns the total.
constexpr int kGradLanes = 4;
__device__ __forceinline__ float grad_sum(const float* __restrict__ parts, uint32_t n_parts, int i, uint32_t j) {
    float g = 0.0f;
    if (i < kMlpParams)
        for (uint32_t c = j; c < n_parts; c += kGradLanes) g += parts[(size_t)c * kMlpParams + i];
#pragma unroll
    for (int o = 1; o < kGradLanes; o <<= 1) g += __shfl_xor_sync(0xffffffffu, g, o);   // pairs, then pairs of pairs
    return g;
}

__global__ void k_mlp_sum_parts(const float* __restrict__ parts, uint32_t n_parts, float* __restrict__ dW) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(t / kGradLanes);
    const float g = grad_sum(parts, n_parts, i, t % kGradLanes);
    if (i < kMlpParams && t % kGradLanes == 0) dW[i] = g;
}

// Adam (Kingma and Ba 2015) on the fp32 master weights; writes the bf16 copy
// in the kernels' tile layout (mlp_tile_index).
// With ema_decay > 0 it also keeps an exponential moving average of the
// weights (zero-started, so ema_corr = 1 / (1 - decay^steps) corrects its bias)
// and writes the corrected average's bf16 copy, which renders read.
__global__ void k_mlp_adam(float* __restrict__ wm, __nv_bfloat16* __restrict__ wb, const float* __restrict__ parts,
                           uint32_t n_parts, float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                           float eps, float bc1, float bc2, float* __restrict__ ema, __nv_bfloat16* __restrict__ emab,
                           float ema_decay, float ema_corr) {
    const uint32_t lane_id = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(lane_id / kGradLanes);
    const float gr = grad_sum(parts, n_parts, i, lane_id % kGradLanes);
    if (i >= kMlpParams || lane_id % kGradLanes != 0) return;
    float mi = b1 * m[i] + (1.0f - b1) * gr;
    float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    float mh = mi / bc1, vh = vi / bc2;
    float wi = wm[i] - lr * mh / (sqrtf(vh) + eps);
    // padded output rows stay zero
    if (i >= kMlpHidden * kMlpLayerParams + kMlpOut * kMlpHid) wi = 0.0f;
    wm[i] = wi;
    const int t = mlp_tile_index(i);
    wb[t] = __float2bfloat16_rn(wi);
    if (ema_decay > 0.0f) {
        float e = ema_decay * ema[i] + (1.0f - ema_decay) * wi;
        ema[i] = e;
        emab[t] = __float2bfloat16_rn(e * ema_corr);
    }
}

// ------------------------------------------------------------- launcher ----
cudaError_t launch_mlp_adam(cudaStream_t st, float* wm, void* wb, const float* dW_parts, uint32_t n_parts, float* m,
                            float* v, float lr, int step, float* ema, void* ema_b, float ema_decay, int ema_step) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
    float corr = ema_decay > 0.0f ? (float)(1.0 / (1.0 - std::pow((double)ema_decay, (double)ema_step))) : 1.0f;
    k_mlp_adam<<<(kMlpParams * kGradLanes + 255) / 256, 256, 0, st>>>(wm, (__nv_bfloat16*)wb, dW_parts, n_parts, m, v,
                                                                      lr, b1, b2, eps, bc1, bc2, ema,
                                                                      (__nv_bfloat16*)ema_b, ema_decay, corr);
    return cudaGetLastError();
}

cudaError_t launch_mlp_sum_parts(cudaStream_t st, const float* dW_parts, uint32_t n_parts, float* dW) {
    k_mlp_sum_parts<<<(kMlpParams * kGradLanes + 255) / 256, 256, 0, st>>>(dW_parts, n_parts, dW);
    return cudaGetLastError();
}

}  // namespace bsm
