// mlp.cu — the radiance cache's optimiser step.
//
//   k_mlp_adam    Adam on the FP32 master weights, BF16 copies for the next pass
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

// Adam (Kingma and Ba 2015) on the fp32 master weights; writes the bf16 copy
// in the kernels' tile layout (mlp_tile_index).
// With ema_decay > 0 it also keeps an exponential moving average of the
// weights (zero-started, so ema_corr = 1 / (1 - decay^steps) corrects its bias)
// and writes the corrected average's bf16 copy, which renders read.
__global__ void k_mlp_adam(float* __restrict__ wm, __nv_bfloat16* __restrict__ wb, const float* __restrict__ dW,
                           float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2, float eps,
                           float bc1, float bc2, float* __restrict__ ema, __nv_bfloat16* __restrict__ emab,
                           float ema_decay, float ema_corr) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    float gr = dW[i];
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
cudaError_t launch_mlp_adam(cudaStream_t st, float* wm, void* wb, const float* dW, float* m, float* v, float lr,
                            int step, float* ema, void* ema_b, float ema_decay, int ema_step) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
    float corr = ema_decay > 0.0f ? (float)(1.0 / (1.0 - std::pow((double)ema_decay, (double)ema_step))) : 1.0f;
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(wm, (__nv_bfloat16*)wb, dW, m, v, lr, b1, b2, eps, bc1, bc2,
                                                         ema, (__nv_bfloat16*)ema_b, ema_decay, corr);
    return cudaGetLastError();
}

}  // namespace bsm
