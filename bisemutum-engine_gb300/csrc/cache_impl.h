// cache_impl.h — the radiance-cache object behind bsm_cache (cache.cpp), shared
// with the render loop (api.cpp).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bsm_pt.h"
#include "pt_device.h"

struct bsm_cache {
    bsm_context* ctx = nullptr;
    int device = 0;
    float* w_master = nullptr;   // fp32 master weights (kMlpParams)
    void* w_bf16 = nullptr;      // bf16 copy read by the kernels
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    float* dW = nullptr;
    float* loss = nullptr;       // device scalar
    float4* samples = nullptr;   // training samples (4 float4 each)
    uint32_t* sample_count = nullptr;
    uint32_t sample_cap = 0;
    bsm::DevView* view_dev = nullptr;
    float* io = nullptr;         // device staging for host-buffer entry points
    size_t io_bytes = 0;
    int step = 0;
    uint32_t frame = 0;
};

namespace bsm {
// Runs train paths + Adam steps for one camera (cache.cpp).
bsm_status cache_train_frame(bsm_cache* c, const DevScene& sc, const DevView& view, const bsm_cache_settings& cs,
                             cudaStream_t st, float* loss_out, uint32_t* samples_out);
}
