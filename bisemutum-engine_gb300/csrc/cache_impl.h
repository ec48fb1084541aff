// cache_impl.h — the radiance-cache object behind bsm_cache (cache.cpp), shared
// with the render loop (api.cpp).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bsm_pt.h"
#include "pt_device.h"

constexpr uint32_t kLossSlots = 64;  // per-step loss slots on the device (read back together)

struct bsm_cache {
    bsm_context* ctx = nullptr;
    int device = 0;
    float* w_master = nullptr;   // fp32 master weights (kMlpParams)
    void* w_bf16 = nullptr;      // bf16 copy read by the kernels
    float* w_ema = nullptr;      // moving average of the master weights (zero-started, bias-corrected on use)
    void* w_ema_bf16 = nullptr;  // bf16 copy of the corrected average, read by renders
    int ema_steps = 0;           // Adam steps averaged (0: renders read w_bf16)
    float ema_decay = 0.0f;      // decay of the running average
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    float* dW = nullptr;         // the summed gradient (bsm_cache_gradient)
    float* dW_parts = nullptr;   // the training kernel's per-CTA gradient slots (mlp_train_parts of them)
    float* loss = nullptr;       // device: one loss per Adam step of a training call (kLossSlots)
    uint32_t* err = nullptr;     // device error word of the training kernels (bit 1: a tensor-core wait timed out)
    float4* samples = nullptr;   // training samples (4 float4 each)
    uint32_t* sample_count = nullptr;
    uint32_t sample_cap = 0;
    // training paths: per-vertex records (vertex v = path x segments + k) and their shadow-ray queue
    float4* tv_raw = nullptr;      // 3 float4 per vertex: the cache's raw inputs
    float4* tv_thr = nullptr;      // path throughput at the vertex
    float4* tv_rad = nullptr;      // radiance gathered at the vertex (NEE through the shadow pass, sky on escape)
    uint32_t* tv_count = nullptr;  // vertices per path
    unsigned long long* tv_fx = nullptr;  // 3 words per vertex: the shadow pass's fixed-point radiance sums
    uint32_t* tv_nsamp = nullptr;  // per block of 256 paths: samples, then the block's first sample
    uint32_t* tv_offs = nullptr;   // each path's first sample within its block
    void* tv_queue = nullptr;      // shadow rays (origin, direction, contribution + vertex, seed), counters, stats
    uint32_t tv_cap = 0;           // vertices the buffers hold
    uint32_t tv_paths = 0;         // paths tv_count holds
    uint32_t tv_lights = 0;        // lights the shadow queue was sized for
    bsm::DevView* view_dev = nullptr;
    float* io = nullptr;         // device staging for host-buffer entry points
    size_t io_bytes = 0;
    int step = 0;
    uint32_t frame = 0;
};

namespace bsm {
// The bf16 weights renders read: the corrected moving average once it holds a step, else the current ones.
inline const void* cache_render_weights(const bsm_cache* c) { return c->ema_steps > 0 ? c->w_ema_bf16 : c->w_bf16; }
// Runs train paths + Adam steps for one camera (cache.cpp).
bsm_status cache_train_frame(bsm_cache* c, const DevScene& sc, const DevView& view, const bsm_cache_settings& cs,
                             const LaunchCfg& lc, cudaStream_t st, float* loss_out, uint32_t* samples_out);
}
