// cache.cpp — host side of the radiance cache: weights, Adam state, training
// on tracer-generated samples, save/load.  The kernels are in mlp.cu and
// train_paths.cu; bsm_render_cached (api.cpp) renders with the cache.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "bsm_pt.h"
#include "cache_impl.h"
#include "mlp.cuh"

using namespace bsm;

namespace {

bsm_status cache_io(bsm_cache* c, size_t bytes) {
    if (c->io_bytes >= bytes) return BSM_OK;
    if (c->io) cudaFree(c->io);
    c->io = nullptr;
    c->io_bytes = 0;
    if (cudaMalloc(&c->io, bytes) != cudaSuccess) return BSM_ERR_OUT_OF_MEMORY;
    c->io_bytes = bytes;
    return BSM_OK;
}

void upload_weights(bsm_cache* c, const float* w) {
    std::vector<__nv_bfloat16> b(kMlpParams);   // in the tensor-core kernels' tile layout
    for (int i = 0; i < kMlpParams; ++i) b[bsm::mlp_tile_index(i)] = __float2bfloat16_rn(w[i]);
    cudaMemcpy(c->w_master, w, kMlpParams * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(c->w_bf16, b.data(), kMlpParams * 2, cudaMemcpyHostToDevice);
    cudaMemset(c->adam_m, 0, kMlpParams * 4);
    cudaMemset(c->adam_v, 0, kMlpParams * 4);
    cudaMemset(c->w_ema, 0, kMlpParams * 4);
    c->step = 0;
    c->ema_steps = 0;
    c->ema_decay = 0.0f;
}

}  // namespace

extern "C" void bsm_cache_settings_default(bsm_cache_settings* cs) {
    if (!cs) return;
    cs->cache_segment = 2;
    cs->train_paths = 32768;
    cs->train_segments = 8;
    cs->train_batch = 16384;
    cs->train_steps = 4;
    cs->lr = 1e-2f;
    cs->ema_decay = 0.99f;
    cs->min_roughness = 0.0f;
    cs->extra_segments = 0;
}

extern "C" uint32_t bsm_cache_param_count(void) { return (uint32_t)kMlpParams; }

extern "C" bsm_status bsm_cache_create(bsm_context* ctx, uint64_t seed, bsm_cache** out) {
    if (!ctx || !out) return BSM_ERR_INVALID_ARG;
    *out = nullptr;
    auto* c = new bsm_cache();
    c->ctx = ctx;
    c->device = ctx_device(ctx);
    cudaSetDevice(c->device);
    bool ok = cudaMalloc((void**)&c->w_master, kMlpParams * 4) == cudaSuccess &&
              cudaMalloc(&c->w_bf16, kMlpParams * 2) == cudaSuccess &&
              cudaMalloc((void**)&c->w_ema, kMlpParams * 4) == cudaSuccess &&
              cudaMalloc(&c->w_ema_bf16, kMlpParams * 2) == cudaSuccess &&
              cudaMalloc((void**)&c->adam_m, kMlpParams * 4) == cudaSuccess &&
              cudaMalloc((void**)&c->adam_v, kMlpParams * 4) == cudaSuccess &&
              cudaMalloc((void**)&c->dW, kMlpParams * 4) == cudaSuccess &&
              mlp_train_parts(c->device) > 0 &&
              cudaMalloc((void**)&c->dW_parts, (size_t)mlp_train_parts(c->device) * kMlpParams * 4) == cudaSuccess &&
              // the output layer's padded rows of every slot are never written: they stay zero
              cudaMemset(c->dW_parts, 0, (size_t)mlp_train_parts(c->device) * kMlpParams * 4) == cudaSuccess &&
              cudaMalloc((void**)&c->loss, kLossSlots * 4) == cudaSuccess &&
              cudaMalloc((void**)&c->err, 16) == cudaSuccess && cudaMemset(c->err, 0, 16) == cudaSuccess &&
              cudaMalloc((void**)&c->sample_count, 4) == cudaSuccess &&
              cudaMalloc((void**)&c->view_dev, sizeof(DevView)) == cudaSuccess;
    if (!ok) {
        bsm_cache_destroy(c);
        return BSM_ERR_OUT_OF_MEMORY;
    }
    // He-uniform initialisation, U(-sqrt(6/fan_in), sqrt(6/fan_in)), from a SplitMix64 stream
    std::vector<float> w(kMlpParams, 0.0f);
    uint64_t st = seed * 0x9e3779b97f4a7c15ULL + 0x632be59bd9b4e019ULL;
    const float lim = std::sqrt(6.0f / 64.0f);
    for (int i = 0; i < kMlpParams; ++i) {
        st += 0x9e3779b97f4a7c15ULL;
        float u = (float)(mix64(st) >> 40) * (1.0f / 16777216.0f);
        w[i] = (2.0f * u - 1.0f) * lim;
        if (i >= kMlpHidden * kMlpLayerParams + kMlpOut * kMlpHid) w[i] = 0.0f;
        else if (i >= kMlpHidden * kMlpLayerParams) w[i] *= 0.1f;  // small initial output
    }
    upload_weights(c, w.data());
    *out = c;
    return BSM_OK;
}

extern "C" void bsm_cache_destroy(bsm_cache* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (void* p : {(void*)c->w_master, c->w_bf16, (void*)c->w_ema, c->w_ema_bf16, (void*)c->adam_m,
                    (void*)c->adam_v, (void*)c->dW, (void*)c->dW_parts, (void*)c->loss, (void*)c->err,
                    (void*)c->samples, (void*)c->sample_count, (void*)c->view_dev, (void*)c->io, (void*)c->tv_raw,
                    (void*)c->tv_thr, (void*)c->tv_rad, (void*)c->tv_count, (void*)c->tv_fx, (void*)c->tv_nsamp,
                    (void*)c->tv_offs, c->tv_queue})
        if (p) cudaFree(p);
    delete c;
}

extern "C" bsm_status bsm_cache_weights(bsm_cache* c, float* get, const float* set) {
    if (!c) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    if (get && cudaMemcpy(get, c->w_master, kMlpParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BSM_ERR_CUDA;
    if (set) upload_weights(c, set);
    return cudaGetLastError() == cudaSuccess ? BSM_OK : BSM_ERR_CUDA;
}

extern "C" bsm_status bsm_cache_render_weights(bsm_cache* c, float* out) {
    if (!c || !out) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    if (c->ema_steps == 0) return cudaMemcpy(out, c->w_master, kMlpParams * 4, cudaMemcpyDeviceToHost) == cudaSuccess
                                      ? BSM_OK : BSM_ERR_CUDA;
    if (cudaMemcpy(out, c->w_ema, kMlpParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BSM_ERR_CUDA;
    double corr = 1.0 / (1.0 - std::pow((double)c->ema_decay, (double)c->ema_steps));
    for (int i = 0; i < kMlpParams; ++i) out[i] = (float)(out[i] * corr);
    return BSM_OK;
}

extern "C" bsm_status bsm_cache_predict(bsm_cache* c, const float* samples, uint32_t n, float* out) {
    if (!c || (!samples && n) || (!out && n)) return BSM_ERR_INVALID_ARG;
    if (n == 0) return BSM_OK;
    cudaSetDevice(c->device);
    size_t in_b = (size_t)n * 64, out_b = (size_t)n * 12, err_off = in_b + ((out_b + 15) & ~(size_t)15);
    if (cache_io(c, err_off + 16)) return BSM_ERR_OUT_OF_MEMORY;
    char* b = (char*)c->io;
    uint32_t* err = (uint32_t*)(b + err_off);
    cudaMemcpy(b, samples, in_b, cudaMemcpyHostToDevice);
    cudaMemset(err, 0, 4);
    if (launch_mlp_predict(c->device, 0, c->w_bf16, (const float4*)b, n, (float*)(b + in_b), err) != cudaSuccess)
        return BSM_ERR_CUDA;
    if (cudaMemcpy(out, b + in_b, out_b, cudaMemcpyDeviceToHost) != cudaSuccess) return BSM_ERR_CUDA;
    uint32_t flag = 0;
    if (cudaMemcpy(&flag, err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BSM_ERR_CUDA;
    return flag ? BSM_ERR_DEVICE_CHECK : BSM_OK;
}

namespace {
// Reads and clears the training kernels' error word (after the work on `st`).
bsm_status take_train_error(bsm_cache* c, cudaStream_t st) {
    uint32_t flag = 0;
    if (cudaMemcpyAsync(&flag, c->err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return BSM_ERR_CUDA;
    if (!flag) return BSM_OK;
    cudaMemsetAsync(c->err, 0, 4, st);
    return BSM_ERR_DEVICE_CHECK;
}

}  // namespace

extern "C" bsm_status bsm_cache_gradient(bsm_cache* c, const float* samples, uint32_t n, float* dW, float* loss) {
    if (!c || !samples || !dW || n == 0) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    size_t in_b = (size_t)n * 64;
    if (cache_io(c, in_b)) return BSM_ERR_OUT_OF_MEMORY;
    cudaMemcpy(c->io, samples, in_b, cudaMemcpyHostToDevice);
    cudaMemset(c->loss, 0, 4);
    uint32_t parts = 0;
    if (launch_mlp_train(c->device, 0, c->w_bf16, (const float4*)c->io, n, c->dW_parts, &parts, c->loss, c->err) !=
            cudaSuccess ||
        launch_mlp_sum_parts(0, c->dW_parts, parts, c->dW) != cudaSuccess)
        return BSM_ERR_CUDA;
    if (cudaMemcpy(dW, c->dW, kMlpParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BSM_ERR_CUDA;
    if (loss) cudaMemcpy(loss, c->loss, 4, cudaMemcpyDeviceToHost);
    return take_train_error(c, 0);
}

namespace {
bsm_status train_device(bsm_cache* c, const float4* samples, uint32_t n, uint32_t batch, float lr, cudaStream_t st,
                        float* mean_loss, float ema_decay = 0.0f) {
    if (ema_decay != c->ema_decay) {  // a new decay starts a new average
        cudaMemsetAsync(c->w_ema, 0, kMlpParams * 4, st);
        c->ema_steps = 0;
        c->ema_decay = ema_decay;
    }
    if (batch == 0) batch = 16384;
    // each step's loss goes to its own device slot; the host reads them once per kLossSlots steps, so
    // the steps are queued back to back without a host round trip
    double loss_sum = 0.0;
    uint32_t steps = 0;
    float host_loss[kLossSlots];
    auto drain = [&](uint32_t k) -> bool {
        if (k == 0) return true;
        if (cudaMemcpyAsync(host_loss, c->loss, k * 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
        if (cudaStreamSynchronize(st) != cudaSuccess) return false;
        for (uint32_t j = 0; j < k; ++j) loss_sum += host_loss[j];
        return true;
    };
    uint32_t slot = 0;
    for (uint32_t off = 0; off < n; off += batch) {
        uint32_t nb = std::min(batch, n - off);
        if (slot == 0) cudaMemsetAsync(c->loss, 0, kLossSlots * 4, st);
        uint32_t parts = 0;
        if (launch_mlp_train(c->device, st, c->w_bf16, samples + 4 * (size_t)off, nb, c->dW_parts, &parts,
                             c->loss + slot, c->err) != cudaSuccess)
            return BSM_ERR_CUDA;
        c->step++;
        if (ema_decay > 0.0f) c->ema_steps++;
        if (launch_mlp_adam(st, c->w_master, c->w_bf16, c->dW_parts, parts, c->adam_m, c->adam_v, lr, c->step,
                            c->w_ema, c->w_ema_bf16, ema_decay, c->ema_steps) != cudaSuccess)
            return BSM_ERR_CUDA;
        ++steps;
        if (++slot == kLossSlots) {
            if (!drain(slot)) return BSM_ERR_CUDA;
            slot = 0;
        }
    }
    if (!drain(slot)) return BSM_ERR_CUDA;
    if (mean_loss) *mean_loss = steps ? (float)(loss_sum / steps) : 0.0f;
    return take_train_error(c, st);
}
}  // namespace

extern "C" bsm_status bsm_cache_train(bsm_cache* c, const float* samples, uint32_t n, uint32_t batch, float lr,
                                      float* loss) {
    if (!c || !samples || n == 0 || !(lr > 0.0f)) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    size_t in_b = (size_t)n * 64;
    if (cache_io(c, in_b)) return BSM_ERR_OUT_OF_MEMORY;
    cudaMemcpy(c->io, samples, in_b, cudaMemcpyHostToDevice);
    return train_device(c, (const float4*)c->io, n, batch, lr, 0, loss);
}

extern "C" bsm_status bsm_cache_save(bsm_cache* c, const char* path) {
    if (!c || !path) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    std::vector<float> w(kMlpParams), m(kMlpParams), v(kMlpParams);
    cudaMemcpy(w.data(), c->w_master, kMlpParams * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(m.data(), c->adam_m, kMlpParams * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(v.data(), c->adam_v, kMlpParams * 4, cudaMemcpyDeviceToHost);
    FILE* f = std::fopen(path, "wb");
    if (!f) return BSM_ERR_INVALID_ARG;
    const uint32_t hdr[4] = {0x43534d42u /* "BMSC" */, 1u, (uint32_t)kMlpParams, (uint32_t)c->step};
    bool ok = std::fwrite(hdr, 4, 4, f) == 4 && std::fwrite(w.data(), 4, kMlpParams, f) == (size_t)kMlpParams &&
              std::fwrite(m.data(), 4, kMlpParams, f) == (size_t)kMlpParams &&
              std::fwrite(v.data(), 4, kMlpParams, f) == (size_t)kMlpParams;
    std::fclose(f);
    return ok ? BSM_OK : BSM_ERR_INVALID_ARG;
}

extern "C" bsm_status bsm_cache_load(bsm_cache* c, const char* path) {
    if (!c || !path) return BSM_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return BSM_ERR_NOT_FOUND;
    uint32_t hdr[4];
    std::vector<float> w(kMlpParams), m(kMlpParams), v(kMlpParams);
    bool ok = std::fread(hdr, 4, 4, f) == 4 && hdr[0] == 0x43534d42u && hdr[1] == 1u && hdr[2] == (uint32_t)kMlpParams &&
              std::fread(w.data(), 4, kMlpParams, f) == (size_t)kMlpParams &&
              std::fread(m.data(), 4, kMlpParams, f) == (size_t)kMlpParams &&
              std::fread(v.data(), 4, kMlpParams, f) == (size_t)kMlpParams;
    std::fclose(f);
    if (!ok) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(c->device);
    upload_weights(c, w.data());
    cudaMemcpy(c->adam_m, m.data(), kMlpParams * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(c->adam_v, v.data(), kMlpParams * 4, cudaMemcpyHostToDevice);
    c->step = (int)hdr[3];
    return BSM_OK;
}

namespace bsm {
// Per-vertex records of the training paths and their shadow-ray queue, grown on demand.
static bsm_status ensure_train_verts(bsm_cache* c, uint32_t paths, uint32_t verts, uint32_t lights1) {
    if (c->tv_cap >= verts && c->tv_paths >= paths && c->tv_lights >= lights1) return BSM_OK;
    if ((uint64_t)verts * lights1 >= (1ull << 32) || (uint64_t)verts >= (1ull << 31)) return BSM_ERR_INVALID_ARG;
    for (void** p : {(void**)&c->tv_raw, (void**)&c->tv_thr, (void**)&c->tv_rad, (void**)&c->tv_count,
                     (void**)&c->tv_fx, (void**)&c->tv_nsamp, (void**)&c->tv_offs, &c->tv_queue})
        if (*p) { cudaFree(*p); *p = nullptr; }
    c->tv_cap = c->tv_paths = c->tv_lights = 0;
    const size_t sh = (size_t)verts * lights1;
    const size_t qbytes = 3 * sh * 16 + ((sh * 4 + 255) & ~(size_t)255) + kCntWords * 4 + 256 + kStatWords * 8;
    bool ok = cudaMalloc((void**)&c->tv_raw, (size_t)verts * 48) == cudaSuccess &&
              cudaMalloc((void**)&c->tv_thr, (size_t)verts * 16) == cudaSuccess &&
              cudaMalloc((void**)&c->tv_rad, (size_t)verts * 16) == cudaSuccess &&
              cudaMalloc((void**)&c->tv_count, (size_t)paths * 4) == cudaSuccess &&
              cudaMalloc((void**)&c->tv_fx, (size_t)verts * 24) == cudaSuccess &&
              cudaMalloc((void**)&c->tv_nsamp, (size_t)paths * 4) == cudaSuccess &&
              cudaMalloc((void**)&c->tv_offs, (size_t)paths * 4) == cudaSuccess &&
              cudaMalloc(&c->tv_queue, qbytes) == cudaSuccess;
    if (!ok) return BSM_ERR_OUT_OF_MEMORY;
    c->tv_cap = verts;
    c->tv_paths = paths;
    c->tv_lights = lights1;
    return BSM_OK;
}

bsm_status cache_train_frame(bsm_cache* c, const DevScene& sc, const DevView& view, const bsm_cache_settings& cs,
                             const LaunchCfg& lc, cudaStream_t st, float* loss_out, uint32_t* samples_out) {
    const uint32_t segs = std::max(1u, std::min(cs.train_segments, 16u));
    const uint32_t cap = cs.train_paths * segs;
    if (c->sample_cap < cap) {
        if (c->samples) cudaFree(c->samples);
        c->samples = nullptr;
        c->sample_cap = 0;
        if (cudaMalloc((void**)&c->samples, (size_t)cap * 64) != cudaSuccess) return BSM_ERR_OUT_OF_MEMORY;
        c->sample_cap = cap;
    }
    const uint32_t lights1 = sc.num_lights + 1u;
    if (bsm_status e = ensure_train_verts(c, cs.train_paths, cap, lights1)) return e;
    // shadow queue view (the fields launch_shadow reads), sized for `cap` vertices x (lights + 1) rays
    const size_t sh = (size_t)cap * lights1;
    char* qb = (char*)c->tv_queue;
    Wavefront q{};
    q.capacity = cap;
    q.sh_o = (float4*)qb;
    q.sh_d = (float4*)(qb + sh * 16);
    q.sh_c = (float4*)(qb + 2 * sh * 16);
    q.sh_seed = (uint32_t*)(qb + 3 * sh * 16);
    q.counters = (uint32_t*)(qb + 3 * sh * 16 + ((sh * 4 + 255) & ~(size_t)255));
    q.stats = (unsigned long long*)((char*)q.counters + ((kCntWords * 4 + 255) & ~(size_t)255));
    q.accum_fx = c->tv_fx;   // the shadow pass adds exact fixed-point sums per vertex
    TrainVerts tv{c->tv_raw, c->tv_thr, c->tv_rad, c->tv_count, segs, c->tv_fx, c->tv_nsamp, c->tv_offs};
    cudaMemcpyAsync(c->view_dev, &view, sizeof(DevView), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(c->tv_fx, 0, (size_t)cap * 24, st);
    cudaMemsetAsync(c->sample_count, 0, 4, st);
    cudaMemsetAsync(q.counters, 0, kCntWords * 4, st);
    launch_train_paths(st, sc, c->view_dev, cs.train_paths, c->frame++, tv, q);
    launch_shadow(lc, st, sc, q, 0, c->tv_rad);
    launch_train_targets(st, cs.train_paths, tv, c->samples, c->sample_count, c->sample_cap);
    if (cudaGetLastError() != cudaSuccess) return BSM_ERR_CUDA;
    uint32_t n = 0;
    cudaMemcpyAsync(&n, c->sample_count, 4, cudaMemcpyDeviceToHost, st);
    if (cudaStreamSynchronize(st) != cudaSuccess) return BSM_ERR_CUDA;
    n = std::min(n, c->sample_cap);
    uint32_t use = std::min(n, cs.train_batch * cs.train_steps);
    if (samples_out) *samples_out = n;
    return train_device(c, c->samples, use, cs.train_batch, cs.lr, st, loss_out, cs.ema_decay);
}
}  // namespace bsm
