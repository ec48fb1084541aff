// pt_noalloc.cu — a render entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc for the duration of a frame: an engine
// that owns every byte of device memory through its own allocator and budget
// (as the bisemutum engine does through its RHI's allocators), a frame loop
// that must not take the implicit device synchronisation an allocation can
// cost, or a host with a fixed memory arena.  bsm_render_noalloc serves them:
// it runs the same wavefront kernels as bsm_render, but its working memory —
// queue counters, the view record and the wavefront queues — lives in one
// file-scope device array of fixed size, and it accumulates into the output
// buffer the caller passes.  It calls no cudaMalloc, cudaFree or other
// allocating routine.
//
// The array is g_noalloc_scratch (64 MiB).  Every GPU that loads this library
// holds it until the process exits.  All calls share it and it keeps the last
// call's contents: calls that overlap on the GPU (two contexts on one device,
// or streams that run concurrently) race on it.  Each call clears what must
// start at zero (counters, statistics, the output sums).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "bsm_pt.h"
#include "pt_device.h"

namespace bsm {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};
LaunchCfg g_lc[kMaxDevices] = {};
bool g_lc_valid[kMaxDevices] = {};

// Device address of the scratch array for the current device (looked up once
// per device; the first call on a device does this set-up).
cudaError_t scratch_for_device(int dev, void** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    if (!g_lc_valid[dev]) {
        g_lc[dev].regcap = 1;
        query_launch_cfg(dev, 128, &g_lc[dev]);
        g_lc_valid[dev] = true;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Turns the per-pixel sums in the caller's buffer into the mean, in place.
__global__ void k_noalloc_mean(float4* acc, uint32_t n, float inv_spp) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = acc[i];
    acc[i] = make_float4(a.x * inv_spp, a.y * inv_spp, a.z * inv_spp, 1.0f);
}

// Scratch layout: counters | stats | view record | wavefront arrays.
constexpr size_t kHeaderBytes = 3 * 256 + 2048;
constexpr size_t align256c(size_t x) { return (x + 255) & ~(size_t)255; }
static_assert(align256c(kCntWords * 4) + align256c(kStatWords * 8) + align256c(sizeof(DevView)) <= kHeaderBytes,
              "the counters, statistics and view record must fit the scratch header");

// 9 float4 path arrays, 3 float4 per shadow slot, and a 4-byte opacity seed per
// shadow slot for scenes with non-opaque triangles
size_t bytes_per_path(uint32_t lights, bool non_opaque) {
    return 9 * 16 + (3 * 16 + (non_opaque ? 4 : 0)) * (size_t)(lights + 1);
}

}  // namespace

uint32_t noalloc_max_paths(uint32_t lights, bool non_opaque) {
    size_t c = (kNoAllocScratchBytes - kHeaderBytes - 16 * 256) / bytes_per_path(lights, non_opaque);
    return (uint32_t)(c & ~(size_t)255);
}

}  // namespace bsm

using namespace bsm;

extern "C" bsm_status bsm_render_noalloc(bsm_context* ctx, uint32_t scene_id, const bsm_camera* cam,
                                         const bsm_pt_settings* s, float* out_rgba) {
    if (!ctx || !cam || !s || !out_rgba) return BSM_ERR_INVALID_ARG;
    if (((uintptr_t)out_rgba & 15u) != 0u) {  // read and written as float4
        ctx_set_error(ctx, "bsm_render_noalloc: out_rgba must be 16-byte aligned");
        return BSM_ERR_INVALID_ARG;
    }
    if (s->block_size != 0 && s->block_size != 64 && s->block_size != 128 && s->block_size != 256) {
        ctx_set_error(ctx, "bsm_render_noalloc: block_size must be 0, 64, 128 or 256");
        return BSM_ERR_INVALID_ARG;
    }
    int dev = ctx_device(ctx);
    if (dev < 0 || dev >= kMaxDevices) return BSM_ERR_INVALID_ARG;
    if (cudaSetDevice(dev) != cudaSuccess) return BSM_ERR_CUDA;
    DevScene sc;
    if (!ctx_scene(ctx, scene_id, &sc)) {
        ctx_set_error(ctx, "bsm_render_noalloc: unknown scene id or BVH not built");
        return BSM_ERR_NOT_FOUND;
    }
    if (ctx_camera_problem(cam) || s->spp == 0 || !(s->ray_length > 0.0f) || s->t_min < 0.0f) {
        ctx_set_error(ctx, "bsm_render_noalloc: invalid camera or settings");
        return BSM_ERR_INVALID_ARG;
    }
    uint32_t max_seg = s->max_segments ? s->max_segments : (std::min(std::max(s->max_bounces, 2u), 16u) - 1u);
    if (max_seg == 0 || max_seg > (uint32_t)kMaxSeg) {
        ctx_set_error(ctx, "bsm_render_noalloc: max_segments must be 1..16");
        return BSM_ERR_INVALID_ARG;
    }
    uint64_t npix = (uint64_t)cam->width * cam->height;
    if (npix >= (1ull << 32)) {
        ctx_set_error(ctx, "bsm_render_noalloc: too many pixels");
        return BSM_ERR_INVALID_ARG;
    }
    const uint32_t lights = std::max(sc.num_lights, 1u);
    const uint32_t max_paths = noalloc_max_paths(lights, sc.has_non_opaque != 0);
    if (s->wavefront_capacity > max_paths) {
        ctx_set_error(ctx, "bsm_render_noalloc: wavefront_capacity exceeds the fixed scratch "
                           "(64 MiB: at most noalloc_max_paths() paths per chunk)");
        return BSM_ERR_INVALID_ARG;
    }
    uint32_t capacity = s->wavefront_capacity ? s->wavefront_capacity : max_paths;
    if (capacity < 1024) {
        ctx_set_error(ctx, "bsm_render_noalloc: wavefront_capacity must be >= 1024");
        return BSM_ERR_INVALID_ARG;
    }

    void* base = nullptr;
    cudaError_t e = scratch_for_device(dev, &base);
    if (e != cudaSuccess) {
        ctx_set_error(ctx, cudaGetErrorString(e));
        return BSM_ERR_CUDA;
    }
    const LaunchCfg& lc = g_lc[dev];
    cudaStream_t st = ctx_stream(ctx);

    char* b = (char*)base;
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = b + off; off += align256(bytes); return p; };
    Wavefront wf{};
    wf.capacity = capacity;
    wf.counters = (uint32_t*)take(kCntWords * 4);
    wf.stats = (unsigned long long*)take(kStatWords * 8);
    DevView* view_dev = (DevView*)take(sizeof(DevView));
    off = kHeaderBytes;
    const size_t C = capacity, SH = C * (lights + 1);
    for (int q = 0; q < 2; ++q) {
        wf.ray_o[q] = (float4*)take(C * 16);
        wf.ray_d[q] = (float4*)take(C * 16);
        wf.path[q] = (uint4*)take(C * 16);
        wf.thr[q] = (float4*)take(C * 16);
    }
    wf.hit = (float4*)take(C * 16);
    wf.sh_o = (float4*)take(SH * 16);
    wf.sh_d = (float4*)take(SH * 16);
    wf.sh_c = (float4*)take(SH * 16);
    wf.sh_seed = sc.has_non_opaque ? (uint32_t*)take(SH * 4) : nullptr;
    if (off > kNoAllocScratchBytes) {  // cannot happen for capacity <= noalloc_max_paths
        ctx_set_error(ctx, "bsm_render_noalloc: scratch layout overflow");
        return BSM_ERR_INVALID_ARG;
    }

    DevView dv{};
    ctx_make_view(cam, &dv);
    dv.ray_length = s->ray_length;
    dv.t_min = s->t_min;
    dv.spp = s->spp;
    dv.sample_offset = s->sample_offset;
    dv.seed = s->seed;
    dv.path_base = 0;
    dv.accum_base = 0;
    dv.max_segments = max_seg;
    dv.flags = s->flags & (BSM_PT_JITTER | BSM_PT_NO_SUN_NEE | BSM_PT_NO_SKY_NEE);

    float4* accum = (float4*)out_rgba;
    uint64_t total = npix * s->spp;
#define NA_CK(call)                                  \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) {                     \
            ctx_set_error(ctx, cudaGetErrorString(e_)); \
            return BSM_ERR_CUDA;                     \
        }                                            \
    } while (0)
    NA_CK(cudaMemcpyAsync(view_dev, &dv, sizeof(dv), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemsetAsync(out_rgba, 0, npix * 16, st));
    NA_CK(cudaMemsetAsync(wf.stats, 0, kStatWords * 8, st));
    // the error word (kCntError) is not cleared here: it keeps a flag until a sync point of the context
    // (bsm_sync, bsm_render_stats_read) reads and clears it
    NA_CK(cudaMemsetAsync(wf.counters, 0, kCntError * 4, st));
    ctx_note_noalloc(ctx, wf.counters);
    for (uint64_t begin = 0; begin < total; begin += capacity) {
        uint32_t count = (uint32_t)std::min<uint64_t>(capacity, total - begin);
        NA_CK(cudaMemsetAsync(wf.counters, 0, kCntError * 4, st));
        launch_camera(lc, st, view_dev, 1, begin, count, wf, max_seg);
        int q = 0;
        for (uint32_t seg = 0; seg < max_seg; ++seg) {
            launch_extend(lc, st, sc, wf, q, seg, false);
            launch_shade(lc, st, sc, view_dev, wf, q, seg, accum);
            launch_shadow(lc, st, sc, wf, seg, accum);
            q ^= 1;
        }
    }
    k_noalloc_mean<<<(uint32_t)((npix + 255) / 256), 256, 0, st>>>(accum, (uint32_t)npix, 1.0f / (float)s->spp);
    NA_CK(cudaGetLastError());
#undef NA_CK
    return BSM_OK;
}
