// api.cpp — host side of the C ABI (include/bsm_pt.h): context, scene upload,
// BVH build, the wavefront render loop and the stage entry points.
//
// Replaces the reference's host orchestration of the pass:
//   PathTracingPass::update_params  (bisemutum/src/renderer/pass/path_tracing.cpp:183-222)
//   PathTracingPass::render         (path_tracing.cpp:224-490): per camera, the
//       history check (:231-245), the bounce loop of camera ray / sample ray /
//       trace / lighting passes (:290-462) and the running-mean accumulation (:464-478).
// The render graph's passes become launches on one CUDA stream; their queue
// sizes stay on the device, and a render's launch sequence is captured once
// into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "bsm_pt.h"
#include "bvh_build.h"
#include "bvh_gpu.h"
#include "cache_impl.h"
#include "pt_device.h"
#include "pt_math.cuh"

using namespace bsm;

namespace {

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct Scene {
    // host copies (kept for rebuilds)
    std::vector<float> positions;
    std::vector<uint32_t> indices;
    std::vector<uint32_t> material_ids;
    std::vector<float> normals;             // per vertex (3 floats), empty when the scene has none
    std::vector<float> transparency;  // per material: 0 opaque, else what the any-hit rule compares against
    uint32_t num_triangles = 0;
    float extent = 1.0f;
    bool has_bvh = false;
    bsm_bvh_stats bvh_stats{};
    bool tuned = false;
    bsm_tune_params tune{};
    DevBuf nodes, tris, materials, texels, sky_alias, pdf_tab, tri_normals;
    // two-level scenes: instances (caller order), their TLAS leaves, refit data
    bool instanced = false;
    std::vector<bsm_instance> instances;
    std::vector<uint32_t> leaf_of;          // caller index -> TLAS leaf (InstDev record)
    std::vector<uint32_t> level_begin;      // TLAS breadth-first level boundaries (levels + 1 entries)
    std::vector<InstDev> inst_host;         // records in leaf order
    DevBuf insts, inst_box, node_box, mat_tr;
    DevScene dev{};
};

// An object-space geometry of two-level scenes: its own BLAS.
struct Geometry {
    DevBuf nodes, tris;
    float lo[3], hi[3];                     // object-space bounds
    uint32_t num_triangles = 0;
    uint32_t max_material = 0;
    uint32_t users = 0;                     // scenes that instance it
};

struct ViewHist {
    bsm_camera cam{};
    uint32_t spp = 0;
    uint32_t accum_base = 0;
    bool valid = false;
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    std::vector<uint8_t> key;
};

}  // namespace

struct bsm_context {
    int device = 0;
    cudaStream_t stream = nullptr;     // the context's own stream (and the one renders are captured on)
    cudaStream_t user_stream = nullptr;  // bsm_set_stream: the caller's stream, or null
    bool has_user_stream = false;
    uint32_t pending_flags = 0;        // device error flags read back but not yet reported
    uint32_t* noalloc_counters = nullptr;  // counters of the last bsm_render_noalloc call (its fixed array)
    bsm_render_stats last_stats{};     // host-side part of the last render's statistics
    bool last_stats_valid = false;
    bool last_stats_timing = false;    // the last render recorded per-stage events
    uint64_t budget = 0;
    uint64_t used = 0;
    std::string err;
    std::map<uint32_t, std::unique_ptr<Scene>> scenes;
    uint32_t next_scene = 1;
    std::map<uint32_t, std::unique_ptr<Geometry>> geoms;
    uint32_t next_geom = 1;
    LaunchCfg lc{};
    int lc_block = 0;
    // wavefront buffers
    Wavefront wf{};
    DevBuf wf_buf;
    uint32_t wf_lights = 0;
    // views and history
    DevBuf views_dev;
    std::vector<DevView> views_host;
    DevBuf accum;                 // float4 per pixel, all views
    DevBuf accum_fx;              // BSM_PT_DETERMINISTIC: one call's 32.32 fixed-point sums, 3 words per pixel
    std::vector<ViewHist> hist;   // per view index
    std::vector<std::pair<uint32_t, uint32_t>> layout;  // (width, height) per view
    DevBuf out_stage;             // device staging for host outputs
    DevBuf tmp;                   // stage entry points (host buffers)
    std::vector<GraphEntry> graphs;
    cudaEvent_t ev[16] = {};
    std::vector<cudaEvent_t> stage_ev;
    std::mutex mu;
    void* server = nullptr;       // serving loop (serve.cpp), null when not started
};

namespace {

void clear_graphs(bsm_context* ctx);

// The stream a context's work runs on: the caller's (bsm_set_stream) or its own.
cudaStream_t WS(const bsm_context* ctx) { return ctx->has_user_stream ? ctx->user_stream : ctx->stream; }

bsm_status fail(bsm_context* ctx, bsm_status st, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return st;
}
// Message for the device error word (counters[kCntError]).
std::string device_flag_text(uint32_t flag) {
    std::string m = "device error flag set:";
    if (flag & 1u) m += " a kernel queue overflowed;";
    if (flag & 2u) m += " a tensor-core wait of the radiance cache timed out;";
    return m;
}
bsm_status cuda_fail(bsm_context* ctx, cudaError_t e, const char* what) {
    return fail(ctx, BSM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                            \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

bsm_status dev_alloc(bsm_context* ctx, DevBuf& b, size_t bytes) {
    if (b.bytes >= bytes && b.ptr) return BSM_OK;
    if (b.ptr) { cudaFree(b.ptr); ctx->used -= b.bytes; b.ptr = nullptr; b.bytes = 0; }
    if (bytes == 0) return BSM_OK;
    if (ctx->budget && ctx->used + bytes > ctx->budget)
        return fail(ctx, BSM_ERR_OUT_OF_MEMORY, "device memory budget exceeded (" + std::to_string(ctx->used + bytes) +
                                                    " > " + std::to_string(ctx->budget) + " bytes)");
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
        b.ptr = nullptr;
        cudaGetLastError();
        return fail(ctx, BSM_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b.bytes = bytes;
    ctx->used += bytes;
    return BSM_OK;
}
void dev_free(bsm_context* ctx, DevBuf& b) {
    if (b.ptr) { cudaFree(b.ptr); ctx->used -= b.bytes; }
    b.ptr = nullptr;
    b.bytes = 0;
}

V3 vnorm(V3 a) { return normalize(a); }

// Camera basis of glm::lookAt(position, position + front, up) (right-handed):
// s = normalize(cross(f, up)), u = cross(s, f).  camera.cpp:96-98.
void make_view(const bsm_camera& c, DevView& v) {
    V3 f = vnorm(v3(c.front[0], c.front[1], c.front[2]));
    V3 s = vnorm(cross(f, v3(c.up[0], c.up[1], c.up[2])));
    V3 u = cross(s, f);
    v.pos[0] = c.position[0]; v.pos[1] = c.position[1]; v.pos[2] = c.position[2];
    v.s[0] = s.x; v.s[1] = s.y; v.s[2] = s.z;
    v.u[0] = u.x; v.u[1] = u.y; v.u[2] = u.z;
    v.f[0] = f.x; v.f[1] = f.y; v.f[2] = f.z;
    v.tan_half = (float)std::tan((double)c.yfov_deg * 3.14159265358979323846 / 360.0);
    v.aspect = (float)c.width / (float)c.height;
    v.width = c.width;
    v.height = c.height;
}

// Why a camera cannot be rendered, or nullptr: a view needs a size, a field of
// view in (0, 180) degrees, finite vectors, and a front that is neither zero
// nor parallel to up (the view basis is built from front x up).
const char* camera_problem(const bsm_camera& c) {
    if (c.width == 0 || c.height == 0) return "view size must be > 0";
    if (!(c.yfov_deg > 0.0f && c.yfov_deg < 180.0f)) return "yfov_deg must be in (0, 180)";
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(c.position[k]) || !std::isfinite(c.front[k]) || !std::isfinite(c.up[k]))
            return "camera position, front and up must be finite";
    double f[3] = {c.front[0], c.front[1], c.front[2]}, u[3] = {c.up[0], c.up[1], c.up[2]};
    double x[3] = {f[1] * u[2] - f[2] * u[1], f[2] * u[0] - f[0] * u[2], f[0] * u[1] - f[1] * u[0]};
    double ff = f[0] * f[0] + f[1] * f[1] + f[2] * f[2], uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    double xx = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    if (!(ff > 0.0) || !(uu > 0.0)) return "camera front and up must not be zero";
    if (!(xx > 1e-12 * ff * uu)) return "camera front must not be parallel to up";
    return nullptr;
}

bool same_camera(const bsm_camera& a, const bsm_camera& b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

// Sky sampling tables: texel weights (r + g + b) * sin(theta at the row centre),
// the pdf of each texel in (u, v) space, and an alias table over the texels
// (Walker's method with Vose's construction): entry k keeps texel k with
// probability prob[k] and otherwise gives its alias.  Two words per entry:
// the bits of prob, the alias.  Sampling is two dependent loads instead of two
// binary searches over CDFs.
void build_sky_tables(const bsm_sky& sky, std::vector<uint32_t>& alias, std::vector<float>& pdf) {
    const uint32_t W = sky.width, H = sky.height;
    const size_t N = (size_t)W * H;
    pdf.assign(N, 0.0f);
    std::vector<double> w((size_t)H * W), rows(H);
    double total = 0.0;
    for (uint32_t i = 0; i < H; ++i) {
        float st, ct;
        sincos_turns(((float)i + 0.5f) / (2.0f * (float)H), &st, &ct);
        double rs = 0.0;
        for (uint32_t j = 0; j < W; ++j) {
            const uint16_t* t = sky.rgba16f + ((size_t)i * W + j) * 4;
            float lum = half_to_float(t[0]) + half_to_float(t[1]) + half_to_float(t[2]);
            double wij = lum > 0.0f ? (double)lum * (double)st : 0.0;
            w[(size_t)i * W + j] = wij;
            rs += wij;
        }
        rows[i] = rs;
        total += rs;
    }
    for (size_t k = 0; k < N; ++k)
        pdf[k] = total > 0.0 ? (float)(w[k] * (double)W * (double)H / total) : 0.0f;
    // Vose: scaled weights q = N w / total; small (q < 1) entries take a large one's excess
    alias.assign(2 * N, 0u);
    std::vector<double> q(N);
    std::vector<uint32_t> small, large;
    for (size_t k = 0; k < N; ++k) {
        q[k] = total > 0.0 ? w[k] * (double)N / total : 1.0;
        (q[k] < 1.0 ? small : large).push_back((uint32_t)k);
    }
    auto put = [&](uint32_t k, float prob, uint32_t a) {
        std::memcpy(&alias[2 * (size_t)k], &prob, 4);
        alias[2 * (size_t)k + 1] = a;
    };
    while (!small.empty() && !large.empty()) {
        uint32_t sm = small.back();
        small.pop_back();
        uint32_t lg = large.back();
        put(sm, (float)q[sm], lg);
        q[lg] = (q[lg] + q[sm]) - 1.0;
        if (q[lg] < 1.0) {
            large.pop_back();
            small.push_back(lg);
        }
    }
    for (uint32_t k : large) put(k, 1.0f, k);
    for (uint32_t k : small) put(k, 1.0f, k);  // rounding leftovers
}

bsm_status ensure_launch_cfg(bsm_context* ctx, uint32_t block, int regcap = 0) {
    int b = block ? (int)block : 128;
    if (b != 64 && b != 128 && b != 256) return fail(ctx, BSM_ERR_INVALID_ARG, "block_size must be 64, 128 or 256");
    int key = b | (regcap << 16);
    if (ctx->lc_block == key) return BSM_OK;
    ctx->lc.regcap = regcap;
    query_launch_cfg(ctx->device, b, &ctx->lc);
    ctx->lc_block = key;
    return BSM_OK;
}

// The launch configuration of a render of scene `sc`: tuned parameters of the scene fill in what the
// settings leave at 0.
bsm_status prepare_launch(bsm_context* ctx, const Scene* sc, const bsm_pt_settings& s) {
    uint32_t block = s.block_size ? s.block_size : (sc->tuned ? sc->tune.block_size : 0u);
    if (bsm_status st = ensure_launch_cfg(ctx, block, sc->tuned ? (int)(sc->tune.register_cap != 0) : 1)) return st;
    ctx->lc.postpone_sp = sc->tuned ? (int)sc->tune.postpone_depth : 16;
    ctx->lc.refill_min = sc->tuned ? (int)sc->tune.refill_lanes : 8;
    return BSM_OK;
}

// Device bytes of the wavefront per path slot (the layout of ensure_wavefront):
// 9 arrays of 16 B (rays, paths and throughputs ping-pong, hits), 64 B of cache
// query, and (lights + 1) shadow records of 3 x 16 B + a 4 B opacity seed.
uint64_t wavefront_bytes_per_path(uint32_t lights) { return 9 * 16 + 64 + (uint64_t)(lights + 1) * (3 * 16 + 4); }

// Paths per chunk when the caller leaves it open: the whole call up to 2^27
// paths (one chunk for a 1920x1080 frame at 64 spp), within half of the device
// memory the context's budget has left.  Bigger chunks keep the late, short
// segments of a frame wide enough to fill the GPU (measured on the terrain at
// 64 spp: 1154 Mrays/s with 2^23-path chunks, 1216 with 2^24, 1249 with 2^25,
// 1273 with one chunk).
uint32_t default_capacity(const bsm_context* ctx, uint64_t total_paths, uint32_t lights) {
    uint64_t left = ctx->budget > ctx->used ? ctx->budget - ctx->used + ctx->wf_buf.bytes : ctx->wf_buf.bytes;
    uint64_t by_mem = left / 2 / wavefront_bytes_per_path(lights);
    uint64_t c = std::min<uint64_t>(std::min<uint64_t>(total_paths, 1ull << 27), by_mem);
    return (uint32_t)std::max<uint64_t>(c, 1024);
}

bsm_status ensure_wavefront(bsm_context* ctx, uint32_t capacity, uint32_t lights) {
    if (ctx->wf.capacity >= capacity && ctx->wf_lights >= lights && ctx->wf_buf.ptr) return BSM_OK;
    // queue slots are 32-bit: the shadow queue holds (lights + 1) records per path
    if ((uint64_t)capacity * (lights + 1) >= (1ull << 32))
        return fail(ctx, BSM_ERR_INVALID_ARG, "wavefront_capacity x (lights + 1) must stay below 2^32");
    size_t C = capacity;
    size_t sh = C * (lights + 1);
    size_t bytes = 0;
    auto sz = [&](size_t n) { size_t off = bytes; bytes += (n + 255) & ~(size_t)255; return off; };
    size_t o_ro0 = sz(C * 16), o_ro1 = sz(C * 16), o_rd0 = sz(C * 16), o_rd1 = sz(C * 16);
    size_t o_p0 = sz(C * 16), o_p1 = sz(C * 16), o_t0 = sz(C * 16), o_t1 = sz(C * 16);
    size_t o_hit = sz(C * 16), o_sho = sz(sh * 16), o_shd = sz(sh * 16), o_shc = sz(sh * 16), o_cq = sz(C * 64);
    size_t o_shs = sz(sh * 4);
    size_t o_cnt = sz(kCntWords * 4), o_st = sz(kStatWords * 8);
    clear_graphs(ctx);  // graphs hold the old pointers
    if (ctx->wf.counters) {  // keep the old buffer's error flags for the next sync point
        uint32_t f = 0;
        if (cudaStreamSynchronize(WS(ctx)) == cudaSuccess &&
            cudaMemcpy(&f, ctx->wf.counters + kCntError, 4, cudaMemcpyDeviceToHost) == cudaSuccess)
            ctx->pending_flags |= f;
    }
    dev_free(ctx, ctx->wf_buf);
    bsm_status s = dev_alloc(ctx, ctx->wf_buf, bytes);
    if (s) { ctx->wf = Wavefront{}; return s; }
    char* b = (char*)ctx->wf_buf.ptr;
    Wavefront& w = ctx->wf;
    w.capacity = capacity;
    w.ray_o[0] = (float4*)(b + o_ro0); w.ray_o[1] = (float4*)(b + o_ro1);
    w.ray_d[0] = (float4*)(b + o_rd0); w.ray_d[1] = (float4*)(b + o_rd1);
    w.path[0] = (uint4*)(b + o_p0); w.path[1] = (uint4*)(b + o_p1);
    w.thr[0] = (float4*)(b + o_t0); w.thr[1] = (float4*)(b + o_t1);
    w.hit = (float4*)(b + o_hit);
    w.sh_o = (float4*)(b + o_sho); w.sh_d = (float4*)(b + o_shd); w.sh_c = (float4*)(b + o_shc);
    w.sh_seed = (uint32_t*)(b + o_shs);
    w.cache_q = (float4*)(b + o_cq);
    w.counters = (uint32_t*)(b + o_cnt);
    w.stats = (unsigned long long*)(b + o_st);
    ctx->wf_lights = lights;
    if (cudaMemset(w.counters, 0, kCntWords * 4) != cudaSuccess) return fail(ctx, BSM_ERR_CUDA, "counter clear failed");
    return BSM_OK;
}

// Reads and clears the device error words of the context's work (its wavefront's
// and the fixed array's of its last allocation-free render) after waiting for
// the work stream.  A flag stays set on the device until a sync point reads it,
// so renders queued back to back cannot hide one another's errors.
bsm_status take_device_flags(bsm_context* ctx, uint32_t* flags) {
    cudaStream_t st = WS(ctx);
    CK(cudaStreamSynchronize(st));
    uint32_t f = ctx->pending_flags;
    ctx->pending_flags = 0;
    uint32_t* words[2] = {ctx->wf.counters ? ctx->wf.counters + kCntError : nullptr,
                          ctx->noalloc_counters ? ctx->noalloc_counters + kCntError : nullptr};
    for (uint32_t* w : words) {
        if (!w) continue;
        uint32_t h = 0;
        CK(cudaMemcpyAsync(&h, w, 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (h) {
            f |= h;
            CK(cudaMemsetAsync(w, 0, 4, st));
        }
    }
    CK(cudaStreamSynchronize(st));
    *flags = f;
    return BSM_OK;
}

// Waits for the work stream and turns set device flags into BSM_ERR_DEVICE_CHECK.
bsm_status check_device_flags(bsm_context* ctx) {
    uint32_t flag = 0;
    bsm_status s = take_device_flags(ctx, &flag);
    if (s) return s;
    if (flag) return fail(ctx, BSM_ERR_DEVICE_CHECK, device_flag_text(flag));
    return BSM_OK;
}

void clear_graphs(bsm_context* ctx) {
    for (auto& g : ctx->graphs) if (g.exec) cudaGraphExecDestroy(g.exec);
    ctx->graphs.clear();
}

Scene* find_scene(bsm_context* ctx, uint32_t id) {
    auto it = ctx->scenes.find(id);
    return it == ctx->scenes.end() ? nullptr : it->second.get();
}

}  // namespace

// ============================================================== context ====
extern "C" int bsm_api_version(void) { return BSM_API_VERSION; }

extern "C" bsm_status bsm_create(bsm_context** out, int device, uint64_t budget) {
    if (!out) return BSM_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) { cudaGetLastError(); return BSM_ERR_NO_DEVICE; }
    if (device < 0 || device >= n) return BSM_ERR_INVALID_ARG;
    auto* ctx = new bsm_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return BSM_ERR_CUDA; }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return BSM_ERR_CUDA; }
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    ctx->budget = budget ? budget : (uint64_t)((double)fr * 0.9);
    for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    *out = ctx;
    return BSM_OK;
}

extern "C" void bsm_destroy(bsm_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->server) bsm_server_stop(ctx);
    cudaStreamSynchronize(WS(ctx));
    cudaStreamSynchronize(ctx->stream);
    for (auto& g : ctx->graphs) if (g.exec) cudaGraphExecDestroy(g.exec);
    for (auto& kv : ctx->scenes) {
        Scene* s = kv.second.get();
        for (DevBuf* b : {&s->nodes, &s->tris, &s->materials, &s->texels, &s->sky_alias, &s->pdf_tab,
                          &s->tri_normals})
            dev_free(ctx, *b);
    }
    dev_free(ctx, ctx->wf_buf);
    dev_free(ctx, ctx->views_dev);
    dev_free(ctx, ctx->accum);
    dev_free(ctx, ctx->accum_fx);
    dev_free(ctx, ctx->out_stage);
    dev_free(ctx, ctx->tmp);
    for (auto& ev : ctx->ev) if (ev) cudaEventDestroy(ev);
    for (auto& ev : ctx->stage_ev) cudaEventDestroy(ev);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" const char* bsm_last_error(const bsm_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" bsm_status bsm_sync(bsm_context* ctx, uint32_t timeout_ms) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    auto t0 = std::chrono::steady_clock::now();
    while (true) {
        cudaError_t e = cudaStreamQuery(WS(ctx));
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return cuda_fail(ctx, e, "cudaStreamQuery");
        auto ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_ms && ms > timeout_ms) return fail(ctx, BSM_ERR_TIMEOUT, "bsm_sync timed out");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return check_device_flags(ctx);
}

extern "C" bsm_status bsm_set_stream(bsm_context* ctx, void* stream) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    if (ctx->server) return fail(ctx, BSM_ERR_BAD_STATE, "the stream cannot change while the server runs");
    cudaSetDevice(ctx->device);
    cudaStream_t next = stream ? (cudaStream_t)stream : ctx->stream;
    if (next != WS(ctx)) {
        // work queued on the old stream keeps its order before work on the new one
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        cudaError_t r = cudaEventRecord(e, WS(ctx));
        if (r == cudaSuccess) r = cudaStreamWaitEvent(next, e, 0);
        cudaEventDestroy(e);
        if (r != cudaSuccess) return cuda_fail(ctx, r, "bsm_set_stream: ordering against the previous stream");
    }
    ctx->user_stream = (cudaStream_t)stream;
    ctx->has_user_stream = stream != nullptr;
    return BSM_OK;
}

extern "C" void* bsm_get_stream(bsm_context* ctx) { return ctx ? (void*)WS(ctx) : nullptr; }

extern "C" bsm_status bsm_device_alloc(bsm_context* ctx, uint64_t bytes, void** ptr) {
    if (!ctx || !ptr) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->budget && ctx->used + bytes > ctx->budget) return fail(ctx, BSM_ERR_OUT_OF_MEMORY, "budget exceeded");
    CK(cudaMalloc(ptr, bytes ? bytes : 1));
    ctx->used += bytes;
    return BSM_OK;
}
extern "C" bsm_status bsm_device_free(bsm_context* ctx, void* ptr) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaFree(ptr));
    return BSM_OK;
}
extern "C" bsm_status bsm_memcpy(bsm_context* ctx, void* dst, const void* src, uint64_t bytes, int kind) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    CK(cudaMemcpyAsync(dst, src, bytes, k, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    return BSM_OK;
}

extern "C" bsm_status bsm_host_alloc(bsm_context* ctx, uint64_t bytes, void** ptr) {
    if (!ctx || !ptr) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    CK(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault));
    return BSM_OK;
}
extern "C" bsm_status bsm_host_free(bsm_context* ctx, void* ptr) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    CK(cudaFreeHost(ptr));
    return BSM_OK;
}

namespace {
bsm_status build_tlas(bsm_context* ctx, Scene* sc);

// Device buffers of a scene; an instanced scene also lets go of its geometries.
void free_scene_buffers(bsm_context* ctx, Scene& sc) {
    for (DevBuf* b : {&sc.nodes, &sc.tris, &sc.materials, &sc.texels, &sc.sky_alias, &sc.pdf_tab, &sc.tri_normals,
                      &sc.insts, &sc.inst_box, &sc.node_box, &sc.mat_tr})
        dev_free(ctx, *b);
    if (sc.instanced)
        for (const bsm_instance& in : sc.instances) {
            auto it = ctx->geoms.find(in.geometry_id);
            if (it != ctx->geoms.end() && it->second->users > 0) it->second->users--;
        }
    sc.instanced = false;
    sc.instances.clear();
}

// Materials, lights, sky and the scene bounds of a scene (both kinds).
// IEEE half of a float, round to nearest even (for resampled sky texels).
uint16_t float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t exp = (x >> 23) & 0xffu;
    uint32_t man = x & 0x7fffffu;
    if (exp == 0xffu) return (uint16_t)(sign | 0x7c00u | (man ? 0x200u : 0u));
    int e = (int)exp - 127 + 15;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {  // subnormal half
        if (e < -10) return (uint16_t)sign;
        man |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - e);
        uint32_t h = man >> shift;
        uint32_t rem = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)e << 10) | (man >> 13);
    uint32_t rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;  // may carry into the exponent: still correct
    return (uint16_t)(sign | h);
}

// A cubemap sky (6 faces +X -X +Y -Y +Z -Z, RGBA16F) resampled to the equirect
// layout of the sky sampler (4 size x 2 size): per texel centre the direction,
// rotated by the sky transform, picks a face by the standard cube face table
// (major axis; +X: (-z, -y), -X: (z, -y), +Y: (x, z), -Y: (x, -z), +Z: (x, -y),
// -Z: (-x, -y)) and is filtered bilinearly inside that face.
void cube_to_equirect(const bsm_sky& sky, std::vector<uint16_t>& out, uint32_t& W, uint32_t& H) {
    const uint32_t S = sky.width;
    W = 4 * S;
    H = 2 * S;
    out.assign((size_t)W * H * 4, 0);
    double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    bool any = false;
    for (int k = 0; k < 9; ++k) any = any || sky.transform[k] != 0.0f;
    if (any)
        for (int k = 0; k < 9; ++k) R[k] = sky.transform[k];
    const double pi = 3.14159265358979323846;
    for (uint32_t i = 0; i < H; ++i) {
        double th = pi * (i + 0.5) / H;
        for (uint32_t j = 0; j < W; ++j) {
            double ph = 2.0 * pi * ((j + 0.5) / W - 0.5);
            double d0[3] = {std::sin(th) * std::cos(ph), std::cos(th), std::sin(th) * std::sin(ph)};
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = R[3 * k] * d0[0] + R[3 * k + 1] * d0[1] + R[3 * k + 2] * d0[2];
            double ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
            int face;
            double sc, tc, ma;
            if (ax >= ay && ax >= az) { face = d[0] > 0 ? 0 : 1; ma = ax; sc = d[0] > 0 ? -d[2] : d[2]; tc = -d[1]; }
            else if (ay >= az) { face = d[1] > 0 ? 2 : 3; ma = ay; sc = d[0]; tc = d[1] > 0 ? d[2] : -d[2]; }
            else { face = d[2] > 0 ? 4 : 5; ma = az; sc = d[2] > 0 ? d[0] : -d[0]; tc = -d[1]; }
            double x = ((sc / ma + 1.0) * 0.5) * S - 0.5, y = ((tc / ma + 1.0) * 0.5) * S - 0.5;
            x = std::min(std::max(x, 0.0), (double)S - 1);
            y = std::min(std::max(y, 0.0), (double)S - 1);
            uint32_t x0 = (uint32_t)x, y0 = (uint32_t)y;
            uint32_t x1 = std::min(x0 + 1, S - 1), y1 = std::min(y0 + 1, S - 1);
            double fx = x - x0, fy = y - y0;
            const uint16_t* F = sky.rgba16f + (size_t)face * S * S * 4;
            for (int c = 0; c < 4; ++c) {
                auto at = [&](uint32_t xx, uint32_t yy) { return (double)half_to_float(F[((size_t)yy * S + xx) * 4 + c]); };
                double v = (at(x0, y0) * (1 - fx) + at(x1, y0) * fx) * (1 - fy) + (at(x0, y1) * (1 - fx) + at(x1, y1) * fx) * fy;
                out[((size_t)i * W + j) * 4 + c] = float_to_half((float)v);
            }
        }
    }
}

bsm_status setup_shading(bsm_context* ctx, Scene* sc, const bsm_material* materials, uint32_t num_materials,
                         const bsm_dir_light* dir_lights, uint32_t num_dir_lights, const bsm_point_light* point_lights,
                         uint32_t num_point_lights, const bsm_rect_light* rect_lights, uint32_t num_rect_lights,
                         const bsm_sky& sky_in, const float lo[3], const float hi[3]) {
    if (num_materials == 0 || !materials) return fail(ctx, BSM_ERR_INVALID_ARG, "scene needs at least one material");
    if ((uint64_t)num_dir_lights + num_point_lights + num_rect_lights > (uint64_t)kMaxLights)
        return fail(ctx, BSM_ERR_INVALID_ARG, "at most " + std::to_string(kMaxLights) + " lights in all");
    if ((num_dir_lights && !dir_lights) || (num_point_lights && !point_lights) || (num_rect_lights && !rect_lights))
        return fail(ctx, BSM_ERR_INVALID_ARG, "light array is NULL");
    if (sky_in.kind > BSM_SKY_CUBEMAP) return fail(ctx, BSM_ERR_INVALID_ARG, "unknown sky kind");
    if (sky_in.kind != BSM_SKY_CONSTANT && (!sky_in.rgba16f || sky_in.width == 0 || sky_in.height == 0))
        return fail(ctx, BSM_ERR_INVALID_ARG, "sky map needs texels");
    if (sky_in.kind == BSM_SKY_CUBEMAP && sky_in.width != sky_in.height)
        return fail(ctx, BSM_ERR_INVALID_ARG, "cubemap faces must be square");
    bsm_sky sky = sky_in;
    std::vector<uint16_t> cube_eq;
    if (sky_in.kind == BSM_SKY_CUBEMAP) {  // resampled once into the sampler's equirect layout
        uint32_t W, H;
        cube_to_equirect(sky_in, cube_eq, W, H);
        sky.kind = BSM_SKY_EQUIRECT;
        sky.width = W;
        sky.height = H;
        sky.rgba16f = cube_eq.data();
    }
    sc->extent = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), std::max(hi[2] - lo[2], 1e-6f));
    // materials: (base.rgb, roughness), (f0.rgb, metallic); f0 = lerp(0.04, base, metallic)
    std::vector<float4> mats(2 * (size_t)num_materials);
    sc->transparency.assign(num_materials, 0.0f);
    for (uint32_t m = 0; m < num_materials; ++m) {
        const bsm_material& M = materials[m];
        if (M.blend_mode > BSM_BLEND_TRANSLUCENT) return fail(ctx, BSM_ERR_INVALID_ARG, "unknown blend mode");
        if (M.blend_mode != BSM_BLEND_OPAQUE && !(M.opacity >= 0.0f && M.opacity <= 1.0f))
            return fail(ctx, BSM_ERR_INVALID_ARG, "opacity must be in [0, 1]");
        // the any-hit rule (rt_gbuffer_hit.hlsl:20-35): alpha test drops the hit below the
        // threshold (utils.hlsl:38), translucent drops it when u < 1 - opacity
        if (M.blend_mode == BSM_BLEND_ALPHA_TEST) sc->transparency[m] = M.opacity < 0.01f ? 1.0f : 0.0f;
        if (M.blend_mode == BSM_BLEND_TRANSLUCENT) sc->transparency[m] = 1.0f - M.opacity;
        float f0[3];
        for (int k = 0; k < 3; ++k) f0[k] = 0.04f + (M.base_color[k] - 0.04f) * M.metallic;
        mats[2 * m] = make_float4(M.base_color[0], M.base_color[1], M.base_color[2], M.roughness);
        mats[2 * m + 1] = make_float4(f0[0], f0[1], f0[2], M.metallic);
    }
    bsm_status st;
    if ((st = dev_alloc(ctx, sc->materials, mats.size() * sizeof(float4)))) return st;
    CK(cudaMemcpy(sc->materials.ptr, mats.data(), mats.size() * sizeof(float4), cudaMemcpyHostToDevice));
    DevScene& ds = sc->dev;
    ds.materials = (const float4*)sc->materials.ptr;
    ds.num_materials = num_materials;
    uint32_t nl = 0;
    auto kind_bits = [](uint32_t k) { float f; std::memcpy(&f, &k, 4); return f; };
    for (uint32_t l = 0; l < num_dir_lights; ++l) {
        const bsm_dir_light& L = dir_lights[l];
        V3 dir = normalize(v3(L.direction[0], L.direction[1], L.direction[2]));
        DevLight& d = ds.lights[nl++];
        d.a = make_float4(dir.x, dir.y, dir.z, kind_bits(kLightDir));
        d.b = make_float4(L.emission[0], L.emission[1], L.emission[2], 0.0f);
        d.c = d.d = make_float4(0, 0, 0, 0);
    }
    for (uint32_t l = 0; l < num_point_lights; ++l) {
        const bsm_point_light& L = point_lights[l];
        if (!(L.range > 0.0f)) return fail(ctx, BSM_ERR_INVALID_ARG, "point light range must be > 0");
        V3 dir = normalize(v3(L.direction[0], L.direction[1], L.direction[2]));
        if (!(L.cos_inner > L.cos_outer)) dir = v3(0.0f, 0.0f, 1.0f);
        DevLight& d = ds.lights[nl++];
        d.a = make_float4(L.position[0], L.position[1], L.position[2], kind_bits(kLightPoint));
        d.b = make_float4(L.emission[0], L.emission[1], L.emission[2], 1.0f / (L.range * L.range));
        d.c = make_float4(dir.x, dir.y, dir.z, L.cos_inner);
        d.d = make_float4(L.cos_outer, 0.0f, 0.0f, 0.0f);
    }
    for (uint32_t l = 0; l < num_rect_lights; ++l) {
        const bsm_rect_light& L = rect_lights[l];
        if (!(L.width > 0.0f && L.height > 0.0f)) return fail(ctx, BSM_ERR_INVALID_ARG, "rect light size must be > 0");
        V3 ax = v3(L.axis_x[0], L.axis_x[1], L.axis_x[2]), ay = v3(L.axis_y[0], L.axis_y[1], L.axis_y[2]);
        V3 c = v3(L.center[0], L.center[1], L.center[2]);
        V3 eu = ax * L.width, ev = ay * L.height;
        V3 corner = c - ax * (0.5f * L.width) - ay * (0.5f * L.height);
        DevLight& d = ds.lights[nl++];
        d.a = make_float4(corner.x, corner.y, corner.z, kind_bits(kLightRect));
        d.b = make_float4(L.emission[0], L.emission[1], L.emission[2], kind_bits(L.two_sided ? 1u : 0u));
        d.c = make_float4(eu.x, eu.y, eu.z, L.width * L.height);
        d.d = make_float4(ev.x, ev.y, ev.z, 0.0f);
    }
    ds.num_lights = nl;
    ds.dir_lights_only = 1u;
    for (uint32_t l = 0; l < nl; ++l)
        if (f2u(ds.lights[l].a.w) != kLightDir) ds.dir_lights_only = 0u;
    ds.sky.kind = sky.kind;
    ds.sky.cr = sky.color[0]; ds.sky.cg = sky.color[1]; ds.sky.cb = sky.color[2];
    if (sky.kind == BSM_SKY_EQUIRECT) {
        const uint32_t W = sky.width, H = sky.height;
        std::vector<uint32_t> alias;
        std::vector<float> pdf;
        build_sky_tables(sky, alias, pdf);
        size_t tb = (size_t)W * H * 8;
        if ((st = dev_alloc(ctx, sc->texels, tb))) return st;
        if ((st = dev_alloc(ctx, sc->sky_alias, alias.size() * 4))) return st;
        if ((st = dev_alloc(ctx, sc->pdf_tab, pdf.size() * 4))) return st;
        CK(cudaMemcpy(sc->texels.ptr, sky.rgba16f, tb, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->sky_alias.ptr, alias.data(), alias.size() * 4, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->pdf_tab.ptr, pdf.data(), pdf.size() * 4, cudaMemcpyHostToDevice));
        ds.sky.width = W; ds.sky.height = H;
        ds.sky.texels = (const ushort4*)sc->texels.ptr;
        ds.sky.alias = (const uint2*)sc->sky_alias.ptr;
        ds.sky.pdf_tab = (const float*)sc->pdf_tab.ptr;
    }
    ds.ray_offset = 2e-5f * sc->extent;
    for (int k = 0; k < 3; ++k) {
        ds.box_lo[k] = lo[k];
        ds.box_inv[k] = 1.0f / std::max(hi[k] - lo[k], 1e-6f);
    }
    return BSM_OK;
}

}  // namespace

namespace {

// Builds a BVH with the device builder from host arrays: uploads them to one
// temporary buffer, runs bvh_gpu.cu's build on the context's own stream and
// adopts the node and triangle buffers it returns.  The scratch the build holds
// counts against the memory budget while it runs.
bsm_status device_bvh(bsm_context* ctx, const float* positions, uint32_t nv, const uint32_t* indices, uint32_t nt,
                      const uint32_t* material_ids, const std::vector<float>& transparency, const bsm_bvh_opts* opts,
                      DevBuf& nodes, DevBuf& tris, bsm_bvh_stats& s) {
    auto a256 = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_pos = a256((size_t)nv * 12), b_idx = indices ? a256((size_t)nt * 12) : 0,
                 b_mat = material_ids ? a256((size_t)nt * 4) : 0, b_tr = a256(transparency.size() * 4 + 4);
    const uint64_t need = b_pos + b_idx + b_mat + b_tr + device_build_scratch_bytes(nt) + device_build_output_bytes(nt);
    if (ctx->budget && ctx->used + need > ctx->budget)
        return fail(ctx, BSM_ERR_OUT_OF_MEMORY, "device BVH build needs " + std::to_string(need) +
                                                    " bytes beyond the memory budget");
    auto t0 = std::chrono::steady_clock::now();
    char* in = nullptr;
    CK(cudaMalloc(&in, b_pos + b_idx + b_mat + b_tr));
    cudaStream_t st = ctx->stream;
    float* d_pos = (float*)in;
    uint32_t* d_idx = indices ? (uint32_t*)(in + b_pos) : nullptr;
    uint32_t* d_mat = material_ids ? (uint32_t*)(in + b_pos + b_idx) : nullptr;
    float* d_tr = transparency.empty() ? nullptr : (float*)(in + b_pos + b_idx + b_mat);
    cudaError_t e = cudaMemcpyAsync(d_pos, positions, (size_t)nv * 12, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && d_idx) e = cudaMemcpyAsync(d_idx, indices, (size_t)nt * 12, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && d_mat) e = cudaMemcpyAsync(d_mat, material_ids, (size_t)nt * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && d_tr)
        e = cudaMemcpyAsync(d_tr, transparency.data(), transparency.size() * 4, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { cudaFree(in); return cuda_fail(ctx, e, "device BVH build: input upload"); }
    DeviceBvhResult r;
    std::string err;
    bool ok = build_cwbvh_device(st, d_pos, nv, d_idx, nt, d_mat, d_tr, (uint32_t)transparency.size(), opts, r, err);
    cudaFree(in);
    if (!ok) return fail(ctx, BSM_ERR_INVALID_ARG, "BVH build failed: " + err);
    if (r.max_depth > (uint32_t)kMaxTraversalDepth) {
        cudaFree(r.nodes);
        cudaFree(r.tris);
        return fail(ctx, BSM_ERR_UNSUPPORTED, "BVH deeper than the traversal stack (" + std::to_string(r.max_depth) + ")");
    }
    dev_free(ctx, nodes);
    dev_free(ctx, tris);
    nodes.ptr = r.nodes;
    nodes.bytes = (size_t)r.num_nodes * sizeof(CwNode);
    tris.ptr = r.tris;
    tris.bytes = (size_t)r.num_tris * sizeof(CwTri);
    ctx->used += nodes.bytes + tris.bytes;
    s = bsm_bvh_stats{};
    s.num_nodes = r.num_nodes;
    s.num_tris = r.num_tris;
    s.max_depth = r.max_depth;
    s.builder = BSM_BUILD_DEVICE;
    s.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    s.sah_cost = r.sah_cost;
    s.node_bytes = nodes.bytes;
    s.tri_bytes = tris.bytes;
    return BSM_OK;
}

bool use_host_builder(const bsm_bvh_opts* opts) { return opts && opts->builder == BSM_BUILD_HOST; }

// The leaf-ordered vertex normals of a scene that has them (after every BVH build: the leaf order changes).
bsm_status make_tri_normals(bsm_context* ctx, Scene* sc) {
    sc->dev.tri_normals = nullptr;
    if (sc->normals.empty()) return BSM_OK;
    bsm_status st;
    if ((st = dev_alloc(ctx, sc->tri_normals, (size_t)sc->num_triangles * 48))) return st;
    const size_t b_n = (sc->normals.size() * 4 + 255) & ~(size_t)255, b_i = sc->indices.size() * 4;
    char* tmp = nullptr;
    CK(cudaMalloc(&tmp, b_n + b_i + 16));
    cudaStream_t s = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(tmp, sc->normals.data(), sc->normals.size() * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && b_i) e = cudaMemcpyAsync(tmp + b_n, sc->indices.data(), b_i, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        launch_gather_normals(s, (const CwTri*)sc->tris.ptr, sc->num_triangles, (const float*)tmp,
                              b_i ? (const uint32_t*)(tmp + b_n) : nullptr, (float4*)sc->tri_normals.ptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "vertex normals");
    sc->dev.tri_normals = (const float4*)sc->tri_normals.ptr;
    return BSM_OK;
}

}  // namespace

// ================================================================ scenes ====
extern "C" bsm_status bsm_scene_upload(bsm_context* ctx, const bsm_scene_desc* d, uint32_t* scene_id) {
    if (!ctx || !d || !scene_id) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (d->num_triangles == 0 || !d->positions || d->num_vertices == 0)
        return fail(ctx, BSM_ERR_INVALID_ARG, "scene needs vertices and triangles");
    if (d->num_materials == 0 || !d->materials) return fail(ctx, BSM_ERR_INVALID_ARG, "scene needs at least one material");
    auto sc = std::make_unique<Scene>();
    sc->positions.assign(d->positions, d->positions + 3 * (size_t)d->num_vertices);
    if (d->indices) {
        sc->indices.assign(d->indices, d->indices + 3 * (size_t)d->num_triangles);
        for (uint32_t x : sc->indices)
            if (x >= d->num_vertices) return fail(ctx, BSM_ERR_INVALID_ARG, "vertex index out of range");
    } else if ((size_t)d->num_vertices < 3 * (size_t)d->num_triangles) {
        return fail(ctx, BSM_ERR_INVALID_ARG, "triangle soup needs 3 vertices per triangle");
    }
    if (d->material_ids) {
        sc->material_ids.assign(d->material_ids, d->material_ids + d->num_triangles);
        for (uint32_t m : sc->material_ids)
            if (m >= d->num_materials) return fail(ctx, BSM_ERR_INVALID_ARG, "material id out of range");
    }
    sc->num_triangles = d->num_triangles;
    if (d->normals) {
        sc->normals.assign(d->normals, d->normals + 3 * (size_t)d->num_vertices);
        for (float x : sc->normals)
            if (!std::isfinite(x)) return fail(ctx, BSM_ERR_INVALID_ARG, "non-finite vertex normal");
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < (size_t)d->num_vertices; ++i)
        for (int k = 0; k < 3; ++k) {
            float p = d->positions[3 * i + k];
            if (!std::isfinite(p)) return fail(ctx, BSM_ERR_INVALID_ARG, "non-finite vertex position");
            lo[k] = std::min(lo[k], p); hi[k] = std::max(hi[k], p);
        }
    bsm_status st = setup_shading(ctx, sc.get(), d->materials, d->num_materials, d->dir_lights, d->num_dir_lights,
                                  d->point_lights, d->num_point_lights, d->rect_lights, d->num_rect_lights, d->sky, lo,
                                  hi);
    if (st) { free_scene_buffers(ctx, *sc); return st; }
    DevScene& ds = sc->dev;
    ds.has_non_opaque = 0;
    for (uint32_t t = 0; t < d->num_triangles; ++t)
        if (sc->transparency[d->material_ids ? d->material_ids[t] : 0] != 0.0f) { ds.has_non_opaque = 1; break; }
    if (ctx->server) {
        free_scene_buffers(ctx, *sc);
        return fail(ctx, BSM_ERR_BAD_STATE, "scenes cannot change while the server runs");
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    uint32_t id = ctx->next_scene++;
    ctx->scenes[id] = std::move(sc);
    *scene_id = id;
    return BSM_OK;
}

extern "C" bsm_status bsm_scene_build_bvh(bsm_context* ctx, uint32_t scene_id, const bsm_bvh_opts* opts,
                                          bsm_bvh_stats* stats) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene id");
    if (ctx->server) return fail(ctx, BSM_ERR_BAD_STATE, "scenes cannot change while the server runs");
    if (sc->instanced) {  // a full rebuild of the TLAS from the current transforms
        cudaStreamSynchronize(WS(ctx));
        bsm_status st = build_tlas(ctx, sc);
        if (!st && stats) *stats = sc->bvh_stats;
        return st;
    }
    if (opts && opts->builder > BSM_BUILD_HOST) return fail(ctx, BSM_ERR_INVALID_ARG, "unknown BVH builder");
    if (!use_host_builder(opts)) {
        bsm_bvh_stats s{};
        bsm_status st = device_bvh(ctx, sc->positions.data(), (uint32_t)(sc->positions.size() / 3),
                                   sc->indices.empty() ? nullptr : sc->indices.data(), sc->num_triangles,
                                   sc->material_ids.empty() ? nullptr : sc->material_ids.data(), sc->transparency,
                                   opts, sc->nodes, sc->tris, s);
        if (st) return st;
        sc->dev.nodes = (const CwNode*)sc->nodes.ptr;
        sc->dev.tris = (const CwTri*)sc->tris.ptr;
        if ((st = make_tri_normals(ctx, sc))) return st;
        sc->has_bvh = true;
        sc->bvh_stats = s;
        clear_graphs(ctx);
        if (stats) *stats = s;
        return BSM_OK;
    }
    BvhBuildResult r;
    std::string err;
    if (!build_cwbvh(sc->positions.data(), sc->indices.empty() ? nullptr : sc->indices.data(), sc->num_triangles,
                     sc->material_ids.empty() ? nullptr : sc->material_ids.data(), opts, r, err))
        return fail(ctx, BSM_ERR_INVALID_ARG, "BVH build failed: " + err);
    if (r.max_depth > (uint32_t)kMaxTraversalDepth)
        return fail(ctx, BSM_ERR_UNSUPPORTED, "BVH deeper than the traversal stack (" + std::to_string(r.max_depth) + ")");
    for (CwTri& t : r.tris) {  // the any-hit rule's operand rides in the spare word
        float tr = t.material < sc->transparency.size() ? sc->transparency[t.material] : 0.0f;
        std::memcpy(&t.pad, &tr, 4);
    }
    bsm_status st;
    dev_free(ctx, sc->nodes);
    dev_free(ctx, sc->tris);
    if ((st = dev_alloc(ctx, sc->nodes, r.nodes.size() * sizeof(CwNode)))) return st;
    if ((st = dev_alloc(ctx, sc->tris, r.tris.size() * sizeof(CwTri)))) return st;
    CK(cudaMemcpy(sc->nodes.ptr, r.nodes.data(), r.nodes.size() * sizeof(CwNode), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sc->tris.ptr, r.tris.data(), r.tris.size() * sizeof(CwTri), cudaMemcpyHostToDevice));
    sc->dev.nodes = (const CwNode*)sc->nodes.ptr;
    sc->dev.tris = (const CwTri*)sc->tris.ptr;
    if ((st = make_tri_normals(ctx, sc))) return st;
    sc->has_bvh = true;
    bsm_bvh_stats s{};
    s.num_nodes = (uint32_t)r.nodes.size();
    s.num_tris = (uint32_t)r.tris.size();
    s.max_depth = r.max_depth;
    s.builder = BSM_BUILD_HOST;
    s.build_ms = r.build_ms;
    s.sah_cost = r.sah_cost;
    s.node_bytes = r.nodes.size() * sizeof(CwNode);
    s.tri_bytes = r.tris.size() * sizeof(CwTri);
    sc->bvh_stats = s;
    clear_graphs(ctx);
    if (stats) *stats = s;
    return BSM_OK;
}

extern "C" bsm_status bsm_bvh_build_host(const bsm_scene_desc* d, const bsm_bvh_opts* opts, void* nodes,
                                         uint64_t nodes_bytes, void* tris, uint64_t tris_bytes,
                                         bsm_bvh_stats* stats) {
    if (!d || !stats || !d->positions || d->num_triangles == 0) return BSM_ERR_INVALID_ARG;
    if (d->indices)
        for (size_t i = 0; i < 3 * (size_t)d->num_triangles; ++i)
            if (d->indices[i] >= d->num_vertices) return BSM_ERR_INVALID_ARG;
    BvhBuildResult r;
    std::string err;
    if (!build_cwbvh(d->positions, d->indices, d->num_triangles, d->material_ids, opts, r, err))
        return BSM_ERR_INVALID_ARG;
    bsm_bvh_stats s{};
    s.num_nodes = (uint32_t)r.nodes.size();
    s.num_tris = (uint32_t)r.tris.size();
    s.max_depth = r.max_depth;
    s.builder = BSM_BUILD_HOST;
    s.build_ms = r.build_ms;
    s.sah_cost = r.sah_cost;
    s.node_bytes = r.nodes.size() * sizeof(CwNode);
    s.tri_bytes = r.tris.size() * sizeof(CwTri);
    *stats = s;
    if (nodes) {
        if (nodes_bytes < s.node_bytes) return BSM_ERR_INVALID_ARG;
        std::memcpy(nodes, r.nodes.data(), s.node_bytes);
    }
    if (tris) {
        if (tris_bytes < s.tri_bytes) return BSM_ERR_INVALID_ARG;
        std::memcpy(tris, r.tris.data(), s.tri_bytes);
    }
    return BSM_OK;
}

extern "C" bsm_status bsm_scene_release(bsm_context* ctx, uint32_t scene_id) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene id");
    if (ctx->server) return fail(ctx, BSM_ERR_BAD_STATE, "scenes cannot change while the server runs");
    cudaStreamSynchronize(WS(ctx));
    free_scene_buffers(ctx, *sc);
    ctx->scenes.erase(scene_id);
    clear_graphs(ctx);
    return BSM_OK;
}

// ============================================================ instancing ====
namespace {

// Object-to-world (row-major 3x4) -> world-to-object: the inverse in double
// (cofactors, determinant along the first row), rounded to float.  The oracle
// evaluates the same expressions in the same order.
bool invert_affine(const float* m, float* inv) {
    double L00 = m[0], L01 = m[1], L02 = m[2], t0 = m[3];
    double L10 = m[4], L11 = m[5], L12 = m[6], t1 = m[7];
    double L20 = m[8], L21 = m[9], L22 = m[10], t2 = m[11];
    double c00 = L11 * L22 - L12 * L21, c01 = L02 * L21 - L01 * L22, c02 = L01 * L12 - L02 * L11;
    double c10 = L12 * L20 - L10 * L22, c11 = L00 * L22 - L02 * L20, c12 = L02 * L10 - L00 * L12;
    double c20 = L10 * L21 - L11 * L20, c21 = L01 * L20 - L00 * L21, c22 = L00 * L11 - L01 * L10;
    double det = L00 * c00 + L01 * c10 + L02 * c20;
    if (!std::isfinite(det) || !(std::fabs(det) > 1e-30)) return false;
    double r[9] = {c00 / det, c01 / det, c02 / det, c10 / det, c11 / det, c12 / det, c20 / det, c21 / det, c22 / det};
    for (int i = 0; i < 3; ++i) {
        inv[4 * i] = (float)r[3 * i];
        inv[4 * i + 1] = (float)r[3 * i + 1];
        inv[4 * i + 2] = (float)r[3 * i + 2];
        inv[4 * i + 3] = (float)(-(r[3 * i] * t0 + r[3 * i + 1] * t1 + r[3 * i + 2] * t2));
    }
    return true;
}

// World box of an instance: the eight transformed corners of the geometry's
// box in double, padded by 1e-5 of the coordinates' magnitude (more than the
// rounding of the float ray transform) and rounded outward to float.
void instance_world_box(const float* m, const float glo[3], const float ghi[3], float lo[3], float hi[3]) {
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
        double p[3] = {(c & 1) ? ghi[0] : glo[0], (c & 2) ? ghi[1] : glo[1], (c & 4) ? ghi[2] : glo[2]};
        for (int k = 0; k < 3; ++k) {
            double w = (double)m[4 * k] * p[0] + (double)m[4 * k + 1] * p[1] + (double)m[4 * k + 2] * p[2] +
                       (double)m[4 * k + 3];
            mn[k] = std::min(mn[k], w);
            mx[k] = std::max(mx[k], w);
        }
    }
    double mag = 0.0;
    for (int k = 0; k < 3; ++k) mag = std::max(mag, std::max(std::fabs(mn[k]), std::fabs(mx[k])));
    double pad = 1e-5 * mag + 1e-30;
    for (int k = 0; k < 3; ++k) {
        float l = (float)(mn[k] - pad), h = (float)(mx[k] + pad);
        while ((double)l > mn[k] - pad) l = std::nextafter(l, -INFINITY);
        while ((double)h < mx[k] + pad) h = std::nextafter(h, INFINITY);
        lo[k] = l;
        hi[k] = h;
    }
}

bool valid_transform(const float* m) {
    for (int i = 0; i < 12; ++i)
        if (!std::isfinite(m[i])) return false;
    float inv[12];
    return invert_affine(m, inv);
}

// Instance records (w2o, o2w, BLAS pointers) and world boxes of every instance, in leaf order.
void fill_instances(bsm_context* ctx, Scene* sc, std::vector<float>& boxes) {
    const uint32_t n = (uint32_t)sc->instances.size();
    sc->inst_host.resize(n);
    boxes.assign(6 * (size_t)n, 0.0f);
    uint32_t prim_base = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const bsm_instance& in = sc->instances[i];
        Geometry* g = ctx->geoms.at(in.geometry_id).get();
        uint32_t leaf = sc->leaf_of[i];
        InstDev& r = sc->inst_host[leaf];
        std::memcpy(r.o2w, in.transform, sizeof(r.o2w));
        invert_affine(in.transform, r.w2o);
        r.nodes = (const CwNode*)g->nodes.ptr;
        r.tris = (const CwTri*)g->tris.ptr;
        r.prim_base = prim_base;
        r.material = in.material_id;
        r.id = i;
        r.pad = 0;
        prim_base += g->num_triangles;
        instance_world_box(in.transform, g->lo, g->hi, &boxes[6 * (size_t)leaf], &boxes[6 * (size_t)leaf + 3]);
    }
}

// Builds the TLAS of an instanced scene from its instances' current world boxes
// (the same SAH builder, one instance per leaf) and uploads it with the records.
bsm_status build_tlas(bsm_context* ctx, Scene* sc) {
    const uint32_t n = (uint32_t)sc->instances.size();
    std::vector<float> corners(6 * (size_t)n);
    std::vector<uint32_t> idx(3 * (size_t)n);
    sc->leaf_of.assign(n, 0);
    for (uint32_t i = 0; i < n; ++i) {
        const bsm_instance& in = sc->instances[i];
        Geometry* g = ctx->geoms.at(in.geometry_id).get();
        instance_world_box(in.transform, g->lo, g->hi, &corners[6 * (size_t)i], &corners[6 * (size_t)i + 3]);
        idx[3 * i] = 2 * i; idx[3 * i + 1] = 2 * i + 1; idx[3 * i + 2] = 2 * i;  // a "triangle" spanning the box
    }
    bsm_bvh_opts opts{};
    opts.max_leaf_tris = 1;
    BvhBuildResult r;
    std::string err;
    if (!build_cwbvh(corners.data(), idx.data(), n, nullptr, &opts, r, err))
        return fail(ctx, BSM_ERR_INVALID_ARG, "TLAS build failed: " + err);
    if (r.max_depth > (uint32_t)kMaxTlasDepth)
        return fail(ctx, BSM_ERR_UNSUPPORTED, "TLAS deeper than " + std::to_string(kMaxTlasDepth) + " levels");
    for (uint32_t l = 0; l < n; ++l) sc->leaf_of[r.tris[l].prim] = l;
    // breadth-first levels: nodes are emitted in BFS order, so each level is a contiguous range
    std::vector<uint32_t> depth(r.nodes.size(), 0);
    for (uint32_t ni = 0; ni < r.nodes.size(); ++ni) {
        const CwNode& nd = r.nodes[ni];
        uint32_t k = 0;
        for (int s = 0; s < 8; ++s)
            if (nd.imask & (1u << s)) depth[nd.child_base + k++] = depth[ni] + 1;
    }
    sc->level_begin.clear();
    for (uint32_t ni = 0; ni < r.nodes.size(); ++ni)
        if (ni == 0 || depth[ni] != depth[ni - 1]) sc->level_begin.push_back(ni);
    sc->level_begin.push_back((uint32_t)r.nodes.size());
    std::vector<float> boxes;
    fill_instances(ctx, sc, boxes);
    bsm_status st;
    dev_free(ctx, sc->nodes);
    if ((st = dev_alloc(ctx, sc->nodes, r.nodes.size() * sizeof(CwNode)))) return st;
    if ((st = dev_alloc(ctx, sc->insts, (size_t)n * sizeof(InstDev)))) return st;
    if ((st = dev_alloc(ctx, sc->inst_box, boxes.size() * 4))) return st;
    if ((st = dev_alloc(ctx, sc->node_box, r.nodes.size() * 6 * 4))) return st;
    CK(cudaMemcpy(sc->nodes.ptr, r.nodes.data(), r.nodes.size() * sizeof(CwNode), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sc->insts.ptr, sc->inst_host.data(), (size_t)n * sizeof(InstDev), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sc->inst_box.ptr, boxes.data(), boxes.size() * 4, cudaMemcpyHostToDevice));
    DevScene& ds = sc->dev;
    ds.nodes = (const CwNode*)sc->nodes.ptr;
    ds.tris = nullptr;
    ds.insts = (const InstDev*)sc->insts.ptr;
    ds.num_instances = n;
    bsm_bvh_stats bs{};
    bs.num_nodes = (uint32_t)r.nodes.size();
    bs.num_tris = n;
    bs.max_depth = r.max_depth;
    bs.build_ms = r.build_ms;
    bs.sah_cost = r.sah_cost;
    bs.node_bytes = r.nodes.size() * sizeof(CwNode);
    bs.tri_bytes = (uint64_t)n * sizeof(InstDev);
    sc->bvh_stats = bs;
    sc->has_bvh = true;
    clear_graphs(ctx);
    return BSM_OK;
}

}  // namespace

extern "C" bsm_status bsm_geometry_create(bsm_context* ctx, const bsm_geometry_desc* d, const bsm_bvh_opts* opts,
                                          uint32_t* geometry_id) {
    if (!ctx || !d || !geometry_id) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (d->num_triangles == 0 || !d->positions || d->num_vertices == 0)
        return fail(ctx, BSM_ERR_INVALID_ARG, "geometry needs vertices and triangles");
    if (d->indices) {
        for (size_t i = 0; i < 3 * (size_t)d->num_triangles; ++i)
            if (d->indices[i] >= d->num_vertices) return fail(ctx, BSM_ERR_INVALID_ARG, "vertex index out of range");
    } else if ((size_t)d->num_vertices < 3 * (size_t)d->num_triangles) {
        return fail(ctx, BSM_ERR_INVALID_ARG, "triangle soup needs 3 vertices per triangle");
    }
    auto g = std::make_unique<Geometry>();
    for (int k = 0; k < 3; ++k) { g->lo[k] = INFINITY; g->hi[k] = -INFINITY; }
    for (size_t i = 0; i < (size_t)d->num_vertices; ++i)
        for (int k = 0; k < 3; ++k) {
            float p = d->positions[3 * i + k];
            if (!std::isfinite(p)) return fail(ctx, BSM_ERR_INVALID_ARG, "non-finite vertex position");
            g->lo[k] = std::min(g->lo[k], p);
            g->hi[k] = std::max(g->hi[k], p);
        }
    if (d->material_ids)
        for (uint32_t t = 0; t < d->num_triangles; ++t) g->max_material = std::max(g->max_material, d->material_ids[t]);
    if (opts && opts->builder > BSM_BUILD_HOST) return fail(ctx, BSM_ERR_INVALID_ARG, "unknown BVH builder");
    if (!use_host_builder(opts)) {
        bsm_bvh_stats s{};
        // the two-level stack bound below holds for any BLAS within the traversal stack
        bsm_status st = device_bvh(ctx, d->positions, d->num_vertices, d->indices, d->num_triangles, d->material_ids,
                                   std::vector<float>(), opts, g->nodes, g->tris, s);
        if (st) return st;
        g->num_triangles = d->num_triangles;
        std::lock_guard<std::mutex> lk(ctx->mu);
        uint32_t id = ctx->next_geom++;
        ctx->geoms[id] = std::move(g);
        *geometry_id = id;
        return BSM_OK;
    }
    BvhBuildResult r;
    std::string err;
    if (!build_cwbvh(d->positions, d->indices, d->num_triangles, d->material_ids, opts, r, err))
        return fail(ctx, BSM_ERR_INVALID_ARG, "BVH build failed: " + err);
    // two-level stack: (TLAS depth - 1) + 3 transition entries + (BLAS depth - 1) <= 11 + 3 + 23 < kStackSize
    if (r.max_depth > (uint32_t)kMaxTraversalDepth)
        return fail(ctx, BSM_ERR_UNSUPPORTED, "geometry BVH deeper than the traversal stack");
    bsm_status st;
    if ((st = dev_alloc(ctx, g->nodes, r.nodes.size() * sizeof(CwNode)))) return st;
    if ((st = dev_alloc(ctx, g->tris, r.tris.size() * sizeof(CwTri)))) { dev_free(ctx, g->nodes); return st; }
    CK(cudaMemcpy(g->nodes.ptr, r.nodes.data(), r.nodes.size() * sizeof(CwNode), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g->tris.ptr, r.tris.data(), r.tris.size() * sizeof(CwTri), cudaMemcpyHostToDevice));
    g->num_triangles = d->num_triangles;
    std::lock_guard<std::mutex> lk(ctx->mu);
    uint32_t id = ctx->next_geom++;
    ctx->geoms[id] = std::move(g);
    *geometry_id = id;
    return BSM_OK;
}

extern "C" bsm_status bsm_geometry_release(bsm_context* ctx, uint32_t geometry_id) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    auto it = ctx->geoms.find(geometry_id);
    if (it == ctx->geoms.end()) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown geometry id");
    if (it->second->users) return fail(ctx, BSM_ERR_BAD_STATE, "geometry is instanced by a scene");
    cudaSetDevice(ctx->device);
    dev_free(ctx, it->second->nodes);
    dev_free(ctx, it->second->tris);
    ctx->geoms.erase(it);
    return BSM_OK;
}

extern "C" bsm_status bsm_scene_create_instanced(bsm_context* ctx, const bsm_instanced_scene_desc* d,
                                                 uint32_t* scene_id) {
    if (!ctx || !d || !scene_id) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->server) return fail(ctx, BSM_ERR_BAD_STATE, "scenes cannot change while the server runs");
    if (d->num_instances == 0 || !d->instances) return fail(ctx, BSM_ERR_INVALID_ARG, "scene needs instances");
    uint64_t total = 0;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < d->num_instances; ++i) {
        const bsm_instance& in = d->instances[i];
        auto it = ctx->geoms.find(in.geometry_id);
        if (it == ctx->geoms.end()) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown geometry id in instance " + std::to_string(i));
        if (in.material_id != kMissPrim ? in.material_id >= d->num_materials : it->second->max_material >= d->num_materials)
            return fail(ctx, BSM_ERR_INVALID_ARG, "material id out of range in instance " + std::to_string(i));
        if (!valid_transform(in.transform))
            return fail(ctx, BSM_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": transform not finite / invertible");
        total += it->second->num_triangles;
        float bl[3], bh[3];
        instance_world_box(in.transform, it->second->lo, it->second->hi, bl, bh);
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], bl[k]); hi[k] = std::max(hi[k], bh[k]); }
    }
    if (total >= 0xffffffffull) return fail(ctx, BSM_ERR_INVALID_ARG, "more than 2^32 - 1 instanced triangles");
    auto sc = std::make_unique<Scene>();
    sc->instanced = true;
    sc->instances.assign(d->instances, d->instances + d->num_instances);
    sc->num_triangles = (uint32_t)total;
    for (const bsm_instance& in : sc->instances) ctx->geoms[in.geometry_id]->users++;
    bsm_status st = setup_shading(ctx, sc.get(), d->materials, d->num_materials, d->dir_lights, d->num_dir_lights,
                                  d->point_lights, d->num_point_lights, d->rect_lights, d->num_rect_lights, d->sky, lo,
                                  hi);
    if (!st) {
        bool any = false;
        for (float t : sc->transparency) any = any || t != 0.0f;
        sc->dev.has_non_opaque = any ? 1u : 0u;
        sc->dev.mat_tr = nullptr;
        if (any) {
            st = dev_alloc(ctx, sc->mat_tr, sc->transparency.size() * 4);
            if (!st && cudaMemcpy(sc->mat_tr.ptr, sc->transparency.data(), sc->transparency.size() * 4,
                                  cudaMemcpyHostToDevice) != cudaSuccess)
                st = fail(ctx, BSM_ERR_CUDA, "material upload failed");
            sc->dev.mat_tr = (const float*)sc->mat_tr.ptr;
        }
    }
    if (!st) st = build_tlas(ctx, sc.get());
    if (st) { free_scene_buffers(ctx, *sc); return st; }
    std::lock_guard<std::mutex> lk(ctx->mu);
    uint32_t id = ctx->next_scene++;
    ctx->scenes[id] = std::move(sc);
    *scene_id = id;
    return BSM_OK;
}

extern "C" bsm_status bsm_scene_update_instances(bsm_context* ctx, uint32_t scene_id, const float* transforms,
                                                 uint32_t num_instances) {
    if (!ctx || !transforms) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene id");
    if (!sc->instanced) return fail(ctx, BSM_ERR_BAD_STATE, "not an instanced scene");
    if (ctx->server) return fail(ctx, BSM_ERR_BAD_STATE, "scenes cannot change while the server runs");
    if (num_instances != sc->instances.size())
        return fail(ctx, BSM_ERR_INVALID_ARG, "transform count differs from the scene's instances");
    for (uint32_t i = 0; i < num_instances; ++i)
        if (!valid_transform(transforms + 12 * (size_t)i))
            return fail(ctx, BSM_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": transform not finite / invertible");
    for (uint32_t i = 0; i < num_instances; ++i)
        std::memcpy(sc->instances[i].transform, transforms + 12 * (size_t)i, 12 * sizeof(float));
    std::vector<float> boxes;
    fill_instances(ctx, sc, boxes);
    // the scene bounds (ray offset, radiance-cache normalisation) follow the instances, as a rebuild's would
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t l = 0; l < sc->inst_host.size(); ++l)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], boxes[6 * l + k]);
            hi[k] = std::max(hi[k], boxes[6 * l + 3 + k]);
        }
    float extent = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), std::max(hi[2] - lo[2], 1e-6f));
    DevScene& ds = sc->dev;
    bool moved_bounds = extent != sc->extent;
    for (int k = 0; k < 3; ++k)
        moved_bounds = moved_bounds || ds.box_lo[k] != lo[k] || ds.box_inv[k] != 1.0f / std::max(hi[k] - lo[k], 1e-6f);
    CK(cudaStreamSynchronize(WS(ctx)));  // no render may read the records while they change
    if (moved_bounds) {
        sc->extent = extent;
        ds.ray_offset = 2e-5f * extent;
        for (int k = 0; k < 3; ++k) {
            ds.box_lo[k] = lo[k];
            ds.box_inv[k] = 1.0f / std::max(hi[k] - lo[k], 1e-6f);
        }
        clear_graphs(ctx);  // captured launches hold the scene record by value
    }
    CK(cudaMemcpyAsync(sc->insts.ptr, sc->inst_host.data(), sc->inst_host.size() * sizeof(InstDev),
                       cudaMemcpyHostToDevice, WS(ctx)));
    CK(cudaMemcpyAsync(sc->inst_box.ptr, boxes.data(), boxes.size() * 4, cudaMemcpyHostToDevice, WS(ctx)));
    // refit bottom-up: one launch per breadth-first level, deepest first
    for (size_t lv = sc->level_begin.size() - 1; lv-- > 0;)
        launch_tlas_refit(WS(ctx), (CwNode*)sc->nodes.ptr, (float*)sc->node_box.ptr, (const float*)sc->inst_box.ptr,
                          sc->level_begin[lv], sc->level_begin[lv + 1]);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(WS(ctx)));
    return BSM_OK;
}

extern "C" bsm_status bsm_scene_device_bytes(bsm_context* ctx, uint32_t scene_id, uint64_t* bytes) {
    if (!ctx || !bytes) return BSM_ERR_INVALID_ARG;
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene id");
    uint64_t b = 0;
    for (DevBuf* x : {&sc->nodes, &sc->tris, &sc->materials, &sc->texels, &sc->sky_alias, &sc->pdf_tab,
                      &sc->tri_normals, &sc->insts, &sc->inst_box, &sc->node_box, &sc->mat_tr})
        b += x->bytes;
    *bytes = b;
    return BSM_OK;
}

extern "C" bsm_status bsm_scene_download_bvh(bsm_context* ctx, uint32_t scene_id, void* nodes, void* tris) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc || !sc->has_bvh) return fail(ctx, BSM_ERR_NOT_FOUND, "scene has no BVH");
    if (nodes) CK(cudaMemcpy(nodes, sc->nodes.ptr, sc->bvh_stats.node_bytes, cudaMemcpyDeviceToHost));
    if (tris) {  // a two-level scene's leaves are its instance records (InstDev, leaf order)
        const void* src = sc->instanced ? sc->insts.ptr : sc->tris.ptr;
        CK(cudaMemcpy(tris, src, sc->bvh_stats.tri_bytes, cudaMemcpyDeviceToHost));
    }
    return BSM_OK;
}

// =============================================================== render ====
extern "C" void bsm_pt_settings_default(bsm_pt_settings* s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    s->ray_length = 100.0f;
    s->max_bounces = 3;
    s->accumulate = 1;
    s->denoise = 1;
    s->spp = 1;
    s->seed = 1;
}

namespace {

// Records the launch sequence of one render (all chunks) on `st` (the capture
// stream when a graph is being recorded, else the work stream).
// With `ev` non-null an event is recorded after every launch (no host waits):
// ev[0] before the first launch, then one per stage; `tags` gets the stage of
// each interval (0 camera, 1 extend, 2 shade, 3 shadow).  With `fx_px` > 0
// (BSM_PT_DETERMINISTIC) the contributions go to fixed-point sums over the
// call's fx_px accumulator pixels, added to the FP32 accumulator at the end.
void record_render(bsm_context* ctx, cudaStream_t st, const Scene* sc, uint32_t n_views, uint64_t total_paths,
                   uint32_t capacity, uint32_t max_seg, bool count_traversal, std::vector<cudaEvent_t>* ev,
                   std::vector<int>* tags, const void* cache_wb = nullptr, uint32_t fx_px = 0) {
    const LaunchCfg& lc = ctx->lc;
    const DevView* views = (const DevView*)ctx->views_dev.ptr;
    float4* accum = (float4*)ctx->accum.ptr;
    Wavefront wf = ctx->wf;
    wf.accum_fx = fx_px ? (unsigned long long*)ctx->accum_fx.ptr : nullptr;
    if (fx_px) cudaMemsetAsync(wf.accum_fx, 0, (size_t)fx_px * 24, st);
    size_t k = 0;
    auto mark = [&](int tag) {
        if (!ev) return;
        if (k >= ev->size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev->push_back(e);
        }
        cudaEventRecord((*ev)[k++], st);
        if (tag >= 0) tags->push_back(tag);
    };
    mark(-1);
    for (uint64_t begin = 0; begin < total_paths; begin += capacity) {
        uint32_t count = (uint32_t)std::min<uint64_t>(capacity, total_paths - begin);
        cudaMemsetAsync(wf.counters, 0, kCntError * 4, st);
        launch_camera(lc, st, views, n_views, begin, count, wf, max_seg);
        mark(0);
        int q = 0;
        for (uint32_t seg = 0; seg < max_seg; ++seg) {
            launch_extend(lc, st, sc->dev, wf, q, seg, count_traversal);
            mark(1);
            launch_shade(lc, st, sc->dev, views, wf, q, seg, accum, cache_wb != nullptr);
            mark(2);
            launch_shadow(lc, st, sc->dev, wf, seg, accum);
            mark(3);
            q ^= 1;
        }
        if (cache_wb)
            launch_mlp_infer(ctx->device, st, cache_wb, wf.cache_q, wf.counters + kCntCache, capacity, accum,
                             wf.accum_fx, wf.counters + kCntError);
    }
    if (fx_px) launch_fold_fixed(st, wf.accum_fx, accum, fx_px);
}

}  // namespace

namespace {

// Statistics of the last render issued on the context, once its work is done:
// the host-side part kept at issue time plus the device's ray counters and the
// device time between the render's two events.
bsm_status read_last_stats(bsm_context* ctx, bsm_render_stats* out) {
    CK(cudaEventSynchronize(ctx->ev[9]));
    unsigned long long h[kStatWords];
    CK(cudaMemcpyAsync(h, ctx->wf.stats, sizeof(h), cudaMemcpyDeviceToHost, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    *out = ctx->last_stats;
    out->extend_rays = out->shadow_rays = 0;
    for (uint32_t k = 0; k < (uint32_t)kMaxSeg; ++k) {
        out->rays_per_segment[k] = h[kStatExtend + k];
        out->extend_rays += h[kStatExtend + k];
        out->shadow_rays += h[kStatShadow + k];
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ctx->ev[8], ctx->ev[9]);
    out->ms_total = ms;
    out->traversal_nodes = h[kStatNodes];
    out->traversal_tris = h[kStatTris];
    return BSM_OK;
}

// One view of a render call: camera plus the per-view sample count, segment
// limit and seed (uniform for bsm_render, per view for bsm_render_batch).
struct ViewReq {
    bsm_camera cam;
    uint32_t spp;
    uint32_t max_seg;
    uint64_t seed;
};

bsm_status render_impl(bsm_context* ctx, uint32_t scene_id, const std::vector<ViewReq>& req,
                       const bsm_pt_settings& s, const bsm_view_output* outputs, bsm_render_stats* stats,
                       const void* cache_wb = nullptr, uint32_t cache_seg = 0, float cache_rough = 0.0f,
                       bool start_recorded = false) {
    const uint32_t n_views = (uint32_t)req.size();
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene id");
    if (!sc->has_bvh) return fail(ctx, BSM_ERR_BAD_STATE, "scene BVH not built (bsm_scene_build_bvh)");
    uint32_t max_seg = 0;
    for (const ViewReq& r : req) {
        if (r.spp == 0) return fail(ctx, BSM_ERR_INVALID_ARG, "spp must be >= 1");
        if (r.max_seg == 0 || r.max_seg > (uint32_t)kMaxSeg)
            return fail(ctx, BSM_ERR_INVALID_ARG, "max_segments must be 1..16");
        max_seg = std::max(max_seg, r.max_seg);
    }
    if (!(s.ray_length > 0.0f)) return fail(ctx, BSM_ERR_INVALID_ARG, "ray_length must be > 0");
    if (s.t_min < 0.0f) return fail(ctx, BSM_ERR_INVALID_ARG, "t_min must be >= 0");
    bsm_status st;
    if ((st = prepare_launch(ctx, sc, s))) return st;
    const bsm_camera* views = nullptr;
    std::vector<bsm_camera> cams(n_views);
    for (uint32_t v = 0; v < n_views; ++v) cams[v] = req[v].cam;
    views = cams.data();

    // view layout and history (path_tracing.cpp:231-245: history kept per camera,
    // reset when it moves or the target changes size)
    bool relayout = ctx->layout.size() != n_views;
    for (uint32_t v = 0; v < n_views && !relayout; ++v)
        relayout = ctx->layout[v].first != views[v].width || ctx->layout[v].second != views[v].height;
    uint64_t total_px = 0;
    for (uint32_t v = 0; v < n_views; ++v) {
        if (const char* why = camera_problem(views[v])) return fail(ctx, BSM_ERR_INVALID_ARG, why);
        total_px += (uint64_t)views[v].width * views[v].height;
    }
    if (total_px >= (1ull << 32)) return fail(ctx, BSM_ERR_INVALID_ARG, "too many pixels in one call");
    if (n_views > 65535) return fail(ctx, BSM_ERR_INVALID_ARG, "at most 65535 views per call");
    if (relayout) {
        cudaStreamSynchronize(WS(ctx));
        clear_graphs(ctx);
        if ((st = dev_alloc(ctx, ctx->accum, total_px * sizeof(float4)))) return st;
        CK(cudaMemsetAsync(ctx->accum.ptr, 0, total_px * sizeof(float4), WS(ctx)));
        ctx->layout.assign(n_views, {0, 0});
        ctx->hist.assign(n_views, ViewHist{});
        uint32_t base = 0;
        for (uint32_t v = 0; v < n_views; ++v) {
            ctx->layout[v] = {views[v].width, views[v].height};
            ctx->hist[v].accum_base = base;
            base += views[v].width * views[v].height;
        }
    }
    ctx->views_host.resize(n_views);
    uint64_t total_paths = 0;
    for (uint32_t v = 0; v < n_views; ++v) {
        ViewHist& h = ctx->hist[v];
        bool reset = !s.accumulate || !h.valid || !same_camera(h.cam, views[v]);
        if (reset) {
            CK(cudaMemsetAsync((float4*)ctx->accum.ptr + h.accum_base, 0,
                               (size_t)views[v].width * views[v].height * sizeof(float4), WS(ctx)));
            h.spp = 0;
            h.cam = views[v];
            h.valid = true;
        }
        DevView& dv = ctx->views_host[v];
        std::memset(&dv, 0, sizeof(dv));
        make_view(views[v], dv);
        dv.ray_length = s.ray_length;
        dv.t_min = s.t_min;
        dv.spp = req[v].spp;
        dv.sample_offset = s.sample_offset + h.spp;
        dv.seed = req[v].seed;
        dv.path_base = total_paths;
        dv.accum_base = h.accum_base;
        dv.max_segments = req[v].max_seg;
        dv.flags = s.flags;
        dv.cache_segment = cache_wb ? cache_seg : 0u;
        dv.cache_min_rough = cache_wb ? cache_rough : 0.0f;
        total_paths += (uint64_t)views[v].width * views[v].height * req[v].spp;
    }
    uint32_t cap_req = s.wavefront_capacity ? s.wavefront_capacity : (sc->tuned ? sc->tune.wavefront_capacity : 0u);
    uint32_t capacity = cap_req ? cap_req : default_capacity(ctx, total_paths, std::max(sc->dev.num_lights, 1u));
    capacity = std::max(capacity, 1024u);
    if ((st = ensure_wavefront(ctx, capacity, std::max(sc->dev.num_lights, 1u)))) return st;
    capacity = std::min(capacity, ctx->wf.capacity);
    if ((st = dev_alloc(ctx, ctx->views_dev, n_views * sizeof(DevView)))) return st;
    CK(cudaMemcpyAsync(ctx->views_dev.ptr, ctx->views_host.data(), n_views * sizeof(DevView), cudaMemcpyHostToDevice,
                       WS(ctx)));
    CK(cudaMemsetAsync(ctx->wf.stats, 0, kStatWords * 8, WS(ctx)));

    bool timing = (s.flags & BSM_PT_STAGE_TIMING) != 0;
    bool counting = (s.flags & BSM_PT_COUNT_TRAVERSAL) != 0;
    bool use_graph = !timing && !counting && !(s.flags & BSM_PT_NO_GRAPH);
    const uint32_t fx_px = (s.flags & BSM_PT_DETERMINISTIC) ? (uint32_t)total_px : 0u;
    if (fx_px && ctx->accum_fx.bytes < (size_t)fx_px * 24) {
        cudaStreamSynchronize(WS(ctx));   // earlier renders may still add to the old sums
        clear_graphs(ctx);
        if ((st = dev_alloc(ctx, ctx->accum_fx, (size_t)fx_px * 24))) return st;
    }
    float stage_ms[4] = {0, 0, 0, 0};
    std::vector<int> tags;
    if (!start_recorded) CK(cudaEventRecord(ctx->ev[8], WS(ctx)));   // start of the device time of this render
    if (use_graph) {
        // key: everything the recorded launches depend on
        std::vector<uint8_t> key(72);
        uint64_t kv[9] = {(uint64_t)scene_id, (uint64_t)n_views, total_paths,
                          capacity | ((uint64_t)ctx->lc.postpone_sp << 32) | ((uint64_t)ctx->lc.refill_min << 40),
                          max_seg | ((uint64_t)(uintptr_t)cache_wb << 8), (uint64_t)(uintptr_t)ctx->wf_buf.ptr,
                          (uint64_t)(uintptr_t)ctx->accum.ptr,
                          (uint64_t)(uintptr_t)ctx->views_dev.ptr ^ ((uint64_t)ctx->lc_block << 56),
                          fx_px ? (uint64_t)(uintptr_t)ctx->accum_fx.ptr : 0u};
        std::memcpy(key.data(), kv, 72);
        cudaGraphExec_t exec = nullptr;
        for (auto& g : ctx->graphs) if (g.key == key) exec = g.exec;
        if (!exec) {
            cudaGraph_t graph;
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            record_render(ctx, ctx->stream, sc, n_views, total_paths, capacity, max_seg, false, nullptr, nullptr,
                          cache_wb, fx_px);
            CK(cudaStreamEndCapture(ctx->stream, &graph));
            CK(cudaGraphInstantiate(&exec, graph, 0));
            cudaGraphDestroy(graph);
            if (ctx->graphs.size() >= 16) {
                cudaGraphExecDestroy(ctx->graphs.front().exec);
                ctx->graphs.erase(ctx->graphs.begin());
            }
            ctx->graphs.push_back({exec, key});
        }
        CK(cudaGraphLaunch(exec, WS(ctx)));
    } else {
        record_render(ctx, WS(ctx), sc, n_views, total_paths, capacity, max_seg, counting,
                      timing ? &ctx->stage_ev : nullptr, &tags, cache_wb, fx_px);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[9], WS(ctx)));
    for (uint32_t v = 0; v < n_views; ++v) ctx->hist[v].spp += req[v].spp;

    // outputs: running mean
    bool host_out = false;
    if (outputs) {
        for (uint32_t v = 0; v < n_views; ++v) {
            const bsm_view_output& o = outputs[v];
            if (!o.rgba) continue;
            uint32_t W = views[v].width, H = views[v].height;
            uint32_t pitch = o.row_pitch_px ? o.row_pitch_px : W;
            if (pitch < W) return fail(ctx, BSM_ERR_INVALID_ARG, "row_pitch_px < width");
            float inv = 1.0f / (float)ctx->hist[v].spp;
            const float4* acc = (const float4*)ctx->accum.ptr + ctx->hist[v].accum_base;
            if (o.location == BSM_DEVICE) {
                launch_resolve(WS(ctx), acc, W, H, inv, (float4*)o.rgba, pitch);
            } else {
                if ((st = dev_alloc(ctx, ctx->out_stage, (size_t)W * H * sizeof(float4)))) return st;
                launch_resolve(WS(ctx), acc, W, H, inv, (float4*)ctx->out_stage.ptr, W);
                CK(cudaMemcpy2DAsync(o.rgba, (size_t)pitch * 16, ctx->out_stage.ptr, (size_t)W * 16, (size_t)W * 16, H,
                                     cudaMemcpyDeviceToHost, WS(ctx)));
                host_out = true;
            }
        }
        CK(cudaGetLastError());
    }
    // host-side statistics of this render; the device counts stay on the device until a read
    bsm_render_stats& ls = ctx->last_stats;
    std::memset(&ls, 0, sizeof(ls));
    ls.paths = total_paths;
    ls.chunks = (uint32_t)((total_paths + capacity - 1) / capacity);
    ls.extend_launches = ls.chunks * max_seg;
    ctx->last_stats_valid = true;
    ctx->last_stats_timing = timing;
    if (timing) {
        CK(cudaStreamSynchronize(WS(ctx)));
        for (size_t i = 0; i < tags.size(); ++i) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ctx->stage_ev[i], ctx->stage_ev[i + 1]);
            stage_ms[tags[i]] += ms;
        }
        ls.ms_camera = stage_ms[0];
        ls.ms_extend = stage_ms[1];
        ls.ms_shade = stage_ms[2];
        ls.ms_shadow = stage_ms[3];
    }
    // Device outputs and no statistics: the call returns with the work queued on the work stream
    // (bsm_sync / bsm_render_stats_read wait for it and report the device error flags).
    if (!host_out && !stats && !timing) return BSM_OK;
    if ((st = check_device_flags(ctx))) return st;
    if (stats) return read_last_stats(ctx, stats);
    return BSM_OK;
}

}  // namespace

extern "C" bsm_status bsm_render(bsm_context* ctx, uint32_t scene_id, const bsm_camera* views, uint32_t n_views,
                                 const bsm_pt_settings* settings, const bsm_view_output* outputs,
                                 bsm_render_stats* stats) {
    if (!ctx || !views || n_views == 0 || !settings) return BSM_ERR_INVALID_ARG;
    if (n_views > 65535) return fail(ctx, BSM_ERR_INVALID_ARG, "at most 65535 views per call");
    const bsm_pt_settings& s = *settings;
    uint32_t max_seg = s.max_segments ? s.max_segments : (std::min(std::max(s.max_bounces, 2u), 16u) - 1u);
    std::vector<ViewReq> req(n_views);
    for (uint32_t v = 0; v < n_views; ++v) req[v] = ViewReq{views[v], s.spp, max_seg, s.seed};
    return render_impl(ctx, scene_id, req, s, outputs, stats);
}

extern "C" bsm_status bsm_render_stats_read(bsm_context* ctx, bsm_render_stats* stats) {
    if (!ctx || !stats) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (!ctx->last_stats_valid || !ctx->wf.stats) return fail(ctx, BSM_ERR_NOT_FOUND, "no render issued yet");
    bsm_status st = check_device_flags(ctx);
    if (st) return st;
    return read_last_stats(ctx, stats);
}

extern "C" bsm_status bsm_render_cached(bsm_context* ctx, uint32_t scene_id, const bsm_camera* cam,
                                        const bsm_pt_settings* settings, bsm_cache* cache,
                                        const bsm_cache_settings* cs_in, const bsm_view_output* output,
                                        bsm_render_stats* stats, float* train_loss) {
    if (!ctx || !cam || !settings || !cache) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc || !sc->has_bvh) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene or BVH not built");
    if (cache->ctx != ctx) return fail(ctx, BSM_ERR_INVALID_ARG, "cache belongs to another context");
    if (const char* why = camera_problem(*cam)) return fail(ctx, BSM_ERR_INVALID_ARG, why);
    bsm_cache_settings cs;
    if (cs_in) cs = *cs_in; else bsm_cache_settings_default(&cs);
    if (cs.cache_segment == 0 || cs.cache_segment >= (uint32_t)kMaxSeg)
        return fail(ctx, BSM_ERR_INVALID_ARG, "cache_segment must be 1..15");
    if (train_loss) *train_loss = 0.0f;
    // the training paths' shadow pass launches with the render's configuration, which a first call on a
    // context has not set yet
    if (bsm_status e = prepare_launch(ctx, sc, *settings)) return e;
    // the frame's device time (stats->ms_total) starts before its training step
    CK(cudaEventRecord(ctx->ev[8], WS(ctx)));
    if (cs.train_steps > 0 && cs.train_paths > 0) {
        DevView dv{};
        make_view(*cam, dv);
        dv.ray_length = settings->ray_length;
        dv.t_min = settings->t_min;
        dv.seed = settings->seed;
        dv.max_segments = std::min(std::max(cs.train_segments, 1u), 16u);
        bsm_status e = cache_train_frame(cache, sc->dev, dv, cs, ctx->lc, WS(ctx), train_loss, nullptr);
        if (e) return fail(ctx, e, "radiance-cache training failed");
    }
    std::vector<ViewReq> req(1);
    if (!(cs.min_roughness >= 0.0f) || cs.cache_segment + 1 + cs.extra_segments > (uint32_t)kMaxSeg)
        return fail(ctx, BSM_ERR_INVALID_ARG, "min_roughness must be >= 0 and cache_segment + extra_segments <= 15");
    req[0] = ViewReq{*cam, settings->spp, cs.cache_segment + 1 + cs.extra_segments, settings->seed};
    return render_impl(ctx, scene_id, req, *settings, output, stats, cache_render_weights(cache), cs.cache_segment,
                       cs.extra_segments ? cs.min_roughness : 0.0f, /*start_recorded=*/true);
}

extern "C" bsm_status bsm_render_batch(bsm_context* ctx, uint32_t scene_id, const bsm_view_desc* views,
                                       uint32_t n_views, const bsm_pt_settings* settings,
                                       const bsm_view_output* outputs, bsm_render_stats* stats) {
    if (!ctx || !views || n_views == 0 || !settings) return BSM_ERR_INVALID_ARG;
    if (n_views > 65535) return fail(ctx, BSM_ERR_INVALID_ARG, "at most 65535 views per call");
    const bsm_pt_settings& s = *settings;
    uint32_t def_seg = s.max_segments ? s.max_segments : (std::min(std::max(s.max_bounces, 2u), 16u) - 1u);
    std::vector<ViewReq> req(n_views);
    for (uint32_t v = 0; v < n_views; ++v)
        req[v] = ViewReq{views[v].camera, views[v].spp ? views[v].spp : s.spp,
                         views[v].max_segments ? views[v].max_segments : def_seg, views[v].seed ? views[v].seed : s.seed};
    return render_impl(ctx, scene_id, req, s, outputs, stats);
}

// ============================================================ autotune ====
namespace {

bool valid_tune(const bsm_tune_params& p) {
    return (p.block_size == 64 || p.block_size == 128 || p.block_size == 256) &&
           (p.wavefront_capacity == 0 || p.wavefront_capacity >= 1024) && p.postpone_depth <= 16 &&
           p.refill_lanes >= 1 && p.refill_lanes <= 32 && p.register_cap <= 1;
}

std::string tune_key(bsm_context* ctx, const Scene* sc, uint64_t paths) {
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, ctx->device);
    int tri_bucket = 0, path_bucket = 0;
    for (uint64_t x = sc->num_triangles; x > 1; x >>= 1) ++tri_bucket;
    for (uint64_t x = paths; x > 1; x >>= 1) ++path_bucket;
    std::string name = prop.name;
    for (char& c : name) if (c == ' ' || c == '|') c = '_';
    return name + "|sm" + std::to_string(prop.multiProcessorCount) + "|tri2^" + std::to_string(tri_bucket) +
           "|paths2^" + std::to_string(path_bucket);
}

}  // namespace

extern "C" bsm_status bsm_set_tuning(bsm_context* ctx, uint32_t scene_id, const bsm_tune_params* p) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene id");
    if (!p) { sc->tuned = false; return BSM_OK; }
    if (!valid_tune(*p)) return fail(ctx, BSM_ERR_INVALID_ARG, "invalid tuning parameters");
    sc->tune = *p;
    sc->tuned = true;
    return BSM_OK;
}

extern "C" bsm_status bsm_autotune(bsm_context* ctx, uint32_t scene_id, const bsm_view_desc* views, uint32_t n_views,
                                   const bsm_pt_settings* settings, const char* cache_path, bsm_tune_result* result) {
    if (!ctx || !views || n_views == 0 || !settings || !result) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc || !sc->has_bvh) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene or BVH not built");
    const bsm_pt_settings& s0 = *settings;
    uint32_t def_seg = s0.max_segments ? s0.max_segments : (std::min(std::max(s0.max_bounces, 2u), 16u) - 1u);
    std::vector<ViewReq> req(n_views);
    uint64_t paths = 0;
    for (uint32_t v = 0; v < n_views; ++v) {
        uint32_t spp = views[v].spp ? views[v].spp : s0.spp;
        req[v] = ViewReq{views[v].camera, std::max(1u, spp / 16), views[v].max_segments ? views[v].max_segments : def_seg,
                         views[v].seed ? views[v].seed : s0.seed};
        paths += (uint64_t)views[v].camera.width * views[v].camera.height * req[v].spp;
    }
    std::memset(result, 0, sizeof(*result));
    std::string key = tune_key(ctx, sc, paths);
    if (cache_path) {
        FILE* f = std::fopen(cache_path, "r");
        if (f) {
            char line[512];
            while (std::fgets(line, sizeof(line), f)) {
                char k[400];
                bsm_tune_params p{};
                float ms = 0.0f;
                if (std::sscanf(line, "%399s %u %u %u %u %u %f", k, &p.block_size, &p.wavefront_capacity,
                                &p.postpone_depth, &p.refill_lanes, &p.register_cap, &ms) == 7 && key == k &&
                    valid_tune(p)) {
                    result->best = p;
                    result->best_ms = ms;
                    result->from_cache = 1;
                }
            }
            std::fclose(f);
            if (result->from_cache) {
                sc->tune = result->best;
                sc->tuned = true;
                return BSM_OK;
            }
        }
    }
    bsm_pt_settings s = s0;
    s.flags &= ~(uint32_t)(BSM_PT_STAGE_TIMING | BSM_PT_COUNT_TRAVERSAL | BSM_PT_NO_GRAPH);
    s.accumulate = 0;
    s.block_size = 0;
    s.wavefront_capacity = 0;
    bool had = sc->tuned;
    bsm_tune_params saved = sc->tune;
    auto measure = [&](const bsm_tune_params& p, float* ms_out) -> bsm_status {
        sc->tune = p;
        sc->tuned = true;
        bsm_render_stats st{};
        bsm_status e = render_impl(ctx, scene_id, req, s, nullptr, &st);  // captures the graph
        if (e) return e;
        float best = 1e30f;
        for (int r = 0; r < 2; ++r) {
            e = render_impl(ctx, scene_id, req, s, nullptr, &st);
            if (e) return e;
            best = std::min(best, st.ms_total);
        }
        *ms_out = best;
        result->tried++;
        result->worst_ms = std::max(result->worst_ms, best);
        return BSM_OK;
    };
    bsm_tune_params cur{128, 0, 16, 8, 1};
    float cur_ms = 0.0f;
    bsm_status e = measure(cur, &cur_ms);
    if (e) { sc->tune = saved; sc->tuned = had; return e; }
    result->default_ms = cur_ms;
    const uint32_t blocks[] = {64, 128, 256};
    const uint32_t caps[] = {1u << 20, 1u << 22, 1u << 24, 1u << 25, 1u << 26, 1u << 27};
    const uint64_t cap_mem = default_capacity(ctx, ~0ull, std::max(sc->dev.num_lights, 1u));
    const uint32_t postpones[] = {0, 4, 8, 16};
    const uint32_t refills[] = {4, 8, 16, 24};
    for (int pass = 0; pass < 2; ++pass) {
        bool improved = false;
        auto try_one = [&](bsm_tune_params p) -> bsm_status {
            float ms;
            bsm_status e2 = measure(p, &ms);
            if (e2) return e2;
            if (ms < cur_ms * 0.995f) { cur = p; cur_ms = ms; improved = true; }
            return BSM_OK;
        };
        for (uint32_t b : blocks) if (b != cur.block_size) { bsm_tune_params p = cur; p.block_size = b; if ((e = try_one(p))) break; }
        for (uint32_t c : caps) {
            if (e) break;
            if ((uint64_t)c > paths * 2 || c > cap_mem || c == cur.wavefront_capacity) continue;
            bsm_tune_params p = cur; p.wavefront_capacity = c;
            e = try_one(p);
        }
        for (uint32_t v : postpones) { if (e) break; if (v != cur.postpone_depth) { bsm_tune_params p = cur; p.postpone_depth = v; e = try_one(p); } }
        for (uint32_t v : refills) { if (e) break; if (v != cur.refill_lanes) { bsm_tune_params p = cur; p.refill_lanes = v; e = try_one(p); } }
        if (!e) { bsm_tune_params p = cur; p.register_cap = cur.register_cap ^ 1u; e = try_one(p); }
        if (e) { sc->tune = saved; sc->tuned = had; return e; }
        if (!improved) break;
    }
    sc->tune = cur;
    sc->tuned = true;
    result->best = cur;
    result->best_ms = cur_ms;
    if (cache_path) {
        FILE* f = std::fopen(cache_path, "a");
        if (f) {
            std::fprintf(f, "%s %u %u %u %u %u %.4f\n", key.c_str(), cur.block_size, cur.wavefront_capacity,
                         cur.postpone_depth, cur.refill_lanes, cur.register_cap, cur_ms);
            std::fclose(f);
        }
    }
    return BSM_OK;
}

extern "C" bsm_status bsm_read_view(bsm_context* ctx, uint32_t view_index, const bsm_view_output* o) {
    if (!ctx || !o || !o->rgba) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (view_index >= ctx->hist.size() || !ctx->hist[view_index].valid || ctx->hist[view_index].spp == 0)
        return fail(ctx, BSM_ERR_NOT_FOUND, "view has no history");
    const ViewHist& h = ctx->hist[view_index];
    uint32_t W = ctx->layout[view_index].first, H = ctx->layout[view_index].second;
    uint32_t pitch = o->row_pitch_px ? o->row_pitch_px : W;
    const float4* acc = (const float4*)ctx->accum.ptr + h.accum_base;
    float inv = 1.0f / (float)h.spp;
    if (o->location == BSM_DEVICE) {
        launch_resolve(WS(ctx), acc, W, H, inv, (float4*)o->rgba, pitch);
        CK(cudaGetLastError());
        return BSM_OK;
    }
    bsm_status st;
    if ((st = dev_alloc(ctx, ctx->out_stage, (size_t)W * H * sizeof(float4)))) return st;
    launch_resolve(WS(ctx), acc, W, H, inv, (float4*)ctx->out_stage.ptr, W);
    CK(cudaMemcpy2DAsync(o->rgba, (size_t)pitch * 16, ctx->out_stage.ptr, (size_t)W * 16, (size_t)W * 16, H,
                         cudaMemcpyDeviceToHost, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    return BSM_OK;
}

extern "C" bsm_status bsm_export_history(bsm_context* ctx, uint32_t view_index, float* sums, uint32_t* spp,
                                         uint32_t location) {
    if (!ctx || !sums || !spp) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (view_index >= ctx->hist.size() || !ctx->hist[view_index].valid)
        return fail(ctx, BSM_ERR_NOT_FOUND, "view has no history");
    const ViewHist& h = ctx->hist[view_index];
    size_t bytes = (size_t)ctx->layout[view_index].first * ctx->layout[view_index].second * sizeof(float4);
    CK(cudaMemcpyAsync(sums, (float4*)ctx->accum.ptr + h.accum_base, bytes,
                       location == BSM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    *spp = h.spp;
    return BSM_OK;
}

extern "C" bsm_status bsm_import_history(bsm_context* ctx, uint32_t view_index, const bsm_camera* cam,
                                         const float* sums, uint32_t spp, uint32_t location) {
    if (!ctx || !sums || !cam) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (view_index >= ctx->hist.size()) return fail(ctx, BSM_ERR_NOT_FOUND, "view slot does not exist (render once first)");
    if (ctx->layout[view_index].first != cam->width || ctx->layout[view_index].second != cam->height)
        return fail(ctx, BSM_ERR_INVALID_ARG, "camera size differs from the view slot");
    ViewHist& h = ctx->hist[view_index];
    size_t bytes = (size_t)cam->width * cam->height * sizeof(float4);
    CK(cudaMemcpyAsync((float4*)ctx->accum.ptr + h.accum_base, sums, bytes,
                       location == BSM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    h.cam = *cam;
    h.spp = spp;
    h.valid = true;
    return BSM_OK;
}

// ===================================================== stage entry points ====
namespace {
bsm_status stage_prep(bsm_context* ctx, uint32_t scene_id, Scene** out) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BSM_ERR_NOT_FOUND, "unknown scene id");
    if (!sc->has_bvh) return fail(ctx, BSM_ERR_BAD_STATE, "scene BVH not built");
    *out = sc;
    return BSM_OK;
}
}  // namespace

extern "C" bsm_status bsm_trace_closest(bsm_context* ctx, uint32_t scene_id, const float* rays, uint32_t n, void* hits,
                                        uint32_t location) {
    Scene* sc;
    bsm_status st = stage_prep(ctx, scene_id, &sc);
    if (st) return st;
    if (n == 0) return BSM_OK;
    if (!rays || !hits) return BSM_ERR_INVALID_ARG;
    if (location == BSM_DEVICE) {
        launch_trace_closest(WS(ctx), sc->dev, (const float4*)rays, n, (uint4*)hits, 128);
        CK(cudaGetLastError());
        return BSM_OK;   // queued on the work stream
    }
    size_t rb = (size_t)n * 32, hb = (size_t)n * 16;
    if ((st = dev_alloc(ctx, ctx->tmp, rb + hb))) return st;
    char* b = (char*)ctx->tmp.ptr;
    CK(cudaMemcpyAsync(b, rays, rb, cudaMemcpyHostToDevice, WS(ctx)));
    launch_trace_closest(WS(ctx), sc->dev, (const float4*)b, n, (uint4*)(b + rb), 128);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(hits, b + rb, hb, cudaMemcpyDeviceToHost, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    return BSM_OK;
}

extern "C" bsm_status bsm_trace_any(bsm_context* ctx, uint32_t scene_id, const float* rays, uint32_t n,
                                    uint8_t* occluded, uint32_t location) {
    Scene* sc;
    bsm_status st = stage_prep(ctx, scene_id, &sc);
    if (st) return st;
    if (n == 0) return BSM_OK;
    if (!rays || !occluded) return BSM_ERR_INVALID_ARG;
    if (location == BSM_DEVICE) {
        launch_trace_any(WS(ctx), sc->dev, (const float4*)rays, n, occluded, 128);
        CK(cudaGetLastError());
        return BSM_OK;   // queued on the work stream
    }
    size_t rb = (size_t)n * 32;
    if ((st = dev_alloc(ctx, ctx->tmp, rb + n + 16))) return st;
    char* b = (char*)ctx->tmp.ptr;
    CK(cudaMemcpyAsync(b, rays, rb, cudaMemcpyHostToDevice, WS(ctx)));
    launch_trace_any(WS(ctx), sc->dev, (const float4*)b, n, (uint8_t*)(b + rb), 128);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(occluded, b + rb, n, cudaMemcpyDeviceToHost, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    return BSM_OK;
}

// Per-ray traversal counters (nodes visited, triangles tested) for the
// traversal-bytes figure; not part of the reference interface.
extern "C" bsm_status bsm_trace_counts(bsm_context* ctx, uint32_t scene_id, const float* rays, uint32_t n,
                                               uint32_t* counts) {
    Scene* sc;
    bsm_status st = stage_prep(ctx, scene_id, &sc);
    if (st) return st;
    if (sc->instanced) return fail(ctx, BSM_ERR_UNSUPPORTED, "traversal counters cover single-level scenes");
    if (n == 0) return BSM_OK;
    size_t rb = (size_t)n * 32, cb = (size_t)n * 8;
    if ((st = dev_alloc(ctx, ctx->tmp, rb + cb))) return st;
    char* b = (char*)ctx->tmp.ptr;
    CK(cudaMemcpyAsync(b, rays, rb, cudaMemcpyHostToDevice, WS(ctx)));
    launch_trace_count(WS(ctx), sc->dev, (const float4*)b, n, (uint2*)(b + rb));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(counts, b + rb, cb, cudaMemcpyDeviceToHost, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    return BSM_OK;
}

extern "C" bsm_status bsm_render_primary(bsm_context* ctx, uint32_t scene_id, const bsm_camera* camera,
                                         const bsm_pt_settings* settings, float near_z, float far_z,
                                         const bsm_primary_output* out) {
    Scene* sc;
    bsm_status st = stage_prep(ctx, scene_id, &sc);
    if (st) return st;
    if (!camera || !out) return fail(ctx, BSM_ERR_INVALID_ARG, "camera and out must not be NULL");
    bsm_pt_settings s;
    bsm_pt_settings_default(&s);
    if (settings) s = *settings;
    const bsm_camera& c = *camera;
    if (const char* why = camera_problem(c)) return fail(ctx, BSM_ERR_INVALID_ARG, why);
    if ((uint64_t)c.width * c.height >= (1ull << 31)) return fail(ctx, BSM_ERR_INVALID_ARG, "view too large");
    if (!(s.ray_length > 0.0f)) return fail(ctx, BSM_ERR_INVALID_ARG, "ray_length must be > 0");
    if (s.t_min < 0.0f) return fail(ctx, BSM_ERR_INVALID_ARG, "t_min must be >= 0");
    if (near_z == 0.0f) near_z = 0.01f;   // camera.hpp:54-55
    if (far_z == 0.0f) far_z = 10000.0f;
    if (!(near_z > 0.0f && far_z > near_z)) return fail(ctx, BSM_ERR_INVALID_ARG, "need 0 < near_z < far_z");
    if (out->location != BSM_HOST && out->location != BSM_DEVICE)
        return fail(ctx, BSM_ERR_INVALID_ARG, "location must be BSM_HOST or BSM_DEVICE");
    DevView v;
    std::memset(&v, 0, sizeof(v));
    make_view(c, v);
    v.ray_length = s.ray_length;
    v.t_min = s.t_min;
    v.seed = s.seed;
    v.sample_offset = s.sample_offset;
    const size_t npix = (size_t)c.width * c.height;
    // device targets: the caller's buffers, or one staging block for host outputs
    float* dst[6] = {out->depth, out->gbuffer[0], out->gbuffer[1], out->gbuffer[2], out->gbuffer[3],
                     out->hit_positions};
    const size_t bytes[6] = {npix * 4, npix * 16, npix * 16, npix * 16, npix * 16, npix * 16};
    float* dev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (out->location == BSM_DEVICE) {
        for (int k = 0; k < 6; ++k) dev[k] = dst[k];
    } else {
        size_t total = 0;
        for (int k = 0; k < 6; ++k)
            if (dst[k]) total += bytes[k];
        if (total == 0) return BSM_OK;
        if ((st = dev_alloc(ctx, ctx->tmp, total))) return st;
        char* b = (char*)ctx->tmp.ptr;
        for (int k = 0; k < 6; ++k)
            if (dst[k]) { dev[k] = (float*)b; b += bytes[k]; }
    }
    float4* gb[4] = {(float4*)dev[1], (float4*)dev[2], (float4*)dev[3], (float4*)dev[4]};
    launch_primary(WS(ctx), sc->dev, v, near_z, far_z, dev[0], gb, (float4*)dev[5]);
    CK(cudaGetLastError());
    if (out->location == BSM_DEVICE) return BSM_OK;   // queued on the work stream
    for (int k = 0; k < 6; ++k)
        if (dst[k]) CK(cudaMemcpyAsync(dst[k], dev[k], bytes[k], cudaMemcpyDeviceToHost, WS(ctx)));
    CK(cudaStreamSynchronize(WS(ctx)));
    return BSM_OK;
}

// ============================================ internals for other entry points ====
namespace bsm {
bool ctx_scene(bsm_context* ctx, uint32_t scene_id, DevScene* out) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    Scene* sc = find_scene(ctx, scene_id);
    if (!sc || !sc->has_bvh) return false;
    *out = sc->dev;
    return true;
}
cudaStream_t ctx_stream(bsm_context* ctx) { return WS(ctx); }
void ctx_note_noalloc(bsm_context* ctx, uint32_t* counters) { ctx->noalloc_counters = counters; }
int ctx_device(bsm_context* ctx) { return ctx->device; }
void ctx_set_error(bsm_context* ctx, const char* msg) { ctx->err = msg; }
void ctx_make_view(const bsm_camera* c, DevView* v) { make_view(*c, *v); }
const char* ctx_camera_problem(const bsm_camera* c) { return camera_problem(*c); }
void*& ctx_server_slot(bsm_context* ctx) { return ctx->server; }
uint32_t ctx_max_lights(bsm_context* ctx) {
    uint32_t m = 1;
    for (auto& kv : ctx->scenes) m = std::max(m, kv.second->dev.num_lights);
    return m;
}
}  // namespace bsm
