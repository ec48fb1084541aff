// serve.cpp — the serving loop: resident scenes, render requests admitted by
// free memory, continuous batching of their paths into shared wavefronts.
//
// No reference counterpart: the engine renders one frame per camera per
// window tick (graphics_manager.cpp:407-427).  Here a worker thread owns the
// device work of a context:
//   * requests (scene, camera, spp, segments, seed, host output) queue FIFO;
//   * a request is admitted when its accumulator (width x height float4, or
//     three 64-bit fixed-point sums per pixel with BSM_SERVER_DETERMINISTIC)
//     fits in the accumulator pool (first-fit), so admission follows free memory;
//   * every lane (a CUDA stream with its own wavefront queues) that is idle
//     takes the next chunk: path ranges of one scene's active requests, up to
//     the chunk capacity, described by one view record per range — requests
//     that arrived while others were on the GPU join the next chunk, the ones
//     with the least work left first (those admitted over 200 ms ago first);
//   * lanes run concurrently, so chunks of different scenes (and of the same
//     scene) overlap on the device;
//   * when all of a request's paths are traced, its mean is resolved into a
//     staging buffer, copied to the request's host output, and its accumulator
//     returns to the pool.
// A request's random numbers depend only on its seed, pixel and sample, never
// on the chunk or slot it ran in, so its image is the same alone and in a mix
// (up to the order of the per-pixel float sums; bit for bit with exact
// fixed-point sums, BSM_SERVER_DETERMINISTIC).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "bsm_pt.h"
#include "pt_device.h"

namespace bsm {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id;
    bsm_request r;
    uint32_t max_seg;
    uint64_t total_paths;
    uint64_t issued = 0;
    uint64_t done = 0;
    uint32_t state = BSM_REQ_QUEUED;
    uint64_t accum_off = 0;      // float4 index into the pool
    uint64_t accum_len = 0;
    double submit_ms = 0, admit_ms = 0, done_ms = 0;
    bool finishing = false;
    bool cancelled = false;      // bsm_server_cancel: no more paths are issued, no output is written
    cudaEvent_t fin_ev = nullptr;
    cudaEvent_t zero_ev = nullptr;   // accumulator cleared (recorded on the admission stream)
    int fin_lane = -1;
};

struct Range {
    Request* req;
    uint64_t first;
    uint32_t count;
};

struct Lane {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    Wavefront wf{};
    void* wf_mem = nullptr;
    DevView* views_dev = nullptr;
    DevView* views_host = nullptr;   // pinned
    float4* stage = nullptr;         // resolve staging for finished requests
    size_t stage_px = 0;
    bool busy = false;
    std::vector<Range> ranges;
};

// first-fit allocator over the accumulator pool (units: float4)
struct Pool {
    uint64_t size = 0;
    std::map<uint64_t, uint64_t> free_;  // offset -> length
    uint64_t used = 0;
    void init(uint64_t n) { size = n; free_.clear(); free_[0] = n; used = 0; }
    bool alloc(uint64_t n, uint64_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                uint64_t rest = it->second - n, o = it->first + n;
                free_.erase(it);
                if (rest) free_[o] = rest;
                used += n;
                return true;
            }
        }
        return false;
    }
    void release(uint64_t off, uint64_t n) {
        used -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
};

struct Server {
    bsm_context* ctx = nullptr;
    int device = 0;
    bsm_server_opts opts{};
    LaunchCfg lc{};
    uint32_t lights = 1;
    cudaStream_t admin = nullptr;      // clears admitted requests' accumulators
    std::vector<Lane> lanes;
    float4* pool_mem = nullptr;              // FP32 sums (one float4 per pixel)
    unsigned long long* pool_fx = nullptr;   // BSM_SERVER_DETERMINISTIC: fixed-point sums (3 words per pixel)
    bool det = false;
    Pool pool;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> queued;
    std::vector<Request*> active;
    std::map<uint64_t, std::unique_ptr<Request>> all;
    uint64_t next_id = 1;
    std::atomic<bool> stop{false};
    std::thread worker;
    Clock::time_point t0;
    bsm_server_stats stats{};
    std::string error;
    unsigned long long* stats_host = nullptr;  // pinned, per lane kStatWords

    double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
};

bool admit_locked(Server& S) {
    bool any = false;
    while (!S.queued.empty()) {
        Request* r = S.queued.front();
        uint64_t off;
        if (!S.pool.alloc(r->accum_len, &off)) break;  // FIFO: wait for memory to free up
        S.queued.pop_front();
        r->accum_off = off;
        if (S.det) cudaMemsetAsync(S.pool_fx + 3 * off, 0, r->accum_len * 24, S.admin);
        else cudaMemsetAsync(S.pool_mem + off, 0, r->accum_len * 16, S.admin);
        cudaEventCreateWithFlags(&r->zero_ev, cudaEventDisableTiming);
        cudaEventRecord(r->zero_ev, S.admin);
        r->state = BSM_REQ_RUNNING;
        r->admit_ms = S.now_ms();
        S.active.push_back(r);
        S.stats.admitted++;
        any = true;
    }
    return any;
}

// Requests admitted longer ago than this are served in arrival order, ahead of the least-work-first rule.
constexpr double kServeAgeMs = 200.0;

// Builds the next chunk for `lane` from the active requests of one scene
// (round-robin over scenes).  Returns the scene id, or 0 when there is no work.
uint32_t build_chunk_locked(Server& S, Lane& lane, uint32_t* rr_scene) {
    lane.ranges.clear();
    // pick the scene: the first active request with unissued paths after the round-robin cursor
    uint32_t scene = 0;
    uint32_t best_after = 0xffffffffu, best_any = 0xffffffffu;
    for (Request* r : S.active) {
        if (r->issued >= r->total_paths || r->cancelled) continue;
        uint32_t sid = r->r.scene_id;
        if (sid > *rr_scene && sid < best_after) best_after = sid;
        if (sid < best_any) best_any = sid;
    }
    scene = best_after != 0xffffffffu ? best_after : best_any;
    if (scene == 0xffffffffu || scene == 0) return 0;
    *rr_scene = scene;
    uint32_t left = S.opts.chunk_paths;
    std::vector<Request*> cand;
    for (Request* r : S.active)
        if (r->r.scene_id == scene && r->issued < r->total_paths && !r->cancelled) cand.push_back(r);
    // Order within the scene: requests admitted more than kServeAgeMs ago first, oldest first; then the
    // others by the work they have left (paths still to issue x segments), least first, so that a small
    // request arriving while a large one of the same scene runs joins the next chunk instead of waiting for
    // the large one's paths.
    const double now = S.now_ms();
    auto key = [&](const Request* r) {
        const bool aged = now - r->admit_ms > kServeAgeMs;
        return std::make_pair(aged ? 0.0 : 1.0, aged ? r->admit_ms : (double)(r->total_paths - r->issued) * r->max_seg);
    };
    std::stable_sort(cand.begin(), cand.end(), [&](const Request* a, const Request* b) { return key(a) < key(b); });
    for (Request* r : cand) {
        if (lane.ranges.size() >= S.opts.max_views_per_chunk || left == 0) break;
        uint64_t n = std::min<uint64_t>(left, r->total_paths - r->issued);
        lane.ranges.push_back(Range{r, r->issued, (uint32_t)n});
        r->issued += n;
        left -= (uint32_t)n;
    }
    return lane.ranges.empty() ? 0 : scene;
}

bool launch_chunk(Server& S, Lane& lane, uint32_t scene) {
    DevScene sc;
    if (!ctx_scene(S.ctx, scene, &sc)) return false;
    uint64_t base = 0;
    uint32_t max_seg = 1;
    for (size_t i = 0; i < lane.ranges.size(); ++i) {
        const Range& rg = lane.ranges[i];
        DevView& dv = lane.views_host[i];
        std::memset(&dv, 0, sizeof(dv));
        ctx_make_view(&rg.req->r.camera, &dv);
        dv.ray_length = 100.0f;
        dv.t_min = 0.0f;
        dv.spp = rg.req->r.spp;
        dv.sample_offset = 0;
        dv.seed = rg.req->r.seed;
        dv.path_base = base;
        dv.first_path = rg.first;
        dv.accum_base = (uint32_t)rg.req->accum_off;
        dv.max_segments = rg.req->max_seg;
        dv.flags = 0;
        base += rg.count;
        max_seg = std::max(max_seg, rg.req->max_seg);
    }
    cudaStream_t st = lane.stream;
    // every request in the chunk must have its accumulator cleared first (admission stream)
    for (const Range& rg : lane.ranges) cudaStreamWaitEvent(st, rg.req->zero_ev, 0);
    cudaMemcpyAsync(lane.views_dev, lane.views_host, lane.ranges.size() * sizeof(DevView), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(lane.wf.counters, 0, kCntWords * 4, st);
    cudaMemsetAsync(lane.wf.stats, 0, kStatWords * 8, st);
    launch_camera(S.lc, st, lane.views_dev, (uint32_t)lane.ranges.size(), 0, (uint32_t)base, lane.wf, max_seg);
    int q = 0;
    for (uint32_t seg = 0; seg < max_seg; ++seg) {
        launch_extend(S.lc, st, sc, lane.wf, q, seg, false);
        launch_shade(S.lc, st, sc, lane.views_dev, lane.wf, q, seg, S.pool_mem);
        launch_shadow(S.lc, st, sc, lane.wf, seg, S.pool_mem);
        q ^= 1;
    }
    size_t li = &lane - S.lanes.data();
    cudaMemcpyAsync(S.stats_host + li * kStatWords, lane.wf.stats, kStatWords * 8, cudaMemcpyDeviceToHost, st);
    cudaEventRecord(lane.ev, st);
    lane.busy = true;
    return cudaGetLastError() == cudaSuccess;
}

// Resolves a finished request into the lane's staging buffer and copies it to
// the request's host output (asynchronously; completion is polled).
void finish_request(Server& S, Lane& lane, Request* r) {
    const bsm_camera& c = r->r.camera;
    size_t px = (size_t)c.width * c.height;
    if (S.det)
        launch_resolve_fixed(lane.stream, S.pool_fx + 3 * r->accum_off, c.width, c.height, 1.0f / (float)r->r.spp,
                             lane.stage, c.width);
    else
        launch_resolve(lane.stream, S.pool_mem + r->accum_off, c.width, c.height, 1.0f / (float)r->r.spp,
                       lane.stage, c.width);
    cudaMemcpyAsync(r->r.out_rgba, lane.stage, px * 16, cudaMemcpyDeviceToHost, lane.stream);
    cudaEventCreateWithFlags(&r->fin_ev, cudaEventDisableTiming);
    cudaEventRecord(r->fin_ev, lane.stream);
    r->finishing = true;
    r->fin_lane = (int)(&lane - S.lanes.data());
}

void worker_main(Server* Sp) {
    Server& S = *Sp;
    cudaSetDevice(S.device);
    uint32_t rr_scene = 0;
    while (!S.stop.load()) {
        bool did = false;
        // completions
        for (Lane& lane : S.lanes) {
            if (!lane.busy) continue;
            if (cudaEventQuery(lane.ev) != cudaSuccess) continue;
            lane.busy = false;
            did = true;
            size_t li = &lane - S.lanes.data();
            std::lock_guard<std::mutex> lk(S.mu);
            for (uint32_t k = 0; k < (uint32_t)kMaxSeg; ++k) {
                S.stats.extend_rays += S.stats_host[li * kStatWords + kStatExtend + k];
                S.stats.shadow_rays += S.stats_host[li * kStatWords + kStatShadow + k];
            }
            for (const Range& rg : lane.ranges) rg.req->done += rg.count;
            // a finished request resolves on this (now idle) lane
            for (const Range& rg : lane.ranges) {
                Request* r = rg.req;
                if (r->done == r->total_paths && !r->finishing && !r->cancelled) finish_request(S, lane, r);
            }
            lane.ranges.clear();
        }
        {
            std::lock_guard<std::mutex> lk(S.mu);
            // finished outputs
            for (size_t i = 0; i < S.active.size();) {
                Request* r = S.active[i];
                if (r->cancelled && !r->finishing && r->done == r->issued) {
                    // no chunk of it is in flight any more: its accumulator goes back to the pool
                    if (r->zero_ev) { cudaEventSynchronize(r->zero_ev); cudaEventDestroy(r->zero_ev); }
                    r->zero_ev = nullptr;
                    r->done_ms = S.now_ms();
                    r->state = BSM_REQ_CANCELLED;
                    S.pool.release(r->accum_off, r->accum_len);
                    S.stats.cancelled++;
                    S.active.erase(S.active.begin() + i);
                    did = true;
                    continue;
                }
                if (r->finishing && cudaEventQuery(r->fin_ev) == cudaSuccess) {
                    cudaEventDestroy(r->fin_ev);
                    r->fin_ev = nullptr;
                    cudaEventDestroy(r->zero_ev);
                    r->zero_ev = nullptr;
                    r->done_ms = S.now_ms();
                    r->state = BSM_REQ_DONE;
                    S.pool.release(r->accum_off, r->accum_len);
                    S.stats.completed++;
                    S.active.erase(S.active.begin() + i);
                    did = true;
                    continue;
                }
                ++i;
            }
            if (admit_locked(S)) did = true;
            // keep lanes whose finish copies are pending busy-free: a finish uses the lane stream,
            // later chunks on that stream simply queue behind it
            for (Lane& lane : S.lanes) {
                if (lane.busy) continue;
                uint32_t scene = build_chunk_locked(S, lane, &rr_scene);
                if (!scene) break;
                if (!launch_chunk(S, lane, scene)) {
                    S.error = "chunk launch failed";
                    for (const Range& rg : lane.ranges) rg.req->state = BSM_REQ_FAILED;
                }
                did = true;
            }
            S.stats.active = (uint32_t)S.active.size();
            S.stats.queued = (uint32_t)S.queued.size();
            S.stats.pool_used_bytes = S.pool.used * (S.det ? 24 : 16);
        }
        S.cv.notify_all();
        if (!did) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

Server* get(bsm_context* ctx) { return (Server*)ctx_server_slot(ctx); }

}  // namespace
}  // namespace bsm

using namespace bsm;

extern "C" bsm_status bsm_server_start(bsm_context* ctx, const bsm_server_opts* o) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    if (get(ctx)) { ctx_set_error(ctx, "server already running"); return BSM_ERR_BAD_STATE; }
    auto S = std::make_unique<Server>();
    S->ctx = ctx;
    S->device = ctx_device(ctx);
    cudaSetDevice(S->device);
    if (o) S->opts = *o;
    if (!S->opts.pool_bytes) S->opts.pool_bytes = 1ull << 30;
    if (!S->opts.chunk_paths) S->opts.chunk_paths = 1u << 21;
    if (!S->opts.lanes) S->opts.lanes = 4;
    if (!S->opts.max_views_per_chunk) S->opts.max_views_per_chunk = 256;
    if (S->opts.lanes > 16 || S->opts.chunk_paths < 1024 || S->opts.max_views_per_chunk > 4096 ||
        (S->opts.flags & ~(uint32_t)BSM_SERVER_DETERMINISTIC)) {
        ctx_set_error(ctx, "server options out of range (lanes <= 16, chunk_paths >= 1024, views <= 4096, flags)");
        return BSM_ERR_INVALID_ARG;
    }
    S->det = (S->opts.flags & BSM_SERVER_DETERMINISTIC) != 0;
    S->lc.regcap = 1;
    query_launch_cfg(S->device, 128, &S->lc);
    S->lights = std::max(ctx_max_lights(ctx), (uint32_t)kMaxLights);
    const size_t C = S->opts.chunk_paths, SH = C * (S->lights + 1);
    auto fail_cleanup = [&](const char* m) {
        for (Lane& l : S->lanes) {
            if (l.wf_mem) cudaFree(l.wf_mem);
            if (l.views_host) cudaFreeHost(l.views_host);
            if (l.stage) cudaFree(l.stage);
            if (l.stream) cudaStreamDestroy(l.stream);
            if (l.ev) cudaEventDestroy(l.ev);
        }
        if (S->pool_mem) cudaFree(S->pool_mem);
        if (S->pool_fx) cudaFree(S->pool_fx);
        if (S->stats_host) cudaFreeHost(S->stats_host);
        ctx_set_error(ctx, m);
        return BSM_ERR_OUT_OF_MEMORY;
    };
    S->lanes.resize(S->opts.lanes);
    const size_t max_px = 1920ull * 1080ull;
    for (Lane& l : S->lanes) {
        size_t bytes = 0;
        auto sz = [&](size_t n) { size_t off = bytes; bytes += (n + 255) & ~(size_t)255; return off; };
        size_t o_ro0 = sz(C * 16), o_ro1 = sz(C * 16), o_rd0 = sz(C * 16), o_rd1 = sz(C * 16);
        size_t o_p0 = sz(C * 16), o_p1 = sz(C * 16), o_t0 = sz(C * 16), o_t1 = sz(C * 16), o_hit = sz(C * 16);
        size_t o_sho = sz(SH * 16), o_shd = sz(SH * 16), o_shc = sz(SH * 16), o_shs = sz(SH * 4);
        size_t o_cnt = sz(kCntWords * 4), o_st = sz(kStatWords * 8);
        size_t o_v = sz(S->opts.max_views_per_chunk * sizeof(DevView));
        if (cudaMalloc(&l.wf_mem, bytes) != cudaSuccess) return fail_cleanup("server: cannot allocate lane queues");
        char* b = (char*)l.wf_mem;
        l.wf.capacity = (uint32_t)C;
        l.wf.ray_o[0] = (float4*)(b + o_ro0); l.wf.ray_o[1] = (float4*)(b + o_ro1);
        l.wf.ray_d[0] = (float4*)(b + o_rd0); l.wf.ray_d[1] = (float4*)(b + o_rd1);
        l.wf.path[0] = (uint4*)(b + o_p0); l.wf.path[1] = (uint4*)(b + o_p1);
        l.wf.thr[0] = (float4*)(b + o_t0); l.wf.thr[1] = (float4*)(b + o_t1);
        l.wf.hit = (float4*)(b + o_hit);
        l.wf.sh_o = (float4*)(b + o_sho); l.wf.sh_d = (float4*)(b + o_shd); l.wf.sh_c = (float4*)(b + o_shc);
        l.wf.sh_seed = (uint32_t*)(b + o_shs);
        l.wf.counters = (uint32_t*)(b + o_cnt);
        l.wf.stats = (unsigned long long*)(b + o_st);
        l.views_dev = (DevView*)(b + o_v);
        if (cudaHostAlloc((void**)&l.views_host, S->opts.max_views_per_chunk * sizeof(DevView), 0) != cudaSuccess)
            return fail_cleanup("server: cannot allocate pinned view records");
        if (cudaMalloc((void**)&l.stage, max_px * 16) != cudaSuccess) return fail_cleanup("server: staging");
        l.stage_px = max_px;
        cudaStreamCreateWithFlags(&l.stream, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&l.ev, cudaEventDisableTiming);
    }
    if (cudaHostAlloc((void**)&S->stats_host, S->lanes.size() * kStatWords * 8, 0) != cudaSuccess)
        return fail_cleanup("server: pinned stats");
    const uint64_t px_bytes = S->det ? 24 : 16;
    uint64_t pool_n = S->opts.pool_bytes / px_bytes;
    if (S->det) {
        if (cudaMalloc((void**)&S->pool_fx, pool_n * 24) != cudaSuccess) return fail_cleanup("server: accumulator pool");
        for (Lane& l : S->lanes) l.wf.accum_fx = S->pool_fx;   // contributions go to the fixed-point sums
    } else if (cudaMalloc((void**)&S->pool_mem, pool_n * 16) != cudaSuccess) {
        return fail_cleanup("server: accumulator pool");
    }
    S->pool.init(pool_n);
    S->stats.pool_bytes = pool_n * px_bytes;
    cudaStreamCreateWithFlags(&S->admin, cudaStreamNonBlocking);
    S->t0 = Clock::now();
    Server* raw = S.release();
    ctx_server_slot(ctx) = raw;
    raw->worker = std::thread(worker_main, raw);
    return BSM_OK;
}

extern "C" bsm_status bsm_server_submit(bsm_context* ctx, const bsm_request* r, uint64_t* id) {
    if (!ctx || !r || !id) return BSM_ERR_INVALID_ARG;
    Server* S = get(ctx);
    if (!S) { ctx_set_error(ctx, "server not running"); return BSM_ERR_BAD_STATE; }
    DevScene sc;
    if (!ctx_scene(ctx, r->scene_id, &sc)) { ctx_set_error(ctx, "unknown scene or BVH not built"); return BSM_ERR_NOT_FOUND; }
    if (!r->out_rgba || r->camera.width == 0 || r->camera.height == 0 || r->spp == 0 ||
        !(r->camera.yfov_deg > 0.0f && r->camera.yfov_deg < 180.0f)) {
        ctx_set_error(ctx, "invalid request");
        return BSM_ERR_INVALID_ARG;
    }
    if (const char* why = ctx_camera_problem(&r->camera)) { ctx_set_error(ctx, why); return BSM_ERR_INVALID_ARG; }
    uint32_t segs = r->max_segments ? r->max_segments : 8;
    if (segs > (uint32_t)kMaxSeg) { ctx_set_error(ctx, "max_segments must be 1..16"); return BSM_ERR_INVALID_ARG; }
    uint64_t px = (uint64_t)r->camera.width * r->camera.height;
    if (px > 1920ull * 1080ull) { ctx_set_error(ctx, "request larger than 1920x1080 pixels"); return BSM_ERR_INVALID_ARG; }
    if (sc.num_lights > S->lights) { ctx_set_error(ctx, "scene has more lights than the server's queues"); return BSM_ERR_INVALID_ARG; }
    std::lock_guard<std::mutex> lk(S->mu);
    if (px > S->pool.size) {
        S->stats.rejected++;
        ctx_set_error(ctx, "request does not fit the accumulator pool");
        return BSM_ERR_ADMISSION;
    }
    auto q = std::make_unique<Request>();
    q->id = S->next_id++;
    q->r = *r;
    q->max_seg = segs;
    q->total_paths = px * r->spp;
    q->accum_len = px;
    q->submit_ms = S->now_ms();
    S->queued.push_back(q.get());
    S->stats.submitted++;
    *id = q->id;
    S->all[q->id] = std::move(q);
    return BSM_OK;
}

static void fill_status(const Request* r, bsm_request_status* st) {
    st->cancelled = r->cancelled ? 1u : 0u;
    st->state = r->state;
    st->submit_ms = r->submit_ms;
    st->admit_ms = r->admit_ms;
    st->done_ms = r->done_ms;
    st->paths = r->total_paths;
}

extern "C" bsm_status bsm_server_poll(bsm_context* ctx, uint64_t id, bsm_request_status* st) {
    if (!ctx || !st) return BSM_ERR_INVALID_ARG;
    Server* S = get(ctx);
    if (!S) return BSM_ERR_BAD_STATE;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return BSM_ERR_NOT_FOUND;
    fill_status(it->second.get(), st);
    return BSM_OK;
}

extern "C" bsm_status bsm_server_wait(bsm_context* ctx, uint64_t id, uint32_t timeout_ms, bsm_request_status* st) {
    if (!ctx || !st) return BSM_ERR_INVALID_ARG;
    Server* S = get(ctx);
    if (!S) return BSM_ERR_BAD_STATE;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return BSM_ERR_NOT_FOUND;
    Request* r = it->second.get();
    auto pred = [&] {
        return r->state == BSM_REQ_DONE || r->state == BSM_REQ_FAILED || r->state == BSM_REQ_CANCELLED;
    };
    if (timeout_ms) {
        if (!S->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) {
            fill_status(r, st);
            return BSM_ERR_TIMEOUT;
        }
    } else {
        S->cv.wait(lk, pred);
    }
    fill_status(r, st);
    if (r->state == BSM_REQ_CANCELLED) return BSM_ERR_CANCELLED;
    return r->state == BSM_REQ_DONE ? BSM_OK : BSM_ERR_CUDA;
}

extern "C" bsm_status bsm_server_cancel(bsm_context* ctx, uint64_t id) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    Server* S = get(ctx);
    if (!S) return BSM_ERR_BAD_STATE;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return BSM_ERR_NOT_FOUND;
    Request* r = it->second.get();
    if (r->state == BSM_REQ_QUEUED) {   // never admitted: nothing of it is on the device
        S->queued.erase(std::find(S->queued.begin(), S->queued.end(), r));
        r->cancelled = true;
        r->state = BSM_REQ_CANCELLED;
        r->done_ms = S->now_ms();
        S->stats.cancelled++;
    } else if (r->state == BSM_REQ_RUNNING) {
        if (r->finishing) {
            // its output copy is already queued: let it land before returning, so that the library
            // writes nothing into out_rgba after this call; the request completes normally
            cudaEvent_t e = r->fin_ev;
            lk.unlock();
            cudaSetDevice(S->device);
            cudaEventSynchronize(e);
            return BSM_OK;
        }
        r->cancelled = true;   // the worker releases it when its chunks in flight are done
    }
    S->cv.notify_all();
    return BSM_OK;
}

extern "C" bsm_status bsm_server_get_stats(bsm_context* ctx, bsm_server_stats* out) {
    if (!ctx || !out) return BSM_ERR_INVALID_ARG;
    Server* S = get(ctx);
    if (!S) return BSM_ERR_BAD_STATE;
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->stats;
    out->elapsed_ms = S->now_ms();
    return BSM_OK;
}

extern "C" bsm_status bsm_server_stop(bsm_context* ctx) {
    if (!ctx) return BSM_ERR_INVALID_ARG;
    Server* S = get(ctx);
    if (!S) return BSM_ERR_BAD_STATE;
    S->stop.store(true);
    S->worker.join();
    cudaSetDevice(S->device);
    for (Lane& l : S->lanes) {
        cudaStreamSynchronize(l.stream);
        cudaFree(l.wf_mem);
        cudaFreeHost(l.views_host);
        cudaFree(l.stage);
        cudaStreamDestroy(l.stream);
        cudaEventDestroy(l.ev);
    }
    cudaStreamSynchronize(S->admin);
    cudaStreamDestroy(S->admin);
    for (auto& kv : S->all) {
        if (kv.second->fin_ev) cudaEventDestroy(kv.second->fin_ev);
        if (kv.second->zero_ev) cudaEventDestroy(kv.second->zero_ev);
    }
    if (S->pool_mem) cudaFree(S->pool_mem);
    if (S->pool_fx) cudaFree(S->pool_fx);
    cudaFreeHost(S->stats_host);
    ctx_server_slot(ctx) = nullptr;
    delete S;
    return BSM_OK;
}
