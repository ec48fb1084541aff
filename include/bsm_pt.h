/*
 * bsm_pt.h — C ABI of the GB300 wavefront path-tracing pass.
 *
 * This library is a drop-in for the path-tracing pass of the bisemutum builtin
 * renderer.  The pass keeps the reference's contract: camera, scene (meshes,
 * materials, directional lights, skybox), spp and bounce settings in, an HDR
 * accumulation buffer out.  Everything behind these entry points runs as
 * hand-written sm_103a CUDA kernels on one GPU.
 *
 * Reference interfaces replaced (paths relative to the bisemutum-engine repo):
 *   - PathTracingPass::update_params / ::render
 *       bisemutum/src/renderer/pass/path_tracing.hpp:27-35
 *       bisemutum/src/renderer/pass/path_tracing.cpp:183-222, 224-490
 *   - BasicRenderer::PathTracingSettings
 *       bisemutum/include/bisemutum/renderer/basic.hpp:76-81
 *   - acceleration structure build (driver BLAS/TLAS)
 *       bisemutum/src/graphics/accel.cpp:11-159
 *   - TraceRay closest hit / any hit
 *       bisemutum/shaders/renderer/raytracing/rt_gbuffer.hlsl:7-36
 *       bisemutum/shaders/renderer/raytracing/hits/rt_gbuffer_hit.hlsl:6-35
 *   - scene inputs: DirLightData (bisemutum/src/renderer/context/lights.hpp:12-22),
 *     skybox colour/texture (bisemutum/src/renderer/context/skybox.cpp),
 *     camera matrices (bisemutum/src/graphics/camera.cpp:73-118).
 *
 * Conventions
 *   - Every call returns a bsm_status; 0 is success, negative values are errors.
 *     bsm_last_error(ctx) returns a message for the last failing call on ctx.
 *   - Plain pointers and sizes only.  A `location` argument says whether a
 *     buffer lives in host memory (BSM_HOST) or device memory (BSM_DEVICE).
 *   - One context per host thread.  Calls on one context are serialised by the
 *     caller; the serving entry points (bsm_server_*) take an internal lock.
 *   - Work runs on the context's stream, or on the caller's stream after
 *     bsm_set_stream.  Calls whose results stay on the device (renders to device
 *     outputs or to the view history, device-located traces, primary outputs on
 *     the device) return with their kernels queued, as the reference's pass only
 *     records work that runs later in RenderGraph::execute
 *     (bisemutum/src/graphics/graphics_manager.cpp:418-419).  Calls that hand a
 *     result to host memory wait for it.  Kernels report overflows and timed-out
 *     waits in a device error word that stays set until a sync point
 *     (bsm_sync, bsm_render_stats_read, or a call that waits) reads it and
 *     returns BSM_ERR_DEVICE_CHECK.
 *   - Scene data passed to bsm_scene_upload is copied; the caller may free its
 *     buffers when the call returns.
 */
#ifndef BSM_PT_H
#define BSM_PT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BSM_API_VERSION 1

#if defined(_WIN32)
#define BSM_API __declspec(dllexport)
#else
#define BSM_API __attribute__((visibility("default")))
#endif

typedef int32_t bsm_status;
enum {
    BSM_OK = 0,
    BSM_ERR_INVALID_ARG = -1,
    BSM_ERR_OUT_OF_MEMORY = -2,
    BSM_ERR_CUDA = -3,
    BSM_ERR_TIMEOUT = -4,
    BSM_ERR_NOT_FOUND = -5,
    BSM_ERR_BAD_STATE = -6,
    BSM_ERR_NO_DEVICE = -7,
    BSM_ERR_UNSUPPORTED = -8,
    BSM_ERR_DEVICE_CHECK = -9,   /* a kernel's own bounds/overflow check or bounded wait fired */
    BSM_ERR_ADMISSION = -10,     /* serving: request does not fit the memory budget */
    BSM_ERR_CANCELLED = -11      /* serving: the request was cancelled (bsm_server_cancel) */
};

enum { BSM_HOST = 0, BSM_DEVICE = 1 };

typedef struct bsm_context bsm_context;

/* ---- context ---------------------------------------------------------- */

/* Creates a context on CUDA device `device_ordinal`.  `mem_budget_bytes`
 * bounds the device memory the context may hold (0 = 90% of free memory).
 * Replaces the graphics-device setup the reference does in
 * GraphicsManager::initialize (bisemutum/src/graphics/graphics_manager.cpp). */
BSM_API bsm_status bsm_create(bsm_context** ctx, int device_ordinal, uint64_t mem_budget_bytes);
BSM_API void bsm_destroy(bsm_context* ctx);
BSM_API const char* bsm_last_error(const bsm_context* ctx);
BSM_API int bsm_api_version(void);
/* Waits for all work on the context's work stream (timeout_ms = 0: no limit;
 * BSM_ERR_TIMEOUT when the limit runs out, the work keeps running), then reads
 * and clears the device error word: BSM_ERR_DEVICE_CHECK if a kernel's check
 * fired since the last sync point. */
BSM_API bsm_status bsm_sync(bsm_context* ctx, uint32_t timeout_ms);
/* Runs the context's later work on `stream` (a cudaStream_t of the context's
 * device, owned by the caller, that must outlive that work), or on the
 * context's own stream again when `stream` is NULL.  Work queued before the
 * switch stays ordered before work queued after it.  Replaces the engine's
 * command encoder that the reference's render graph records the pass into
 * (GraphicsManager::execute_in_this_frame, graphics_manager.cpp:407-427).
 * Refused while the serving loop runs (it uses streams of its own). */
BSM_API bsm_status bsm_set_stream(bsm_context* ctx, void* stream);
/* The stream the context's work runs on (cudaStream_t). */
BSM_API void* bsm_get_stream(bsm_context* ctx);

/* Device memory helpers for callers without their own allocator. */
BSM_API bsm_status bsm_device_alloc(bsm_context* ctx, uint64_t bytes, void** ptr);
BSM_API bsm_status bsm_device_free(bsm_context* ctx, void* ptr);
/* kind: 0 host->device, 1 device->host, 2 device->device (synchronous). */
BSM_API bsm_status bsm_memcpy(bsm_context* ctx, void* dst, const void* src, uint64_t bytes, int kind);

/* ---- scene description (DirLightData, skybox, GPU scene buffers) ------ */

/* BlendMode (graphics/material.hpp): opaque surfaces always stop rays; the
 * others run the any-hit rule of rt_gbuffer_hit.hlsl:20-35 on every candidate
 * hit: alpha test ignores the hit when opacity < 0.01 (utils.hlsl:38),
 * translucent ignores it when a per-ray uniform u < 1 - opacity (stochastic
 * opacity).  Shadow rays follow the same rule. */
enum { BSM_BLEND_OPAQUE = 0, BSM_BLEND_ALPHA_TEST = 1, BSM_BLEND_TRANSLUCENT = 2 };

typedef struct bsm_material {
    float base_color[3];   /* SurfaceData::base_color (utils.hlsl:5-16) */
    float roughness;       /* perceptual roughness, alpha = max(r^2, 1e-3) */
    float metallic;        /* f0 = lerp(0.04, base_color, metallic) (import_model.cpp:217-219) */
    float emission[3];     /* kept for the descriptor; the reference PT drops it (gbuffer.hlsl) */
    float opacity;         /* SurfaceData::opacity in [0, 1]; used by the non-opaque blend modes */
    uint32_t blend_mode;   /* BSM_BLEND_* (0 = opaque) */
} bsm_material;

typedef struct bsm_dir_light {
    float direction[3];    /* unit vector pointing TO the light (lights.cpp:59-65) */
    float emission[3];     /* colour * strength; the radiance term of dir_light_eval (lights.hlsl:10-13) */
} bsm_dir_light;

/* PointLightData (renderer/context/lights.hpp:24-36): a point light, or a
 * spot light when cos_inner > cos_outer; point_light_eval (lights.hlsl:15-25). */
typedef struct bsm_point_light {
    float position[3];
    float emission[3];      /* colour * strength */
    float range;            /* attenuation range (saturate(1 - (d^2 / range^2)^2) / max(d^2, 0.001)) */
    float direction[3];     /* unit vector pointing TO the light (the spot's axis reversed) */
    float cos_inner;        /* spot: cos of the inner / outer half angles; point light: both 0 */
    float cos_outer;
} bsm_point_light;

/* RectLightData (lights.hpp:38-53): a rectangle with corners c + R(+-w, +-h, 0).
 * It emits towards its local -z (the side from which the corners run
 * counter-clockwise, which the reference's LTC integral counts positive,
 * lights.hlsl:421), or both sides when two_sided.  Untextured. */
typedef struct bsm_rect_light {
    float center[3];
    float axis_x[3];        /* unit local x (width direction) in world space */
    float axis_y[3];        /* unit local y (height direction) */
    float width, height;
    float emission[3];      /* colour * strength: radiance of the surface */
    uint32_t two_sided;
} bsm_rect_light;

enum { BSM_SKY_CONSTANT = 0, BSM_SKY_EQUIRECT = 1, BSM_SKY_CUBEMAP = 2 };
typedef struct bsm_sky {
    uint32_t kind;          /* BSM_SKY_* */
    float color[3];         /* constant radiance, or a multiplier of the map (skybox_color) */
    uint32_t width, height; /* equirect size (row 0 looks at +y, column 0 at azimuth -pi), or the cube face size */
    const uint16_t* rgba16f;/* RGBA IEEE half texels (host): width*height, or 6 faces +X -X +Y -Y +Z -Z */
    float transform[9];     /* cubemap: row-major rotation applied to a direction before the lookup
                               (skybox_transform, deferred_lighting_secondary.hlsl:25); zeros = identity */
} bsm_sky;

typedef struct bsm_scene_desc {
    uint32_t num_vertices;
    const float* positions;       /* 3 * num_vertices */
    uint32_t num_triangles;
    const uint32_t* indices;      /* 3 * num_triangles, or NULL for a triangle soup */
    const uint32_t* material_ids; /* num_triangles, or NULL (all material 0) */
    uint32_t num_materials;
    const bsm_material* materials;
    uint32_t num_dir_lights;
    const bsm_dir_light* dir_lights;
    bsm_sky sky;
    uint32_t num_point_lights;        /* dir + point + rect lights: at most 8 */
    const bsm_point_light* point_lights;
    uint32_t num_rect_lights;
    const bsm_rect_light* rect_lights;
    const float* normals;             /* 3 * num_vertices vertex normals (world space, any length), or NULL:
                                         hits shade with the interpolated, normalised vertex normal
                                         (hit.hlsl:55-71, 158), else with the geometric normal; either is
                                         faced towards the ray */
} bsm_scene_desc;

enum { BSM_COLLAPSE_SAH_OPTIMAL = 0, BSM_COLLAPSE_GREEDY = 1 };
enum { BSM_BUILD_DEVICE = 0, BSM_BUILD_HOST = 1 };
typedef struct bsm_bvh_opts {
    uint32_t sah_bins;        /* 0 = 32 (the device builder takes 4..32, the host builder 4..256) */
    uint32_t max_leaf_tris;   /* 1..2, 0 = 2 */
    uint32_t num_threads;     /* host builder threads; 0 = hardware concurrency */
    uint32_t collapse;        /* binary -> 8-wide: BSM_COLLAPSE_SAH_OPTIMAL (dynamic programming over a
                                 binary tree of single-triangle leaves) or BSM_COLLAPSE_GREEDY (open the
                                 largest child) */
    float tri_cost;           /* SAH-optimal collapse: cost of a triangle test relative to a node test; 0 = 1.0 */
    uint32_t builder;         /* BSM_BUILD_DEVICE (default: sm_103a kernels) or BSM_BUILD_HOST (C++ threads) */
} bsm_bvh_opts;

typedef struct bsm_bvh_stats {
    uint32_t num_nodes;       /* 8-wide compressed nodes (80 B each) */
    uint32_t num_tris;
    uint32_t max_depth;
    uint32_t builder;         /* BSM_BUILD_* that built it */
    double build_ms;          /* build time (wall clock, uploads and waits included) */
    double sah_cost;          /* SAH cost of the binary BVH before collapsing */
    uint64_t node_bytes;
    uint64_t tri_bytes;
} bsm_bvh_stats;

/* Copies a scene to the device.  Replaces the GPU-scene upload the reference
 * does in GpuSceneSystem (bisemutum/src/graphics/gpu_scene_system.cpp). */
BSM_API bsm_status bsm_scene_upload(bsm_context* ctx, const bsm_scene_desc* desc, uint32_t* scene_id);
/* SAH-binned build of the compressed 8-wide BVH, on the device by default
 * (opts->builder); replaces the driver BLAS/TLAS build of
 * AccelerationStructure (bisemutum/src/graphics/accel.cpp:11-159), which the
 * reference also runs on the GPU (graphics_manager.cpp:475-478).  Synchronous.
 * A two-level scene rebuilds its TLAS from the current transforms. */
BSM_API bsm_status bsm_scene_build_bvh(bsm_context* ctx, uint32_t scene_id, const bsm_bvh_opts* opts,
                                       bsm_bvh_stats* stats);
BSM_API bsm_status bsm_scene_release(bsm_context* ctx, uint32_t scene_id);
/* Host-only build of the same BVH into caller buffers (no device needed).
 * Call with nodes == tris == NULL to get the sizes in `stats`, then again
 * with buffers of stats->node_bytes and stats->tri_bytes. */
BSM_API bsm_status bsm_bvh_build_host(const bsm_scene_desc* desc, const bsm_bvh_opts* opts, void* nodes,
                                      uint64_t nodes_bytes, void* tris, uint64_t tris_bytes,
                                      bsm_bvh_stats* stats);
/* Device bytes held by one scene (BVH + triangles + materials + sky). */
BSM_API bsm_status bsm_scene_device_bytes(bsm_context* ctx, uint32_t scene_id, uint64_t* bytes);
/* Copies the built BVH back to the host (node_bytes / tri_bytes as in the stats).
 * Either pointer may be NULL.  Used by tests that check the BVH invariants. */
BSM_API bsm_status bsm_scene_download_bvh(bsm_context* ctx, uint32_t scene_id, void* nodes, void* tris);

/* ---- camera and settings (Camera, PathTracingSettings) ----------------- */

typedef struct bsm_camera {
    float position[3];
    float front[3];          /* view direction (lookAt(position, position + front, up)) */
    float up[3];
    float yfov_deg;          /* vertical field of view (camera.cpp:96-98) */
    uint32_t width, height;
} bsm_camera;

enum {
    BSM_PT_JITTER = 1u << 0,        /* jitter primary rays inside the pixel (reference: centre) */
    BSM_PT_NO_SUN_NEE = 1u << 1,
    BSM_PT_NO_SKY_NEE = 1u << 2,    /* sky only through BSDF-sampled escapes */
    BSM_PT_STAGE_TIMING = 1u << 3,  /* record per-stage CUDA events into bsm_render_stats */
    BSM_PT_NO_GRAPH = 1u << 4,      /* launch stages directly instead of replaying a CUDA graph */
    BSM_PT_COUNT_TRAVERSAL = 1u << 5, /* count BVH nodes visited / triangles tested by the extend stage */
    BSM_PT_DETERMINISTIC = 1u << 6  /* bit-reproducible images: the call's contributions are summed per pixel
                                       as 32.32 fixed-point integers (exact, so the order of the additions does
                                       not matter) and added to the view's history once; negative
                                       contributions count as 0, and a pixel's sum over one call must stay
                                       below 2^32 per channel.  Default: FP32 atomics, whose last bits
                                       depend on the order in which the GPU adds them. bsm_render,
                                       bsm_render_batch and bsm_render_cached; the serving loop ignores it */
};

typedef struct bsm_pt_settings {
    float ray_length;          /* PathTracingSettings::ray_length, default 100 (basic.hpp:77) */
    uint32_t max_bounces;      /* PathTracingSettings::max_bounces (>=2); segments = max_bounces - 1 */
    uint32_t accumulate;       /* PathTracingSettings::accumulate: add to the view's history */
    uint32_t denoise;          /* PathTracingSettings::denoise: accepted and ignored, as in the reference PT */
    uint32_t spp;              /* samples per pixel in this call */
    uint32_t max_segments;     /* extend stages including the primary ray; 0 = max_bounces - 1 */
    uint64_t seed;             /* scene seed for the PCG32 per-pixel streams */
    uint32_t sample_offset;    /* index of the first sample (progressive rendering) */
    uint32_t flags;            /* BSM_PT_* */
    float t_min;               /* ray TMin; 0 = default 0 (origins are offset instead) */
    float ray_offset;          /* origin offset along the geometric normal; 0 = 2e-5 * scene extent */
    uint32_t wavefront_capacity; /* paths in flight per chunk; 0 = the whole call up to 2^27 paths, within
                                    half of the device memory the budget has left */
    uint32_t block_size;       /* threads per block of the traversal kernels; 0 = tuned default */
} bsm_pt_settings;

/* Fills `s` with the reference defaults plus spp = 1, seed = 1. */
BSM_API void bsm_pt_settings_default(bsm_pt_settings* s);

typedef struct bsm_view_output {
    float* rgba;             /* width*height RGBA fp32 (mean radiance), row pitch below */
    uint32_t row_pitch_px;   /* 0 = width */
    uint32_t location;       /* BSM_HOST or BSM_DEVICE */
} bsm_view_output;

#define BSM_MAX_SEGMENTS 16
typedef struct bsm_render_stats {
    uint64_t paths;
    uint64_t extend_rays;                 /* rays that entered the closest-hit kernel */
    uint64_t shadow_rays;                 /* rays that entered the any-hit kernel */
    uint64_t rays_per_segment[BSM_MAX_SEGMENTS];
    uint32_t chunks;
    uint32_t extend_launches;
    float ms_total;                       /* device time of the whole render (events) */
    float ms_camera, ms_extend, ms_shade, ms_shadow, ms_resolve; /* BSM_PT_STAGE_TIMING only */
    uint64_t traversal_nodes;             /* BSM_PT_COUNT_TRAVERSAL only: nodes visited by extend rays */
    uint64_t traversal_tris;              /* BSM_PT_COUNT_TRAVERSAL only: triangles tested by extend rays */
} bsm_render_stats;

/* Renders `n_views` views of one scene (PathTracingPass::render for each
 * camera).  With settings->accumulate the samples are added to the view's
 * history (kept per view index, reset when the camera or size changes, as
 * path_tracing.cpp:224-245 does); outputs receive the running mean.
 * `outputs` may be NULL to keep the result on the device (bsm_read_view).
 * `stats` may be NULL.
 * Asynchronous when every output is in device memory (or `outputs` is NULL),
 * `stats` is NULL and BSM_PT_STAGE_TIMING is not set: the call queues the
 * render on the work stream and returns; bsm_sync or bsm_render_stats_read
 * wait for it.  A host output, a non-NULL `stats` or stage timing make the
 * call wait for the render (and report device errors).  The first render of a
 * new view layout or a larger wavefront allocates and waits. */
BSM_API bsm_status bsm_render(bsm_context* ctx, uint32_t scene_id, const bsm_camera* views, uint32_t n_views,
                              const bsm_pt_settings* settings, const bsm_view_output* outputs,
                              bsm_render_stats* stats);
/* Waits for the last render issued on the context (bsm_render, bsm_render_batch,
 * bsm_render_cached) and returns its statistics; BSM_ERR_DEVICE_CHECK if a device
 * error flag is set (the flag is then cleared).  BSM_ERR_NOT_FOUND before any
 * render.  No reference counterpart (the engine's profiler scopes, not its
 * pass, time the frame). */
BSM_API bsm_status bsm_render_stats_read(bsm_context* ctx, bsm_render_stats* stats);
/* One view of a batched render: its camera, samples per pixel, segment limit
 * and seed (0 = the value in the settings). */
typedef struct bsm_view_desc {
    bsm_camera camera;
    uint32_t spp;
    uint32_t max_segments;
    uint64_t seed;
} bsm_view_desc;

/* Renders many views of different sizes and sample counts in one wavefront:
 * all views' paths share the queues and one CUDA graph replays the whole
 * bounce loop.  Each view's result equals a bsm_render of that view alone with
 * the same spp, segments and seed (same paths; per-pixel sums in another
 * order).  Replaces a loop of PathTracingPass::render over cameras
 * (graphics_manager.cpp:407-427 runs one per enabled camera). */
BSM_API bsm_status bsm_render_batch(bsm_context* ctx, uint32_t scene_id, const bsm_view_desc* views,
                                    uint32_t n_views, const bsm_pt_settings* settings,
                                    const bsm_view_output* outputs, bsm_render_stats* stats);

/* Launch parameters the autotuner chooses. */
typedef struct bsm_tune_params {
    uint32_t block_size;          /* threads per block of the traversal kernels: 64, 128 or 256 */
    uint32_t wavefront_capacity;  /* paths per chunk (queue capacity) */
    uint32_t postpone_depth;      /* traversal stack entries open to postponed triangle groups (0..16) */
    uint32_t refill_lanes;        /* idle lanes that make a warp fetch new rays (1..32) */
    uint32_t register_cap;        /* 1: traversal kernels limited to 64 registers (more warps per SM) */
} bsm_tune_params;

typedef struct bsm_tune_result {
    bsm_tune_params best;
    float best_ms;                /* device time of the tuning workload with `best` */
    float default_ms;             /* ... with the built-in defaults */
    uint32_t tried;               /* configurations timed (0 when read from the cache file) */
    uint32_t from_cache;
    float worst_ms;               /* ... with the slowest configuration timed (what a bad choice costs) */
    uint32_t reserved;
} bsm_tune_result;

/* Picks block size, queue capacity and traversal stack budget for a scene and
 * a workload (views + settings) by timing short renders (each view at
 * max(1, spp / 16) samples), coordinate descent over the four parameters.  The
 * result is kept for the scene (used whenever the settings leave these fields
 * at 0) and, when `cache_path` is not NULL, appended to that text file keyed
 * by GPU name, SM count, scene size and path count, and read back from it on
 * later calls.  No reference counterpart (the driver picks these for its RT
 * pipeline). */
BSM_API bsm_status bsm_autotune(bsm_context* ctx, uint32_t scene_id, const bsm_view_desc* views, uint32_t n_views,
                                const bsm_pt_settings* settings, const char* cache_path, bsm_tune_result* result);
/* Sets a scene's launch parameters by hand (NULL clears them). */
BSM_API bsm_status bsm_set_tuning(bsm_context* ctx, uint32_t scene_id, const bsm_tune_params* params);

/* Reads the current mean of a view's history into `out`. */
BSM_API bsm_status bsm_read_view(bsm_context* ctx, uint32_t view_index, const bsm_view_output* out);
/* Exports / imports a view's raw history (sum RGB + sample count) so a render
 * can resume to more samples.  `sums` holds width*height*4 floats. */
BSM_API bsm_status bsm_export_history(bsm_context* ctx, uint32_t view_index, float* sums, uint32_t* spp,
                                      uint32_t location);
BSM_API bsm_status bsm_import_history(bsm_context* ctx, uint32_t view_index, const bsm_camera* camera,
                                      const float* sums, uint32_t spp, uint32_t location);

/* ---- stage entry points (TraceRay closest hit / any hit) --------------- */

/* rays: n * 8 floats (ox, oy, oz, tmin, dx, dy, dz, tmax).
 * hits: n * 4 words (t as f32, primitive id as u32, u, v as f32); a miss has
 * primitive id 0xffffffff and t = tmax.  Replaces TraceRay in rt_gbuffer_rgen
 * with the closest-hit shader (rt_gbuffer.hlsl:7-36, rt_gbuffer_hit.hlsl:6-18).
 * With location BSM_DEVICE both buffers are device memory and the call is
 * asynchronous on the work stream; with BSM_HOST it waits. */
BSM_API bsm_status bsm_trace_closest(bsm_context* ctx, uint32_t scene_id, const float* rays, uint32_t n,
                                     void* hits, uint32_t location);
/* occluded: n bytes, 1 if any triangle lies in (tmin, tmax].  Replaces the
 * any-hit path (rt_gbuffer_hit.hlsl:20-35) for opaque geometry. */
BSM_API bsm_status bsm_trace_any(bsm_context* ctx, uint32_t scene_id, const float* rays, uint32_t n,
                                 uint8_t* occluded, uint32_t location);

/* Per-ray traversal counters: counts[2*i] = BVH nodes visited, counts[2*i+1] =
 * triangles tested, for the closest-hit traversal of ray i (host buffers).
 * No reference counterpart: it measures the traversal working set. */
BSM_API bsm_status bsm_trace_counts(bsm_context* ctx, uint32_t scene_id, const float* rays, uint32_t n,
                                    uint32_t* counts);

/* ---- primary-hit outputs (depth, G-buffer) ------------------------------ */

/* The outputs of PathTracingPass::render besides the colour
 * (path_tracing.hpp:20-25, OutputData{depth, velocity, gbuffer}; velocity is
 * invalid there too).  Each array is width*height, row-major, tightly packed;
 * a NULL pointer skips that output. */
typedef struct bsm_primary_output {
    float* depth;           /* f32 reverse-Z device depth of the primary hit, 0 on a miss
                               (pt_depth.hlsl:7-16, depth.hlsl:3-4) */
    float* gbuffer[4];      /* float4 each: base_color, normal_roughness, fresnel, material_0 as
                               pack_surface_to_gbuffer packs them (renderer/gbuffer.hlsl:6-31);
                               zero on a miss */
    float* hit_positions;   /* float4: (position, t), or (direction, -1) on a miss (rt_gbuffer.hlsl:28-35) */
    uint32_t location;      /* BSM_HOST or BSM_DEVICE */
} bsm_primary_output;

/* Traces one pixel-centre camera ray per pixel and writes the primary-hit
 * outputs: the "PT Trace GBuffer #1" and "PT Depth" passes of
 * PathTracingPass::render (path_tracing.cpp:362-395, 437-448).  The primary
 * hit is the one the colour pass's first segment finds for an unjittered
 * sample (same ray, same t_min / ray_length from `settings`; NULL = defaults).
 * `near_z` / `far_z` are the camera's clip planes for the reverse-Z
 * projection (camera.hpp:54-55; 0 = the reference defaults 0.01 / 10000).
 * Asynchronous on the work stream for device outputs; waits for host outputs. */
BSM_API bsm_status bsm_render_primary(bsm_context* ctx, uint32_t scene_id, const bsm_camera* camera,
                                      const bsm_pt_settings* settings, float near_z, float far_z,
                                      const bsm_primary_output* out);

/* Page-locked host memory for fast host<->device copies (cudaHostAlloc). */
BSM_API bsm_status bsm_host_alloc(bsm_context* ctx, uint64_t bytes, void** ptr);
BSM_API bsm_status bsm_host_free(bsm_context* ctx, void* ptr);

/* Renders one view without allocating any device memory.  No counterpart in
 * the reference: it exists for callers that cannot call cudaMalloc while they
 * render — an engine that owns all device memory through its own allocator and
 * budget, a frame loop that must not take the synchronisation an allocation can
 * cost, a host with a fixed memory arena.  The scene must already be resident
 * (bsm_scene_upload + bsm_scene_build_bvh, done at set-up).  The working memory
 * (queue counters, the view record, the wavefront queues) is one fixed 64 MiB
 * device array inside the library, held by every GPU that loads it until the
 * process exits; it bounds a chunk to wavefront_capacity paths (0 = the
 * maximum, 279,552 paths for one light in an opaque scene, 270,336 when
 * some material is not opaque); a larger wavefront_capacity is
 * rejected with BSM_ERR_INVALID_ARG.  Any image size works: paths run in chunks.
 * `out_rgba` is a caller-owned device buffer of width*height RGBA floats,
 * tightly packed and 16-byte aligned (else BSM_ERR_INVALID_ARG); it receives
 * the per-pixel sums and then the mean of this call's samples.  Settings the
 * call does not use: `accumulate` (every call writes a fresh mean), `denoise`,
 * and flags other than BSM_PT_JITTER, BSM_PT_NO_SUN_NEE and BSM_PT_NO_SKY_NEE;
 * `block_size` must be 0, 64, 128 or 256 and the kernels run with 128.  The
 * first call on a device looks up the array's device address (set-up); make
 * that first call before any stream capture.  All calls share the array and it
 * keeps the last call's contents, so calls that overlap on the GPU race (that
 * includes the array's device error word, which a sync point of any context
 * that called this entry point reads and clears).  The call is asynchronous on
 * the work stream; bsm_sync waits for it and reports a queue overflow of the
 * call as BSM_ERR_DEVICE_CHECK. */
BSM_API bsm_status bsm_render_noalloc(bsm_context* ctx, uint32_t scene_id, const bsm_camera* camera,
                                      const bsm_pt_settings* settings, float* out_rgba);

/* ---- serving: resident scenes, requests admitted by memory, continuous batching ---- */

typedef struct bsm_server_opts {
    uint64_t pool_bytes;          /* accumulator pool: admission budget (16 B per pixel, 24 with
                                     BSM_SERVER_DETERMINISTIC); 0 = 1 GiB */
    uint32_t chunk_paths;         /* paths per in-flight chunk (queue capacity of a lane); 0 = 2^21 */
    uint32_t lanes;               /* chunks in flight at once, one CUDA stream each; 0 = 4 */
    uint32_t max_views_per_chunk; /* request ranges one chunk can hold; 0 = 256 */
    uint32_t flags;               /* BSM_SERVER_* (0: FP32 atomic sums) */
} bsm_server_opts;

enum {
    /* every request sums its contributions as exact 32.32 fixed-point integers (24 B per pixel of the pool
       instead of 16), as BSM_PT_DETERMINISTIC does for bsm_render: a result is then the same bit for bit
       alone, in any mix of requests, and as bsm_render with that flag renders it */
    BSM_SERVER_DETERMINISTIC = 1u << 0
};

typedef struct bsm_request {
    uint32_t scene_id;
    bsm_camera camera;            /* at most 1920 x 1080 pixels */
    uint32_t spp;
    uint32_t max_segments;        /* 0 = 8 */
    uint64_t seed;
    float* out_rgba;              /* host buffer of width*height RGBA floats, written when done;
                                     must stay valid until the request is done */
} bsm_request;

enum { BSM_REQ_QUEUED = 0, BSM_REQ_RUNNING = 1, BSM_REQ_DONE = 2, BSM_REQ_FAILED = 3, BSM_REQ_CANCELLED = 4 };

typedef struct bsm_request_status {
    uint32_t state;               /* BSM_REQ_* */
    uint32_t cancelled;           /* bsm_server_cancel was called (the state may still be DONE) */
    double submit_ms, admit_ms, done_ms;  /* since bsm_server_start */
    uint64_t paths;
} bsm_request_status;

typedef struct bsm_server_stats {
    uint64_t submitted, admitted, completed, rejected;
    uint64_t extend_rays, shadow_rays;
    uint64_t pool_bytes, pool_used_bytes;
    uint32_t active, queued;
    double elapsed_ms;
    uint64_t cancelled;
} bsm_server_stats;

/* Starts the serving loop on a context: a worker thread that admits requests
 * in arrival order as accumulator memory frees up and packs the paths of all
 * admitted requests of a scene into shared wavefront chunks, several chunks in
 * flight on separate streams.  A request's image equals bsm_render of the same
 * camera, spp, segments and seed.  Scenes must not be uploaded or released
 * while the server runs.  No reference counterpart (the engine renders its
 * cameras once per window frame, graphics_manager.cpp:407-427). */
BSM_API bsm_status bsm_server_start(bsm_context* ctx, const bsm_server_opts* opts);
/* Queues a request; BSM_ERR_ADMISSION if it can never fit the pool. */
BSM_API bsm_status bsm_server_submit(bsm_context* ctx, const bsm_request* request, uint64_t* request_id);
BSM_API bsm_status bsm_server_poll(bsm_context* ctx, uint64_t request_id, bsm_request_status* status);
/* Waits for a request (timeout_ms = 0: no limit); BSM_ERR_TIMEOUT when it runs out,
 * BSM_ERR_CANCELLED for a cancelled request. */
BSM_API bsm_status bsm_server_wait(bsm_context* ctx, uint64_t request_id, uint32_t timeout_ms,
                                   bsm_request_status* status);
BSM_API bsm_status bsm_server_get_stats(bsm_context* ctx, bsm_server_stats* stats);
/* Cancels a request.  A queued one is dropped at once; a running one issues no
 * more paths and gives its accumulator back to the pool when its chunks in
 * flight finish (state BSM_REQ_CANCELLED).  If its output copy is already
 * queued the call waits for it and the request completes normally.  Either way
 * the library writes nothing into the request's out_rgba after the call
 * returns, so the caller may free it.  No-op on finished requests.  No
 * reference counterpart (the engine has no request queue). */
BSM_API bsm_status bsm_server_cancel(bsm_context* ctx, uint64_t request_id);
/* Stops the worker after the chunks in flight; queued requests are dropped. */
BSM_API bsm_status bsm_server_stop(bsm_context* ctx);

/* ---- radiance cache (learned) ------------------------------------------ */

/* A small BF16 MLP (64 encoded inputs, 4 hidden ReLU layers of 64, RGB out,
 * FP32 accumulation on the tensor cores) trained online on the path vertices
 * the tracer generates.  Paths terminate into it after a short prefix.  No
 * reference counterpart: the engine's DDGI probes (ddgi_update.cpp) are its
 * closest relative, and the plain pass stays the fallback and the yardstick
 * of its error. */
typedef struct bsm_cache bsm_cache;

typedef struct bsm_cache_settings {
    uint32_t cache_segment;   /* hits of this segment query the cache (2 = after two bounces) */
    uint32_t train_paths;     /* full-length training paths per frame (32768) */
    uint32_t train_segments;  /* their maximum segments (8) */
    uint32_t train_batch;     /* samples per Adam step (16384) */
    uint32_t train_steps;     /* Adam steps per frame (4); 0 = render only */
    float lr;                 /* Adam learning rate (1e-2) */
    float ema_decay;          /* renders read an exponential moving average of the weights with this
                                 decay per Adam step (bias-corrected); 0 = the current weights */
    float min_roughness;      /* a hit of the cache segment or later whose roughness is below this does not
                                 query the cache: the path shades it and goes on (a near-mirror vertex's
                                 outgoing radiance holds a sun glint the network cannot resolve) */
    uint32_t extra_segments;  /* segments a path may go past cache_segment looking for a rough enough hit;
                                 the last one queries the cache whatever its roughness */
} bsm_cache_settings;

BSM_API void bsm_cache_settings_default(bsm_cache_settings* cs);
/* Number of network parameters (fp32 master weights, row-major W0..W3 [64][64], W4 [8][64]). */
BSM_API uint32_t bsm_cache_param_count(void);
/* Creates a cache on ctx's device with He-uniform random weights from `seed`. */
BSM_API bsm_status bsm_cache_create(bsm_context* ctx, uint64_t seed, bsm_cache** cache);
BSM_API void bsm_cache_destroy(bsm_cache* cache);
/* Reads (get != NULL) and/or writes (set != NULL) the fp32 master weights; a write resets Adam. */
BSM_API bsm_status bsm_cache_weights(bsm_cache* cache, float* get, const float* set);
/* Reads the weights renders use (bsm_cache_param_count floats): the bias-corrected moving average of the
 * master weights over the Adam steps taken with ema_decay > 0, or the master weights before any. */
BSM_API bsm_status bsm_cache_render_weights(bsm_cache* cache, float* out);
/* samples: n x 16 floats (12 raw inputs, 3 target radiance, 1 unused), host memory.
 * Prediction (n x 3) / gradient of the mean relative L2 loss (bsm_cache_param_count floats).
 * Prediction runs the render's tcgen05 inference kernel; BSM_ERR_DEVICE_CHECK if one of its bounded
 * tensor-core waits gave up (a render reports the same through its device error word). */
BSM_API bsm_status bsm_cache_predict(bsm_cache* cache, const float* samples, uint32_t n, float* out);
BSM_API bsm_status bsm_cache_gradient(bsm_cache* cache, const float* samples, uint32_t n, float* dW, float* loss);
/* Adam steps over `samples` in batches; returns the mean loss. */
BSM_API bsm_status bsm_cache_train(bsm_cache* cache, const float* samples, uint32_t n, uint32_t batch, float lr,
                                   float* loss);
BSM_API bsm_status bsm_cache_save(bsm_cache* cache, const char* path);
BSM_API bsm_status bsm_cache_load(bsm_cache* cache, const char* path);

/* One frame with the cache: optionally trains on `train_paths` fresh full-length
 * paths of this camera, then renders with paths terminated into the cache at
 * `cache_segment` (settings->max_segments is ignored).  `train_loss` may be NULL.
 * stats->ms_total is the device time of the whole frame, training included. */
BSM_API bsm_status bsm_render_cached(bsm_context* ctx, uint32_t scene_id, const bsm_camera* camera,
                                     const bsm_pt_settings* settings, bsm_cache* cache,
                                     const bsm_cache_settings* cache_settings, const bsm_view_output* output,
                                     bsm_render_stats* stats, float* train_loss);

/* ---- instancing: two-level scenes --------------------------------------- */

/* An object-space mesh with its own BVH (the reference's per-mesh BLAS,
 * accel.cpp:11-87).  Material ids index the materials of the scenes that
 * instance it. */
typedef struct bsm_geometry_desc {
    uint32_t num_vertices;
    const float* positions;       /* 3 * num_vertices, object space */
    uint32_t num_triangles;
    const uint32_t* indices;      /* 3 * num_triangles, or NULL for a soup */
    const uint32_t* material_ids; /* num_triangles, or NULL (all 0) */
} bsm_geometry_desc;

BSM_API bsm_status bsm_geometry_create(bsm_context* ctx, const bsm_geometry_desc* desc, const bsm_bvh_opts* opts,
                                       uint32_t* geometry_id);
/* Fails with BSM_ERR_BAD_STATE while a scene instances the geometry. */
BSM_API bsm_status bsm_geometry_release(bsm_context* ctx, uint32_t geometry_id);

/* One drawable of a two-level scene (the reference's TLAS instance,
 * accel.cpp:104-132). */
typedef struct bsm_instance {
    uint32_t geometry_id;
    uint32_t material_id;     /* material of every triangle, or 0xffffffff: the geometry's ids */
    float transform[12];      /* object to world, row-major 3x4 (rows of Transform::matrix()) */
} bsm_instance;

typedef struct bsm_instanced_scene_desc {
    uint32_t num_instances;
    const bsm_instance* instances;
    uint32_t num_materials;
    const bsm_material* materials;
    uint32_t num_dir_lights;
    const bsm_dir_light* dir_lights;
    bsm_sky sky;
    uint32_t num_point_lights;
    const bsm_point_light* point_lights;
    uint32_t num_rect_lights;
    const bsm_rect_light* rect_lights;
} bsm_instanced_scene_desc;

/* Creates a scene over instances of geometries: a TLAS (the same compressed
 * 8-wide BVH, one instance per leaf) over the instances' world boxes; rays
 * enter an instance's BLAS in its object space.  The scene renders and
 * traces like any other (bsm_render*, bsm_trace_*, the server, the cache);
 * primitive ids are global: the sum of the earlier instances' triangle
 * counts plus the triangle's index in its geometry.  bsm_scene_build_bvh on
 * it rebuilds the TLAS from the current transforms. */
BSM_API bsm_status bsm_scene_create_instanced(bsm_context* ctx, const bsm_instanced_scene_desc* desc,
                                              uint32_t* scene_id);
/* New object-to-world transforms (12 floats per instance, in creation order)
 * and a refit of the TLAS on the GPU: the world boxes change, the tree's
 * topology stays (the reference rebuilds its TLAS every frame,
 * accel.cpp:139-158; a refit keeps the per-frame cost to one small kernel per
 * TLAS level).  The scene bounds (ray offsets, radiance-cache inputs) follow
 * the new instance boxes, as after a rebuild; when they change, the next
 * render re-captures its CUDA graph.  Synchronous. */
BSM_API bsm_status bsm_scene_update_instances(bsm_context* ctx, uint32_t scene_id, const float* transforms,
                                              uint32_t num_instances);

/* ---- the reference's on-disk formats ----------------------------------- */

/* SubmeshDesc (graphics/mesh.hpp:16-22); topology 3 = triangle_list (rhi/pipeline.hpp:34-43). */
typedef struct bsm_submesh {
    uint32_t base_vertex;
    uint32_t index_offset;
    uint32_t num_indices;     /* with no index data: the number of vertices; ~0 = to the end */
    uint32_t topology;
} bsm_submesh;

/* MeshData (graphics/mesh.hpp:24-80): the arrays of a StaticMesh asset.  Each
 * attribute array has its own element count (0 / NULL when absent). */
typedef struct bsm_mesh_data {
    uint32_t num_vertices;
    const float* positions;   /* 3 * num_vertices */
    uint32_t num_normals;
    const float* normals;     /* 3 * num_normals */
    uint32_t num_tangents;
    const float* tangents;    /* 4 * num_tangents */
    uint32_t num_colors;
    const float* colors;      /* 3 * num_colors */
    uint32_t num_texcoords;
    const float* texcoords;   /* 2 * num_texcoords */
    uint32_t num_texcoords2;
    const float* texcoords2;  /* 2 * num_texcoords2 */
    uint32_t num_indices;
    const uint32_t* indices;
    uint32_t num_submeshes;
    const bsm_submesh* submeshes;
    void* handle;             /* owner of the arrays (bsm_static_mesh_free) */
} bsm_mesh_data;

/* Reads a .static_mesh.biasset file image (StaticMesh::load,
 * scene_basic/static_mesh.cpp:10-31): magic 0x0b1a55e7, type name
 * "StaticMesh", version 1 (raw MeshData stream) or 2 (zlib-compressed
 * MeshData stream, prelude/byte_stream.cpp:28-41).  Truncated or corrupt
 * files are rejected (the reference reads past them silently); `error`
 * (may be NULL) receives the reason.  Arrays belong to the library until
 * bsm_static_mesh_free. */
BSM_API bsm_status bsm_static_mesh_read(const void* bytes, uint64_t size, bsm_mesh_data* mesh, char* error,
                                        uint32_t error_len);
BSM_API void bsm_static_mesh_free(bsm_mesh_data* mesh);
/* Writes a .static_mesh.biasset image of `mesh` (StaticMesh::save,
 * static_mesh.cpp:33-42), version 1 or 2 (zlib stream of stored blocks).
 * With out == NULL only *out_size is set. */
BSM_API bsm_status bsm_static_mesh_write(const bsm_mesh_data* mesh, uint32_t version, void* out,
                                         uint64_t out_capacity, uint64_t* out_size);

typedef struct bsm_project_info {
    bsm_camera camera;                 /* first CameraComponent (camera_system.cpp:17-29) */
    float near_z, far_z;               /* its clip planes (for bsm_render_primary) */
    uint32_t has_camera;
    uint32_t camera_orthographic;      /* orthographic cameras are not supported by the pass */
    bsm_pt_settings settings;          /* defaults + the path_tracing block of a BasicRendererOverrideVolume */
    uint32_t num_objects;
    uint32_t num_drawables;            /* (object, submesh) pairs placed in the scene */
    uint32_t num_skipped_submeshes;    /* non-triangle-list topologies */
    uint32_t num_materials_approximated; /* material functions beyond constant assignments */
    uint32_t num_non_opaque_materials; /* alpha-test / translucent blend modes (any-hit opacity rule) */
    uint32_t num_unsupported_lights;   /* textured rect lights (traced with their constant emission) */
    uint32_t has_skybox;               /* a SkyboxComponent (its cube texture is not read: sky is black) */
    char error[256];                   /* reason of a failed load */
} bsm_project_info;

/* Loads a reference project directory (project.toml -> asset_metadata.toml,
 * scene.toml; runtime/scene.cpp:103-135) into a scene description: every
 * StaticMeshComponent + MeshRendererComponent object's submeshes
 * (static_mesh_render_system.cpp:56-79) in world space (Transform,
 * math/transform.cpp:120-124, parents applied), its materials from their
 * TOML (scene_basic/material.cpp:12-53; constant base colour / roughness /
 * f0 / metallic / opacity, blend mode), directional, point / spot and rect
 * light components (renderer/context/lights.cpp:55-65, 120-139, 210-228), and
 * the first camera.  Arrays belong
 * to the library until bsm_project_free. */
BSM_API bsm_status bsm_project_load(const char* project_dir, bsm_scene_desc* desc, bsm_project_info* info);
BSM_API void bsm_project_free(bsm_scene_desc* desc);
/* Parses a TOML text with the reader bsm_project_load uses (syntax check). */
BSM_API bsm_status bsm_toml_check(const char* text, char* error, uint32_t error_len);

/* ---- synthetic scenes --------------------------------------------------- */

enum {
    BSM_SCENE_ROOM = 0,     /* 12 quads + 64 icospheres, constant sky (20,504 triangles) */
    BSM_SCENE_TERRAIN = 1   /* fBm heightfield + UV spheres, baked gradient sky */
};
typedef struct bsm_scene_gen_params {
    uint32_t kind;           /* BSM_SCENE_* */
    uint64_t seed;
    uint32_t grid;           /* terrain vertices per side (512 for 1,482,242 triangles) */
    uint32_t spheres;        /* terrain: UV spheres (2000); room: icospheres (64) */
    uint32_t sky_width, sky_height; /* terrain sky map (1024 x 512) */
} bsm_scene_gen_params;

/* Generates a procedural scene.  The arrays in `desc` belong to the library
 * until bsm_scene_gen_free(desc).  `camera` receives the scene's fixed camera
 * (width/height left as passed in). */
BSM_API bsm_status bsm_scene_generate(const bsm_scene_gen_params* params, bsm_scene_desc* desc,
                                      bsm_camera* camera);
BSM_API void bsm_scene_gen_free(bsm_scene_desc* desc);

#ifdef __cplusplus
}
#endif
#endif /* BSM_PT_H */
