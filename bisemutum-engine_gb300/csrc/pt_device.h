// pt_device.h — device-side structures of the wavefront pass and the launch
// wrappers the host orchestration (api.cpp) calls.
//
// HBM layout of one wavefront chunk (capacity C paths, L directional lights):
//   ray_o[2][C]  float4  origin.xyz, tmin            (ping-pong queues)
//   ray_d[2][C]  float4  direction.xyz, tmax
//   path[2][C]   uint4   accum index, flags (segment | max segments | view),
//                        PCG32 state low/high word
//   thr[2][C]    float4  throughput.rgb, pdf of the sampled direction
//   hit[C]       float4  t, leaf triangle index, u, v
//   sh_o/sh_d/sh_c[(L+1) C] float4  shadow rays and their contributions: sun
//                rays fill the queue from the front, sky rays from the back, so
//                a warp of the any-hit kernel traces rays of one kind
//   sh_seed[(L+1) C] uint32  opacity seed of each shadow ray (scenes with
//                non-opaque triangles; extension rays use the path's PCG word)
//   counters     uint32  queue sizes per segment, work counters, error flags
//   stats        uint64  rays per segment (summed over chunks)
// All queues are structures of arrays read with 128-bit loads.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bvh_layout.h"

namespace bsm {

constexpr int kMaxLights = 8;     // directional + point/spot + rect lights of a scene

// A light of the scene, four float4 (kind in a.w's bits):
//   directional: a = (direction to the light, 0), b = (emission, 0)
//   point/spot:  a = (position, 1), b = (emission, 1 / range^2), c = (direction to the light, cos_inner),
//                d = (cos_outer, 0, 0, 0)
//   rect:        a = (corner (-w, -h), 2), b = (emission, two_sided), c = (edge along x, area),
//                d = (edge along y, 0); the unit normal (local +z) is normalize(cross(c, d))
enum : uint32_t { kLightDir = 0, kLightPoint = 1, kLightRect = 2 };
struct DevLight { float4 a, b, c, d; };
constexpr int kMaxSeg = 16;

struct DevSky {
    uint32_t kind;             // BSM_SKY_CONSTANT / BSM_SKY_EQUIRECT
    uint32_t width, height;
    float cr, cg, cb;          // colour / multiplier
    const ushort4* texels;     // width*height RGBA16F
    const uint2* alias;        // height * width alias entries (bits of the keep probability, alias texel)
    const float* pdf_tab;      // height * width: pdf in (u,v) space
};

struct DevScene {
    const CwNode* nodes;       // the BVH; in a two-level scene the TLAS
    const CwTri* tris;         // leaf-ordered triangles (null in a two-level scene)
    const float4* tri_normals; // single-level scenes with vertex normals: 3 per leaf triangle (xyz), else null
    const InstDev* insts;      // two-level scene: instances in TLAS leaf order, else null
    uint32_t num_instances;
    const float* mat_tr;       // two-level scene with non-opaque materials: per-material transparency, else null
    const float4* materials;   // 2 per material: (base.rgb, roughness), (f0.rgb, metallic)
    uint32_t num_materials;
    uint32_t num_lights;       // all kinds; the shadow queue has num_lights + 1 slots per path
    DevLight lights[kMaxLights];
    DevSky sky;
    uint32_t has_non_opaque;   // some triangle has a transparency (alpha test / translucent)
    uint32_t dir_lights_only;  // every light is directional (the shading kernel's slim variant)
    float ray_offset;          // origin offset along the geometric normal
    float box_lo[3];           // scene bounds: radiance-cache inputs are normalised to them
    float box_inv[3];
};

struct DevView {
    float pos[3]; float tan_half;
    float s[3]; float aspect;
    float u[3]; float ray_length;
    float f[3]; float t_min;
    uint32_t width, height, spp, sample_offset;
    uint64_t seed;
    uint64_t path_base;        // first path index of this view in the render's path space
    uint32_t accum_base;       // first accumulator pixel of this view
    uint32_t max_segments;
    uint32_t flags;            // BSM_PT_* bits that reach the device
    uint32_t cache_segment;    // >0: hits of this segment query the radiance cache instead of shading
    uint64_t first_path;       // index (within the view) of the path at path_base; >0 when a view is split
    float cache_min_rough;     // hits smoother than this do not query the cache (but the last segment's do)
    uint32_t pad;
};

// counters[] word offsets
enum : uint32_t {
    kCntQueue = 0,                 // [kMaxSeg + 1] extend queue size entering segment s
    kCntShadow = kCntQueue + 17,   // [kMaxSeg] sun shadow rays of segment s (queue front)
    kCntWork = kCntShadow + 16,    // [2 * kMaxSeg] persistent-kernel work counters
    kCntSky = kCntWork + 32,       // [kMaxSeg] sky shadow rays of segment s (queue back)
    kCntCache = kCntSky + 16,      // radiance-cache queries of the chunk
    kCntError = kCntCache + 1,     // error flags (bit 0: queue overflow, bit 1: a tensor-core wait timed out);
                                   // words below it are cleared per chunk
    kCntWords = kCntError + 1
};
// stats[] (uint64) offsets
enum : uint32_t {
    kStatExtend = 0,               // [kMaxSeg]
    kStatShadow = kMaxSeg,         // [kMaxSeg]
    kStatNodes = 2 * kMaxSeg,      // traversal counters (counting extend variant)
    kStatTris = 2 * kMaxSeg + 1,
    kStatWords = 2 * kMaxSeg + 2
};

struct Wavefront {
    uint32_t capacity;
    float4* ray_o[2];
    float4* ray_d[2];
    uint4* path[2];
    float4* thr[2];
    float4* hit;
    float4* sh_o;
    float4* sh_d;
    float4* sh_c;
    uint32_t* sh_seed;         // [(L+1) C] opacity seeds of the shadow rays (written for non-opaque scenes)
    float4* cache_q;           // radiance-cache queries (4 float4 each), capacity C; may be null
    // BSM_PT_DETERMINISTIC: the call's per-pixel sums as 32.32 fixed point (3 words per accumulator pixel);
    // null: contributions go to the FP32 accumulator by atomics
    unsigned long long* accum_fx;
    uint32_t* counters;
    unsigned long long* stats;
};

struct LaunchCfg {
    int grid_persistent;    // blocks for the persistent traversal kernels
    int grid_persistent2;   // blocks for the persistent two-level traversal kernels
    int block_trace;        // threads per block, traversal
    int block_shade;        // threads per block, shading / camera
    int grid_shade;
    int postpone_sp = 16;   // traversal stack budget for postponed triangle groups
    int refill_min = 8;     // idle lanes that trigger a warp refill
    int regcap = 1;         // 1: traversal kernels compiled for 4 blocks of 256 (64 registers); the default
};

#if defined(__CUDACC__)
// Adds the contribution (x, y, z) to accumulator pixel `idx` of 32.32 fixed-point sums: each positive value
// is rounded once to a multiple of 2^-32 and added as an integer, which makes the sums independent of the
// order of the additions.  Zero, negative and NaN values add nothing.
__device__ __forceinline__ void accum_fixed_add(unsigned long long* fx, uint32_t idx, float x, float y, float z) {
    unsigned long long* p = fx + 3 * (size_t)idx;
    if (x > 0.0f) atomicAdd(p, __float2ull_rn(x * 4294967296.0f));
    if (y > 0.0f) atomicAdd(p + 1, __float2ull_rn(y * 4294967296.0f));
    if (z > 0.0f) atomicAdd(p + 2, __float2ull_rn(z * 4294967296.0f));
}
#endif

// ---- launch wrappers (pt_kernels.cu) ----
void launch_camera(const LaunchCfg& lc, cudaStream_t st, const DevView* views, uint32_t n_views,
                   uint64_t path_begin, uint32_t path_count, const Wavefront& wf, uint32_t max_segments);
void launch_extend(const LaunchCfg& lc, cudaStream_t st, const DevScene& sc, const Wavefront& wf, int q,
                   uint32_t seg, bool count_traversal);
// `cache`: some view of the launch queries the radiance cache
void launch_shade(const LaunchCfg& lc, cudaStream_t st, const DevScene& sc, const DevView* views,
                  const Wavefront& wf, int q, uint32_t seg, float4* accum, bool cache = false);
void launch_shadow(const LaunchCfg& lc, cudaStream_t st, const DevScene& sc, const Wavefront& wf, uint32_t seg,
                   float4* accum);
void launch_resolve(cudaStream_t st, const float4* accum, uint32_t width, uint32_t height, float inv_spp,
                    float4* out, uint32_t pitch_px);
// accum[p] += fx[3p .. 3p + 2] * 2^-32 for the n accumulator pixels (one add per pixel: deterministic)
void launch_fold_fixed(cudaStream_t st, const unsigned long long* fx, float4* accum, uint32_t n);
// launch_resolve from fixed-point sums: out = (fx * 2^-32 as float) * inv_spp, alpha 1 (the same values as a
// fold into a cleared accumulator followed by launch_resolve)
void launch_resolve_fixed(cudaStream_t st, const unsigned long long* fx, uint32_t width, uint32_t height,
                          float inv_spp, float4* out, uint32_t pitch_px);
void launch_trace_closest(cudaStream_t st, const DevScene& sc, const float4* rays, uint32_t n, uint4* hits,
                          int block);
void launch_trace_any(cudaStream_t st, const DevScene& sc, const float4* rays, uint32_t n, uint8_t* occluded,
                      int block);
void launch_trace_count(cudaStream_t st, const DevScene& sc, const float4* rays, uint32_t n, uint2* counts);
// Vertex normals of every leaf triangle in leaf order (3 float4 each) from per-vertex normals (3 floats each,
// indexed by `idx`, or a soup when idx is null); all pointers are device memory.
void launch_gather_normals(cudaStream_t st, const CwTri* tris, uint32_t n, const float* vn, const uint32_t* idx,
                           float4* out);
void launch_tlas_refit(cudaStream_t st, CwNode* nodes, float* node_box, const float* inst_box, uint32_t begin,
                       uint32_t end);
void launch_primary(cudaStream_t st, const DevScene& sc, const DevView& v, float near_z, float far_z, float* depth,
                    float4* const gb[4], float4* hitpos);
// radiance cache: the network's tensor-core kernels (mlp_tc.cu; `err`: a device word that gets bit 1 if a
// tensor-core wait timed out) and Adam (mlp.cu)
cudaError_t launch_mlp_infer(int device, cudaStream_t st, const void* wb, const float4* queries, const uint32_t* count,
                             uint32_t capacity, float4* accum, unsigned long long* accum_fx, uint32_t* err);
cudaError_t launch_mlp_predict(int device, cudaStream_t st, const void* wb, const float4* samples, uint32_t n,
                               float* out, uint32_t* err);
// gradient of the mean relative L2 loss over n samples added to dW, the loss to loss[0]; a tensor-core wait
// that timed out sets bit 1 of *err
// Each CTA writes its share of the gradient to its own slot, dW_parts + cta x kMlpParams (rows 3..7 of the
// output layer are not written: they keep the zeros the slots start with); *parts = the CTAs launched.
cudaError_t launch_mlp_train(int device, cudaStream_t st, const void* wb, const float4* samples, uint32_t n,
                             float* dW_parts, uint32_t* parts, float* loss, uint32_t* err);
// Gradient slots written by launch_mlp_train (at most mlp_train_parts(device) of them).
uint32_t mlp_train_parts(int device);
// dW = sum over the n_parts gradient slots, in slot order (mlp.cu)
cudaError_t launch_mlp_sum_parts(cudaStream_t st, const float* dW_parts, uint32_t n_parts, float* dW);
// Adam step; with ema_decay > 0 also updates the weights' moving average `ema` and writes its
// bias-corrected bf16 copy `ema_b` (ema_step: steps averaged, this one included)
// The gradient is the sum of the n_parts slots of dW_parts, taken in slot order.
cudaError_t launch_mlp_adam(cudaStream_t st, float* wm, void* wb, const float* dW_parts, uint32_t n_parts, float* m,
                            float* v, float lr, int step, float* ema, void* ema_b, float ema_decay, int ema_step);
// training paths (train_paths.cu): full-length paths that record per-vertex cache samples.
// Vertex v = path x segments + k.  The path kernel writes each vertex's raw inputs (3 float4), throughput
// and directly gathered radiance, and queues its next-event shadow rays in `shadow` (sun/light rays from the
// front, sky rays from the back, contribution.w = the vertex's bits); the shadow pass (launch_shadow with the
// queue's accum_fx = fx) adds the unoccluded ones as exact fixed-point sums; the targets kernels turn each
// vertex into a training sample, written at an offset from a scan of the per-path counts, so the samples'
// order (and everything trained on them) does not depend on the order of the GPU's atomics.
struct TrainVerts {
    float4* raw;
    float4* thr;
    float4* rad;
    uint32_t* count;   // vertices per path
    uint32_t segments;
    unsigned long long* fx;   // 3 words per vertex: the shadow pass's 32.32 fixed-point sums
    uint32_t* nsamp;          // per block of 256 paths: its sample count, then (scanned) its first sample
    uint32_t* offs;           // each path's first sample within its block
};
void launch_train_paths(cudaStream_t st, const DevScene& sc, const DevView* view, uint32_t n_paths, uint32_t frame,
                        const TrainVerts& tv, const Wavefront& shadow);
// Samples of the n_paths paths at scanned offsets; *count = their total (those past max_samples are dropped).
void launch_train_targets(cudaStream_t st, uint32_t n_paths, const TrainVerts& tv, float4* samples, uint32_t* count,
                          uint32_t max_samples);

// Fills the persistent-kernel grids from the device's SM count and occupancy
// (for the kernel variant lc->regcap selects).
void query_launch_cfg(int device, int block_trace, LaunchCfg* lc);

}  // namespace bsm

struct bsm_context;
struct bsm_camera;

namespace bsm {
// Context internals for entry points defined outside api.cpp.
bool ctx_scene(bsm_context* ctx, uint32_t scene_id, DevScene* out);
cudaStream_t ctx_stream(bsm_context* ctx);   // the work stream (the caller's after bsm_set_stream)
// Records where an allocation-free render keeps its counters, so that the context's sync points read
// and clear that call's device error word too.
void ctx_note_noalloc(bsm_context* ctx, uint32_t* counters);
int ctx_device(bsm_context* ctx);
void ctx_set_error(bsm_context* ctx, const char* msg);
void ctx_make_view(const bsm_camera* c, DevView* v);
const char* ctx_camera_problem(const bsm_camera* c);   // nullptr when the camera can be rendered
void*& ctx_server_slot(bsm_context* ctx);
uint32_t ctx_max_lights(bsm_context* ctx);

}  // namespace bsm
