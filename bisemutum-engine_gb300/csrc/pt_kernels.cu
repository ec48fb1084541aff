// pt_kernels.cu — the sm_103a kernels of the wavefront path-tracing pass.
//
// One render is a sequence of chunks; each chunk runs
//   k_camera  -> [k_extend -> k_shade -> k_shadow] x segments
// over device-resident queues whose sizes live in device counters, so no
// stage waits for the host and a whole render can be captured as one CUDA
// graph.  Stage <-> reference shader:
//   k_camera   generate_camera_ray_cs   (direction_sample/generate_camera_ray.hlsl:4-16)
//   k_extend   rt_gbuffer_rgen/rchit/rmiss (rt_gbuffer.hlsl:7-36, hits/rt_gbuffer_hit.hlsl:6-18)
//   k_shade    deferred_lighting_secondary_cs + sample_secondary_ray_cs
//              (deferred_lighting_secondary.hlsl:11-111, sample_secondary_ray.hlsl:11-69)
//   k_shadow   the visibility term of the direct light (there: shadow maps,
//              lights.hlsl:27-104; here: any-hit rays)
//   k_resolve  additive blit + pt_accumulate_cs (path_tracing.cpp:436-478, pt_accumulate.hlsl:3-11)
// Compiled with --fmad=false: every float operation outside the explicit
// __fmaf_rn of the box test rounds once, as on the CPU oracle.
#include <cuda_runtime.h>

#include "bsm_pt.h"
#include "pt_device.h"
#include "pt_sky.cuh"
#include "pt_trace.cuh"
#include "pt_scene.cuh"
#include "pt_lights.cuh"
#include "pt_gbuffer.cuh"
#include "bvh_quant.h"
#include "mlp.cuh"

namespace bsm {

// Warp-aggregated queue allocation: one atomic per warp, slots in lane order.
// Must be reached by all 32 lanes (pred may be false).
__device__ __forceinline__ uint32_t warp_alloc(bool pred, uint32_t* counter) {
    uint32_t b = __ballot_sync(0xffffffffu, pred);
    uint32_t base = 0;
    int lane = threadIdx.x & 31;
    if (b != 0u && lane == __ffs(b) - 1) base = atomicAdd(counter, (uint32_t)__popc(b));
    base = __shfl_sync(0xffffffffu, base, b != 0u ? __ffs(b) - 1 : 0);
    return base + (uint32_t)__popc(b & lanemask_lt());
}

// Queue slots for the threads of a block with `pred`, grouped by the direction
// of `dir`: its octant and its dominant axis, 24 bins (one atomic on `counter`
// per block).  Consecutive slots then hold rays heading the same way from
// neighbouring paths, which keeps the warps of the next traversal and shading
// launches coherent.  The lanes of a warp that share a bin take their ranks
// from one shared-memory atomic; warp 0 scans the bins.  Every
// thread of the block must call it with the same `parity`, alternating 0 / 1
// from call to call, after s_dir_cnt[0] was cleared: each call clears the
// other parity's counters for the next one, so it needs two block barriers
// instead of three.  Returns 0 for threads without pred.
constexpr uint32_t kDirBins = 24;   // octant x dominant axis
static_assert(kDirBins <= 32, "one warp scans the bins");
__shared__ uint32_t s_dir_cnt[2][kDirBins + 1];
__device__ __forceinline__ uint32_t block_alloc_by_direction(bool pred, V3 dir, uint32_t* counter, int parity) {
    __shared__ uint32_t s_off[2][kDirBins], s_base[2];
    const float ax = fabsf(dir.x), ay = fabsf(dir.y), az = fabsf(dir.z);
    const uint32_t dom = (ax >= ay && ax >= az) ? 0u : (ay >= az ? 1u : 2u);
    uint32_t key = pred ? ((dir.x < 0.0f ? 1u : 0u) | (dir.y < 0.0f ? 2u : 0u) | (dir.z < 0.0f ? 4u : 0u)) * 3u + dom
                        : kDirBins;
    // one shared atomic per bin present in the warp (the lanes of a bin share it)
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    const uint32_t leader = (uint32_t)__ffs(peers) - 1u;
    uint32_t rank = 0;
    if ((threadIdx.x & 31u) == leader && pred) rank = atomicAdd(&s_dir_cnt[parity][key], (uint32_t)__popc(peers));
    rank = __shfl_sync(0xffffffffu, rank, (int)leader) + (uint32_t)__popc(peers & lanemask_lt());
    __syncthreads();
    if (threadIdx.x < 32) {   // exclusive prefix over the bins by warp 0, one bin per lane
        const uint32_t lane = threadIdx.x;
        const uint32_t c = lane < kDirBins ? s_dir_cnt[parity][lane] : 0u;
        uint32_t x = c;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane < kDirBins) s_off[parity][lane] = x - c;
        const uint32_t total = __shfl_sync(0xffffffffu, x, 31);
        if (lane == 0) s_base[parity] = total ? atomicAdd(counter, total) : 0u;
    }
    if (threadIdx.x <= kDirBins) s_dir_cnt[parity ^ 1][threadIdx.x] = 0u;
    __syncthreads();
    return pred ? s_base[parity] + s_off[parity][key] + rank : 0u;
}

// A path's contribution to its pixel: FP32 atomics, or the call's fixed-point sums when `fx` is set
// (BSM_PT_DETERMINISTIC).
__device__ __forceinline__ void accum_add(float4* accum, unsigned long long* fx, uint32_t idx, V3 c) {
    if (fx) accum_fixed_add(fx, idx, c.x, c.y, c.z);
    else atomicAdd(accum + idx, make_float4(c.x, c.y, c.z, 0.0f));
}

// ---------------------------------------------------------------- camera ----
// generate_camera_ray.hlsl:9-11 restated without the matrices: the inverse
// reverse-Z projection of (ndc, 1, 1) is (ndc.x * aspect * tan, ndc.y * tan, -1),
// rotated by the camera basis.  (jx, jy) is the position inside the pixel.
__device__ __forceinline__ V3 camera_dir(const DevView& v, uint32_t px, uint32_t py, float jx, float jy) {
    float uvx = ((float)px + jx) / (float)v.width;
    float uvy = ((float)py + jy) / (float)v.height;
    float ndx = uvx * 2.0f - 1.0f;
    float ndy = 1.0f - uvy * 2.0f;
    V3 dl = normalize(v3(ndx * v.aspect * v.tan_half, ndy * v.tan_half, -1.0f));
    V3 s = v3(v.s[0], v.s[1], v.s[2]), u = v3(v.u[0], v.u[1], v.u[2]), f = v3(v.f[0], v.f[1], v.f[2]);
    return normalize(s * dl.x + u * dl.y + (-f) * dl.z);
}

__global__ void k_camera(const DevView* __restrict__ views, uint32_t n_views, uint64_t path_begin,
                         uint32_t path_count, Wavefront wf, uint32_t max_segments_cap) {
    uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid == 0) wf.counters[kCntQueue + 0] = path_count;
    if (gid >= path_count) return;
    uint64_t p = path_begin + gid;
    // view lookup (views sorted by path_base)
    uint32_t lo = 0, hi = n_views - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (views[mid].path_base <= p) lo = mid; else hi = mid - 1;
    }
    const DevView& v = views[lo];
    uint64_t local = p - v.path_base + v.first_path;
    // pixel-major order: the samples of a pixel are neighbours in the queue, so a warp traces the (near-)
    // identical camera rays of one or a few pixels together, and their later rays start from the same
    // points.  Every path's random stream depends only on its pixel and sample, so the order changes no
    // result (measured on the 1920x1080x64 terrain frame: 1274 -> 1515 Mrays/s against sample-major).
    uint32_t pixel = (uint32_t)(local / v.spp);
    uint32_t sample = (uint32_t)(local - (uint64_t)pixel * v.spp);
    uint32_t px = pixel % v.width, py = pixel / v.width;
    Pcg g = pcg_seed(path_initstate(v.seed, v.sample_offset + sample, pixel), (uint64_t)pixel);
    float jx = 0.5f, jy = 0.5f;
    if (v.flags & BSM_PT_JITTER) { jx = pcg_uniform(g); jy = pcg_uniform(g); }
    V3 dw = camera_dir(v, px, py, jx, jy);
    uint32_t maxseg = v.max_segments < max_segments_cap ? v.max_segments : max_segments_cap;
    wf.ray_o[0][gid] = make_float4(v.pos[0], v.pos[1], v.pos[2], v.t_min);
    wf.ray_d[0][gid] = make_float4(dw.x, dw.y, dw.z, v.ray_length);
    wf.path[0][gid] = make_uint4(v.accum_base + pixel, (maxseg << 8) | (lo << 16), (uint32_t)g.state,
                                 (uint32_t)(g.state >> 32));
    wf.thr[0][gid] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
}

// ---------------------------------------------------------------- extend ----
template <bool kCount, int kMinBlocks, bool kOpacity>
__global__ void __launch_bounds__(256, kMinBlocks) k_extend(DevScene sc, const float4* __restrict__ ray_o,
                                                const float4* __restrict__ ray_d, const uint4* __restrict__ path,
                                                float4* __restrict__ hit, uint32_t* counters,
                                                unsigned long long* stats, uint32_t seg, int postpone_sp,
                                                int refill_min) {
    uint32_t n = counters[kCntQueue + seg];
    if (blockIdx.x == 0 && threadIdx.x == 0) stats[kStatExtend + seg] += n;
    TraceCounters c{0, 0};
    trace_queue<false, kCount, kOpacity>(
        sc.nodes, sc.tris, n, counters + kCntWork + 2 * seg,
        [&](uint32_t i, float4& o, float4& d) { o = ray_o[i]; d = ray_d[i]; },
        [&](uint32_t i, uint32_t leaf, float t, float u, float v) {
            hit[i] = make_float4(t, __uint_as_float(leaf), u, v);
        },
        [&](uint32_t i) { return path[i].z; },   // the path's PCG32 word
        &c, postpone_sp, refill_min);
    if (kCount) {
        uint32_t cn = c.nodes, ct = c.tris;
        for (int off = 16; off > 0; off >>= 1) {
            cn += __shfl_xor_sync(0xffffffffu, cn, off);
            ct += __shfl_xor_sync(0xffffffffu, ct, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(stats + kStatNodes, (unsigned long long)cn);
            atomicAdd(stats + kStatTris, (unsigned long long)ct);
        }
    }
}

// ---------------------------------------------------------------- shadow ----
template <int kMinBlocks, bool kOpacity>
__global__ void __launch_bounds__(256, kMinBlocks) k_shadow(DevScene sc, Wavefront wf, uint32_t seg, float4* accum,
                                                            int postpone_sp, int refill_min) {
    const uint32_t n_sun = wf.counters[kCntShadow + seg], n_sky = wf.counters[kCntSky + seg];
    const uint32_t sh_cap = wf.capacity * (sc.num_lights + 1u);
    const uint32_t n = n_sun + n_sky;
    if (blockIdx.x == 0 && threadIdx.x == 0) wf.stats[kStatShadow + seg] += n;
    const float4* __restrict__ so = wf.sh_o;
    const float4* __restrict__ sd = wf.sh_d;
    const float4* __restrict__ scn = wf.sh_c;
    // work index i < n_sun: sun ray i; otherwise sky ray at the back of the queue
    auto slot = [=](uint32_t i) { return i < n_sun ? i : sh_cap - 1u - (i - n_sun); };
    trace_queue<true, false, kOpacity>(
        sc.nodes, sc.tris, n, wf.counters + kCntWork + 2 * seg + 1,
        [&](uint32_t i, float4& o, float4& d) { uint32_t k = slot(i); o = so[k]; d = sd[k]; },
        [&](uint32_t i, uint32_t leaf, float, float, float) {
            if (leaf == kMissPrim) {
                float4 c = scn[slot(i)];
                accum_add(accum, wf.accum_fx, __float_as_uint(c.w), v3(c.x, c.y, c.z));
            }
        },
        [&](uint32_t i) { return wf.sh_seed ? wf.sh_seed[slot(i)] : 0u; },
        nullptr, postpone_sp, refill_min);
}

// ------------------------------------------------- two-level extend / shadow ----
// Two-level scenes: persistent warps over the queue with trace_queue2 (TLAS
// leaves enter instances).  The hit record carries the instance in place of u.
template <bool kOpacity>
__global__ void __launch_bounds__(256, 4) k_extend2(DevScene sc, const float4* __restrict__ ray_o,
                                                    const float4* __restrict__ ray_d, const uint4* __restrict__ path,
                                                    float4* __restrict__ hit, uint32_t* counters,
                                                    unsigned long long* stats, uint32_t seg, int postpone_sp,
                                                    int refill_min) {
    const uint32_t n = counters[kCntQueue + seg];
    if (blockIdx.x == 0 && threadIdx.x == 0) stats[kStatExtend + seg] += n;
    trace_queue2<false, kOpacity>(
        sc.nodes, sc.insts, sc.mat_tr, n, counters + kCntWork + 2 * seg,
        [&](uint32_t i, float4& o, float4& d) { o = ray_o[i]; d = ray_d[i]; },
        [&](uint32_t i, uint32_t leaf, float t, float, float v, uint32_t inst) {
            hit[i] = make_float4(t, __uint_as_float(leaf), __uint_as_float(inst), v);
        },
        [&](uint32_t i) { return path[i].z; },   // the path's PCG32 word
        postpone_sp, refill_min);
}

template <bool kOpacity>
__global__ void __launch_bounds__(256, 4) k_shadow2(DevScene sc, Wavefront wf, uint32_t seg, float4* accum,
                                                    int postpone_sp, int refill_min) {
    const uint32_t n_sun = wf.counters[kCntShadow + seg], n_sky = wf.counters[kCntSky + seg];
    const uint32_t sh_cap = wf.capacity * (sc.num_lights + 1u);
    const uint32_t n = n_sun + n_sky;
    if (blockIdx.x == 0 && threadIdx.x == 0) wf.stats[kStatShadow + seg] += n;
    const float4* __restrict__ so = wf.sh_o;
    const float4* __restrict__ sd = wf.sh_d;
    const float4* __restrict__ scn = wf.sh_c;
    auto slot = [=](uint32_t i) { return i < n_sun ? i : sh_cap - 1u - (i - n_sun); };
    trace_queue2<true, kOpacity>(
        sc.nodes, sc.insts, sc.mat_tr, n, wf.counters + kCntWork + 2 * seg + 1,
        [&](uint32_t i, float4& o, float4& d) { uint32_t k = slot(i); o = so[k]; d = sd[k]; },
        [&](uint32_t i, uint32_t leaf, float, float, float, uint32_t) {
            if (leaf == kMissPrim) {
                float4 c = scn[slot(i)];
                accum_add(accum, wf.accum_fx, __float_as_uint(c.w), v3(c.x, c.y, c.z));
            }
        },
        [&](uint32_t i) { return wf.sh_seed ? wf.sh_seed[slot(i)] : 0u; },
        postpone_sp, refill_min);
}

// ----------------------------------------------------------------- shade ----
// kGeneral: point, spot or rect lights, or radiance-cache queries; the slim
// variant (directional lights only, no cache) leaves that code out.
template <bool kGeneral>
__global__ void __launch_bounds__(512, 2) k_shade(DevScene sc, const DevView* __restrict__ views, Wavefront wf,
                                               int q, uint32_t seg, float4* accum) {
    const uint32_t n = wf.counters[kCntQueue + seg];
    const uint32_t cap = wf.capacity;
    const uint32_t sh_cap = cap * (sc.num_lights + 1u);
    const float4* __restrict__ in_o = wf.ray_o[q];
    const float4* __restrict__ in_d = wf.ray_d[q];
    const uint4* __restrict__ in_p = wf.path[q];
    const float4* __restrict__ in_t = wf.thr[q];
    float4* out_o = wf.ray_o[q ^ 1];
    float4* out_d = wf.ray_d[q ^ 1];
    uint4* out_p = wf.path[q ^ 1];
    float4* out_t = wf.thr[q ^ 1];
    const uint32_t stride = gridDim.x * blockDim.x;
    if (threadIdx.x <= kDirBins) s_dir_cnt[0][threadIdx.x] = 0u;
    __syncthreads();
    int parity = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride, parity ^= 1) {
        uint32_t i = base + threadIdx.x;
        bool active = i < n;
        float4 o4 = make_float4(0, 0, 0, 0), d4 = make_float4(0, 0, 1, 0), h4 = make_float4(0, 0, 0, 0);
        float4 t4 = make_float4(0, 0, 0, 0);
        uint4 m4 = make_uint4(0, 0, 0, 0);
        if (active) { o4 = in_o[i]; d4 = in_d[i]; h4 = wf.hit[i]; t4 = in_t[i]; m4 = in_p[i]; }
        uint32_t leaf = active ? __float_as_uint(h4.y) : kMissPrim;
        bool is_hit = active && leaf != kMissPrim;
        uint32_t segi = m4.y & 0xffu, maxseg = (m4.y >> 8) & 0xffu, view_id = m4.y >> 16;
        V3 thr = v3(t4.x, t4.y, t4.z);
        V3 d = v3(d4.x, d4.y, d4.z);
        bool sky_nee = sc.num_lights + 1u > 0u;  // placeholder, refined below per view
        uint32_t vflags = 0;
        uint32_t stream = 0;
        uint32_t cache_seg = 0;
        float cache_rough = 0.0f;
        if (active) {
            const DevView& v = views[view_id];
            vflags = v.flags;
            stream = m4.x - v.accum_base;
            cache_seg = v.cache_segment;
            cache_rough = v.cache_min_rough;
        }
        sky_nee = (vflags & BSM_PT_NO_SKY_NEE) == 0u;
        if (active && !is_hit) {
            // deferred_lighting_secondary.hlsl:23-29: skybox x weight on a miss,
            // here with the MIS weight against sky next-event estimation.
            V3 le = sky_eval(sc.sky, d);
            float w = 1.0f;
            if (segi > 0u && sky_nee) {
                float pb = t4.w;
                float pl = sky_pdf(sc.sky, d);
                float pb2 = pb * pb, pl2 = pl * pl;
                w = pb2 + pl2 > 0.0f ? pb2 / (pb2 + pl2) : 1.0f;
            }
            V3 c = thr * le * w;
            if (max_comp(c) > 0.0f) accum_add(accum, wf.accum_fx, m4.x, c);
        }
        // surface at the hit: N shades (the interpolated vertex normal where the scene has them), Ng offsets
        V3 N = v3(0.0f, 0.0f, 1.0f), Ng = N, P = v3(0.0f, 0.0f, 0.0f);
        Surface surf;
        surf.base_color = v3s(0.5f); surf.f0 = v3s(0.04f); surf.f90 = v3s(1.0f); surf.roughness = 0.5f; surf.ior = 1.5f;
        if (is_hit) {
            V3 ng, edge;
            uint32_t mi;
            hit_geometry(sc, leaf, sc.insts ? __float_as_uint(h4.z) : kMissPrim, ng, edge, mi);
            if (dot(ng, d) > 0.0f) ng = -ng;
            Ng = ng;
            N = ng;
            if (sc.tri_normals) {
                N = shading_normal(sc, leaf, h4.z, h4.w, ng);
                if (dot(N, d) > 0.0f) N = -N;
            }
            P = v3(o4.x, o4.y, o4.z) + d * h4.x;
            float4 m0 = sc.materials[2 * mi], m1 = sc.materials[2 * mi + 1];
            surf.base_color = v3(m0.x, m0.y, m0.z);
            surf.roughness = m0.w;
            surf.f0 = v3(m1.x, m1.y, m1.z);
        }
        Frame fr = create_frame(N);
        V3 V = -d;
        Pcg g;
        g.state = ((uint64_t)m4.w << 32) | m4.z;
        g.inc = ((uint64_t)stream << 1) | 1u;
        float u_sky0 = 0.0f, u_sky1 = 0.0f, u_sky2 = 0.0f, u_lobe = 0.0f, u_b0 = 0.0f, u_b1 = 0.0f;
        if (is_hit) {
            u_sky0 = pcg_uniform(g); u_sky1 = pcg_uniform(g); u_sky2 = pcg_uniform(g); u_lobe = pcg_uniform(g);
            u_b0 = pcg_uniform(g); u_b1 = pcg_uniform(g);
        }
        // radiance cache: a hit of the cache segment (or a later one, when the earlier hits were too smooth)
        // becomes a query (NRC-style termination) — the cache's prediction includes the direct light there
        bool cache_q = kGeneral && is_hit && cache_seg != 0u && segi >= cache_seg &&
                       (surf.roughness >= cache_rough || segi + 1u >= maxseg);
        {
            uint32_t slot = warp_alloc(cache_q, wf.counters + kCntCache);
            if (cache_q) {
                if (slot < cap && wf.cache_q) {
                    float raw[kMlpRaw];
                    mlp_raw_inputs(P, v3(sc.box_lo[0], sc.box_lo[1], sc.box_lo[2]),
                                   v3(sc.box_inv[0], sc.box_inv[1], sc.box_inv[2]), -d, N, surf.roughness,
                                   surf.base_color, (float)segi * 0.125f, raw);
                    float4* qd = wf.cache_q + 4 * (size_t)slot;
                    qd[0] = make_float4(raw[0], raw[1], raw[2], raw[3]);
                    qd[1] = make_float4(raw[4], raw[5], raw[6], raw[7]);
                    qd[2] = make_float4(raw[8], raw[9], raw[10], raw[11]);
                    qd[3] = make_float4(thr.x, thr.y, thr.z, __uint_as_float(m4.x));
                } else {
                    atomicOr(wf.counters + kCntError, 1u);
                }
            }
        }
        if (cache_q) is_hit = false;  // no NEE, no continuation at a cache vertex
        V3 org = P + Ng * sc.ray_offset;
        const DevView* vp = views + view_id;
        float ray_len = is_hit ? vp->ray_length : 0.0f;
        float tmin = is_hit ? vp->t_min : 0.0f;
        float rx = 0.001f, ry = 0.001f;
        aniso_roughness(surf.roughness, &rx, &ry);
        V3 lv = to_local(fr, V);
        float p_spec = spec_probability(surf, lv.z);
        // next-event estimation towards the lights (lights.hlsl:10-25; rect lights sampled by area),
        // deferred_lighting_secondary.hlsl:51-96.  Rect lights draw their two uniforms here, after
        // the vertex's six, in light order.
        for (uint32_t l = 0; l < (uint32_t)kMaxLights; ++l) {
            if (l >= sc.num_lights) break;
            const DevLight& lt = sc.lights[l];
            V3 c = v3s(0.0f), L = v3s(0.0f);
            float smax = ray_len;
            float ur0 = 0.0f, ur1 = 0.0f;
            if (kGeneral && is_hit && __float_as_uint(lt.a.w) == kLightRect) {
                ur0 = pcg_uniform(g);
                ur1 = pcg_uniform(g);
            }
            bool emit = false;
            if (is_hit && (vflags & BSM_PT_NO_SUN_NEE) == 0u) {
                V3 e;
                bool lit;
                if (kGeneral) {
                    lit = light_sample(lt, P, ur0, ur1, ray_len, L, smax, e);
                } else {  // directional: light_sample's first case
                    L = v3(lt.a.x, lt.a.y, lt.a.z);
                    e = v3(lt.b.x, lt.b.y, lt.b.z);
                    smax = ray_len;
                    lit = true;
                }
                if (lit) {
                    V3 f = surface_eval_lit(N, fr.x, fr.y, V, L, surf);
                    c = thr * e * f;
                    emit = max_comp(c) > 0.0f;
                }
            }
            uint32_t slot = warp_alloc(emit, wf.counters + kCntShadow + seg);
            if (emit) {
                if (slot < cap * sc.num_lights) {
                    wf.sh_o[slot] = make_float4(org.x, org.y, org.z, tmin);
                    wf.sh_d[slot] = make_float4(L.x, L.y, L.z, smax);
                    wf.sh_c[slot] = make_float4(c.x, c.y, c.z, __uint_as_float(m4.x));
                    if (sc.has_non_opaque && wf.sh_seed) wf.sh_seed[slot] = (uint32_t)g.state;
                } else {
                    atomicOr(wf.counters + kCntError, 1u);
                }
            }
        }
        // next-event estimation: sky, MIS (power heuristic) against BSDF sampling
        {
            V3 c = v3s(0.0f), L = v3s(0.0f);
            bool emit = false;
            if (is_hit && sky_nee) {
                float pl;
                V3 le;
                L = sky_sample(sc.sky, u_sky0, u_sky1, u_sky2, pl, le);
                if (pl > 0.0f) {
                    V3 f = surface_eval_lit(N, fr.x, fr.y, V, L, surf);
                    if (max_comp(f) > 0.0f) {
                        V3 ll = to_local(fr, L);
                        float pb = mixture_pdf(lv, ll, rx, ry, p_spec);
                        float pl2 = pl * pl, pb2 = pb * pb;
                        float w = pl2 / (pl2 + pb2);
                        c = thr * le * f * (w / pl);
                        emit = max_comp(c) > 0.0f;
                    }
                }
            }
            uint32_t slot = warp_alloc(emit, wf.counters + kCntSky + seg);
            if (emit) {
                if (slot < cap) {
                    uint32_t k = sh_cap - 1u - slot;   // sky rays fill the queue from the back
                    wf.sh_o[k] = make_float4(org.x, org.y, org.z, tmin);
                    wf.sh_d[k] = make_float4(L.x, L.y, L.z, ray_len);
                    wf.sh_c[k] = make_float4(c.x, c.y, c.z, __uint_as_float(m4.x));
                    if (sc.has_non_opaque && wf.sh_seed) wf.sh_seed[k] = (uint32_t)g.state;
                } else {
                    atomicOr(wf.counters + kCntError, 1u);
                }
            }
        }
        // next direction: lobe mixture (sample_secondary_ray.hlsl:16-28 termination, :51-64 weight)
        bool cont = false;
        V3 nthr = v3s(0.0f), L = v3s(0.0f);
        float pdf = 0.0f;
        if (is_hit && segi + 1u < maxseg && max_comp(thr) >= 0.001f) {
            V3 ll;
            if (u_lobe < p_spec) {
                V3 h = ggx_vndf_sample(lv, rx, ry, u_b0, u_b1);
                ll = reflect(-lv, h);
            } else {
                ll = cos_hemisphere_sample(u_b0, u_b1);
            }
            if (ll.z > 0.0f) {
                L = to_world(fr, ll);
                pdf = mixture_pdf(lv, ll, rx, ry, p_spec);
                V3 f = surface_eval_lit(N, fr.x, fr.y, V, L, surf);
                V3 w = pdf > 0.0f ? f / pdf : v3s(0.0f);
                if (!isfinite(w.x) || !isfinite(w.y) || !isfinite(w.z)) w = v3s(0.0f);
                nthr = thr * w;
                cont = max_comp(nthr) > 0.0f;
            }
        }
        // the next rays, grouped by direction per block (sorting the sky shadow rays by octant measured no gain)
        uint32_t slot = block_alloc_by_direction(cont, L, wf.counters + kCntQueue + seg + 1, parity);
        if (cont) {
            if (slot < cap) {
                out_o[slot] = make_float4(org.x, org.y, org.z, tmin);
                out_d[slot] = make_float4(L.x, L.y, L.z, ray_len);
                out_p[slot] = make_uint4(m4.x, (m4.y & 0xffffff00u) | (segi + 1u), (uint32_t)g.state,
                                         (uint32_t)(g.state >> 32));
                out_t[slot] = make_float4(nthr.x, nthr.y, nthr.z, pdf);
            } else {
                atomicOr(wf.counters + kCntError, 1u);
            }
        }
    }
}

// --------------------------------------------------------------- resolve ----
// The call's fixed-point sums added to the FP32 accumulator, one add per pixel and channel.
__global__ void k_fold_fixed(const unsigned long long* __restrict__ fx, float4* __restrict__ accum, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long* p = fx + 3 * (size_t)i;
    float4 a = accum[i];
    a.x += (float)((double)p[0] * 0x1p-32);
    a.y += (float)((double)p[1] * 0x1p-32);
    a.z += (float)((double)p[2] * 0x1p-32);
    accum[i] = a;
}

__global__ void k_resolve_fixed(const unsigned long long* __restrict__ fx, uint32_t width, uint32_t height,
                                float inv_spp, float4* __restrict__ out, uint32_t pitch) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= width || y >= height) return;
    const unsigned long long* p = fx + 3 * ((size_t)y * width + x);
    out[(size_t)y * pitch + x] = make_float4((float)((double)p[0] * 0x1p-32) * inv_spp,
                                             (float)((double)p[1] * 0x1p-32) * inv_spp,
                                             (float)((double)p[2] * 0x1p-32) * inv_spp, 1.0f);
}

__global__ void k_resolve(const float4* __restrict__ accum, uint32_t width, uint32_t height, float inv_spp,
                          float4* __restrict__ out, uint32_t pitch) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t y = blockIdx.y;
    if (x >= width || y >= height) return;
    float4 a = accum[(size_t)y * width + x];
    out[(size_t)y * pitch + x] = make_float4(a.x * inv_spp, a.y * inv_spp, a.z * inv_spp, 1.0f);
}

// ------------------------------------------------------- vertex normals ----
// The three vertex normals of every leaf triangle, in leaf order, from the
// scene's per-vertex normals (indexed like the positions).
__global__ void k_gather_normals(const CwTri* __restrict__ tris, uint32_t n, const float* __restrict__ vn,
                                 const uint32_t* __restrict__ idx, float4* __restrict__ out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t prim = tris[i].prim;
    for (int k = 0; k < 3; ++k) {
        const size_t v = idx ? idx[3 * (size_t)prim + k] : 3 * (size_t)prim + k;
        out[3 * (size_t)i + k] = make_float4(vn[3 * v], vn[3 * v + 1], vn[3 * v + 2], 0.0f);
    }
}

// ------------------------------------------------------ stage entry points ----
__global__ void __launch_bounds__(256) k_trace_closest(DevScene sc, const float4* __restrict__ rays, uint32_t n,
                                                       uint4* __restrict__ hits) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 o = rays[2 * (size_t)i], d = rays[2 * (size_t)i + 1];
    RayPre r = make_ray(o, d);
    float t, u, v;
    uint32_t inst;
    uint32_t leaf = trace_scene<false>(sc, r, d.w, t, u, v, inst, 0u);
    uint32_t prim = kMissPrim;
    if (leaf != kMissPrim)
        prim = inst != kMissPrim ? sc.insts[inst].prim_base + sc.insts[inst].tris[leaf].prim : sc.tris[leaf].prim;
    hits[i] = make_uint4(__float_as_uint(t), prim, __float_as_uint(u), __float_as_uint(v));
}

// ------------------------------------------------------ primary outputs ----
// One pixel-centre camera ray per pixel and its closest hit, as the reference's
// first trace of a frame (generate_camera_ray.hlsl:9-15, rt_gbuffer.hlsl:7-36),
// written as the pass's primary-hit outputs: reverse-Z depth (pt_depth.hlsl:7-16),
// the packed G-buffer (gbuffer.hlsl:18-31) and hit positions.  The normal is the
// geometric one faced towards the ray (as k_shade), the tangent the triangle's
// first edge.  A miss writes depth 0, hit position (direction, -1) and a zero
// G-buffer.  Outputs are tightly packed width*height arrays; any may be null.
__global__ void __launch_bounds__(256) k_primary(DevScene sc, DevView v, float near_z, float far_z,
                                                 float* __restrict__ depth, float4* __restrict__ gb0,
                                                 float4* __restrict__ gb1, float4* __restrict__ gb2,
                                                 float4* __restrict__ gb3, float4* __restrict__ hitpos) {
    uint32_t npix = v.width * v.height;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    uint32_t px = i % v.width, py = i / v.width;
    V3 dw = camera_dir(v, px, py, 0.5f, 0.5f);
    V3 eye = v3(v.pos[0], v.pos[1], v.pos[2]);
    RayPre r = make_ray(make_float4(eye.x, eye.y, eye.z, v.t_min), make_float4(dw.x, dw.y, dw.z, v.ray_length));
    float t, hu, hv;
    // opacity decisions of sample 0 of an unjittered render (its camera-ray PCG word)
    Pcg pg = pcg_seed(path_initstate(v.seed, v.sample_offset, i), (uint64_t)i);
    uint32_t inst;
    uint32_t leaf = trace_scene<false>(sc, r, v.ray_length, t, hu, hv, inst, (uint32_t)pg.state);
    float g[16];
    float z = 0.0f;
    float4 hp;
    if (leaf == kMissPrim) {
#pragma unroll
        for (int k = 0; k < 16; ++k) g[k] = 0.0f;
        hp = make_float4(dw.x, dw.y, dw.z, -1.0f);
    } else {
        V3 ng, edge;
        uint32_t mi;
        hit_geometry(sc, leaf, inst, ng, edge, mi);
        if (dot(ng, dw) > 0.0f) ng = -ng;
        if (sc.tri_normals) {
            ng = shading_normal(sc, leaf, hu, hv, ng);
            if (dot(ng, dw) > 0.0f) ng = -ng;
        }
        V3 T = normalize(edge);
        float4 m0 = sc.materials[2 * mi], m1 = sc.materials[2 * mi + 1];
        pack_gbuffer(ng, T, v3(m0.x, m0.y, m0.z), v3(m1.x, m1.y, m1.z), m0.w, g);
        V3 P = eye + dw * t;
        z = reverse_z_depth(eye, v3(v.f[0], v.f[1], v.f[2]), P, near_z, far_z);
        hp = make_float4(P.x, P.y, P.z, t);
    }
    if (depth) depth[i] = z;
    if (gb0) gb0[i] = make_float4(g[0], g[1], g[2], g[3]);
    if (gb1) gb1[i] = make_float4(g[4], g[5], g[6], g[7]);
    if (gb2) gb2[i] = make_float4(g[8], g[9], g[10], g[11]);
    if (gb3) gb3[i] = make_float4(g[12], g[13], g[14], g[15]);
    if (hitpos) hitpos[i] = hp;
}

__global__ void __launch_bounds__(256) k_trace_any(DevScene sc, const float4* __restrict__ rays, uint32_t n,
                                                   uint8_t* __restrict__ occluded) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 o = rays[2 * (size_t)i], d = rays[2 * (size_t)i + 1];
    RayPre r = make_ray(o, d);
    float t, u, v;
    uint32_t inst;
    uint32_t leaf = trace_scene<true>(sc, r, d.w, t, u, v, inst, 0u);
    occluded[i] = leaf == kMissPrim ? 0 : 1;
}

__global__ void __launch_bounds__(256) k_trace_count(DevScene sc, const float4* __restrict__ rays, uint32_t n,
                                                     uint2* __restrict__ counts) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 o = rays[2 * (size_t)i], d = rays[2 * (size_t)i + 1];
    RayPre r = make_ray(o, d);
    float t, u, v;
    TraceCounters c{0, 0};
    trace_ray<false, true>(r, d.w, sc.nodes, sc.tris, t, u, v, &c);
    counts[i] = make_uint2(c.nodes, c.tris);
}

// ------------------------------------------------------------- TLAS refit ----
// Refits the TLAS for new instance boxes, one BFS level per launch from the
// deepest up (nodes of a level are contiguous in the builder's breadth-first
// order).  A node's eight child boxes come from the instance boxes of its leaf
// slots (TLAS leaves hold one instance) and from the boxes its internal
// children wrote one launch earlier; the node's frame and bytes are then
// quantised outward exactly as the host builder does (tlas_quantise).
__global__ void k_tlas_refit(CwNode* __restrict__ nodes, float* __restrict__ node_box,
                             const float* __restrict__ inst_box, uint32_t begin, uint32_t end) {
    uint32_t ni = begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (ni >= end) return;
    CwNode n = nodes[ni];
    float lo[8][3], hi[8][3];
    uint32_t used = 0;
    for (int s = 0; s < 8; ++s) {
        bool inner = (n.imask >> s) & 1u;
        if (!inner && ((n.tri_mask >> (2 * s)) & 3u) == 0u) continue;
        used |= 1u << s;
        const float* b;
        if (inner) {
            uint32_t ci = n.child_base + (uint32_t)__popc((uint32_t)n.imask & ((1u << s) - 1u));
            b = node_box + 6 * (size_t)ci;
        } else {
            b = inst_box + 6 * (size_t)(n.tri_base + (uint32_t)__popc((uint32_t)n.tri_mask & ((1u << (2 * s)) - 1u)));
        }
        for (int k = 0; k < 3; ++k) { lo[s][k] = b[k]; hi[s][k] = b[3 + k]; }
    }
    float nlo[3], nhi[3];
    tlas_quantise(n, lo, hi, used, nlo, nhi);
    nodes[ni] = n;
    for (int k = 0; k < 3; ++k) { node_box[6 * (size_t)ni + k] = nlo[k]; node_box[6 * (size_t)ni + 3 + k] = nhi[k]; }
}

// ------------------------------------------------------------ launchers ----
void launch_tlas_refit(cudaStream_t st, CwNode* nodes, float* node_box, const float* inst_box, uint32_t begin,
                       uint32_t end) {
    if (end <= begin) return;
    k_tlas_refit<<<(end - begin + 127) / 128, 128, 0, st>>>(nodes, node_box, inst_box, begin, end);
}
void launch_camera(const LaunchCfg& lc, cudaStream_t st, const DevView* views, uint32_t n_views,
                   uint64_t path_begin, uint32_t path_count, const Wavefront& wf, uint32_t max_segments) {
    uint32_t blocks = (path_count + lc.block_shade - 1) / lc.block_shade;
    if (blocks == 0) blocks = 1;
    k_camera<<<blocks, lc.block_shade, 0, st>>>(views, n_views, path_begin, path_count, wf, max_segments);
}
void launch_gather_normals(cudaStream_t st, const CwTri* tris, uint32_t n, const float* vn, const uint32_t* idx,
                           float4* out) {
    if (n) k_gather_normals<<<(n + 255) / 256, 256, 0, st>>>(tris, n, vn, idx, out);
}

void launch_extend(const LaunchCfg& lc, cudaStream_t st, const DevScene& sc, const Wavefront& wf, int q,
                   uint32_t seg, bool count_traversal) {
#define BSM_EXTEND(C, B, O)                                                                                    \
    k_extend<C, B, O><<<lc.grid_persistent, lc.block_trace, 0, st>>>(sc, wf.ray_o[q], wf.ray_d[q], wf.path[q], \
                                                                     wf.hit, wf.counters, wf.stats, seg,        \
                                                                     lc.postpone_sp, lc.refill_min)
    const bool op = sc.has_non_opaque != 0;
    if (sc.insts) {
        if (op)
            k_extend2<true><<<lc.grid_persistent2, lc.block_trace, 0, st>>>(
                sc, wf.ray_o[q], wf.ray_d[q], wf.path[q], wf.hit, wf.counters, wf.stats, seg, lc.postpone_sp,
                lc.refill_min);
        else
            k_extend2<false><<<lc.grid_persistent2, lc.block_trace, 0, st>>>(
                sc, wf.ray_o[q], wf.ray_d[q], wf.path[q], wf.hit, wf.counters, wf.stats, seg, lc.postpone_sp,
                lc.refill_min);
    }
    else if (count_traversal) { if (op) BSM_EXTEND(true, 1, true); else BSM_EXTEND(true, 1, false); }
    else if (lc.regcap) { if (op) BSM_EXTEND(false, 4, true); else BSM_EXTEND(false, 4, false); }
    else { if (op) BSM_EXTEND(false, 1, true); else BSM_EXTEND(false, 1, false); }
#undef BSM_EXTEND
}
void launch_shade(const LaunchCfg& lc, cudaStream_t st, const DevScene& sc, const DevView* views,
                  const Wavefront& wf, int q, uint32_t seg, float4* accum, bool cache) {
    if (cache || !sc.dir_lights_only)
        k_shade<true><<<lc.grid_shade, lc.block_shade, 0, st>>>(sc, views, wf, q, seg, accum);
    else
        k_shade<false><<<lc.grid_shade, lc.block_shade, 0, st>>>(sc, views, wf, q, seg, accum);
}
void launch_shadow(const LaunchCfg& lc, cudaStream_t st, const DevScene& sc, const Wavefront& wf, uint32_t seg,
                   float4* accum) {
#define BSM_SHADOW(B, O) \
    k_shadow<B, O><<<lc.grid_persistent, lc.block_trace, 0, st>>>(sc, wf, seg, accum, lc.postpone_sp, lc.refill_min)
    const bool op = sc.has_non_opaque != 0;
    if (sc.insts) {
        if (op)
            k_shadow2<true><<<lc.grid_persistent2, lc.block_trace, 0, st>>>(sc, wf, seg, accum, lc.postpone_sp,
                                                                            lc.refill_min);
        else
            k_shadow2<false><<<lc.grid_persistent2, lc.block_trace, 0, st>>>(sc, wf, seg, accum, lc.postpone_sp,
                                                                             lc.refill_min);
    } else if (lc.regcap) { if (op) BSM_SHADOW(4, true); else BSM_SHADOW(4, false); }
    else { if (op) BSM_SHADOW(1, true); else BSM_SHADOW(1, false); }
#undef BSM_SHADOW
}
void launch_resolve(cudaStream_t st, const float4* accum, uint32_t width, uint32_t height, float inv_spp,
                    float4* out, uint32_t pitch_px) {
    dim3 grid((width + 255) / 256, height);
    k_resolve<<<grid, 256, 0, st>>>(accum, width, height, inv_spp, out, pitch_px);
}
void launch_resolve_fixed(cudaStream_t st, const unsigned long long* fx, uint32_t width, uint32_t height,
                          float inv_spp, float4* out, uint32_t pitch_px) {
    dim3 grid((width + 255) / 256, height);
    k_resolve_fixed<<<grid, 256, 0, st>>>(fx, width, height, inv_spp, out, pitch_px);
}
void launch_fold_fixed(cudaStream_t st, const unsigned long long* fx, float4* accum, uint32_t n) {
    if (n == 0) return;
    k_fold_fixed<<<(unsigned)(((uint64_t)n + 255) / 256), 256, 0, st>>>(fx, accum, n);
}
void launch_trace_closest(cudaStream_t st, const DevScene& sc, const float4* rays, uint32_t n, uint4* hits,
                          int block) {
    if (n == 0) return;
    k_trace_closest<<<(n + block - 1) / block, block, 0, st>>>(sc, rays, n, hits);
}
void launch_trace_any(cudaStream_t st, const DevScene& sc, const float4* rays, uint32_t n, uint8_t* occluded,
                      int block) {
    if (n == 0) return;
    k_trace_any<<<(n + block - 1) / block, block, 0, st>>>(sc, rays, n, occluded);
}
void launch_primary(cudaStream_t st, const DevScene& sc, const DevView& v, float near_z, float far_z, float* depth,
                    float4* const gb[4], float4* hitpos) {
    uint32_t npix = v.width * v.height;
    if (npix == 0) return;
    k_primary<<<(npix + 255) / 256, 256, 0, st>>>(sc, v, near_z, far_z, depth, gb[0], gb[1], gb[2], gb[3], hitpos);
}
void launch_trace_count(cudaStream_t st, const DevScene& sc, const float4* rays, uint32_t n, uint2* counts) {
    if (n == 0) return;
    k_trace_count<<<(n + 127) / 128, 128, 0, st>>>(sc, rays, n, counts);
}

// Occupancy-derived grid of the persistent kernels: every SM filled.
void query_launch_cfg(int device, int block_trace, LaunchCfg* lc) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int per_sm_ext = 0, per_sm_sh = 0, per_sm_shade = 0;
    if (lc->regcap) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_ext, k_extend<false, 4, true>, block_trace, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_sh, k_shadow<4, true>, block_trace, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_ext, k_extend<false, 1, true>, block_trace, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_sh, k_shadow<1, true>, block_trace, 0);
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_shade, k_shade<true>, 512, 0);
    int per_sm2_ext = 0, per_sm2_sh = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2_ext, k_extend2<true>, block_trace, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2_sh, k_shadow2<true>, block_trace, 0);
    int per_sm2 = per_sm2_ext < per_sm2_sh ? per_sm2_ext : per_sm2_sh;
    if (per_sm2 < 1) per_sm2 = 1;
    lc->grid_persistent2 = sms * per_sm2;
    int per_sm = per_sm_ext < per_sm_sh ? per_sm_ext : per_sm_sh;
    if (per_sm < 1) per_sm = 1;
    if (per_sm_shade < 1) per_sm_shade = 1;
    lc->block_trace = block_trace;
    lc->grid_persistent = sms * per_sm;
    lc->block_shade = 512;   // the direction grouping of the next rays spans a block
    lc->grid_shade = sms * per_sm_shade * 4;
}

}  // namespace bsm
