// train_paths.cu — training data for the radiance cache, generated by the tracer.
//
// One thread follows one full-length path (the plain pass's stages: closest
// hit, sun/light and sky next-event estimation, lobe sampling, sky on escape
// with MIS) and records every vertex k it reaches: the cache's raw inputs, the
// path throughput there, and the radiance gathered there directly (the sky on
// escape).  Its next-event shadow rays are not traced in the thread: they go
// to a shadow queue, which the persistent any-hit kernel traces afterwards in
// one launch, adding each unoccluded contribution to its vertex.  A thread's
// serial chain is thus its closest-hit rays only (the shadow pass adds exact
// fixed-point sums, so a vertex's radiance does not depend on the order of the
// additions).  The targets kernels then
// form T_k = (sum of radiance at vertices j >= k) / throughput_k, the radiance
// the rest of the path carried back to vertex k: the (input, T_k) pairs are
// what the network learns, so that a path cut short at a vertex can be
// finished with throughput x cache(vertex).  Each path's samples go to an
// offset from a scan of the per-path counts, so their order is fixed.
// Pixels are drawn per frame by a hash of (frame, path index); random numbers
// are PCG32 streams keyed to the pixel and a per-frame sample index.
#include <cuda_runtime.h>

#include "bsm_pt.h"
#include "mlp.cuh"
#include "pt_device.h"
#include "pt_sky.cuh"
#include "pt_trace.cuh"
#include "pt_scene.cuh"
#include "pt_lights.cuh"

namespace bsm {

// A slot of `ctr` for each calling lane, one atomic per group of converged lanes.
__device__ __forceinline__ uint32_t agg_alloc(uint32_t* ctr) {
    const uint32_t m = __activemask(), lane = threadIdx.x & 31u;
    const uint32_t leader = (uint32_t)__ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(ctr, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ void queue_shadow(const Wavefront& q, uint32_t slot, V3 o, float tmin, V3 d, float tmax,
                                             V3 c, uint32_t vertex, uint32_t seed) {
    q.sh_o[slot] = make_float4(o.x, o.y, o.z, tmin);
    q.sh_d[slot] = make_float4(d.x, d.y, d.z, tmax);
    q.sh_c[slot] = make_float4(c.x, c.y, c.z, __uint_as_float(vertex));
    q.sh_seed[slot] = seed;
}

__global__ void __launch_bounds__(128, 4) k_train_paths(DevScene sc, const DevView* __restrict__ view, uint32_t n_paths,
                                                     uint32_t frame, TrainVerts tv, Wavefront q) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_paths) return;
    const DevView& v = *view;
    uint32_t npix = v.width * v.height;
    uint32_t pixel = (uint32_t)(mix64(((uint64_t)frame << 32) ^ (uint64_t)i ^ 0x5851f42d4c957f2dULL) % npix);
    uint32_t px = pixel % v.width, py = pixel / v.width;
    Pcg g = pcg_seed(sample_initstate(v.seed ^ 0x7f4a7c159e3779b9ULL, frame * n_paths + i), (uint64_t)pixel);
    float uvx = ((float)px + pcg_uniform(g)) / (float)v.width;
    float uvy = ((float)py + pcg_uniform(g)) / (float)v.height;
    V3 dl = normalize(v3((uvx * 2.0f - 1.0f) * v.aspect * v.tan_half, (1.0f - uvy * 2.0f) * v.tan_half, -1.0f));
    V3 sx = v3(v.s[0], v.s[1], v.s[2]), ux = v3(v.u[0], v.u[1], v.u[2]), fx = v3(v.f[0], v.f[1], v.f[2]);
    V3 d = normalize(sx * dl.x + ux * dl.y + (-fx) * dl.z);
    V3 o = v3(v.pos[0], v.pos[1], v.pos[2]);
    V3 thr = v3s(1.0f);
    float last_pdf = 0.0f;
    int nv = 0;
    const V3 box_lo = v3(sc.box_lo[0], sc.box_lo[1], sc.box_lo[2]);
    const V3 box_inv = v3(sc.box_inv[0], sc.box_inv[1], sc.box_inv[2]);
    const uint32_t segs = tv.segments;
    const uint32_t v0 = i * segs;                               // this path's first vertex
    const uint32_t sh_back = q.capacity * (sc.num_lights + 1u) - 1u;
    for (uint32_t seg = 0; seg < segs; ++seg) {
        RayPre r = make_ray(make_float4(o.x, o.y, o.z, v.t_min), make_float4(d.x, d.y, d.z, v.ray_length));
        float t, hu, hv;
        uint32_t inst;
        uint32_t leaf = trace_scene<false>(sc, r, v.ray_length, t, hu, hv, inst, (uint32_t)g.state);
        if (leaf == kMissPrim) {
            if (nv > 0) {
                V3 le = sky_eval(sc.sky, d);
                float pl = sky_pdf(sc.sky, d), pb = last_pdf;
                float w = (pb * pb + pl * pl) > 0.0f ? pb * pb / (pb * pb + pl * pl) : 1.0f;
                float4& rad = tv.rad[v0 + nv - 1];
                V3 e = thr * le * w;
                rad = make_float4(rad.x + e.x, rad.y + e.y, rad.z + e.z, 0.0f);
            }
            break;
        }
        V3 N, edge;
        uint32_t mi;
        hit_geometry(sc, leaf, inst, N, edge, mi);
        if (dot(N, d) > 0.0f) N = -N;
        const V3 Ng = N;
        if (sc.tri_normals) {
            N = shading_normal(sc, leaf, hu, hv, N);
            if (dot(N, d) > 0.0f) N = -N;
        }
        V3 P = o + d * t;
        float4 m0 = sc.materials[2 * mi], m1 = sc.materials[2 * mi + 1];
        Surface surf;
        surf.base_color = v3(m0.x, m0.y, m0.z);
        surf.roughness = m0.w;
        surf.f0 = v3(m1.x, m1.y, m1.z);
        surf.f90 = v3s(1.0f);
        surf.ior = 1.5f;
        V3 V = -d;
        const uint32_t vk = v0 + (uint32_t)nv++;
        {
            float raw[kMlpRaw];
            mlp_raw_inputs(P, box_lo, box_inv, V, N, surf.roughness, surf.base_color, (float)seg * 0.125f, raw);
            float4* rw = tv.raw + 3 * (size_t)vk;
            rw[0] = make_float4(raw[0], raw[1], raw[2], raw[3]);
            rw[1] = make_float4(raw[4], raw[5], raw[6], raw[7]);
            rw[2] = make_float4(raw[8], raw[9], raw[10], raw[11]);
        }
        tv.thr[vk] = make_float4(thr.x, thr.y, thr.z, 0.0f);
        tv.rad[vk] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        Frame fr = create_frame(N);
        V3 org = P + Ng * sc.ray_offset;
        float u_sky0 = pcg_uniform(g), u_sky1 = pcg_uniform(g), u_sky2 = pcg_uniform(g), u_lobe = pcg_uniform(g),
              u_b0 = pcg_uniform(g), u_b1 = pcg_uniform(g);
        float rx, ry;
        aniso_roughness(surf.roughness, &rx, &ry);
        V3 lv = to_local(fr, V);
        float p_spec = spec_probability(surf, lv.z);
        for (uint32_t l = 0; l < sc.num_lights; ++l) {
            const DevLight& lt = sc.lights[l];
            float ur0 = 0.0f, ur1 = 0.0f;
            if (__float_as_uint(lt.a.w) == kLightRect) { ur0 = pcg_uniform(g); ur1 = pcg_uniform(g); }
            V3 L, e;
            float smax;
            if (!light_sample(lt, P, ur0, ur1, v.ray_length, L, smax, e)) continue;
            V3 f = surface_eval_lit(N, fr.x, fr.y, V, L, surf);
            V3 c = thr * e * f;
            if (max_comp(c) > 0.0f)
                queue_shadow(q, agg_alloc(q.counters + kCntShadow), org, v.t_min, L, smax, c, vk, (uint32_t)g.state);
        }
        {
            float pl;
            V3 le;
            V3 L = sky_sample(sc.sky, u_sky0, u_sky1, u_sky2, pl, le);
            if (pl > 0.0f) {
                V3 f = surface_eval_lit(N, fr.x, fr.y, V, L, surf);
                if (max_comp(f) > 0.0f) {
                    float pb = mixture_pdf(lv, to_local(fr, L), rx, ry, p_spec);
                    V3 c = thr * le * f * ((pl * pl) / (pl * pl + pb * pb) / pl);
                    if (max_comp(c) > 0.0f)
                        queue_shadow(q, sh_back - agg_alloc(q.counters + kCntSky), org, v.t_min, L, v.ray_length, c,
                                     vk, (uint32_t)g.state);
                }
            }
        }
        if (seg + 1 >= segs || max_comp(thr) < 0.001f) break;
        V3 ll = u_lobe < p_spec ? reflect(-lv, ggx_vndf_sample(lv, rx, ry, u_b0, u_b1)) : cos_hemisphere_sample(u_b0, u_b1);
        if (!(ll.z > 0.0f)) break;
        V3 L = to_world(fr, ll);
        float pdf = mixture_pdf(lv, ll, rx, ry, p_spec);
        V3 f = surface_eval_lit(N, fr.x, fr.y, V, L, surf);
        V3 w = pdf > 0.0f ? f / pdf : v3s(0.0f);
        if (!isfinite(w.x) || !isfinite(w.y) || !isfinite(w.z)) break;
        thr = thr * w;
        if (!(max_comp(thr) > 0.0f)) break;
        o = org;
        d = L;
        last_pdf = pdf;
    }
    tv.count[i] = (uint32_t)nv;
}

// A vertex's gathered radiance: what its path thread wrote (the sky on escape) plus the shadow pass's exact
// fixed-point sums of its unoccluded next-event rays.
__device__ __forceinline__ V3 vertex_radiance(const TrainVerts& tv, uint32_t v) {
    const float4 r = tv.rad[v];
    const unsigned long long* p = tv.fx + 3 * (size_t)v;
    return v3(r.x + (float)((double)p[0] * 0x1p-32), r.y + (float)((double)p[1] * 0x1p-32),
              r.z + (float)((double)p[2] * 0x1p-32));
}

// Targets of path i: the radiance carried back to each vertex k (from the last vertex down), divided by the
// throughput there; emit(vertex, target) for each finite one, in that order.
template <class Emit>
__device__ __forceinline__ void path_targets(const TrainVerts& tv, uint32_t i, Emit emit) {
    const uint32_t v0 = i * tv.segments;
    const int nv = (int)tv.count[i];
    V3 acc = v3s(0.0f);
    for (int k = nv - 1; k >= 0; --k) {
        acc = acc + vertex_radiance(tv, v0 + (uint32_t)k);
        const float4 tk4 = tv.thr[v0 + k];
        const V3 tk = v3(tk4.x, tk4.y, tk4.z);
        if (!(tk.x > 0.0f && tk.y > 0.0f && tk.z > 0.0f)) continue;
        const V3 target = v3(acc.x / tk.x, acc.y / tk.y, acc.z / tk.z);
        if (!isfinite(target.x) || !isfinite(target.y) || !isfinite(target.z)) continue;
        emit(v0 + (uint32_t)k, target);
    }
}

// Inclusive sum of x over the threads of a block of kScanBlock threads up to this one; *total = the block's sum.
constexpr uint32_t kScanBlock = 256;
__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t x, uint32_t* total) {
    __shared__ uint32_t s_warp[kScanBlock / 32];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[w] = x;
    __syncthreads();
    uint32_t before = 0, all = 0;
#pragma unroll
    for (uint32_t k = 0; k < kScanBlock / 32; ++k) {
        const uint32_t t = s_warp[k];
        before += k < w ? t : 0u;
        all += t;
    }
    __syncthreads();   // s_warp is reused by the next call
    *total = all;
    return x + before;
}

// Per-path sample counts: each path's offset within its block (tv.offs) and each block's total (tv.nsamp[block]).
__global__ void __launch_bounds__(kScanBlock) k_train_count(uint32_t n_paths, TrainVerts tv) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t c = 0;
    if (i < n_paths) path_targets(tv, i, [&](uint32_t, V3) { ++c; });
    uint32_t total;
    const uint32_t incl = block_inclusive_scan(c, &total);
    if (i < n_paths) tv.offs[i] = incl - c;
    if (threadIdx.x == 0) tv.nsamp[blockIdx.x] = total;
}

// Exclusive scan, in place, of the n block totals by one block (in tiles of kScanBlock); *total = their sum.
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(uint32_t* cnt, uint32_t n, uint32_t* total) {
    uint32_t carry = 0;
    for (uint32_t b = 0; b < n; b += kScanBlock) {
        const uint32_t i = b + threadIdx.x;
        const uint32_t x = i < n ? cnt[i] : 0u;
        uint32_t sum;
        const uint32_t incl = block_inclusive_scan(x, &sum);
        if (i < n) cnt[i] = carry + incl - x;
        carry += sum;
    }
    if (threadIdx.x == 0) *total = carry;
}

// Writes path i's samples from its scanned offset on (those past max_samples are dropped); blocks of
// kScanBlock paths, as k_train_count's.
__global__ void __launch_bounds__(kScanBlock) k_train_targets(uint32_t n_paths, TrainVerts tv, float4* samples,
                                                              uint32_t max_samples) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_paths) return;
    uint32_t slot = tv.nsamp[blockIdx.x] + tv.offs[i];   // the block's first sample + the path's offset in it
    path_targets(tv, i, [&](uint32_t v, V3 target) {
        if (slot < max_samples) {
            const float4* rw = tv.raw + 3 * (size_t)v;
            float4* sd = samples + 4 * (size_t)slot;
            sd[0] = rw[0];
            sd[1] = rw[1];
            sd[2] = rw[2];
            sd[3] = make_float4(target.x, target.y, target.z, 0.0f);
        }
        ++slot;
    });
}

void launch_train_paths(cudaStream_t st, const DevScene& sc, const DevView* view, uint32_t n_paths, uint32_t frame,
                        const TrainVerts& tv, const Wavefront& shadow) {
    if (n_paths == 0) return;
    k_train_paths<<<(n_paths + 127) / 128, 128, 0, st>>>(sc, view, n_paths, frame, tv, shadow);
}

void launch_train_targets(cudaStream_t st, uint32_t n_paths, const TrainVerts& tv, float4* samples, uint32_t* count,
                          uint32_t max_samples) {
    if (n_paths == 0) return;
    const uint32_t blocks = (n_paths + kScanBlock - 1) / kScanBlock;
    k_train_count<<<blocks, kScanBlock, 0, st>>>(n_paths, tv);
    k_scan_blocks<<<1, kScanBlock, 0, st>>>(tv.nsamp, blocks, count);
    k_train_targets<<<blocks, kScanBlock, 0, st>>>(n_paths, tv, samples, max_samples);
}

}  // namespace bsm
