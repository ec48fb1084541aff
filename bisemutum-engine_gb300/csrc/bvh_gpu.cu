// bvh_gpu.cu — device build of the compressed 8-wide BVH (sm_103a).
//
// Replaces the driver-side BLAS build the reference requests through
// AccelerationStructure and runs on the GPU (bisemutum/src/graphics/accel.cpp:77-87,
// recorded by GraphicsManager::execute_immediately, graphics_manager.cpp:475-478).
// The tree is defined as in the host builder (bvh_build.cpp): a binary BVH by
// binned SAH over triangle centroids (Wald 2007), collapsed into 8-wide nodes by
// the SAH-optimal dynamic programme of Ylitie, Karras and Laine (HPG 2017) or by
// opening the largest child, children placed in octant slots, child boxes
// quantised outward to 8 bits per plane (bvh_quant.h).  Four phases:
//   1. triangle boxes and the scene's box and centroid bounds, one thread per
//      triangle;
//   2. the binary BVH top-down, one breadth-first level per round while a node
//      holds more than kSmall triangles.  Per level every CTA bins one chunk of
//      one node's triangle references into 3 x 32 centroid bins in shared
//      memory and merges them into the node's bins with one atomic per bin
//      value; one warp per node picks the split of least SAH cost; a stable
//      partition writes the children's references (warp ballots, one CTA per
//      chunk); the children become leaves, small nodes or next-level nodes.
//      Nodes of at most kSmall triangles are then finished by one warp each,
//      with their references in shared memory;
//   3. the collapse's dynamic programme bottom-up: a thread per binary leaf
//      climbs towards the root and stops at every node whose other child is not
//      done yet (the second thread to arrive computes the node; Karras 2012);
//   4. the 8-wide nodes top-down, one level per round: each node gathers its up
//      to eight children and assigns octant slots, a scan over the level gives
//      each node its first child and first triangle, and a second pass writes
//      the quantised node, its leaf triangles and the next level's queue, so
//      nodes and triangles come out in breadth-first order as on the host.
// Split decisions use exact bin counts and boxes (order-independent atomics on
// ordered float keys), and every partition is stable, so the tree does not
// depend on the order in which CTAs run.
#include "bvh_gpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "bvh_quant.h"

namespace bsm {
namespace {

constexpr uint32_t kNone = 0xffffffffu;
constexpr int kBins = 32;                  // lanes of a warp: one bin per lane
constexpr uint32_t kChunk = 4096;          // references per CTA in a level pass
constexpr uint32_t kSmall = 128;           // nodes of at most this many triangles are finished by one warp
constexpr int kSmallWarps = 4;             // warps per CTA of the small-node kernel
constexpr uint32_t kLevelThreads = 256;
constexpr uint8_t kDecLeaf = 0xff, kDecInner = 0xfe, kDecSame = 0xfd;
constexpr uint32_t kKeyLo = 0xffffffffu;   // initial key of a minimum
constexpr uint32_t kKeyHi = 0u;            // initial key of a maximum

// error bits of Counters::error
enum : uint32_t {
    kErrIndex = 1, kErrFinite = 2, kErrNodes = 4, kErrGather = 8, kErrLeaf = 16, kErrStack = 32, kErrClimb = 64,
    kErrWide = 128
};

struct BNode {                 // binary node
    float lo[3];
    uint32_t left;             // kNone: a leaf
    float hi[3];
    uint32_t right;
    uint32_t first, count;     // reference range (all nodes)
    uint32_t parent, pad;
};
static_assert(sizeof(BNode) == 48, "BNode must be 48 bytes");

struct Task {                  // a node still to split: its reference range and centroid bounds
    uint32_t node, begin, end, pad;
    float clo[3], chi[3];
};
struct Chunk {                 // a CTA's share of one task in a level pass
    uint32_t task, begin, end, pad;
    uint32_t left_base, right_base, pad2[2];
};
struct Bin { uint32_t cnt, lo[3], hi[3]; };      // box as ordered float keys
struct Split { int axis; int bin; uint32_t leaf; uint32_t nl; };
struct ChildAcc { uint32_t box[2][6]; uint32_t cen[2][6]; };   // per side: lo xyz, hi xyz (keys)
struct Counters { uint32_t nodes, next_tasks, small_tasks, error, ni_total, nt_total, pad[2]; };
struct WideRec { uint32_t child[8]; uint32_t ni, nt; };     // binary node per slot (kNone: empty slot)

// Order-preserving map of floats to unsigned keys (-0 below +0), so that
// unsigned atomicMin/atomicMax compute float minima and maxima exactly.
__device__ __forceinline__ uint32_t fkey(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float funkey(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ float area6(const float* lo, const float* hi) {
    float dx = fmaxf(0.0f, hi[0] - lo[0]), dy = fmaxf(0.0f, hi[1] - lo[1]), dz = fmaxf(0.0f, hi[2] - lo[2]);
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__device__ __forceinline__ int bin_of(float c, float lo, float scale, int B) {
    int b = (int)((c - lo) * scale);
    return min(max(b, 0), B - 1);
}

__device__ __forceinline__ float axis_scale(const Task& t, int a, int B) {
    float ext = t.chi[a] - t.clo[a];
    return ext > 0.0f ? (float)B / ext : 0.0f;
}

__device__ __forceinline__ float centroid(const float4& l, const float4& h, int a) {
    return a == 0 ? 0.5f * (l.x + h.x) : (a == 1 ? 0.5f * (l.y + h.y) : 0.5f * (l.z + h.z));
}

__device__ __forceinline__ float warp_min(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ------------------------------------------------------------ phase 1 ----
__global__ void __launch_bounds__(256) k_tri_boxes(const float* __restrict__ pos, uint32_t nv,
                                                   const uint32_t* __restrict__ idx, uint32_t nt,
                                                   float4* __restrict__ tlo, float4* __restrict__ thi,
                                                   uint32_t* __restrict__ gkeys, Counters* cnt) {
    __shared__ float s_red[8][12];
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    float v[12];   // box lo, box hi, centroid lo, centroid hi
    for (int k = 0; k < 3; ++k) { v[k] = v[6 + k] = INFINITY; v[3 + k] = v[9 + k] = -INFINITY; }
    if (t < nt) {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int c = 0; c < 3; ++c) {
            uint32_t vi = idx ? idx[3 * (size_t)t + c] : 3 * t + c;
            if (vi >= nv) { atomicOr(&cnt->error, kErrIndex); vi = 0; }
            for (int k = 0; k < 3; ++k) {
                float p = pos[3 * (size_t)vi + k];
                if (!isfinite(p)) atomicOr(&cnt->error, kErrFinite);
                lo[k] = fminf(lo[k], p);
                hi[k] = fmaxf(hi[k], p);
            }
        }
        tlo[t] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        thi[t] = make_float4(hi[0], hi[1], hi[2], 0.0f);
        for (int k = 0; k < 3; ++k) {
            float c = 0.5f * (lo[k] + hi[k]);
            v[k] = lo[k]; v[3 + k] = hi[k]; v[6 + k] = c; v[9 + k] = c;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 12; ++k) {
        bool mx = (k % 6) >= 3;
        v[k] = mx ? warp_max(v[k]) : warp_min(v[k]);
        if (lane == 0) s_red[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        const int k = threadIdx.x;
        bool mx = (k % 6) >= 3;
        float r = s_red[0][k];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = mx ? fmaxf(r, s_red[w][k]) : fminf(r, s_red[w][k]);
        if (mx) atomicMax(&gkeys[k], fkey(r)); else atomicMin(&gkeys[k], fkey(r));
    }
}

__global__ void k_iota(uint32_t* a, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

// ------------------------------------------------------------ phase 2 ----
__global__ void k_bins_init(Bin* bins, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Bin b;
    b.cnt = 0;
    for (int k = 0; k < 3; ++k) { b.lo[k] = kKeyLo; b.hi[k] = kKeyHi; }
    bins[i] = b;
}

__global__ void k_acc_init(ChildAcc* acc, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ChildAcc a;
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 3; ++k) {
            a.box[s][k] = kKeyLo; a.box[s][3 + k] = kKeyHi;
            a.cen[s][k] = kKeyLo; a.cen[s][3 + k] = kKeyHi;
        }
    acc[i] = a;
}

// Bins one chunk of one task's references by centroid, per axis, into shared
// bins, then merges the non-empty bins into the task's bins.
__global__ void __launch_bounds__(kLevelThreads) k_bin(const Chunk* __restrict__ chunks,
                                                       const Task* __restrict__ tasks,
                                                       const uint32_t* __restrict__ refs,
                                                       const float4* __restrict__ tlo,
                                                       const float4* __restrict__ thi, Bin* __restrict__ gbins,
                                                       int B) {
    __shared__ Bin sb[3 * kBins];
    for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
        sb[i].cnt = 0;
        for (int k = 0; k < 3; ++k) { sb[i].lo[k] = kKeyLo; sb[i].hi[k] = kKeyHi; }
    }
    __syncthreads();
    const Chunk ch = chunks[blockIdx.x];
    const Task tk = tasks[ch.task];
    float sc[3];
    for (int a = 0; a < 3; ++a) sc[a] = axis_scale(tk, a, B);
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
        const uint32_t r = refs[i];
        const float4 l = tlo[r], h = thi[r];
        const uint32_t kl[3] = {fkey(l.x), fkey(l.y), fkey(l.z)}, kh[3] = {fkey(h.x), fkey(h.y), fkey(h.z)};
        for (int a = 0; a < 3; ++a) {
            if (!(sc[a] > 0.0f)) continue;
            Bin& b = sb[a * kBins + bin_of(centroid(l, h, a), tk.clo[a], sc[a], B)];
            atomicAdd(&b.cnt, 1u);
            for (int k = 0; k < 3; ++k) { atomicMin(&b.lo[k], kl[k]); atomicMax(&b.hi[k], kh[k]); }
        }
    }
    __syncthreads();
    Bin* g = gbins + (size_t)ch.task * 3 * kBins;
    for (int i = threadIdx.x; i < 3 * kBins; i += blockDim.x) {
        if (sb[i].cnt == 0) continue;
        atomicAdd(&g[i].cnt, sb[i].cnt);
        for (int k = 0; k < 3; ++k) { atomicMin(&g[i].lo[k], sb[i].lo[k]); atomicMax(&g[i].hi[k], sb[i].hi[k]); }
    }
}

// The least-cost split over three axes of binned SAH (bvh_build.cpp Builder::build):
// cost(split before bin b) = area(left) * n_left + area(right) * n_right, axes
// in order and bins ascending, the first minimum kept.  One warp; lane = bin.
// `bins(a)` returns this lane's bin of axis a.  Returns the axis (-1: none).
template <class GetBin>
__device__ int warp_best_split(const Task& tk, int B, GetBin bins, int* best_bin, uint32_t* best_nl, float* best_cost) {
    const int lane = threadIdx.x & 31;
    float best = INFINITY;
    int bax = -1, bbin = 0;
    uint32_t bnl = 0;
    for (int a = 0; a < 3; ++a) {
        if (!(tk.chi[a] - tk.clo[a] > 0.0f)) continue;
        Bin b = bins(a);
        uint32_t n = lane < B ? b.cnt : 0u;
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {
            lo[k] = n ? funkey(b.lo[k]) : INFINITY;
            hi[k] = n ? funkey(b.hi[k]) : -INFINITY;
        }
        // inclusive prefix (bins 0..lane) and suffix (bins lane..31)
        uint32_t ln = n, rn = n;
        float llo[3], lhi[3], rlo[3], rhi[3];
        for (int k = 0; k < 3; ++k) { llo[k] = rlo[k] = lo[k]; lhi[k] = rhi[k] = hi[k]; }
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t un = __shfl_up_sync(0xffffffffu, ln, off), dn = __shfl_down_sync(0xffffffffu, rn, off);
            float ul[3], uh[3], dl[3], dh[3];
            for (int k = 0; k < 3; ++k) {
                ul[k] = __shfl_up_sync(0xffffffffu, llo[k], off);
                uh[k] = __shfl_up_sync(0xffffffffu, lhi[k], off);
                dl[k] = __shfl_down_sync(0xffffffffu, rlo[k], off);
                dh[k] = __shfl_down_sync(0xffffffffu, rhi[k], off);
            }
            if (lane >= off) {
                ln += un;
                for (int k = 0; k < 3; ++k) { llo[k] = fminf(llo[k], ul[k]); lhi[k] = fmaxf(lhi[k], uh[k]); }
            }
            if (lane + off < 32) {
                rn += dn;
                for (int k = 0; k < 3; ++k) { rlo[k] = fminf(rlo[k], dl[k]); rhi[k] = fmaxf(rhi[k], dh[k]); }
            }
        }
        // split before bin `lane`: left = prefix of lane - 1, right = suffix of lane
        uint32_t pn = __shfl_up_sync(0xffffffffu, ln, 1);
        float pl[3], ph[3];
        for (int k = 0; k < 3; ++k) {
            pl[k] = __shfl_up_sync(0xffffffffu, llo[k], 1);
            ph[k] = __shfl_up_sync(0xffffffffu, lhi[k], 1);
        }
        float cost = INFINITY;
        if (lane >= 1 && lane < B && pn > 0 && rn > 0) cost = area6(pl, ph) * (float)pn + area6(rlo, rhi) * (float)rn;
        float m = cost;
        int ml = lane;
        for (int o = 16; o > 0; o >>= 1) {
            float om = __shfl_xor_sync(0xffffffffu, m, o);
            int ol = __shfl_xor_sync(0xffffffffu, ml, o);
            if (om < m || (om == m && ol < ml)) { m = om; ml = ol; }
        }
        uint32_t nl_at = __shfl_sync(0xffffffffu, pn, ml);
        if (m < best) { best = m; bax = a; bbin = ml; bnl = nl_at; }
    }
    *best_bin = bbin;
    *best_nl = bnl;
    *best_cost = best;
    return bax;
}

// Split or leaf of a node of `cnt` triangles and box area `parent_area`, as bvh_build.cpp decides.
__device__ __forceinline__ Split decide(int bax, int bbin, uint32_t bnl, float best, uint32_t cnt, float parent_area,
                                        uint32_t max_leaf) {
    Split s;
    s.leaf = 0;
    s.axis = bax;
    s.bin = bbin;
    s.nl = bnl;
    float split_cost = parent_area > 0.0f ? 1.0f + best / parent_area : INFINITY;
    if (bax < 0) {
        if (cnt <= max_leaf) s.leaf = 1;
        else s.nl = cnt / 2;   // every centroid in one place: split by index
    } else if (cnt <= max_leaf && (float)cnt <= split_cost) {
        s.leaf = 1;
    }
    if (s.leaf) s.nl = cnt;
    return s;
}

__global__ void k_split(const Task* __restrict__ tasks, uint32_t ntasks, const Bin* __restrict__ gbins,
                        const BNode* __restrict__ nodes, Split* __restrict__ splits, int B, uint32_t max_leaf) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= ntasks) return;   // whole warps
    const Task tk = tasks[w];
    int bbin;
    uint32_t bnl;
    float best;
    int bax = warp_best_split(tk, B, [&](int a) {
        Bin e;
        e.cnt = 0;
        return lane < B ? gbins[((size_t)w * 3 + a) * kBins + lane] : e;
    }, &bbin, &bnl, &best);
    const BNode nd = nodes[tk.node];
    Split s = decide(bax, bbin, bnl, best, tk.end - tk.begin, area6(nd.lo, nd.hi), max_leaf);
    if (lane == 0) splits[w] = s;
}

__device__ __forceinline__ bool goes_left(const Task& tk, const Split& sp, uint32_t i, const float4& l,
                                          const float4& h, int B) {
    if (sp.leaf) return true;
    if (sp.axis < 0) return i - tk.begin < sp.nl;
    const int a = sp.axis;
    return bin_of(centroid(l, h, a), tk.clo[a], axis_scale(tk, a, B), B) < sp.bin;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_tmp) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_tmp[w];
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(kLevelThreads) k_count_left(const Chunk* __restrict__ chunks,
                                                              const Task* __restrict__ tasks,
                                                              const Split* __restrict__ splits,
                                                              const uint32_t* __restrict__ refs,
                                                              const float4* __restrict__ tlo,
                                                              const float4* __restrict__ thi,
                                                              uint32_t* __restrict__ chunk_left, int B) {
    __shared__ uint32_t s_tmp[32];
    const Chunk ch = chunks[blockIdx.x];
    const Task tk = tasks[ch.task];
    const Split sp = splits[ch.task];
    uint32_t n = 0;
    for (uint32_t i = ch.begin + threadIdx.x; i < ch.end; i += blockDim.x) {
        uint32_t r = refs[i];
        n += goes_left(tk, sp, i, tlo[r], thi[r], B) ? 1u : 0u;
    }
    n = block_sum(n, s_tmp);
    if (threadIdx.x == 0) chunk_left[blockIdx.x] = n;
}

// Stable partition of one chunk: left references to left_base.., right ones to
// right_base.. (both in chunk order); the children's boxes and centroid bounds
// are reduced over the block and merged into the task's accumulator.
__global__ void __launch_bounds__(kLevelThreads) k_partition(const Chunk* __restrict__ chunks,
                                                             const Task* __restrict__ tasks,
                                                             const Split* __restrict__ splits,
                                                             const uint32_t* __restrict__ in,
                                                             uint32_t* __restrict__ out,
                                                             const float4* __restrict__ tlo,
                                                             const float4* __restrict__ thi,
                                                             ChildAcc* __restrict__ acc, int B) {
    __shared__ uint32_t s_wl[kLevelThreads / 32], s_wr[kLevelThreads / 32];
    __shared__ float s_red[kLevelThreads / 32][24];
    const Chunk ch = chunks[blockIdx.x];
    const Task tk = tasks[ch.task];
    const Split sp = splits[ch.task];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    float v[24];   // side s: box lo(3) hi(3), centroid lo(3) hi(3) at 12 s
    for (int s = 0; s < 2; ++s)
        for (int k = 0; k < 3; ++k) {
            v[12 * s + k] = v[12 * s + 6 + k] = INFINITY;
            v[12 * s + 3 + k] = v[12 * s + 9 + k] = -INFINITY;
        }
    uint32_t lb = ch.left_base, rb = ch.right_base;
    for (uint32_t base = ch.begin; base < ch.end; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool act = i < ch.end;
        uint32_t r = 0;
        float4 l = make_float4(0, 0, 0, 0), h = l;
        bool left = false;
        if (act) {
            r = in[i];
            l = tlo[r];
            h = thi[r];
            left = goes_left(tk, sp, i, l, h, B);
        }
        const bool right = act && !left;
        const uint32_t wl = __ballot_sync(0xffffffffu, left), wr = __ballot_sync(0xffffffffu, right);
        if (lane == 0) { s_wl[warp] = __popc(wl); s_wr[warp] = __popc(wr); }
        __syncthreads();
        uint32_t pl = 0, pr = 0, tl = 0, tr = 0;
        for (int w = 0; w < nw; ++w) {
            if (w < warp) { pl += s_wl[w]; pr += s_wr[w]; }
            tl += s_wl[w];
            tr += s_wr[w];
        }
        if (left) out[lb + pl + __popc(wl & lt)] = r;
        if (right) out[rb + pr + __popc(wr & lt)] = r;
        lb += tl;
        rb += tr;
        __syncthreads();
        if (act) {
            float* s = v + (left ? 0 : 12);
            const float lo[3] = {l.x, l.y, l.z}, hi[3] = {h.x, h.y, h.z};
            for (int k = 0; k < 3; ++k) {
                float c = 0.5f * (lo[k] + hi[k]);
                s[k] = fminf(s[k], lo[k]);
                s[3 + k] = fmaxf(s[3 + k], hi[k]);
                s[6 + k] = fminf(s[6 + k], c);
                s[9 + k] = fmaxf(s[9 + k], c);
            }
        }
    }
    for (int k = 0; k < 24; ++k) {
        const bool mx = (k % 6) >= 3;
        v[k] = mx ? warp_max(v[k]) : warp_min(v[k]);
        if (lane == 0) s_red[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 24) {
        const int k = threadIdx.x;
        const bool mx = (k % 6) >= 3;
        float r = s_red[0][k];
        for (int w = 1; w < nw; ++w) r = mx ? fmaxf(r, s_red[w][k]) : fminf(r, s_red[w][k]);
        if (r == INFINITY || r == -INFINITY) return;   // that side is empty in this chunk
        const int side = k / 12, j = k % 12;
        uint32_t* dst = j < 6 ? &acc[ch.task].box[side][j] : &acc[ch.task].cen[side][j - 6];
        if (mx) atomicMax(dst, fkey(r)); else atomicMin(dst, fkey(r));
    }
}

// Children of every split task: two binary nodes each; a child of one triangle
// is a leaf, a child of at most kSmall goes to the small list, any other to the
// next level.  Leaves and small children copy their references to `final`.
__global__ void k_make_children(const Task* __restrict__ tasks, uint32_t ntasks, const Split* __restrict__ splits,
                                const ChildAcc* __restrict__ acc, const uint32_t* __restrict__ refs,
                                BNode* __restrict__ nodes, uint32_t* __restrict__ final_refs, Task* __restrict__ next,
                                uint32_t next_cap, Task* __restrict__ small, uint32_t small_cap, Counters* cnt,
                                uint32_t max_nodes) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntasks) return;
    const Task tk = tasks[i];
    const Split sp = splits[i];
    if (sp.leaf) {
        for (uint32_t k = tk.begin; k < tk.end; ++k) final_refs[k] = refs[k];
        return;
    }
    const uint32_t id = atomicAdd(&cnt->nodes, 2u);
    if (id + 2u > max_nodes) { atomicOr(&cnt->error, kErrNodes); return; }
    nodes[tk.node].left = id;
    nodes[tk.node].right = id + 1u;
    const ChildAcc& a = acc[i];
    for (int s = 0; s < 2; ++s) {
        const uint32_t cb = s ? tk.begin + sp.nl : tk.begin, ce = s ? tk.end : tk.begin + sp.nl;
        BNode n;
        for (int k = 0; k < 3; ++k) { n.lo[k] = funkey(a.box[s][k]); n.hi[k] = funkey(a.box[s][3 + k]); }
        n.left = n.right = kNone;
        n.first = cb;
        n.count = ce - cb;
        n.parent = tk.node;
        n.pad = 0;
        nodes[id + s] = n;
        if (n.count <= 1u) {
            for (uint32_t k = cb; k < ce; ++k) final_refs[k] = refs[k];
            continue;
        }
        Task c;
        c.node = id + s;
        c.begin = cb;
        c.end = ce;
        c.pad = 0;
        for (int k = 0; k < 3; ++k) { c.clo[k] = funkey(a.cen[s][k]); c.chi[k] = funkey(a.cen[s][3 + k]); }
        if (n.count <= kSmall) {
            for (uint32_t k = cb; k < ce; ++k) final_refs[k] = refs[k];
            uint32_t slot = atomicAdd(&cnt->small_tasks, 1u);
            if (slot < small_cap) small[slot] = c; else atomicOr(&cnt->error, kErrNodes);
        } else {
            uint32_t slot = atomicAdd(&cnt->next_tasks, 1u);
            if (slot < next_cap) next[slot] = c; else atomicOr(&cnt->error, kErrNodes);
        }
    }
}

// Finishes the subtree of one small node per warp with its references in
// shared memory: the same binned SAH splits, a stable warp partition, children
// pushed on a per-warp stack (every entry holds two or more references of a
// disjoint range, so at most kSmall / 2 entries are live).
__global__ void __launch_bounds__(kSmallWarps * 32) k_small(const Task* __restrict__ small, uint32_t nsmall,
                                                            uint32_t* __restrict__ final_refs,
                                                            const float4* __restrict__ tlo,
                                                            const float4* __restrict__ thi, BNode* __restrict__ nodes,
                                                            Counters* cnt, int B, uint32_t max_leaf,
                                                            uint32_t max_nodes) {
    __shared__ uint32_t s_refs[kSmallWarps][kSmall], s_tmp[kSmallWarps][kSmall];
    __shared__ Bin s_bins[kSmallWarps][3 * kBins];
    __shared__ uint32_t s_stack[kSmallWarps][kSmall / 2][3];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ti = blockIdx.x * kSmallWarps + warp;
    if (ti >= nsmall) return;   // whole warps; no block-wide barrier below
    const uint32_t lt = (1u << lane) - 1u;
    const Task root = small[ti];
    const uint32_t n0 = root.end - root.begin;
    if (n0 > kSmall) { if (lane == 0) atomicOr(&cnt->error, kErrStack); return; }
    uint32_t* R = s_refs[warp];
    uint32_t* T = s_tmp[warp];
    Bin* SB = s_bins[warp];
    for (uint32_t i = lane; i < n0; i += 32) R[i] = final_refs[root.begin + i];
    int sp = 0;
    if (lane == 0) { s_stack[warp][0][0] = root.node; s_stack[warp][0][1] = 0; s_stack[warp][0][2] = n0; }
    sp = 1;
    __syncwarp();
    bool failed = false;
    while (sp > 0 && !failed) {
        --sp;
        const uint32_t node = s_stack[warp][sp][0], b = s_stack[warp][sp][1], e = s_stack[warp][sp][2];
        __syncwarp();
        const uint32_t n = e - b;
        // centroid bounds
        Task tk;
        tk.node = node;
        tk.begin = b;
        tk.end = e;
        float cl[3] = {INFINITY, INFINITY, INFINITY}, chv[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = b + lane; i < e; i += 32) {
            uint32_t r = R[i];
            float4 l = tlo[r], h = thi[r];
            for (int a = 0; a < 3; ++a) {
                float c = centroid(l, h, a);
                cl[a] = fminf(cl[a], c);
                chv[a] = fmaxf(chv[a], c);
            }
        }
        for (int a = 0; a < 3; ++a) { tk.clo[a] = warp_min(cl[a]); tk.chi[a] = warp_max(chv[a]); }
        // bins
        for (int i = lane; i < 3 * kBins; i += 32) {
            SB[i].cnt = 0;
            for (int k = 0; k < 3; ++k) { SB[i].lo[k] = kKeyLo; SB[i].hi[k] = kKeyHi; }
        }
        __syncwarp();
        float sc[3];
        for (int a = 0; a < 3; ++a) sc[a] = axis_scale(tk, a, B);
        for (uint32_t i = b + lane; i < e; i += 32) {
            uint32_t r = R[i];
            float4 l = tlo[r], h = thi[r];
            const uint32_t kl[3] = {fkey(l.x), fkey(l.y), fkey(l.z)}, kh[3] = {fkey(h.x), fkey(h.y), fkey(h.z)};
            for (int a = 0; a < 3; ++a) {
                if (!(sc[a] > 0.0f)) continue;
                Bin& bb = SB[a * kBins + bin_of(centroid(l, h, a), tk.clo[a], sc[a], B)];
                atomicAdd(&bb.cnt, 1u);
                for (int k = 0; k < 3; ++k) { atomicMin(&bb.lo[k], kl[k]); atomicMax(&bb.hi[k], kh[k]); }
            }
        }
        __syncwarp();
        int bbin;
        uint32_t bnl;
        float best;
        int bax = warp_best_split(tk, B, [&](int a) {
            Bin z;
            z.cnt = 0;
            return lane < B ? SB[a * kBins + lane] : z;
        }, &bbin, &bnl, &best);
        const BNode nd = nodes[node];
        Split s = decide(bax, bbin, bnl, best, n, area6(nd.lo, nd.hi), max_leaf);
        __syncwarp();
        if (s.leaf) continue;
        if (s.axis >= 0) {   // stable partition through T
            uint32_t lc = 0, rc = 0;
            for (uint32_t base = b; base < e; base += 32) {
                const uint32_t i = base + lane;
                const bool act = i < e;
                uint32_t r = act ? R[i] : 0u;
                bool left = false;
                if (act) left = goes_left(tk, s, i, tlo[r], thi[r], B);
                const bool right = act && !left;
                const uint32_t wl = __ballot_sync(0xffffffffu, left), wr = __ballot_sync(0xffffffffu, right);
                if (left) T[b + lc + __popc(wl & lt)] = r;
                if (right) T[b + s.nl + rc + __popc(wr & lt)] = r;
                lc += __popc(wl);
                rc += __popc(wr);
            }
            __syncwarp();
            for (uint32_t i = b + lane; i < e; i += 32) R[i] = T[i];
            __syncwarp();
        }
        const uint32_t mid = b + s.nl;
        // children's boxes
        float bl[2][6];
        for (int c = 0; c < 2; ++c) {
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            const uint32_t cb = c ? mid : b, ce = c ? e : mid;
            for (uint32_t i = cb + lane; i < ce; i += 32) {
                float4 l = tlo[R[i]], h = thi[R[i]];
                lo[0] = fminf(lo[0], l.x); lo[1] = fminf(lo[1], l.y); lo[2] = fminf(lo[2], l.z);
                hi[0] = fmaxf(hi[0], h.x); hi[1] = fmaxf(hi[1], h.y); hi[2] = fmaxf(hi[2], h.z);
            }
            for (int k = 0; k < 3; ++k) { bl[c][k] = warp_min(lo[k]); bl[c][3 + k] = warp_max(hi[k]); }
        }
        uint32_t id = 0;
        if (lane == 0) id = atomicAdd(&cnt->nodes, 2u);
        id = __shfl_sync(0xffffffffu, id, 0);
        if (id + 2u > max_nodes) {
            if (lane == 0) atomicOr(&cnt->error, kErrNodes);
            failed = true;
            break;
        }
        if (lane == 0) {
            nodes[node].left = id;
            nodes[node].right = id + 1u;
            for (int c = 0; c < 2; ++c) {
                BNode cn;
                for (int k = 0; k < 3; ++k) { cn.lo[k] = bl[c][k]; cn.hi[k] = bl[c][3 + k]; }
                cn.left = cn.right = kNone;
                cn.first = root.begin + (c ? mid : b);
                cn.count = c ? e - mid : mid - b;
                cn.parent = node;
                cn.pad = 0;
                nodes[id + c] = cn;
            }
        }
        // push right then left (left is finished first); single-reference children are leaves
        const uint32_t ranges[2][2] = {{mid, e}, {b, mid}};
        for (int c = 0; c < 2; ++c) {
            const uint32_t cb = ranges[c][0], ce = ranges[c][1];
            if (ce - cb <= 1u) continue;
            if (sp >= (int)(kSmall / 2)) {
                if (lane == 0) atomicOr(&cnt->error, kErrStack);
                failed = true;
                break;
            }
            if (lane == 0) {
                s_stack[warp][sp][0] = id + (c == 0 ? 1u : 0u);
                s_stack[warp][sp][1] = cb;
                s_stack[warp][sp][2] = ce;
            }
            ++sp;
        }
        __syncwarp();
    }
    __syncwarp();
    for (uint32_t i = lane; i < n0; i += 32) final_refs[root.begin + i] = R[i];
}

// ------------------------------------------------------------ phase 3 ----
// cost(n, i) for i = 1..8 and the decisions, as the host's Collapse::run.
__global__ void k_collapse(const BNode* __restrict__ nodes, uint32_t n, uint32_t* __restrict__ visits,
                           float* __restrict__ cost, uint8_t* __restrict__ dec, uint8_t* __restrict__ isplit,
                           uint32_t max_leaf, float tri_cost, Counters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BNode L = nodes[i];
    if (L.left != kNone) return;   // climbs start at leaves
    {
        const float a = area6(L.lo, L.hi);
        const float leaf = L.count <= max_leaf ? a * (float)L.count * tri_cost : INFINITY;
        for (int k = 0; k < 8; ++k) {
            cost[8 * (size_t)i + k] = leaf;
            dec[8 * (size_t)i + k] = k == 0 ? kDecLeaf : kDecSame;
        }
    }
    __threadfence();
    uint32_t x = L.parent;
    for (uint32_t guard = 0; x != kNone; ++guard) {
        if (guard > n) { atomicOr(&cnt->error, kErrClimb); return; }
        if (atomicAdd(&visits[x], 1u) == 0u) return;   // the other child is not done yet
        __threadfence();
        const BNode X = nodes[x];
        float cl[8], cr[8];
        for (int k = 0; k < 8; ++k) {
            cl[k] = __ldcg(&cost[8 * (size_t)X.left + k]);
            cr[k] = __ldcg(&cost[8 * (size_t)X.right + k]);
        }
        float dist[9];
        uint8_t arg[9];
        for (int j = 2; j <= 8; ++j) {
            dist[j] = INFINITY;
            arg[j] = 1;
            for (int k = 1; k < j; ++k) {
                float v = cl[k - 1] + cr[j - k - 1];
                if (v < dist[j]) { dist[j] = v; arg[j] = (uint8_t)k; }
            }
        }
        const float a = area6(X.lo, X.hi);
        const float leaf = X.count <= max_leaf ? a * (float)X.count * tri_cost : INFINITY;
        const float inner = a + dist[8];   // node cost 1
        float c[8];
        uint8_t d[8];
        if (leaf <= inner) { c[0] = leaf; d[0] = kDecLeaf; } else { c[0] = inner; d[0] = kDecInner; }
        for (int k = 2; k <= 8; ++k) {
            if (c[k - 2] <= dist[k]) { c[k - 1] = c[k - 2]; d[k - 1] = kDecSame; }
            else { c[k - 1] = dist[k]; d[k - 1] = arg[k]; }
        }
        for (int k = 0; k < 8; ++k) {
            cost[8 * (size_t)x + k] = c[k];
            dec[8 * (size_t)x + k] = d[k];
        }
        isplit[x] = arg[8];
        __threadfence();
        x = X.parent;
    }
}

__global__ void k_sah_cost(const BNode* __restrict__ nodes, uint32_t n, double* out) {
    __shared__ double s[8];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        const BNode b = nodes[i];
        v = (double)area6(b.lo, b.hi) * (b.left == kNone ? (double)b.count : 1.0);
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
        atomicAdd(out, t);
    }
}

// ------------------------------------------------------------ phase 4 ----
struct WideCfg {
    const BNode* nodes;
    const uint8_t* dec;
    const uint8_t* isplit;
    bool optimal;
    uint32_t max_leaf;
};

__device__ __forceinline__ bool wide_leaf(const WideCfg& w, uint32_t x) {
    if (w.optimal) return w.dec[8 * (size_t)x] == kDecLeaf;
    const BNode& b = w.nodes[x];
    return b.left == kNone || b.count <= w.max_leaf;
}

// Children of a wide node and their octant slots (bvh_build.cpp: gather, then
// the greedy slot assignment by the children's offsets from the node centre).
__global__ void k_wide_gather(const uint32_t* __restrict__ queue, uint32_t nq, WideCfg w, WideRec* __restrict__ rec,
                              uint32_t* __restrict__ ni_out, uint32_t* __restrict__ nt_out, Counters* cnt) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const uint32_t bi = queue[q];
    uint32_t ch[8];
    int nc = 0;
    bool bad = false;
    const BNode& bn = w.nodes[bi];
    if (wide_leaf(w, bi)) {
        ch[nc++] = bi;   // a root that is a single leaf
    } else if (w.optimal) {
        uint32_t stx[16], sti[16];
        int sp = 0;
        const uint32_t k = w.isplit[bi];
        stx[sp] = bn.right; sti[sp++] = 8u - k;
        stx[sp] = bn.left; sti[sp++] = k;
        while (sp > 0) {
            --sp;
            const uint32_t x = stx[sp];
            uint32_t i = sti[sp];
            while (i > 1u && w.dec[8 * (size_t)x + i - 1] == kDecSame) --i;
            if (i <= 1u) {
                if (nc >= 8) { bad = true; break; }
                ch[nc++] = x;
                continue;
            }
            const uint32_t k2 = w.dec[8 * (size_t)x + i - 1];
            if (sp + 2 > 16 || k2 == 0u || k2 >= i || w.nodes[x].left == kNone) { bad = true; break; }
            stx[sp] = w.nodes[x].right; sti[sp++] = i - k2;
            stx[sp] = w.nodes[x].left; sti[sp++] = k2;
        }
    } else {
        ch[nc++] = bn.left;
        ch[nc++] = bn.right;
        while (nc < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (int i = 0; i < nc; ++i) {
                if (wide_leaf(w, ch[i])) continue;
                const BNode& c = w.nodes[ch[i]];
                float a = area6(c.lo, c.hi);
                if (a > best_area) { best_area = a; best = i; }
            }
            if (best < 0) break;
            const uint32_t open = ch[best];
            ch[best] = w.nodes[open].left;
            ch[nc++] = w.nodes[open].right;
        }
    }
    WideRec r;
    for (int s = 0; s < 8; ++s) r.child[s] = kNone;
    r.ni = r.nt = 0;
    if (bad || nc == 0) {
        atomicOr(&cnt->error, kErrGather);
        rec[q] = r;
        ni_out[q] = 0;
        nt_out[q] = 0;
        return;
    }
    float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < nc; ++i) {
        const BNode& c = w.nodes[ch[i]];
        for (int k = 0; k < 3; ++k) { nlo[k] = fminf(nlo[k], c.lo[k]); nhi[k] = fmaxf(nhi[k], c.hi[k]); }
    }
    float ctr[3];
    for (int k = 0; k < 3; ++k) ctr[k] = 0.5f * (nlo[k] + nhi[k]);
    bool slot_used[8] = {false, false, false, false, false, false, false, false};
    bool done[8] = {false, false, false, false, false, false, false, false};
    for (int round = 0; round < nc; ++round) {
        float best = -INFINITY;
        int bi2 = -1, bs = -1;
        for (int i = 0; i < nc; ++i) {
            if (done[i]) continue;
            const BNode& c = w.nodes[ch[i]];
            float d[3];
            for (int k = 0; k < 3; ++k) d[k] = 0.5f * (c.lo[k] + c.hi[k]) - ctr[k];
            for (int s = 0; s < 8; ++s) {
                if (slot_used[s]) continue;
                float cost = ((s & 1) ? d[0] : -d[0]) + ((s & 2) ? d[1] : -d[1]) + ((s & 4) ? d[2] : -d[2]);
                if (cost > best || bi2 < 0) { best = cost; bi2 = i; bs = s; }
            }
        }
        slot_used[bs] = true;
        done[bi2] = true;
        r.child[bs] = ch[bi2];
    }
    for (int i = 0; i < nc; ++i) {
        if (wide_leaf(w, ch[i])) r.nt += w.nodes[ch[i]].count;
        else r.ni += 1;
    }
    rec[q] = r;
    ni_out[q] = r.ni;
    nt_out[q] = r.nt;
}

// Exclusive scans of two count arrays in place (one block), totals to cnt.
__global__ void __launch_bounds__(1024) k_scan2(uint32_t* __restrict__ a, uint32_t* __restrict__ b, uint32_t n,
                                               Counters* cnt) {
    __shared__ uint32_t s_a[32], s_b[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t carry_a = 0, carry_b = 0;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t va = i < n ? a[i] : 0u, vb = i < n ? b[i] : 0u;
        uint32_t xa = va, xb = vb;   // inclusive warp scans
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t ta = __shfl_up_sync(0xffffffffu, xa, o), tb = __shfl_up_sync(0xffffffffu, xb, o);
            if (lane >= o) { xa += ta; xb += tb; }
        }
        if (lane == 31) { s_a[warp] = xa; s_b[warp] = xb; }
        __syncthreads();
        if (warp == 0) {
            uint32_t ya = lane < (int)(blockDim.x >> 5) ? s_a[lane] : 0u;
            uint32_t yb = lane < (int)(blockDim.x >> 5) ? s_b[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t ta = __shfl_up_sync(0xffffffffu, ya, o), tb = __shfl_up_sync(0xffffffffu, yb, o);
                if (lane >= o) { ya += ta; yb += tb; }
            }
            s_a[lane] = ya;   // inclusive totals of warps 0..lane
            s_b[lane] = yb;
        }
        __syncthreads();
        const uint32_t wa = warp ? s_a[warp - 1] : 0u, wb = warp ? s_b[warp - 1] : 0u;
        if (i < n) {
            a[i] = carry_a + wa + xa - va;
            b[i] = carry_b + wb + xb - vb;
        }
        carry_a += s_a[31];
        carry_b += s_b[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) { cnt->ni_total = carry_a; cnt->nt_total = carry_b; }
}

struct TriSrc {
    const float* pos;
    const uint32_t* idx;
    const uint32_t* mat;
    const float* transp;
    uint32_t num_materials;
    const uint32_t* final_refs;
};

__device__ void emit_tri(const TriSrc& s, uint32_t t, CwTri* out) {
    CwTri c;
    float v[3][3];
    for (int k = 0; k < 3; ++k) {
        const size_t vi = s.idx ? s.idx[3 * (size_t)t + k] : 3 * (size_t)t + k;
        v[k][0] = s.pos[3 * vi];
        v[k][1] = s.pos[3 * vi + 1];
        v[k][2] = s.pos[3 * vi + 2];
    }
    c.v0x = v[0][0]; c.v0y = v[0][1]; c.v0z = v[0][2];
    c.v1x = v[1][0]; c.v1y = v[1][1]; c.v1z = v[1][2];
    c.v2x = v[2][0]; c.v2y = v[2][1]; c.v2z = v[2][2];
    c.prim = t;
    c.material = s.mat ? s.mat[t] : 0u;
    const float tr = (s.transp && c.material < s.num_materials) ? s.transp[c.material] : 0.0f;
    c.pad = __float_as_uint(tr);
    *out = c;
}

__global__ void k_wide_write(const uint32_t* __restrict__ queue, uint32_t nq, const WideRec* __restrict__ rec,
                             const uint32_t* __restrict__ ni_off, const uint32_t* __restrict__ nt_off, WideCfg w,
                             TriSrc src, CwNode* __restrict__ wnodes, uint32_t wnode_cap, CwTri* __restrict__ wtris,
                             uint32_t num_tris, uint32_t* __restrict__ next_queue, uint32_t level_base,
                             uint32_t next_base, uint32_t tri_base0, Counters* cnt) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const WideRec R = rec[q];
    float lo[8][3], hi[8][3];
    uint32_t used = 0;
    for (int s = 0; s < 8; ++s) {
        for (int k = 0; k < 3; ++k) { lo[s][k] = 0.0f; hi[s][k] = 0.0f; }
        if (R.child[s] == kNone) continue;
        used |= 1u << s;
        const BNode& c = w.nodes[R.child[s]];
        for (int k = 0; k < 3; ++k) { lo[s][k] = c.lo[k]; hi[s][k] = c.hi[k]; }
    }
    CwNode node;
    memset(&node, 0, sizeof(node));
    float nlo[3], nhi[3];
    if (used) tlas_quantise(node, lo, hi, used, nlo, nhi);
    node.child_base = next_base + ni_off[q];
    node.tri_base = tri_base0 + nt_off[q];
    uint32_t k = 0, toff = 0;
    for (int s = 0; s < 8; ++s) {
        const uint32_t x = R.child[s];
        if (x == kNone) continue;
        if (wide_leaf(w, x)) {
            const uint32_t c = w.nodes[x].count;
            if (c == 0u || c > kMaxLeafTris || node.tri_base + toff + c > num_tris) {
                atomicOr(&cnt->error, kErrLeaf);
                continue;
            }
            node.tri_mask |= (uint16_t)(((1u << c) - 1u) << (2 * s));
            // the subtree's leaves, left first (at most two references)
            uint32_t st[4];
            int sp = 0;
            st[sp++] = x;
            while (sp > 0) {
                const uint32_t y = st[--sp];
                const BNode& yb = w.nodes[y];
                if (yb.left == kNone) {
                    for (uint32_t j = 0; j < yb.count; ++j)
                        emit_tri(src, src.final_refs[yb.first + j], &wtris[node.tri_base + toff++]);
                } else if (sp + 2 <= 4) {
                    st[sp++] = yb.right;
                    st[sp++] = yb.left;
                } else {
                    atomicOr(&cnt->error, kErrLeaf);
                    break;
                }
            }
        } else {
            node.imask |= (uint8_t)(1u << s);
            next_queue[ni_off[q] + k] = x;
            ++k;
        }
    }
    if (level_base + q >= wnode_cap) { atomicOr(&cnt->error, kErrWide); return; }
    wnodes[level_base + q] = node;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Scratch layout for num_tris triangles (all offsets 256-byte aligned).
struct Layout {
    size_t tlo, thi, refs0, refs1, final_refs, bnodes, visits, cost, dec, isplit, tasks0, tasks1, small, bins,
        splits, acc, chunks, chunk_left, queue0, queue1, rec, ni, nt, wnodes, counters, gkeys, sah, total;
    uint32_t max_nodes, task_cap, small_cap, chunk_cap, wnode_cap;
};

Layout make_layout(uint32_t T) {
    Layout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += align256(std::max<size_t>(bytes, 16)); return o; };
    L.max_nodes = 2 * T;
    L.task_cap = T / kSmall + 2;
    L.small_cap = T / 2 + 2;
    L.chunk_cap = T / kChunk + L.task_cap + 2;
    L.wnode_cap = T + 1;
    L.tlo = take((size_t)T * 16);
    L.thi = take((size_t)T * 16);
    L.refs0 = take((size_t)T * 4);
    L.refs1 = take((size_t)T * 4);
    L.final_refs = take((size_t)T * 4);
    L.bnodes = take((size_t)L.max_nodes * sizeof(BNode));
    L.visits = take((size_t)L.max_nodes * 4);
    L.cost = take((size_t)L.max_nodes * 32);
    L.dec = take((size_t)L.max_nodes * 8);
    L.isplit = take((size_t)L.max_nodes);
    L.tasks0 = take((size_t)L.task_cap * sizeof(Task));
    L.tasks1 = take((size_t)L.task_cap * sizeof(Task));
    L.small = take((size_t)L.small_cap * sizeof(Task));
    L.bins = take((size_t)L.task_cap * 3 * kBins * sizeof(Bin));
    L.splits = take((size_t)L.task_cap * sizeof(Split));
    L.acc = take((size_t)L.task_cap * sizeof(ChildAcc));
    L.chunks = take((size_t)L.chunk_cap * sizeof(Chunk));
    L.chunk_left = take((size_t)L.chunk_cap * 4);
    L.queue0 = take((size_t)L.wnode_cap * 4);
    L.queue1 = take((size_t)L.wnode_cap * 4);
    L.rec = take((size_t)L.wnode_cap * sizeof(WideRec));
    L.ni = take((size_t)L.wnode_cap * 4);
    L.nt = take((size_t)L.wnode_cap * 4);
    L.wnodes = take((size_t)L.wnode_cap * sizeof(CwNode));
    L.counters = take(sizeof(Counters));
    L.gkeys = take(12 * 4);
    L.sah = take(8);
    L.total = off;
    return L;
}

uint32_t blocks_for(uint64_t n, uint32_t threads) { return (uint32_t)std::max<uint64_t>(1, (n + threads - 1) / threads); }

std::string error_text(uint32_t e) {
    std::string m;
    if (e & kErrIndex) m += " vertex index out of range;";
    if (e & kErrFinite) m += " non-finite vertex position;";
    if (e & kErrNodes) m += " node or task capacity exceeded;";
    if (e & kErrGather) m += " wide-node gather failed;";
    if (e & kErrLeaf) m += " leaf size out of range;";
    if (e & kErrStack) m += " small-node stack overflow;";
    if (e & kErrClimb) m += " collapse climb did not end;";
    if (e & kErrWide) m += " wide-node capacity exceeded;";
    return m;
}

}  // namespace

uint64_t device_build_scratch_bytes(uint32_t num_tris) { return make_layout(num_tris).total; }
uint64_t device_build_output_bytes(uint32_t num_tris) {
    return (uint64_t)(num_tris + 1) * sizeof(CwNode) + (uint64_t)num_tris * sizeof(CwTri);
}

bool build_cwbvh_device(cudaStream_t st, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t T,
                        const uint32_t* mat, const float* transparency, uint32_t num_materials,
                        const bsm_bvh_opts* opts_in, DeviceBvhResult& out, std::string& err) {
    auto t0 = std::chrono::steady_clock::now();
    out = DeviceBvhResult{};
    if (T == 0) { err = "scene has no triangles"; return false; }
    if (T >= kTriGroupFlag) { err = "more than 2^31 - 1 triangles in one BVH"; return false; }
    bsm_bvh_opts opts{};
    if (opts_in) opts = *opts_in;
    if (opts.sah_bins > (uint32_t)kBins) { err = "the device builder takes at most 32 SAH bins"; return false; }
    const int B = opts.sah_bins ? (int)std::max(opts.sah_bins, 4u) : kBins;
    const uint32_t max_leaf = opts.max_leaf_tris ? std::min(opts.max_leaf_tris, kMaxLeafTris) : kMaxLeafTris;
    const bool optimal = opts.collapse == BSM_COLLAPSE_SAH_OPTIMAL;
    const uint32_t bin_leaf = optimal ? 1u : max_leaf;   // the collapse chooses the leaves itself
    const float tri_cost = opts.tri_cost > 0.0f ? opts.tri_cost : 1.0f;

    const Layout L = make_layout(T);
    char* base = nullptr;
    cudaError_t e = cudaMalloc(&base, L.total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("device BVH scratch: ") + cudaGetErrorString(e);
        return false;
    }
    CwTri* wtris = nullptr;
    e = cudaMalloc(&wtris, (size_t)T * sizeof(CwTri));
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(base);
        err = std::string("device BVH triangles: ") + cudaGetErrorString(e);
        return false;
    }
    auto P = [&](size_t o) { return (void*)(base + o); };
    float4* tlo = (float4*)P(L.tlo);
    float4* thi = (float4*)P(L.thi);
    uint32_t* refs[2] = {(uint32_t*)P(L.refs0), (uint32_t*)P(L.refs1)};
    uint32_t* final_refs = (uint32_t*)P(L.final_refs);
    BNode* bnodes = (BNode*)P(L.bnodes);
    Task* tasks[2] = {(Task*)P(L.tasks0), (Task*)P(L.tasks1)};
    Task* small = (Task*)P(L.small);
    Bin* bins = (Bin*)P(L.bins);
    Split* splits = (Split*)P(L.splits);
    ChildAcc* acc = (ChildAcc*)P(L.acc);
    Chunk* chunks = (Chunk*)P(L.chunks);
    uint32_t* chunk_left = (uint32_t*)P(L.chunk_left);
    Counters* cnt = (Counters*)P(L.counters);
    uint32_t* gkeys = (uint32_t*)P(L.gkeys);
    double* sah = (double*)P(L.sah);

    bool ok = false;
    std::string why;
#define DB_CK(call)                                                          \
    do {                                                                     \
        cudaError_t e_ = (call);                                             \
        if (e_ != cudaSuccess) { why = std::string(#call) + ": " + cudaGetErrorString(e_); goto done; } \
    } while (0)
    {
        // ---- phase 1 ----
        uint32_t keys0[12];
        for (int k = 0; k < 12; ++k) keys0[k] = (k % 6) >= 3 ? kKeyHi : kKeyLo;
        DB_CK(cudaMemsetAsync(cnt, 0, sizeof(Counters), st));
        DB_CK(cudaMemsetAsync(sah, 0, 8, st));
        DB_CK(cudaMemcpyAsync(gkeys, keys0, sizeof(keys0), cudaMemcpyHostToDevice, st));
        DB_CK(cudaMemsetAsync(bnodes, 0xff, (size_t)L.max_nodes * sizeof(BNode), st));   // left = right = kNone
        DB_CK(cudaMemsetAsync(P(L.visits), 0, (size_t)L.max_nodes * 4, st));
        k_tri_boxes<<<blocks_for(T, 256), 256, 0, st>>>(pos, nv, idx, T, tlo, thi, gkeys, cnt);
        k_iota<<<blocks_for(T, 256), 256, 0, st>>>(refs[0], T);
        DB_CK(cudaGetLastError());
        uint32_t keys[12];
        Counters hc;
        DB_CK(cudaMemcpyAsync(keys, gkeys, sizeof(keys), cudaMemcpyDeviceToHost, st));
        DB_CK(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
        DB_CK(cudaStreamSynchronize(st));
        if (hc.error) { why = "device BVH build:" + error_text(hc.error); goto done; }
        auto unkey = [](uint32_t k) {
            uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
            float f;
            std::memcpy(&f, &b, 4);
            return f;
        };
        // root node 0
        BNode root;
        for (int k = 0; k < 3; ++k) { root.lo[k] = unkey(keys[k]); root.hi[k] = unkey(keys[3 + k]); }
        root.left = root.right = kNone;
        root.first = 0;
        root.count = T;
        root.parent = kNone;
        root.pad = 0;
        DB_CK(cudaMemcpyAsync(bnodes, &root, sizeof(root), cudaMemcpyHostToDevice, st));
        uint32_t one = 1;
        DB_CK(cudaMemcpyAsync(&cnt->nodes, &one, 4, cudaMemcpyHostToDevice, st));
        Task rt;
        rt.node = 0;
        rt.begin = 0;
        rt.end = T;
        rt.pad = 0;
        for (int k = 0; k < 3; ++k) { rt.clo[k] = unkey(keys[6 + k]); rt.chi[k] = unkey(keys[9 + k]); }
        uint32_t nsmall = 0, ntasks = 0;
        int cur = 0;   // refs[cur] holds the current level's references
        if (T == 1) {
            DB_CK(cudaMemcpyAsync(final_refs, refs[0], 4, cudaMemcpyDeviceToDevice, st));
        } else if (T <= kSmall) {
            DB_CK(cudaMemcpyAsync(final_refs, refs[0], (size_t)T * 4, cudaMemcpyDeviceToDevice, st));
            DB_CK(cudaMemcpyAsync(small, &rt, sizeof(rt), cudaMemcpyHostToDevice, st));
            nsmall = 1;
            DB_CK(cudaMemcpyAsync(&cnt->small_tasks, &nsmall, 4, cudaMemcpyHostToDevice, st));
        } else {
            DB_CK(cudaMemcpyAsync(tasks[0], &rt, sizeof(rt), cudaMemcpyHostToDevice, st));
            ntasks = 1;
        }
        // ---- phase 2: levels of large nodes ----
        std::vector<Task> htasks;
        std::vector<Chunk> hchunks;
        std::vector<uint32_t> hleft;
        std::vector<Split> hsplit;
        int tq = 0;   // tasks[tq] holds the current level's tasks
        for (uint32_t level = 0; ntasks > 0; ++level) {
            if (level > T) { why = "device BVH build: levels do not end"; goto done; }
            htasks.resize(ntasks);
            DB_CK(cudaMemcpyAsync(htasks.data(), tasks[tq], ntasks * sizeof(Task), cudaMemcpyDeviceToHost, st));
            DB_CK(cudaStreamSynchronize(st));
            hchunks.clear();
            for (uint32_t t = 0; t < ntasks; ++t)
                for (uint32_t b = htasks[t].begin; b < htasks[t].end; b += kChunk) {
                    Chunk c{};
                    c.task = t;
                    c.begin = b;
                    c.end = std::min(htasks[t].end, b + kChunk);
                    hchunks.push_back(c);
                }
            const uint32_t nch = (uint32_t)hchunks.size();
            if (nch > L.chunk_cap) { why = "device BVH build: chunk capacity exceeded"; goto done; }
            DB_CK(cudaMemcpyAsync(chunks, hchunks.data(), nch * sizeof(Chunk), cudaMemcpyHostToDevice, st));
            k_bins_init<<<blocks_for((uint64_t)ntasks * 3 * kBins, 256), 256, 0, st>>>(bins, ntasks * 3 * kBins);
            k_bin<<<nch, kLevelThreads, 0, st>>>(chunks, tasks[tq], refs[cur], tlo, thi, bins, B);
            k_split<<<blocks_for((uint64_t)ntasks * 32, 256), 256, 0, st>>>(tasks[tq], ntasks, bins, bnodes, splits, B,
                                                                          bin_leaf);
            k_count_left<<<nch, kLevelThreads, 0, st>>>(chunks, tasks[tq], splits, refs[cur], tlo, thi, chunk_left, B);
            DB_CK(cudaGetLastError());
            hleft.resize(nch);
            hsplit.resize(ntasks);
            DB_CK(cudaMemcpyAsync(hleft.data(), chunk_left, nch * 4, cudaMemcpyDeviceToHost, st));
            DB_CK(cudaMemcpyAsync(hsplit.data(), splits, ntasks * sizeof(Split), cudaMemcpyDeviceToHost, st));
            DB_CK(cudaStreamSynchronize(st));
            {
                uint32_t prev_task = kNone, lsum = 0, rsum = 0;
                for (uint32_t c = 0; c < nch; ++c) {
                    Chunk& ck = hchunks[c];
                    const Task& tk = htasks[ck.task];
                    if (ck.task != prev_task) { prev_task = ck.task; lsum = 0; rsum = 0; }
                    const uint32_t nl = hsplit[ck.task].nl;
                    ck.left_base = tk.begin + lsum;
                    ck.right_base = tk.begin + nl + rsum;
                    lsum += hleft[c];
                    rsum += (ck.end - ck.begin) - hleft[c];
                    if (c + 1 == nch || hchunks[c + 1].task != ck.task) {
                        if (lsum != nl) { why = "device BVH build: partition count mismatch"; goto done; }
                    }
                }
            }
            DB_CK(cudaMemcpyAsync(chunks, hchunks.data(), nch * sizeof(Chunk), cudaMemcpyHostToDevice, st));
            k_acc_init<<<blocks_for(ntasks, 256), 256, 0, st>>>(acc, ntasks);
            k_partition<<<nch, kLevelThreads, 0, st>>>(chunks, tasks[tq], splits, refs[cur], refs[cur ^ 1], tlo, thi,
                                                       acc, B);
            DB_CK(cudaMemsetAsync(&cnt->next_tasks, 0, 4, st));
            k_make_children<<<blocks_for(ntasks, 128), 128, 0, st>>>(tasks[tq], ntasks, splits, acc, refs[cur ^ 1],
                                                                      bnodes, final_refs, tasks[tq ^ 1], L.task_cap,
                                                                      small, L.small_cap, cnt, L.max_nodes);
            DB_CK(cudaGetLastError());
            DB_CK(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
            DB_CK(cudaStreamSynchronize(st));
            if (hc.error) { why = "device BVH build:" + error_text(hc.error); goto done; }
            ntasks = hc.next_tasks;
            nsmall = hc.small_tasks;
            tq ^= 1;
            cur ^= 1;
        }
        if (nsmall > 0)
            k_small<<<blocks_for(nsmall, kSmallWarps), kSmallWarps * 32, 0, st>>>(small, nsmall, final_refs, tlo, thi,
                                                                                 bnodes, cnt, B, bin_leaf,
                                                                                 L.max_nodes);
        DB_CK(cudaGetLastError());
        DB_CK(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
        DB_CK(cudaStreamSynchronize(st));
        if (hc.error) { why = "device BVH build:" + error_text(hc.error); goto done; }
        const uint32_t nb = hc.nodes;
        // ---- phase 3 ----
        if (optimal)
            k_collapse<<<blocks_for(nb, 256), 256, 0, st>>>(bnodes, nb, (uint32_t*)P(L.visits), (float*)P(L.cost),
                                                            (uint8_t*)P(L.dec), (uint8_t*)P(L.isplit), max_leaf,
                                                            tri_cost, cnt);
        k_sah_cost<<<blocks_for(nb, 256), 256, 0, st>>>(bnodes, nb, sah);
        DB_CK(cudaGetLastError());
        // ---- phase 4 ----
        WideCfg wc;
        wc.nodes = bnodes;
        wc.dec = (const uint8_t*)P(L.dec);
        wc.isplit = (const uint8_t*)P(L.isplit);
        wc.optimal = optimal;
        wc.max_leaf = max_leaf;
        TriSrc ts;
        ts.pos = pos;
        ts.idx = idx;
        ts.mat = mat;
        ts.transp = transparency;
        ts.num_materials = num_materials;
        ts.final_refs = final_refs;
        uint32_t* queue[2] = {(uint32_t*)P(L.queue0), (uint32_t*)P(L.queue1)};
        uint32_t zero = 0;
        DB_CK(cudaMemcpyAsync(queue[0], &zero, 4, cudaMemcpyHostToDevice, st));   // the binary root
        uint32_t nq = 1, level_base = 0, tri_cursor = 0, depth = 0;
        int qc = 0;
        while (nq > 0) {
            ++depth;
            if (level_base + nq > L.wnode_cap) { why = "device BVH build: wide-node capacity exceeded"; goto done; }
            k_wide_gather<<<blocks_for(nq, 128), 128, 0, st>>>(queue[qc], nq, wc, (WideRec*)P(L.rec),
                                                               (uint32_t*)P(L.ni), (uint32_t*)P(L.nt), cnt);
            k_scan2<<<1, 1024, 0, st>>>((uint32_t*)P(L.ni), (uint32_t*)P(L.nt), nq, cnt);
            DB_CK(cudaGetLastError());
            DB_CK(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
            DB_CK(cudaStreamSynchronize(st));
            if (hc.error) { why = "device BVH build:" + error_text(hc.error); goto done; }
            const uint32_t next_base = level_base + nq;
            if ((uint64_t)next_base + hc.ni_total > L.wnode_cap || (uint64_t)tri_cursor + hc.nt_total > T) {
                why = "device BVH build: wide level exceeds its capacity";
                goto done;
            }
            k_wide_write<<<blocks_for(nq, 128), 128, 0, st>>>(queue[qc], nq, (const WideRec*)P(L.rec),
                                                              (const uint32_t*)P(L.ni), (const uint32_t*)P(L.nt), wc,
                                                              ts, (CwNode*)P(L.wnodes), L.wnode_cap, wtris, T,
                                                              queue[qc ^ 1], level_base, next_base, tri_cursor, cnt);
            DB_CK(cudaGetLastError());
            level_base = next_base;
            tri_cursor += hc.nt_total;
            nq = hc.ni_total;
            qc ^= 1;
        }
        DB_CK(cudaMemcpyAsync(&hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
        double hsah = 0.0;
        DB_CK(cudaMemcpyAsync(&hsah, sah, 8, cudaMemcpyDeviceToHost, st));
        DB_CK(cudaStreamSynchronize(st));
        if (hc.error) { why = "device BVH build:" + error_text(hc.error); goto done; }
        if (tri_cursor != T) { why = "device BVH build: triangle count mismatch"; goto done; }
        CwNode* nodes_out = nullptr;
        DB_CK(cudaMalloc(&nodes_out, (size_t)level_base * sizeof(CwNode)));
        e = cudaMemcpyAsync(nodes_out, P(L.wnodes), (size_t)level_base * sizeof(CwNode), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaFree(nodes_out);
            why = std::string("device BVH nodes: ") + cudaGetErrorString(e);
            goto done;
        }
        const double ra = (double)((root.hi[0] - root.lo[0]) * (root.hi[1] - root.lo[1]) +
                                   (root.hi[1] - root.lo[1]) * (root.hi[2] - root.lo[2]) +
                                   (root.hi[2] - root.lo[2]) * (root.hi[0] - root.lo[0])) * 2.0;
        out.nodes = nodes_out;
        out.tris = wtris;
        out.num_nodes = level_base;
        out.num_tris = T;
        out.max_depth = depth;
        out.sah_cost = ra > 0.0 ? hsah / ra : 0.0;
        ok = true;
    }
done:
#undef DB_CK
    cudaStreamSynchronize(st);
    cudaFree(base);
    if (!ok) {
        cudaFree(wtris);
        cudaGetLastError();
        err = why.empty() ? "device BVH build failed" : why;
        return false;
    }
    out.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return true;
}

}  // namespace bsm
