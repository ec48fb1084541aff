// pt_trace.cuh — device-side ray traversal of the compressed 8-wide BVH.
//
// Replaces TraceRay on the RT cores (bisemutum/shaders/renderer/raytracing/
// rt_gbuffer.hlsl:17-25) with a software traversal:
//   * node test: eight quantised child boxes per 80-byte node; a plane is
//     rebuilt from its byte with one PRMT, then one fused multiply-add gives
//     its slab distance; three-input min/max close the slabs into an 8-bit
//     child hit mask.  Two table lookups turn the mask into the internal
//     children in octant order (the highest bit is the nearest child; Ylitie,
//     Karras, Laine, HPG 2017) and into the hit triangles (two bits per slot);
//   * node groups (base index + hit bits) on a per-thread stack; triangle
//     groups are postponed onto the stack while few lanes of the warp have
//     triangles, so node and triangle work stay converged;
//   * persistent warps refill lanes whose rays finished from a global queue
//     counter (one atomic per refill per warp);
//   * triangle test: the watertight ray/triangle intersection of Woop,
//     Benthin and Wald (JCGT 2013) with its double-precision fallback on zero
//     edge functions, in plain IEEE single precision in a fixed order, so t
//     and the hit primitive are reproducible bit for bit on a CPU.
// Ties at equal t resolve to the lower primitive id, which makes the closest
// hit independent of the BVH's shape.
// Non-opaque triangles carry their transparency (1 - opacity, or 1 / 0 for an
// alpha-tested surface below / above the threshold) in the spare word of the
// triangle record; a candidate hit on one is ignored when the ray's opacity
// uniform is below it (the any-hit shader's IgnoreHit, rt_gbuffer_hit.hlsl:20-35).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bvh_layout.h"
#include "pt_math.cuh"

namespace bsm {

// Far-plane pad: a box is kept when max(near) <= min(far) * (1 + 2^-20).  The
// builder also pads every child box outward by one quantisation step, so the
// rounding of the slab arithmetic never culls a box that holds a hit.
#define BSM_BOX_PAD 1.00000095f
constexpr int kStackSize = 40;        // node groups (<= tree depth) + postponed triangle groups
constexpr int kPostponeMaxSp = 16;    // largest stack budget for postponed triangle groups

struct RayPre {
    float ox, oy, oz, tmin;
    float dx, dy, dz;
    float idx, idy, idz;     // 1 / direction, a component below 1e-20 in magnitude taken as +-1e-20
    uint32_t oct_key;        // 7 ^ (sign bits): child visiting key = slot ^ oct_key
    int kx, ky, kz;          // watertight axis permutation
    float Sx, Sy, Sz;        // watertight shear
};

__device__ __forceinline__ float sel3(int k, float x, float y, float z) {
    return k == 0 ? x : (k == 1 ? y : z);
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ float box_dir(float x) { return fabsf(x) < 1e-20f ? copysignf(1e-20f, x) : x; }

__device__ __forceinline__ RayPre make_ray(float4 o, float4 d) {
    RayPre r;
    r.ox = o.x; r.oy = o.y; r.oz = o.z; r.tmin = o.w;
    r.dx = d.x; r.dy = d.y; r.dz = d.z;
    // The box test's reciprocals: a zero (or tiny) component is taken as
    // +-1e-20, which keeps every slab constant finite.  An infinite reciprocal
    // would make the folded slab constants inf - inf = NaN, which min/max drop:
    // the slab would stop culling, and a ray parallel to an axis (a sky sample
    // at the zenith, for instance) would visit every node its other slabs
    // allow.  The 1e-20 slope moves the ray by at most 1e-20 t across the
    // slab, far inside the half quantisation step of padding left for a hit at
    // t below 1e17 times the node's extent.  The triangle test uses the true
    // direction.
    // __frcp_rn: the correctly rounded 1 / x, the same bits as the IEEE division 1.0f / x
    r.idx = __frcp_rn(box_dir(d.x));
    r.idy = __frcp_rn(box_dir(d.y));
    r.idz = __frcp_rn(box_dir(d.z));
    uint32_t oct = (r.idx < 0.0f ? 1u : 0u) | (r.idy < 0.0f ? 2u : 0u) | (r.idz < 0.0f ? 4u : 0u);
    r.oct_key = 7u ^ oct;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) { kz = 2; }
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    float dkz = sel3(kz, d.x, d.y, d.z);
    if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = __fdiv_rn(sel3(kx, d.x, d.y, d.z), dkz);
    r.Sy = __fdiv_rn(sel3(ky, d.x, d.y, d.z), dkz);
    r.Sz = __frcp_rn(dkz);
    return r;
}

// Rays that are traced: origin and direction finite, direction not zero (a
// zero direction is skipped as a miss, rt_gbuffer.hlsl:13-15) and tmin <= tmax.
// Every other ray (a NaN or infinite component, an empty or NaN interval) is a
// miss without traversal.
__device__ __forceinline__ bool finite_bits(float x) { return (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u; }
__device__ __forceinline__ bool ray_traceable(const RayPre& r, float tmax) {
    bool fin = finite_bits(r.ox) & finite_bits(r.oy) & finite_bits(r.oz) & finite_bits(r.dx) & finite_bits(r.dy) &
               finite_bits(r.dz);
    return fin && !(r.dx == 0.0f && r.dy == 0.0f && r.dz == 0.0f) && r.tmin <= tmax;
}

// Watertight test.  Returns true and writes t/u/v when the triangle is hit at
// t in (tmin, tbest], preferring the lower primitive id on a tie at tbest.
__device__ __forceinline__ bool tri_test(const RayPre& r, float4 a, float4 b, float4 c, float tbest,
                                         uint32_t prim, uint32_t best_prim, float& t_out, float& u_out,
                                         float& v_out) {
    float Ax0 = a.x - r.ox, Ay0 = a.y - r.oy, Az0 = a.z - r.oz;
    float Bx0 = b.x - r.ox, By0 = b.y - r.oy, Bz0 = b.z - r.oz;
    float Cx0 = c.x - r.ox, Cy0 = c.y - r.oy, Cz0 = c.z - r.oz;
    float Akx = sel3(r.kx, Ax0, Ay0, Az0), Aky = sel3(r.ky, Ax0, Ay0, Az0), Akz = sel3(r.kz, Ax0, Ay0, Az0);
    float Bkx = sel3(r.kx, Bx0, By0, Bz0), Bky = sel3(r.ky, Bx0, By0, Bz0), Bkz = sel3(r.kz, Bx0, By0, Bz0);
    float Ckx = sel3(r.kx, Cx0, Cy0, Cz0), Cky = sel3(r.ky, Cx0, Cy0, Cz0), Ckz = sel3(r.kz, Cx0, Cy0, Cz0);
    float Ax = __fsub_rn(Akx, __fmul_rn(r.Sx, Akz));
    float Ay = __fsub_rn(Aky, __fmul_rn(r.Sy, Akz));
    float Bx = __fsub_rn(Bkx, __fmul_rn(r.Sx, Bkz));
    float By = __fsub_rn(Bky, __fmul_rn(r.Sy, Bkz));
    float Cx = __fsub_rn(Ckx, __fmul_rn(r.Sx, Ckz));
    float Cy = __fsub_rn(Cky, __fmul_rn(r.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    float Az = __fmul_rn(r.Sz, Akz), Bz = __fmul_rn(r.Sz, Bkz), Cz = __fmul_rn(r.Sz, Ckz);
    float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    // conservative rejections before the division (exact sign logic, padded bound)
    float Ts = det < 0.0f ? -T : T;
    float adet = fabsf(det);
    if (Ts <= 0.0f && r.tmin >= 0.0f) return false;
    if (Ts > adet * tbest * BSM_BOX_PAD) return false;
    float rcp = __frcp_rn(det);
    float t = __fmul_rn(T, rcp);
    if (!(t > r.tmin)) return false;
    if (!(t < tbest || (t == tbest && prim < best_prim))) return false;
    t_out = t;
    u_out = __fmul_rn(U, rcp);
    v_out = __fmul_rn(V, rcp);
    return true;
}

// Lookup tables of the node test, in global memory (read through L1):
// child_perm[key][m] moves bit s of m to bit s ^ key (octant order of the
// internal children); spread2[m] moves bit s of m to bit 2s (the first
// triangle bit of slot s).
struct ChildPermTable { uint8_t v[8 * 256]; };
struct Spread2Table { uint16_t v[256]; };
constexpr ChildPermTable make_child_perm() {
    ChildPermTable t{};
    for (int k = 0; k < 8; ++k)
        for (int m = 0; m < 256; ++m) {
            int y = 0;
            for (int b = 0; b < 8; ++b)
                if ((m >> b) & 1) y |= 1 << (b ^ k);
            t.v[k * 256 + m] = (uint8_t)y;
        }
    return t;
}
constexpr Spread2Table make_spread2() {
    Spread2Table t{};
    for (int m = 0; m < 256; ++m) {
        int y = 0;
        for (int b = 0; b < 8; ++b)
            if ((m >> b) & 1) y |= 1 << (2 * b);
        t.v[m] = (uint16_t)y;
    }
    return t;
}
static __device__ ChildPermTable g_child_perm = make_child_perm();
static __device__ Spread2Table g_spread2 = make_spread2();

// Byte k of w as the float 2^23 + byte (one PRMT).  The slab constants below
// absorb the 2^23 offset: t = (2^23 + q) s + (a - 2^23 s).  Rounding the folded
// constant costs at most half a quantisation step of the plane, inside the one
// step by which the builder pads every child box outward, so the test stays
// conservative.
__device__ __forceinline__ float qbyte(uint32_t w, uint32_t k) {
    return __uint_as_float(__byte_perm(w, 0x4b000000u, 0x7440u | k));
}

// Intersects the eight children of node `ni`; returns the group of internal
// children hit (child base, hit bits 24..31 in octant order | imask) and the
// group of triangles hit (triangle base, hit bits 0..15 | the node's
// tri_mask in bits 16..31, which locates each triangle: next_tri).
__device__ __forceinline__ void node_test(const RayPre& r, const CwNode* __restrict__ nodes, uint32_t ni, float tbest,
                                          uint2& G, uint2& T) {
    const uint4* p = reinterpret_cast<const uint4*>(nodes + ni);
    uint4 n0 = __ldg(p + 0), n1 = __ldg(p + 1), n2 = __ldg(p + 2), n3 = __ldg(p + 3), n4 = __ldg(p + 4);
    uint32_t ew = n0.w;
    // slab distance of plane q: q * s + a (near planes) and (q * s + a) * pad (far planes)
    float sx = __uint_as_float((ew & 0xffu) << 23) * r.idx;
    float sy = __uint_as_float(((ew >> 8) & 0xffu) << 23) * r.idy;
    float sz = __uint_as_float(((ew >> 16) & 0xffu) << 23) * r.idz;
    float ax = (__uint_as_float(n0.x) - r.ox) * r.idx;
    float ay = (__uint_as_float(n0.y) - r.oy) * r.idy;
    float az = (__uint_as_float(n0.z) - r.oz) * r.idz;
    ax = __fsub_rn(ax, 8388608.0f * sx);
    ay = __fsub_rn(ay, 8388608.0f * sy);
    az = __fsub_rn(az, 8388608.0f * sz);
    float sxf = sx * BSM_BOX_PAD, syf = sy * BSM_BOX_PAD, szf = sz * BSM_BOX_PAD;
    float axf = ax * BSM_BOX_PAD, ayf = ay * BSM_BOX_PAD, azf = az * BSM_BOX_PAD;
    uint32_t imask = ew >> 24;
    bool nx = r.idx < 0.0f, ny = r.idy < 0.0f, nz = r.idz < 0.0f;
    uint32_t nlx0 = nx ? n3.z : n2.x, nlx1 = nx ? n3.w : n2.y;
    uint32_t nfx0 = nx ? n2.x : n3.z, nfx1 = nx ? n2.y : n3.w;
    uint32_t nly0 = ny ? n4.x : n2.z, nly1 = ny ? n4.y : n2.w;
    uint32_t nfy0 = ny ? n2.z : n4.x, nfy1 = ny ? n2.w : n4.y;
    uint32_t nlz0 = nz ? n4.z : n3.x, nlz1 = nz ? n4.w : n3.y;
    uint32_t nfz0 = nz ? n3.x : n4.z, nfz1 = nz ? n3.y : n4.w;
    uint32_t hm = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint32_t k = (uint32_t)(c & 3);
        const bool lo = c < 4;
        float tnx = __fmaf_rn(qbyte(lo ? nlx0 : nlx1, k), sx, ax);
        float tny = __fmaf_rn(qbyte(lo ? nly0 : nly1, k), sy, ay);
        float tnz = __fmaf_rn(qbyte(lo ? nlz0 : nlz1, k), sz, az);
        float tfx = __fmaf_rn(qbyte(lo ? nfx0 : nfx1, k), sxf, axf);
        float tfy = __fmaf_rn(qbyte(lo ? nfy0 : nfy1, k), syf, ayf);
        float tfz = __fmaf_rn(qbyte(lo ? nfz0 : nfz1, k), szf, azf);
        float tn = max3f(tnx, tny, fmaxf(tnz, r.tmin));
        float tf = min3f(tfx, tfy, fminf(tfz, tbest));
        hm |= (tn <= tf) ? (1u << c) : 0u;
    }
    // hit slots that are empty have neither an imask nor a tri_mask bit, so they drop out here
    uint32_t inner = __ldg(&g_child_perm.v[r.oct_key * 256u + (hm & imask)]);
    uint32_t tm = n1.z & 0xffffu;
    uint32_t th = ((uint32_t)__ldg(&g_spread2.v[hm]) * 3u) & tm;
    G = make_uint2(n1.x, (inner << 24) | imask);
    T = make_uint2(n1.y, th | (tm << 16));
}

// Takes the next (lowest) hit triangle of group T, whose hit bits 0..15 must
// not be empty, and returns its index.
__device__ __forceinline__ uint32_t next_tri(uint2& T) {
    uint32_t bit = (uint32_t)__ffs(T.y) - 1u;
    T.y &= T.y - 1u;
    return T.x + (uint32_t)__popc((T.y >> 16) & ((1u << bit) - 1u));
}
__device__ __forceinline__ bool has_tris(const uint2& T) { return (T.y & 0xffffu) != 0u; }

struct TraceCounters { uint32_t nodes, tris; };

// Single-ray closest / any hit (used by the stage entry points).  Returns the
// leaf-ordered triangle index (kMissPrim on a miss); t = tmax on a miss.
// Rule of a candidate hit on a triangle of transparency `tr` (0 = opaque).
__device__ __forceinline__ bool keep_hit(const RayPre& r, float tr, uint32_t oseed) {
    return tr == 0.0f || !(opacity_random(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, oseed) < tr);
}

template <bool kAnyHit, bool kCount>
__device__ __forceinline__ uint32_t trace_ray(const RayPre& r, float tmax, const CwNode* __restrict__ nodes,
                                              const CwTri* __restrict__ tris, float& t_out, float& u_out,
                                              float& v_out, TraceCounters* cnt, uint32_t oseed = 0u) {
    float tbest = tmax;
    uint32_t best_leaf = kMissPrim, best_prim = kMissPrim;
    float bu = 0.0f, bv = 0.0f;
    uint2 stack[kStackSize];
    int sp = 0;
    uint32_t root_slot = 7u ^ r.oct_key;
    uint2 G = make_uint2(0u, ray_traceable(r, tmax) ? (0x80000000u | (1u << root_slot)) : 0u);
    uint2 T = make_uint2(0u, 0u);
    while (true) {
        while (has_tris(T)) {
            uint32_t ti = next_tri(T);
            const float4* tp = reinterpret_cast<const float4*>(tris + ti);
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            uint32_t prim = __float_as_uint(a.w);
            if (kCount) cnt->tris++;
            float t, u, v;
            if (tri_test(r, a, b, c, tbest, prim, best_prim, t, u, v) && keep_hit(r, c.w, oseed)) {
                if (kAnyHit) { t_out = t; u_out = u; v_out = v; return ti; }
                tbest = t; best_leaf = ti; best_prim = prim; bu = u; bv = v;
            }
        }
        if ((G.y & 0xff000000u) == 0u) {
            if (sp == 0) break;
            G = stack[--sp];
        }
        uint32_t bit = 31u - (uint32_t)__clz(G.y & 0xff000000u);
        G.y &= ~(1u << bit);
        uint32_t slot = (bit - 24u) ^ r.oct_key;
        uint32_t ni = G.x + (uint32_t)__popc(G.y & 0xffu & ((1u << slot) - 1u));
        if ((G.y & 0xff000000u) != 0u) stack[sp++] = G;
        if (kCount) cnt->nodes++;
        node_test(r, nodes, ni, tbest, G, T);
    }
    t_out = tbest;
    u_out = bu;
    v_out = bv;
    return best_leaf;
}

// ---------------------------------------------------------- two-level ----
// Row-major 3x4 transform of a point / direction, in a fixed operation order
// (the oracle evaluates the same sums).
__device__ __forceinline__ float4 xform_point(const float* m, float x, float y, float z, float w) {
    return make_float4(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[1], y)), __fmul_rn(m[2], z)), m[3]),
                       __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4], x), __fmul_rn(m[5], y)), __fmul_rn(m[6], z)), m[7]),
                       __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[8], x), __fmul_rn(m[9], y)), __fmul_rn(m[10], z)), m[11]),
                       w);
}
__device__ __forceinline__ float4 xform_dir(const float* m, float x, float y, float z, float w) {
    return make_float4(__fadd_rn(__fadd_rn(__fmul_rn(m[0], x), __fmul_rn(m[1], y)), __fmul_rn(m[2], z)),
                       __fadd_rn(__fadd_rn(__fmul_rn(m[4], x), __fmul_rn(m[5], y)), __fmul_rn(m[6], z)),
                       __fadd_rn(__fadd_rn(__fmul_rn(m[8], x), __fmul_rn(m[9], y)), __fmul_rn(m[10], z)), w);
}
__device__ __forceinline__ void load_xform(const float* src, float* m) {
    const float4* p = reinterpret_cast<const float4*>(src);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    m[0] = a.x; m[1] = a.y; m[2] = a.z; m[3] = a.w;
    m[4] = b.x; m[5] = b.y; m[6] = b.z; m[7] = b.w;
    m[8] = c.x; m[9] = c.y; m[10] = c.z; m[11] = c.w;
}

// Closest / any hit in a two-level scene (the reference's TLAS over per-mesh
// BLASes, accel.cpp:104-132).  The TLAS's leaves are instances: entering one
// pushes the rest of the current node's work and an exit marker, moves the
// ray into the instance's space and traverses its BLAS on the same stack;
// popping the marker restores the world ray.  Triangles are tested in object
// space; ties resolve to the lower global primitive id (instance prim_base +
// primitive).  `mat_tr` (per material: transparency of the any-hit rule, or
// null when every material is opaque) and the world ray give the opacity
// decision.  Returns the leaf triangle index within the instance's geometry
// and the instance (TLAS leaf index) in `inst_out`.
constexpr uint32_t kStackExit = 0xffffffffu;
template <bool kAnyHit>
__device__ __forceinline__ uint32_t trace_ray2(const RayPre& rw, float tmax, const CwNode* __restrict__ tlas,
                                               const InstDev* __restrict__ insts, const float* __restrict__ mat_tr,
                                               float& t_out, float& u_out, float& v_out, uint32_t& inst_out,
                                               uint32_t oseed) {
    float tbest = tmax, bu = 0.0f, bv = 0.0f;
    uint32_t best_leaf = kMissPrim, best_prim = kMissPrim, best_inst = kMissPrim;
    uint2 stack[kStackSize];
    int sp = 0;
    RayPre r = rw;
    const CwNode* nodes = tlas;
    const CwTri* tris = nullptr;
    uint32_t inst = kMissPrim, prim_base = 0u, mat_override = kMissPrim;
    uint2 G = make_uint2(0u, ray_traceable(rw, tmax) ? (0x80000000u | (1u << (7u ^ rw.oct_key))) : 0u);
    uint2 T = make_uint2(0u, 0u);
    while (true) {
        while (has_tris(T)) {
            uint32_t ti = next_tri(T);
            if (inst == kMissPrim) {
                // enter instance ti; this node's remaining work waits below an exit marker.
                // The depth limits (TLAS <= kMaxTlasDepth, BLAS <= kMaxTraversalDepth) keep sp
                // below kStackSize - kMaxTraversalDepth here; the guard only keeps writes in bounds.
                if (sp > kStackSize - 3 - kMaxTraversalDepth) { T.y = 0u; G.y = 0u; sp = 0; break; }
                if ((G.y & 0xff000000u) != 0u) stack[sp++] = G;
                if (has_tris(T)) stack[sp++] = make_uint2(T.x | kTriGroupFlag, T.y);
                stack[sp++] = make_uint2(kStackExit, 0u);
                const InstDev* I = insts + ti;
                float m[12];
                load_xform(I->w2o, m);
                r = make_ray(xform_point(m, rw.ox, rw.oy, rw.oz, rw.tmin), xform_dir(m, rw.dx, rw.dy, rw.dz, 0.0f));
                nodes = I->nodes;
                tris = I->tris;
                prim_base = I->prim_base;
                mat_override = I->material;
                inst = ti;
                G = make_uint2(0u, 0x80000000u | (1u << (7u ^ r.oct_key)));
                T = make_uint2(0u, 0u);
                break;
            }
            const float4* tp = reinterpret_cast<const float4*>(tris + ti);
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            uint32_t prim = prim_base + __float_as_uint(a.w);
            float t, u, v;
            if (tri_test(r, a, b, c, tbest, prim, best_prim, t, u, v)) {
                float tr = 0.0f;
                if (mat_tr) tr = mat_tr[mat_override != kMissPrim ? mat_override : __float_as_uint(b.w)];
                if (keep_hit(rw, tr, oseed)) {
                    if (kAnyHit) { t_out = t; u_out = u; v_out = v; inst_out = inst; return ti; }
                    tbest = t; best_leaf = ti; best_prim = prim; best_inst = inst; bu = u; bv = v;
                }
            }
        }
        if ((G.y & 0xff000000u) == 0u) {
            if (has_tris(T)) continue;
            if (sp == 0) break;
            uint2 e = stack[--sp];
            if (e.y == 0u) {  // exit marker: back to the world ray and the TLAS
                r = rw;
                nodes = tlas;
                tris = nullptr;
                inst = kMissPrim;
                prim_base = 0u;
                mat_override = kMissPrim;
                G = make_uint2(0u, 0u);
                continue;
            }
            if (e.x & kTriGroupFlag) {  // instances of a leaf group
                T = make_uint2(e.x & ~kTriGroupFlag, e.y);
                G = make_uint2(0u, 0u);
                continue;
            }
            G = e;
        }
        uint32_t bit = 31u - (uint32_t)__clz(G.y & 0xff000000u);
        G.y &= ~(1u << bit);
        uint32_t slot = (bit - 24u) ^ r.oct_key;
        uint32_t ni = G.x + (uint32_t)__popc(G.y & 0xffu & ((1u << slot) - 1u));
        if ((G.y & 0xff000000u) != 0u && sp < kStackSize) stack[sp++] = G;
        node_test(r, nodes, ni, tbest, G, T);
    }
    t_out = tbest;
    u_out = bu;
    v_out = bv;
    inst_out = best_inst;
    return best_leaf;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Persistent, warp-synchronous traversal of a queue of n rays.  Every lane of
// the warp runs this loop together (all ballots use the full mask).  `load`
// (index -> (origin/tmin, direction/tmax)) supplies rays; `finish(index, leaf,
// t, u, v)` receives each result (leaf = kMissPrim on a miss; for any-hit the
// first hit found); with kOpacity, `seed(index)` gives the ray's opacity seed,
// read only when a candidate hit lies on a non-opaque triangle (scenes without
// one use the kOpacity = false instantiation, which skips the rule).
// `postpone_sp` (<= kPostponeMaxSp) is the stack depth below which triangle
// groups may be postponed (0 disables postponing); `refill_min` is the number
// of idle lanes that makes the warp fetch new rays.  Both are tuning knobs.
template <bool kAnyHit, bool kCount, bool kOpacity, class Load, class Finish, class Seed>
__device__ __forceinline__ void trace_queue(const CwNode* __restrict__ nodes, const CwTri* __restrict__ tris,
                                            uint32_t n, uint32_t* work, Load load, Finish finish, Seed seed,
                                            TraceCounters* cnt, int postpone_sp, int refill_min) {
    postpone_sp = postpone_sp < kPostponeMaxSp ? postpone_sp : kPostponeMaxSp;
    const uint32_t lane = threadIdx.x & 31u;
    bool has = false;
    bool exhausted = false;  // warp-uniform
    RayPre r;
    float tbest = 0.0f, bu = 0.0f, bv = 0.0f;
    uint32_t best_leaf = kMissPrim, best_prim = kMissPrim, idx = 0;
    uint2 G = make_uint2(0, 0), T = make_uint2(0, 0);
    uint2 stack[kStackSize];
    int sp = 0;
    while (true) {
        // refill lanes whose ray finished (one atomic per warp)
        const uint32_t idle = __ballot_sync(0xffffffffu, !has);
        uint32_t act = ~idle;   // lanes holding a ray in this iteration (taken again after a refill)
        if (!exhausted && (__popc(idle) >= refill_min || idle == 0xffffffffu)) {
            uint32_t cntn = (uint32_t)__popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(work, cntn);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (!has) {
                uint32_t i = base + (uint32_t)__popc(idle & lanemask_lt());
                if (i < n) {
                    float4 o, d;
                    load(i, o, d);
                    r = make_ray(o, d);
                    tbest = d.w;
                    best_leaf = kMissPrim; best_prim = kMissPrim; bu = 0.0f; bv = 0.0f;
                    G = make_uint2(0u, ray_traceable(r, d.w) ? (0x80000000u | (1u << (7u ^ r.oct_key))) : 0u);
                    T = make_uint2(0u, 0u);
                    sp = 0;
                    idx = i;
                    has = true;
                }
            }
            if (base + cntn >= n) exhausted = true;
            act = __ballot_sync(0xffffffffu, has);
        }
        if (act == 0u) break;
        const int n_act = __popc(act);
        // node step
        if (has) {
            if (G.x & kTriGroupFlag) {
                T = make_uint2(G.x & ~kTriGroupFlag, G.y);  // a postponed triangle group popped from the stack
                G = make_uint2(0u, 0u);
            } else if ((G.y & 0xff000000u) != 0u) {
                uint32_t bit = 31u - (uint32_t)__clz(G.y & 0xff000000u);
                G.y &= ~(1u << bit);
                uint32_t slot = (bit - 24u) ^ r.oct_key;
                uint32_t ni = G.x + (uint32_t)__popc(G.y & 0xffu & ((1u << slot) - 1u));
                if ((G.y & 0xff000000u) != 0u) stack[sp++] = G;
                if (kCount) cnt->nodes++;
                node_test(r, nodes, ni, tbest, G, T);
            }
        }
        // triangle steps, postponed while fewer than 1/4 of the active lanes have triangles
        while (true) {
            bool want = has && has_tris(T);
            uint32_t m = __ballot_sync(0xffffffffu, want);
            if (m == 0u) break;
            if (__popc(m) * 4 < n_act) {
                if (want && sp < postpone_sp) { stack[sp++] = make_uint2(T.x | kTriGroupFlag, T.y); T.y = 0u; }
                if (__ballot_sync(0xffffffffu, has && has_tris(T)) == 0u) break;
                want = has && has_tris(T);
            }
            if (want) {
                uint32_t ti = next_tri(T);
                const float4* tp = reinterpret_cast<const float4*>(tris + ti);
                float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                uint32_t prim = __float_as_uint(a.w);
                if (kCount) cnt->tris++;
                float t, u, v;
                if (tri_test(r, a, b, c, tbest, prim, best_prim, t, u, v) &&
                    (!kOpacity || c.w == 0.0f || keep_hit(r, c.w, seed(idx)))) {
                    tbest = t; best_leaf = ti; best_prim = prim; bu = u; bv = v;
                    if (kAnyHit) { T.y = 0u; G.y = 0u; sp = 0; }
                }
            }
        }
        // next group, or done
        if (has && (G.y & 0xff000000u) == 0u && !has_tris(T)) {
            if (sp > 0 && !(kAnyHit && best_leaf != kMissPrim)) {
                G = stack[--sp];
            } else {
                finish(idx, best_leaf, tbest, bu, bv);
                has = false;
            }
        }
    }
}

}  // namespace bsm

namespace bsm {

// two-level: TLAS node groups (<= 12) + postponed TLAS groups (< 16) + 2 groups and an exit marker at an
// instance entry + BLAS node groups (<= 24) + postponed BLAS groups (<= 16)
constexpr int kStackSize2 = 80;
static_assert(kMaxTlasDepth + 3 + kMaxTraversalDepth + 2 * kPostponeMaxSp <= kStackSize2, "two-level stack budget");

// Persistent, warp-synchronous traversal of a queue of rays through a two-level
// scene (TLAS over per-geometry BLASes), with trace_queue's refill and
// triangle postponing.  A TLAS leaf "triangle" is an instance: a lane that
// reaches one pushes the rest of its TLAS work and an exit marker, moves its
// ray into the instance's space and continues in the BLAS on the same stack;
// popping the marker reloads the world ray's origin and direction (`load`),
// takes its divided constants from shared memory and returns to the TLAS.
// Leaf groups (instances in the TLAS, triangles in a BLAS) are postponed while
// the stack holds fewer than `postpone_sp` entries above the current BVH's
// base (0 in the TLAS, the exit marker in a BLAS), so the stack stays within
// kStackSize2 (TLAS depth <= kMaxTlasDepth, BLAS depth <= kMaxTraversalDepth).
// Results and the opacity rule are those of trace_ray2: object-space
// triangle tests with t unchanged, ties to the lower global primitive id,
// candidate hits on non-opaque triangles decided with the world ray.
// `finish(index, leaf, t, u, v, instance)`.
template <bool kAnyHit, bool kOpacity, class Load, class Finish, class Seed>
__device__ __forceinline__ void trace_queue2(const CwNode* __restrict__ tlas, const InstDev* __restrict__ insts,
                                             const float* __restrict__ mat_tr, uint32_t n, uint32_t* work, Load load,
                                             Finish finish, Seed seed, int postpone_sp, int refill_min) {
    postpone_sp = postpone_sp < kPostponeMaxSp ? postpone_sp : kPostponeMaxSp;
    const uint32_t lane = threadIdx.x & 31u;
    bool has = false;
    bool exhausted = false;  // warp-uniform
    RayPre r;
    float tbest = 0.0f, bu = 0.0f, bv = 0.0f;
    uint32_t best_leaf = kMissPrim, best_prim = kMissPrim, best_inst = kMissPrim, idx = 0;
    const CwNode* nodes = tlas;
    const CwTri* tris = nullptr;   // nullptr: traversing the TLAS
    uint32_t inst = kMissPrim, prim_base = 0u, mat_override = kMissPrim;
    uint2 G = make_uint2(0, 0), T = make_uint2(0, 0);
    uint2 stack[kStackSize2];
    int sp = 0, sp_blas = 0;       // sp_blas: stack depth just above the current BLAS's exit marker
    // the world ray's divided constants (reciprocals, shear, axis order), kept per thread so that leaving an
    // instance reloads only origin and direction (blocks have at most 256 threads: __launch_bounds__)
    __shared__ float4 s_world[256][2];
    while (true) {
        uint32_t idle = __ballot_sync(0xffffffffu, !has);
        if (!exhausted && (__popc(idle) >= refill_min || idle == 0xffffffffu)) {
            uint32_t cntn = (uint32_t)__popc(idle);
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(work, cntn);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (!has) {
                uint32_t i = base + (uint32_t)__popc(idle & lanemask_lt());
                if (i < n) {
                    float4 o, d;
                    load(i, o, d);
                    r = make_ray(o, d);
                    s_world[threadIdx.x][0] = make_float4(
                        r.idx, r.idy, r.idz,
                        __uint_as_float(r.oct_key | ((uint32_t)r.kx << 4) | ((uint32_t)r.ky << 8) | ((uint32_t)r.kz << 12)));
                    s_world[threadIdx.x][1] = make_float4(r.Sx, r.Sy, r.Sz, 0.0f);
                    tbest = d.w;
                    best_leaf = kMissPrim; best_prim = kMissPrim; best_inst = kMissPrim; bu = 0.0f; bv = 0.0f;
                    nodes = tlas; tris = nullptr; inst = kMissPrim; prim_base = 0u; mat_override = kMissPrim;
                    G = make_uint2(0u, ray_traceable(r, d.w) ? (0x80000000u | (1u << (7u ^ r.oct_key))) : 0u);
                    T = make_uint2(0u, 0u);
                    sp = 0;
                    sp_blas = 0;
                    idx = i;
                    has = true;
                }
            }
            if (base + cntn >= n) exhausted = true;
        }
        const uint32_t act = __ballot_sync(0xffffffffu, has);
        if (act == 0u) break;
        // node step
        if (has) {
            if (G.x & kTriGroupFlag) {
                T = make_uint2(G.x & ~kTriGroupFlag, G.y);  // a postponed triangle group popped from the stack
                G = make_uint2(0u, 0u);
            } else if ((G.y & 0xff000000u) != 0u) {
                uint32_t bit = 31u - (uint32_t)__clz(G.y & 0xff000000u);
                G.y &= ~(1u << bit);
                uint32_t slot = (bit - 24u) ^ r.oct_key;
                uint32_t ni = G.x + (uint32_t)__popc(G.y & 0xffu & ((1u << slot) - 1u));
                if ((G.y & 0xff000000u) != 0u) stack[sp++] = G;
                node_test(r, nodes, ni, tbest, G, T);
            }
        }
        // leaf steps: instances in the TLAS, triangles in a BLAS (both postponed while few lanes have them)
        while (true) {
            bool want = has && has_tris(T);
            uint32_t m = __ballot_sync(0xffffffffu, want);
            if (m == 0u) break;
            if (__popc(m) * 4 < __popc(act)) {
                if (want && sp < sp_blas + postpone_sp) {
                    stack[sp++] = make_uint2(T.x | kTriGroupFlag, T.y);
                    T.y = 0u;
                }
                if (__ballot_sync(0xffffffffu, has && has_tris(T)) == 0u) break;
                want = has && has_tris(T);
            }
            if (!want) continue;
            uint32_t ti = next_tri(T);
            if (tris == nullptr) {
                // enter instance ti: this node's remaining work waits below an exit marker
                if ((G.y & 0xff000000u) != 0u) stack[sp++] = G;
                if (has_tris(T)) stack[sp++] = make_uint2(T.x | kTriGroupFlag, T.y);
                stack[sp++] = make_uint2(kStackExit, 0u);
                sp_blas = sp;
                const InstDev* I = insts + ti;
                float mx[12];
                load_xform(I->w2o, mx);
                r = make_ray(xform_point(mx, r.ox, r.oy, r.oz, r.tmin), xform_dir(mx, r.dx, r.dy, r.dz, 0.0f));
                nodes = I->nodes;
                tris = I->tris;
                prim_base = I->prim_base;
                mat_override = I->material;
                inst = ti;
                G = make_uint2(0u, 0x80000000u | (1u << (7u ^ r.oct_key)));
                T = make_uint2(0u, 0u);
                continue;
            }
            const float4* tp = reinterpret_cast<const float4*>(tris + ti);
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            uint32_t prim = prim_base + __float_as_uint(a.w);
            float t, u, v;
            if (tri_test(r, a, b, c, tbest, prim, best_prim, t, u, v)) {
                bool keep = true;
                if (kOpacity && mat_tr) {
                    float tr = mat_tr[mat_override != kMissPrim ? mat_override : __float_as_uint(b.w)];
                    if (tr != 0.0f) {   // the rule reads the world ray
                        float4 o4, d4;
                        load(idx, o4, d4);
                        keep = keep_hit(make_ray(o4, d4), tr, seed(idx));
                    }
                }
                if (keep) {
                    tbest = t; best_leaf = ti; best_prim = prim; best_inst = inst; bu = u; bv = v;
                    if (kAnyHit) { T.y = 0u; G.y = 0u; sp = 0; }
                }
            }
        }
        // next group, or done
        if (has && (G.y & 0xff000000u) == 0u && !has_tris(T)) {
            const bool done = kAnyHit && best_leaf != kMissPrim;
            uint2 e = make_uint2(0u, 0u);
            if (!done && sp > 0) {
                e = stack[--sp];
                if (e.y == 0u) {  // exit marker: back to the world ray and the TLAS
                    float4 o4, d4, c0 = s_world[threadIdx.x][0], c1 = s_world[threadIdx.x][1];
                    load(idx, o4, d4);
                    const uint32_t pk = __float_as_uint(c0.w);
                    r.ox = o4.x; r.oy = o4.y; r.oz = o4.z; r.tmin = o4.w;
                    r.dx = d4.x; r.dy = d4.y; r.dz = d4.z;
                    r.idx = c0.x; r.idy = c0.y; r.idz = c0.z;
                    r.oct_key = pk & 15u;
                    r.kx = (int)((pk >> 4) & 15u); r.ky = (int)((pk >> 8) & 15u); r.kz = (int)((pk >> 12) & 15u);
                    r.Sx = c1.x; r.Sy = c1.y; r.Sz = c1.z;
                    nodes = tlas; tris = nullptr; inst = kMissPrim; prim_base = 0u; mat_override = kMissPrim;
                    sp_blas = 0;
                    e = sp > 0 ? stack[--sp] : make_uint2(0u, 0u);
                }
            }
            if (e.y != 0u) {
                G = e;
            } else {
                finish(idx, best_leaf, tbest, bu, bv, best_inst);
                has = false;
            }
        }
    }
}

}  // namespace bsm
