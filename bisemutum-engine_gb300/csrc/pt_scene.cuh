// pt_scene.cuh — traversal and hit geometry over either kind of scene: one BVH
// over world-space triangles, or a two-level scene (TLAS over instances of
// object-space geometries).  Shared by the wavefront kernels, the primary
// outputs and the radiance-cache training paths.
#pragma once
#include "pt_device.h"
#include "pt_trace.cuh"

namespace bsm {

template <bool kAnyHit>
__device__ __forceinline__ uint32_t trace_scene(const DevScene& sc, const RayPre& r, float tmax, float& t, float& u,
                                                float& v, uint32_t& inst, uint32_t oseed) {
    if (sc.insts) return trace_ray2<kAnyHit>(r, tmax, sc.nodes, sc.insts, sc.mat_tr, t, u, v, inst, oseed);
    inst = kMissPrim;
    return trace_ray<kAnyHit, false>(r, tmax, sc.nodes, sc.tris, t, u, v, nullptr, oseed);
}

// n' = transpose(linear part of m) n: normals go from object to world space
// with the transpose of the world-to-object transform.
__device__ __forceinline__ V3 xform_normal(const float* m, V3 n) {
    return v3(__fadd_rn(__fadd_rn(__fmul_rn(m[0], n.x), __fmul_rn(m[4], n.y)), __fmul_rn(m[8], n.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[1], n.x), __fmul_rn(m[5], n.y)), __fmul_rn(m[9], n.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[2], n.x), __fmul_rn(m[6], n.y)), __fmul_rn(m[10], n.z)));
}

// The hit triangle's unit geometric normal and first edge in world space (the
// normal not yet faced towards the ray) and its material.
__device__ __forceinline__ void hit_geometry(const DevScene& sc, uint32_t leaf, uint32_t inst, V3& ng, V3& edge,
                                             uint32_t& material) {
    const CwTri* tris = inst != kMissPrim ? sc.insts[inst].tris : sc.tris;
    const float4* tp = reinterpret_cast<const float4*>(tris + leaf);
    float4 a = tp[0], b = tp[1], c = tp[2];
    V3 va = v3(a.x, a.y, a.z), vb = v3(b.x, b.y, b.z), vc = v3(c.x, c.y, c.z);
    ng = normalize(cross(vb - va, vc - va));
    edge = vb - va;
    material = __float_as_uint(b.w);
    if (inst != kMissPrim) {
        const InstDev* I = sc.insts + inst;
        float m[12];
        load_xform(I->w2o, m);
        ng = normalize(xform_normal(m, ng));
        load_xform(I->o2w, m);
        float4 e = xform_dir(m, edge.x, edge.y, edge.z, 0.0f);
        edge = v3(e.x, e.y, e.z);
        if (I->material != kMissPrim) material = I->material;
    }
    if (material >= sc.num_materials) material = 0;
}

// The shading normal of a hit on a scene that carries vertex normals.  The
// reference's fetch_vertex_attributes (bisemutum/shaders/core/raytracing/
// hit.hlsl:55-71, 158) interpolates n0 + (n1 - n0) b1 + (n2 - n0) b2, b1 and b2
// the barycentric weights of the second and third vertex, and normalises the
// result.  A hit's (u, v) are the weights of the first and second vertex, so
// b1 = v and b2 = 1 - u - v.  A zero interpolated normal falls back to `ng`.
__device__ __forceinline__ V3 shading_normal(const DevScene& sc, uint32_t leaf, float u, float v, V3 ng) {
    const float4* np = sc.tri_normals + 3 * (size_t)leaf;
    const float4 a = np[0], b = np[1], c = np[2];
    const V3 n0 = v3(a.x, a.y, a.z), n1 = v3(b.x, b.y, b.z), n2 = v3(c.x, c.y, c.z);
    const float b1 = v, b2 = 1.0f - u - v;
    V3 n = n0 + (n1 - n0) * b1 + (n2 - n0) * b2;
    return dot(n, n) > 0.0f ? normalize(n) : ng;
}

}  // namespace bsm
