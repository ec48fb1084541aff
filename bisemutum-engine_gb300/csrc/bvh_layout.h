// bvh_layout.h — in-memory layout of the compressed 8-wide BVH and of the
// leaf-ordered triangles, shared by the host builder and the CUDA traversal.
//
// The reference never sees its BVH: the graphics driver builds BLAS/TLAS
// (bisemutum/src/graphics/accel.cpp:77-87, 139-158).  This layout follows the
// published compressed wide BVH of Ylitie, Karras and Laine, "Efficient
// Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs" (HPG 2017):
// one 80-byte node holds the quantisation frame of its box and eight child
// boxes quantised outward to 8 bits per plane.  Where the paper keeps a meta
// byte per child (triangle offset and count), this layout keeps one 16-bit
// mask of two bits per slot, so that a node test turns its 8-bit child hit
// mask into the triangle hits with one table lookup and one AND.
#pragma once
#include <stdint.h>

namespace bsm {

// 80 bytes = 5 x 16-byte loads.
struct alignas(16) CwNode {
    float px, py, pz;        // origin of the quantisation grid (node box minimum)
    uint8_t ex, ey, ez;      // per-axis scale 2^(e - 127)
    uint8_t imask;           // bit s: child slot s is an internal node
    uint32_t child_base;     // index of the first internal child (children stored in slot order)
    uint32_t tri_base;       // index of the first triangle of this node's leaf slots (stored in slot order)
    uint16_t tri_mask;       // bits 2s, 2s + 1: leaf slot s holds a first / a second triangle; the triangle
                             // of bit b is tri_base + popc(tri_mask & ((1 << b) - 1))
    uint8_t pad[6];
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(CwNode) == 80, "CwNode must be 80 bytes");
constexpr uint32_t kMaxLeafTris = 2;          // triangles per leaf slot (the tri_mask has two bits per slot)
constexpr uint32_t kTriGroupFlag = 0x80000000u;  // marks a triangle group on a traversal stack (bases < 2^31)

// Leaf-ordered triangle: three float4 (48 bytes).  w of the first vertex holds
// the primitive id (input triangle index) and w of the second the material id.
struct alignas(16) CwTri {
    float v0x, v0y, v0z; uint32_t prim;
    float v1x, v1y, v1z; uint32_t material;
    float v2x, v2y, v2z; uint32_t pad;
};
static_assert(sizeof(CwTri) == 48, "CwTri must be 48 bytes");

// One instance of a two-level scene, stored in the TLAS's leaf order (the
// TLAS's leaf "triangle" index is the index of this record).  The world-to-
// object transform (row-major 3x4) takes a world ray into the geometry's
// space; t is the same in both spaces because the direction is not
// renormalised.  Normals go back with the transpose of its 3x3 part.
struct alignas(16) InstDev {
    float w2o[12];
    float o2w[12];           // object-to-world (tangents of the primary outputs)
    const CwNode* nodes;     // the geometry's BLAS
    const CwTri* tris;
    uint32_t prim_base;      // global primitive id of the instance's triangle 0
    uint32_t material;       // material for every triangle, or kMissPrim: the geometry's ids
    uint32_t id;             // the caller's instance index
    uint32_t pad;
};
static_assert(sizeof(InstDev) == 128, "InstDev must be 128 bytes");

constexpr uint32_t kMissPrim = 0xffffffffu;
constexpr int kMaxTlasDepth = 12;        // TLAS levels the two-level stack budget accepts
constexpr int kMaxTraversalDepth = 24;   // deepest BVH the traversal stack accepts

}  // namespace bsm
