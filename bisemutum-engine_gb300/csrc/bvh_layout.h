// bvh_layout.h — in-memory layout of the compressed 8-wide BVH and of the
// leaf-ordered triangles, shared by the host builder and the CUDA traversal.
//
// The reference never sees its BVH: the graphics driver builds BLAS/TLAS
// (bisemutum/src/graphics/accel.cpp:77-87, 139-158).  This layout follows the
// published compressed wide BVH of Ylitie, Karras and Laine, "Efficient
// Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs" (HPG 2017):
// one 80-byte node holds the quantisation frame of its box and eight child
// boxes quantised outward to 8 bits per plane.
#pragma once
#include <stdint.h>

namespace bsm {

// 80 bytes = 5 x 16-byte loads.
struct alignas(16) CwNode {
    float px, py, pz;        // origin of the quantisation grid (node box minimum)
    uint8_t ex, ey, ez;      // per-axis scale 2^(e - 127)
    uint8_t imask;           // bit s: child slot s is an internal node
    uint32_t child_base;     // index of the first internal child (children stored in slot order)
    uint32_t tri_base;       // index of the first triangle referenced by this node's leaves
    uint8_t meta[8];         // per slot: 0 = empty; internal: 0x20 | (24 + slot);
                             //           leaf: (unary triangle count << 5) | triangle offset (0..23)
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(CwNode) == 80, "CwNode must be 80 bytes");

// Leaf-ordered triangle: three float4 (48 bytes).  w of the first vertex holds
// the primitive id (input triangle index) and w of the second the material id.
struct alignas(16) CwTri {
    float v0x, v0y, v0z; uint32_t prim;
    float v1x, v1y, v1z; uint32_t material;
    float v2x, v2y, v2z; uint32_t pad;
};
static_assert(sizeof(CwTri) == 48, "CwTri must be 48 bytes");

constexpr uint32_t kMissPrim = 0xffffffffu;
constexpr int kMaxTraversalDepth = 24;   // deepest BVH the traversal stack accepts

}  // namespace bsm
