// pt_gbuffer.cuh — the primary-hit outputs of the path-tracing pass besides the
// colour: the packed G-buffer and the reverse-Z device depth.
//
// The reference writes them from its first trace of each frame:
//   rt_gbuffer_rgen (renderer/raytracing/rt_gbuffer.hlsl:28-35): G-buffer of the
//     hit, and hit_positions = (origin + direction * t, t), or (direction, -1)
//     on a miss;
//   pt_depth_fs (renderer/raytracing/pt_depth.hlsl:7-16): clip-space z / w of the
//     hit position, DEVICE_Z_FARTHEST = 0 on a miss (core/utils/depth.hlsl:3-4);
//   pack_surface_to_gbuffer (renderer/gbuffer.hlsl:18-31) with the packing
//     helpers of core/utils/pack.hlsl (6-8 unorm16x2, 14-16 rg11b10, 83-93
//     octahedral normal, 113-121 normal + tangent).
// The packed formats are the reference's bit for bit (a caller unpacks them with
// the reference's unpack_* functions), so the arithmetic follows the same steps.
#pragma once
#include "pt_bsdf.cuh"

namespace bsm {

struct F2 { float x, y; };

// pack.hlsl:6-8 — low and high 16 bits as x / 65536.
BSM_HD F2 pack_u32_unorm16x2(uint32_t x) {
    F2 r;
    r.x = (float)(x & 0xffffu) / 65536.0f;
    r.y = (float)(x >> 16) / 65536.0f;
    return r;
}

// pack.hlsl:14-16 — 11/11/10-bit unsigned fixed point, truncated.
BSM_HD uint32_t pack_rg11b10(V3 c) {
    return (uint32_t)(c.x * 2047.0f) | ((uint32_t)(c.y * 2047.0f) << 11) | ((uint32_t)(c.z * 1023.0f) << 22);
}

// pack.hlsl:83-93 — octahedral map of a unit vector to [-1, 1]^2.
BSM_HD F2 oct_encode(V3 n) {
    float l1 = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
    n = n / l1;
    F2 r;
    if (n.z >= 0.0f) {
        r.x = n.x;
        r.y = n.y;
    } else {
        r.x = (1.0f - fabsf(n.y)) * (n.x >= 0.0f ? 1.0f : -1.0f);
        r.y = (1.0f - fabsf(n.x)) * (n.y >= 0.0f ? 1.0f : -1.0f);
    }
    return r;
}

// pack.hlsl:113-121 — octahedral normal, and the tangent as the L1-normalised
// x of its projection on the normal's frame with the sign of y in the sign.
BSM_HD V3 pack_normal_tangent(V3 N, V3 T) {
    F2 o = oct_encode(N);
    Frame fr = create_frame(N);
    float px = dot(T, fr.x), py = dot(T, fr.y);
    float l1 = fabsf(px) + fabsf(py);
    px = px / l1;
    py = py / l1;
    float qx = px * 0.5f + 0.5f;
    return v3(o.x, o.y, py < 0.0f ? -qx : qx);
}

// gbuffer.hlsl:18-31 for the lit surface model (core/material.hlsl:4) with the
// reference defaults f90 = 1, anisotropy = 0, ior = 1.5 (material/utils.hlsl:18-31).
// g[0] base colour, g[1] normal + roughness, g[2] fresnel, g[3] material_0.
BSM_HD void pack_gbuffer(V3 N, V3 T, V3 base, V3 f0, float roughness, float g[16]) {
    g[0] = base.x; g[1] = base.y; g[2] = base.z; g[3] = 1.0f;
    V3 nt = pack_normal_tangent(N, T);
    g[4] = nt.x; g[5] = nt.y; g[6] = nt.z; g[7] = roughness;
    F2 a = pack_u32_unorm16x2(pack_rg11b10(f0));
    F2 b = pack_u32_unorm16x2(pack_rg11b10(v3s(1.0f)));
    g[8] = a.x; g[9] = a.y; g[10] = b.x; g[11] = b.y;
    g[12] = 0.0f; g[13] = 1.0f / 1.5f; g[14] = 0.0f; g[15] = 1.0f / 256.0f;
}

// pt_depth.hlsl:13-15 with the reverse-Z perspective of math.cpp:5-11
// (m22 = near / (far - near), m32 = near * far / (far - near), w = -z_view):
// depth = (m22 * z_view + m32) / -z_view, z_view = -dot(front, P - eye).
BSM_HD float reverse_z_depth(V3 eye, V3 front, V3 P, float near_z, float far_z) {
    float inv = 1.0f / (far_z - near_z);
    float m22 = near_z * inv;
    float m32 = near_z * far_z * inv;
    float zv = -dot(front, P - eye);
    return (m22 * zv + m32) / -zv;
}

}  // namespace bsm
