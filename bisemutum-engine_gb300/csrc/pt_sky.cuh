// pt_sky.cuh — skybox radiance, importance sampling and pdf.
//
// The reference looks the skybox up only when a ray misses
// (deferred_lighting_secondary.hlsl:23-29: skybox sample x skybox_color x
// weight) and never samples it.  This pass keeps that lookup for escaped
// rays and adds next-event estimation towards the sky:
//   constant sky: uniform sphere directions, pdf 1 / (4 pi);
//   equirect sky: piecewise-constant 2-D distribution over texels weighted by
//     (r + g + b) * sin(theta at the row centre); an alias table (Walker,
//     Vose's construction) picks a texel in two loads, and two uniforms place
//     the direction inside it.  pdf(omega) = p_uv / (2 pi^2 sin theta).
// Equirect convention: row 0 looks at +y, column j spans azimuth
// phi = 2 pi (j / W - 0.5) .. 2 pi ((j + 1) / W - 0.5), phi = atan2(z, x).
#pragma once
#include "pt_bsdf.cuh"
#include "pt_device.h"

namespace bsm {

#define BSM_TWO_PI_SQR 19.7392082f

__device__ __forceinline__ V3 texel_rgb(const DevSky& s, uint32_t i, uint32_t j) {
    ushort4 t = s.texels[(size_t)i * s.width + j];
    return v3(half_to_float(t.x) * s.cr, half_to_float(t.y) * s.cg, half_to_float(t.z) * s.cb);
}

__device__ __forceinline__ void dir_to_texel(const DevSky& s, V3 d, uint32_t& i, uint32_t& j, float& sin_theta) {
    float rxz = sqrtf(d.x * d.x + d.z * d.z);
    float theta = atan2_det(rxz, d.y);              // [0, pi]
    float phi = atan2_det(d.z, d.x);                // [-pi, pi]
    float v = theta * BSM_INV_PI;
    float u = phi * (0.5f * BSM_INV_PI) + 0.5f;
    int ii = (int)floorf(v * (float)s.height);
    int jj = (int)floorf(u * (float)s.width);
    ii = ii < 0 ? 0 : (ii >= (int)s.height ? (int)s.height - 1 : ii);
    jj = jj < 0 ? 0 : (jj >= (int)s.width ? (int)s.width - 1 : jj);
    i = (uint32_t)ii; j = (uint32_t)jj;
    sin_theta = rxz;
}

__device__ __forceinline__ V3 sky_eval(const DevSky& s, V3 d) {
    if (s.kind == 0u) return v3(s.cr, s.cg, s.cb);
    uint32_t i, j; float st;
    dir_to_texel(s, d, i, j, st);
    return texel_rgb(s, i, j);
}

__device__ __forceinline__ float sky_pdf(const DevSky& s, V3 d) {
    if (s.kind == 0u) return BSM_INV_FOUR_PI;
    uint32_t i, j; float st;
    dir_to_texel(s, d, i, j, st);
    if (!(st > 0.0f)) return 0.0f;
    return s.pdf_tab[(size_t)i * s.width + j] / (BSM_TWO_PI_SQR * st);
}

// Samples a sky direction; returns pdf 0 when nothing can be sampled.  An
// equirect sky picks a texel with the alias table (u0: the entry, u1: keep or
// alias, its remainder the row position inside the texel; u2: the column
// position), then the direction inside the texel.
__device__ __forceinline__ V3 sky_sample(const DevSky& s, float u0, float u1, float u2, float& pdf, V3& le) {
    if (s.kind == 0u) {
        pdf = BSM_INV_FOUR_PI;
        le = v3(s.cr, s.cg, s.cb);
        return uniform_sphere_sample(u0, u1);
    }
    const uint32_t n = s.width * s.height;
    uint32_t k = (uint32_t)(u0 * (float)n);
    k = k < n ? k : n - 1u;
    uint2 e = s.alias[k];
    float keep = __uint_as_float(e.x);
    uint32_t t;
    float fy;
    if (u1 < keep) {
        t = k;
        fy = u1 / keep;
    } else {
        t = e.y;
        fy = (u1 - keep) / (1.0f - keep);
    }
    fy = fminf(fmaxf(fy, 0.0f), 0.99999994f);
    float fx = u2;
    uint32_t i = t / s.width, j = t - i * s.width;
    float st, ct, sp, cp;
    sincos_turns(((float)i + fy) / (2.0f * (float)s.height), &st, &ct);
    sincos_turns(((float)j + fx) / (float)s.width - 0.5f, &sp, &cp);
    V3 d = v3(st * cp, ct, st * sp);
    float p = s.pdf_tab[(size_t)i * s.width + j];
    pdf = (st > 0.0f && p > 0.0f) ? p / (BSM_TWO_PI_SQR * st) : 0.0f;
    le = texel_rgb(s, i, j);
    return d;
}

}  // namespace bsm
