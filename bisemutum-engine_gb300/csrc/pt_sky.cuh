// pt_sky.cuh — skybox radiance, importance sampling and pdf.
//
// The reference looks the skybox up only when a ray misses
// (deferred_lighting_secondary.hlsl:23-29: skybox sample x skybox_color x
// weight) and never samples it.  This pass keeps that lookup for escaped
// rays and adds next-event estimation towards the sky:
//   constant sky: uniform sphere directions, pdf 1 / (4 pi);
//   equirect sky: piecewise-constant 2-D distribution over texels weighted by
//     (r + g + b) * sin(theta at the row centre); the marginal CDF picks a row,
//     the row's conditional CDF a column, and the remainders place the
//     direction inside the texel.  pdf(omega) = p_uv / (2 pi^2 sin theta).
// Equirect convention: row 0 looks at +y, column j spans azimuth
// phi = 2 pi (j / W - 0.5) .. 2 pi ((j + 1) / W - 0.5), phi = atan2(z, x).
#pragma once
#include "pt_bsdf.cuh"
#include "pt_device.h"

namespace bsm {

#define BSM_TWO_PI_SQR 19.7392082f

BSM_HD uint32_t cdf_search(const float* cdf, uint32_t n, float u) {
    // largest i in [0, n-1] with cdf[i] <= u (cdf has n + 1 entries, cdf[0] = 0, cdf[n] = 1)
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (cdf[mid] <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
}

BSM_HD float cdf_remainder(const float* cdf, uint32_t i, float u) {
    float w = cdf[i + 1] - cdf[i];
    float f = w > 0.0f ? (u - cdf[i]) / w : 0.5f;
    return fminf(fmaxf(f, 0.0f), 0.99999994f);
}

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

// Samples a sky direction; returns pdf 0 when nothing can be sampled.
__device__ __forceinline__ V3 sky_sample(const DevSky& s, float u0, float u1, float& pdf, V3& le) {
    if (s.kind == 0u) {
        pdf = BSM_INV_FOUR_PI;
        le = v3(s.cr, s.cg, s.cb);
        return uniform_sphere_sample(u0, u1);
    }
    uint32_t i = cdf_search(s.cdf_marg, s.height, u0);
    float fy = cdf_remainder(s.cdf_marg, i, u0);
    const float* row = s.cdf_cond + (size_t)i * (s.width + 1);
    uint32_t j = cdf_search(row, s.width, u1);
    float fx = cdf_remainder(row, j, u1);
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
