// pt_bsdf.cuh — the reference's lit surface model (GGX metallic-roughness plus
// Lambert), its orthonormal frame and direction samplers, plus the lobe
// mixture this pass samples with.
//
// Evaluation follows the reference shaders formula for formula, in the same
// operation order:
//   bisemutum/shaders/core/material/utils.hlsl:40-121  (Schlick, anisotropic
//       roughness, GGX NDF, G1, height-correlated visibility, VNDF sample/pdf)
//   bisemutum/shaders/core/material/lit.hlsl:5-35      (surface_eval_lit)
//   bisemutum/shaders/core/utils/frame.hlsl:9-18       (create_frame(normal))
//   bisemutum/shaders/core/utils/sampling.hlsl:13-31   (sphere / cosine samplers)
// The material conventions are the reference's material function
// (bisemutum/src/scene_basic/menu_actions/import_model.cpp:217-219): f0 =
// lerp(0.04, base_color, metallic), f90 = 1, base colour not scaled by metallic.
#pragma once
#include "pt_math.cuh"

namespace bsm {

struct Surface {
    V3 base_color;
    V3 f0;
    V3 f90;
    float roughness;
    float ior;
};

// utils.hlsl:40-42
BSM_HD V3 schlick_mix(V3 f0, V3 f90, float cos_theta) {
    return lerp(f0, f90, pow5(1.0f - cos_theta));
}
// utils.hlsl:44-51
BSM_HD V3 schlick_fresnel(V3 f0, V3 f90, float cos_theta, float ior) {
    if (cos_theta < 0.0f) {
        float eta = 1.0f / ior;
        float sin_theta_sqr = eta * eta * (1.0f - cos_theta * cos_theta);
        cos_theta = sqrtf(fmaxf(1.0f - sin_theta_sqr, 0.0f));
    }
    return schlick_mix(f0, f90, cos_theta);
}
// utils.hlsl:54-59 with anisotropy = 0 (sqrt(1 - 0 * 0.9) = 1).
BSM_HD void aniso_roughness(float roughness, float* rx, float* ry) {
    float aniso = sqrtf(1.0f - 0.0f * 0.9f);
    float r2 = roughness * roughness;
    *rx = fmaxf(r2 / aniso, 0.001f);
    *ry = fmaxf(r2 * aniso, 0.001f);
}
// utils.hlsl:62-65
BSM_HD float ggx_ndf(V3 h, float rx, float ry) {
    float a = pow2(h.x / rx) + pow2(h.y / ry) + pow2(h.z);
    return BSM_INV_PI / (rx * ry * a * a);
}
// utils.hlsl:67-70
BSM_HD float ggx_g1(V3 v, float rx, float ry) {
    float a = (pow2(rx * v.x) + pow2(ry * v.y)) / fmaxf(v.z * v.z, 0.0001f);
    return 2.0f / (1.0f + sqrtf(1.0f + a));
}
// utils.hlsl:92-96
BSM_HD float ggx_visible_hc(V3 v, V3 l, float rx, float ry) {
    float a = l.z * sqrtf(pow2(rx * v.x) + pow2(ry * v.y) + pow2(v.z));
    float b = v.z * sqrtf(pow2(rx * l.x) + pow2(ry * l.y) + pow2(l.z));
    return 0.5f / fmaxf(a + b, 0.0001f);
}
// utils.hlsl:98-116; cos/sin(TWO_PI * u) come from sincos_turns(u).
BSM_HD V3 ggx_vndf_sample(V3 v, float rx, float ry, float u0, float u1) {
    if (v.z < 0.0f) v = -v;
    V3 vh = normalize(v3(rx * v.x, ry * v.y, v.z));
    float len_sqr = vh.x * vh.x + vh.y * vh.y;
    V3 t1v = len_sqr > 0.0f ? v3(-vh.y, vh.x, 0.0f) / sqrtf(len_sqr) : v3(1.0f, 0.0f, 0.0f);
    V3 t2v = cross(vh, t1v);
    float r = sqrtf(u0);
    float sp, cp;
    sincos_turns(u1, &sp, &cp);
    float t1 = r * cp;
    float t2 = r * sp;
    float s = 0.5f * (1.0f + vh.z);
    t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
    V3 nh = t1 * t1v + t2 * t2v + sqrtf(fmaxf(1.0f - t1 * t1 - t2 * t2, 0.0f)) * vh;
    return normalize(v3(rx * nh.x, ry * nh.y, fmaxf(nh.z, 0.0f)));
}
// utils.hlsl:118-121
BSM_HD float ggx_vndf_pdf(V3 h, V3 v, float rx, float ry) {
    return ggx_g1(v, rx, ry) * ggx_ndf(h, rx, ry) * fmaxf(dot(h, v), 0.0f) / fmaxf(v.z, 0.0001f);
}

// frame.hlsl:9-18 (Duff et al. 2017 branchless ONB): x = tangent, y = bitangent, z = normal.
struct Frame { V3 x, y, z; };
BSM_HD Frame create_frame(V3 n) {
    Frame f;
    f.z = n;
    float sign = n.z > 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    f.x = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f.y = v3(b, sign + n.y * n.y * a, -n.y);
    return f;
}
BSM_HD V3 to_local(const Frame& f, V3 v) { return v3(dot(v, f.x), dot(v, f.y), dot(v, f.z)); }
BSM_HD V3 to_world(const Frame& f, V3 v) { return v.x * f.x + v.y * f.y + v.z * f.z; }

// lit.hlsl:5-35, returning diffuse + specular (material.hlsl surface_eval).
BSM_HD V3 surface_eval_lit(V3 N, V3 T, V3 B, V3 V, V3 L, const Surface& s) {
    V3 H = normalize(V + L);
    V3 lh = v3(dot(H, T), dot(H, B), dot(H, N));
    V3 lv = v3(dot(V, T), dot(V, B), dot(V, N));
    V3 ll = v3(dot(L, T), dot(L, B), dot(L, N));
    if (lv.z <= 0.0f || ll.z <= 0.0f) return v3s(0.0f);
    V3 fr = schlick_fresnel(s.f0, s.f90, fmaxf(dot(V, H), 0.0f), s.ior);
    V3 diffuse = (v3s(1.0f) - fr) * s.base_color * BSM_INV_PI * fmaxf(ll.z, 0.0f);
    float rx, ry;
    aniso_roughness(s.roughness, &rx, &ry);
    float ndf = ggx_ndf(lh, rx, ry);
    float vis = ggx_visible_hc(lv, ll, rx, ry);
    V3 specular = fr * ndf * vis * fmaxf(ll.z, 0.0f);
    return diffuse + specular;
}

// sampling.hlsl:13-21 uniform_sphere_sample.
BSM_HD V3 uniform_sphere_sample(float u0, float u1) {
    float z = u1 * 2.0f - 1.0f;
    float r = sqrtf(fmaxf(1.0f - z * z, 0.0f));
    float sp, cp;
    sincos_turns(u0, &sp, &cp);
    return v3(cp * r, sp * r, z);
}
// sampling.hlsl:24-31 cos_hemisphere_sample / pdf.
BSM_HD V3 cos_hemisphere_sample(float u0, float u1) {
    float r = sqrtf(u1);
    float sp, cp;
    sincos_turns(u0, &sp, &cp);
    return v3(cp * r, sp * r, sqrtf(fmaxf(1.0f - u1, 0.0f)));
}

// ---- lobe mixture used to sample the next direction ----
// The reference samples GGX-VNDF only (sample_secondary_ray.hlsl:51-56, marked
// "TODO - sample full bsdf").  This pass picks the specular lobe with
// probability p_spec (Fresnel weight at the view angle, clamped to
// [0.1, 0.9]) and the cosine lobe otherwise, and weights by the mixture pdf.
BSM_HD float spec_probability(const Surface& s, float ndotv) {
    V3 fn = schlick_mix(s.f0, s.f90, ndotv);
    float ws = fn.x + fn.y + fn.z;
    float wd = (1.0f - fn.x) * s.base_color.x + (1.0f - fn.y) * s.base_color.y + (1.0f - fn.z) * s.base_color.z;
    float p = ws / (ws + wd);
    return fminf(fmaxf(p, 0.1f), 0.9f);
}
// Mixture pdf (solid angle) of sampling local direction ll from local view lv.
BSM_HD float mixture_pdf(V3 lv, V3 ll, float rx, float ry, float p_spec) {
    if (ll.z <= 0.0f) return 0.0f;
    V3 h = normalize(lv + ll);
    float hv = fabsf(dot(h, lv));
    float pdf_spec = hv > 0.0f ? ggx_vndf_pdf(h, lv, rx, ry) / (4.0f * hv) : 0.0f;
    return p_spec * pdf_spec + (1.0f - p_spec) * (ll.z * BSM_INV_PI);
}

}  // namespace bsm
