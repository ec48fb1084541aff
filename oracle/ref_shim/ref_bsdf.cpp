// ref_bsdf.cpp — TEST INFRASTRUCTURE: compiles the reference's shader math
// (bisemutum/shaders/core/utils/math.hlsl, core/material/utils.hlsl,
// core/material/lit.hlsl, core/utils/frame.hlsl, core/utils/sampling.hlsl,
// the G-buffer packing of core/utils/pack.hlsl and renderer/gbuffer.hlsl, and
// the light evaluation of renderer/lights.hlsl)
// through hlsl_shim.h and exposes it to the golden-vector generator.  The
// sources are read where they lie in the reference tree by oracle/build.py,
// which only rewrites `out T x` / `inout T x` parameters to `T& x`; the result
// is built into oracle/_ref/ and never shipped.
#include "hlsl_shim.h"

#include "ref_sources.inc"  // generated: the reference files and extracted functions, concatenated

#define REF_API extern "C" __attribute__((visibility("default")))

// in: N3 V3 L3 base3 f0_3 roughness; out: diffuse + specular of surface_eval_lit
// with the frame of create_frame(N) (frame.hlsl:9-18) as T, B.
REF_API void ref_eval_lit(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 16 * (size_t)i;
        float3 N(a[0], a[1], a[2]), V(a[3], a[4], a[5]), L(a[6], a[7], a[8]);
        SurfaceData s = surface_data_default();
        s.base_color = float3(a[9], a[10], a[11]);
        s.f0_color = float3(a[12], a[13], a[14]);
        s.roughness = a[15];
        Frame fr = create_frame(N);
        float3 d, sp;
        surface_eval_lit(N, fr.x, fr.y, V, L, s, d, sp);
        float3 r = d + sp;
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
}
// in: V3 rx ry u0 u1; out: h3, ggx_vndf_sample_pdf(h, v)
REF_API void ref_vndf(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 7 * (size_t)i;
        float3 v(a[0], a[1], a[2]);
        float3 h = ggx_vndf_sample(v, a[3], a[4], float2(a[5], a[6]));
        out[4 * i] = h.x; out[4 * i + 1] = h.y; out[4 * i + 2] = h.z;
        out[4 * i + 3] = ggx_vndf_sample_pdf(h, v, a[3], a[4]);
    }
}
// in: N3; out: frame.x, frame.y
REF_API void ref_frame(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        Frame f = create_frame(float3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
        float* o = out + 6 * (size_t)i;
        o[0] = f.x.x; o[1] = f.x.y; o[2] = f.x.z; o[3] = f.y.x; o[4] = f.y.y; o[5] = f.y.z;
    }
}
// in: roughness; out: (roughness_x, roughness_y) of get_anisotropic_roughness(r, 0)
REF_API void ref_aniso(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) get_anisotropic_roughness(in[i], 0.0f, out[2 * i], out[2 * i + 1]);
}
// in: u0 u1; out: cos_hemisphere_sample (3), uniform_sphere_sample (3)
REF_API void ref_samplers(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        float2 u(in[2 * i], in[2 * i + 1]);
        float3 c = cos_hemisphere_sample(u);
        float3 s = uniform_sphere_sample(u);
        float* o = out + 6 * (size_t)i;
        o[0] = c.x; o[1] = c.y; o[2] = c.z; o[3] = s.x; o[4] = s.y; o[5] = s.z;
    }
}
REF_API float ref_inv_pi(void) { return INV_PI; }
// in: V3 N3 T3 base3 f0_3 roughness; out: the four float4 of
// pack_surface_to_gbuffer (gbuffer.hlsl:18-31) for the lit surface model
// (material.hlsl:4) with the default f90, anisotropy and ior (utils.hlsl:18-31).
REF_API void ref_gbuffer(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 16 * (size_t)i;
        SurfaceData s = surface_data_default();
        s.base_color = float3(a[9], a[10], a[11]);
        s.f0_color = float3(a[12], a[13], a[14]);
        s.roughness = a[15];
        GBuffer g = pack_surface_to_gbuffer(float3(a[0], a[1], a[2]), float3(a[3], a[4], a[5]),
                                            float3(a[6], a[7], a[8]), s, 1u);
        const float4* q[4] = {&g.base_color, &g.normal_roughness, &g.fresnel, &g.material_0};
        for (int k = 0; k < 4; ++k) {
            float* o = out + 16 * (size_t)i + 4 * k;
            o[0] = q[k]->x; o[1] = q[k]->y; o[2] = q[k]->z; o[3] = q[k]->w;
        }
    }
}
// in: the four float4 of a packed G-buffer; out: unpack_gbuffer_to_surface
// (gbuffer.hlsl:33-45): N3 T3 base3 f0_3 f90_3 roughness anisotropy ior model, 0.
REF_API void ref_gbuffer_unpack(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 16 * (size_t)i;
        GBuffer g;
        g.base_color = float4(a[0], a[1], a[2], a[3]);
        g.normal_roughness = float4(a[4], a[5], a[6], a[7]);
        g.fresnel = float4(a[8], a[9], a[10], a[11]);
        g.material_0 = float4(a[12], a[13], a[14], a[15]);
        float3 N, T;
        SurfaceData s;
        uint model;
        unpack_gbuffer_to_surface(g, N, T, s, model);
        const float v[20] = {N.x, N.y, N.z, T.x, T.y, T.z, s.base_color.x, s.base_color.y, s.base_color.z,
                             s.f0_color.x, s.f0_color.y, s.f0_color.z, s.f90_color.x, s.f90_color.y, s.f90_color.z,
                             s.roughness, s.anisotropy, s.ior, (float)model, 0.0f};
        for (int k = 0; k < 20; ++k) out[20 * (size_t)i + k] = v[k];
    }
}

// in: light position3, emission3, range, direction to the light3, cos_inner, cos_outer, P3 (16 floats);
// out: point_light_eval's radiance (3) and light_dir (3) (renderer/lights.hlsl:15-25).
REF_API void ref_point_light(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 16 * (size_t)i;
        PointLightData L{};
        L.position = float3(a[0], a[1], a[2]);
        L.emission = float3(a[3], a[4], a[5]);
        L.range_sqr_inv = 1.0f / (a[6] * a[6]);
        L.direction = float3(a[7], a[8], a[9]);
        L.cos_inner = a[10];
        L.cos_outer = a[11];
        float3 dir;
        float3 e = point_light_eval(L, float3(a[12], a[13], a[14]), dir);
        float* o = out + 6 * (size_t)i;
        o[0] = e.x; o[1] = e.y; o[2] = e.z; o[3] = dir.x; o[4] = dir.y; o[5] = dir.z;
    }
}
// in: direction to the light3, emission3, P3; out: dir_light_eval's radiance (3) and light_dir (3)
// (renderer/lights.hlsl:10-13).
REF_API void ref_dir_light(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 9 * (size_t)i;
        DirLightData L{};
        L.direction = float3(a[0], a[1], a[2]);
        L.emission = float3(a[3], a[4], a[5]);
        float3 dir;
        float3 e = dir_light_eval(L, float3(a[6], a[7], a[8]), dir);
        float* o = out + 6 * (size_t)i;
        o[0] = e.x; o[1] = e.y; o[2] = e.z; o[3] = dir.x; o[4] = dir.y; o[5] = dir.z;
    }
}
