// pt_lights.cuh — next-event samples of the scene's lights (device and host).
//
//   directional  dir_light_eval (renderer/lights.hlsl:10-13): the emission along
//                the direction to the light
//   point / spot point_light_eval (lights.hlsl:15-25): emission x
//                saturate(1 - (d^2 / range^2)^2) / max(d^2, 0.001), times the
//                spot ramp clamp(cos, cos_outer, cos_inner) when cos_inner > cos_outer
//   rect         the reference integrates it analytically with linearly
//                transformed cosines (lights.hlsl:164-513, unshadowed); here it is
//                a sampled area light: a uniform point on the rectangle gives
//                radiance x cos_light x area / d^2, visibility by a shadow ray.
// The BSDF and its cosine are applied by the caller (surface_eval_lit).
#pragma once
#include "pt_device.h"
#include "pt_math.cuh"

namespace bsm {

// Sample of light `lt` from surface point P with uniforms (u0, u1) (rect lights
// only): direction L to the light, shadow-ray length, arriving radiance e.
// Returns false when the light sends nothing towards P.
BSM_HD bool light_sample(const DevLight& lt, V3 P, float u0, float u1, float ray_len, V3& L, float& tmax, V3& e) {
    const uint32_t kind = f2u(lt.a.w);
    if (kind == kLightDir) {
        L = v3(lt.a.x, lt.a.y, lt.a.z);
        e = v3(lt.b.x, lt.b.y, lt.b.z);
        tmax = ray_len;
        return true;
    }
    V3 lvec;
    if (kind == kLightPoint) {
        lvec = v3(lt.a.x, lt.a.y, lt.a.z) - P;
    } else {
        V3 eu = v3(lt.c.x, lt.c.y, lt.c.z), ev = v3(lt.d.x, lt.d.y, lt.d.z);
        lvec = (v3(lt.a.x, lt.a.y, lt.a.z) + eu * u0 + ev * u1) - P;
    }
    float d2 = dot(lvec, lvec);
    if (!(d2 > 0.0f)) return false;
    float dist = sqrtf(d2);
    L = lvec / dist;
    tmax = fminf(dist, ray_len);
    if (kind == kLightPoint) {
        float x = d2 * lt.b.w;
        float att = fminf(fmaxf(1.0f - x * x, 0.0f), 1.0f) / fmaxf(d2, 0.001f);
        float ci = lt.c.w, co = lt.d.x;
        if (ci > co) {
            float ct = fminf(fmaxf(dot(L, v3(lt.c.x, lt.c.y, lt.c.z)), co), ci);
            att = att * ((ct - co) / fmaxf(ci - co, 0.001f));
        }
        e = v3(lt.b.x, lt.b.y, lt.b.z) * att;
        return att > 0.0f;
    }
    V3 n = normalize(cross(v3(lt.c.x, lt.c.y, lt.c.z), v3(lt.d.x, lt.d.y, lt.d.z)));
    float cl = dot(L, n);  // emits towards -n: it faces P when L runs along +n
    if (f2u(lt.b.w) != 0u) cl = fabsf(cl);
    if (!(cl > 0.0f)) return false;
    e = v3(lt.b.x, lt.b.y, lt.b.z) * (cl * lt.c.w / d2);
    return true;
}

}  // namespace bsm
