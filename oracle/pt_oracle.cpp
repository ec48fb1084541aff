// pt_oracle.cpp — CPU ORACLE of the wavefront path-tracing pass.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA pass and
// the timed CPU baseline; the product library never links or calls it.
//
// It restates, in plain multithreaded C++, the stages of the bisemutum
// builtin renderer's path-tracing pass (paths relative to the reference repo):
//   camera rays      bisemutum/shaders/renderer/raytracing/direction_sample/generate_camera_ray.hlsl:9-15
//                    with the reverse-Z projection of bisemutum/src/math/math.cpp:5-11 and
//                    lookAt/perspective of bisemutum/src/graphics/camera.cpp:96-98
//   closest / any hit rt_gbuffer.hlsl:17-35 (TraceRay, TMin, TMax = ray_length)
//   lighting         deferred_lighting_secondary.hlsl:23-29 (sky on a miss), :51-60
//                    (directional light x visibility x surface_eval), lights.hlsl:10-13
//   BSDF             bisemutum/shaders/core/material/utils.hlsl:40-121, lit.hlsl:5-35
//   frame            bisemutum/shaders/core/utils/frame.hlsl:9-18
//   samplers         bisemutum/shaders/core/utils/sampling.hlsl:13-31
//   next direction   sample_secondary_ray.hlsl:16-28 (termination), :51-64 (weight, NaN guard)
//   accumulation     pt_accumulate.hlsl:3-11 (running mean = sum / samples)
//   primary outputs  pt_depth.hlsl:7-16 (reverse-Z depth), renderer/gbuffer.hlsl:18-31 and
//                    core/utils/pack.hlsl:6-16, 83-93, 113-121 (G-buffer packing)
// and the decisions the CUDA pass takes where the reference has none (PCG32
// streams keyed to pixel and sample, next-event estimation towards the sun
// and the importance-sampled sky with MIS, lobe-mixture sampling).  It keeps
// its own binary SAH BVH: the closest hit does not depend on the tree, and
// agreement with the GPU's compressed 8-wide BVH is itself part of the check.
// Arithmetic is IEEE single precision in the same order as the CUDA kernels
// (built with -ffp-contract=off), so primitive ids, t values and path
// decisions agree bit for bit.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#define ORC_API extern "C" __attribute__((visibility("default")))

namespace orc {

// ------------------------------------------------------------- vectors ----
struct F3 { float x, y, z; };
static inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
static inline F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline F3 neg(F3 a) { return f3(-a.x, -a.y, -a.z); }
static inline F3 mul(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline F3 muls(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
static inline F3 smul(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
static inline F3 divs(F3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
static inline float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline F3 cross3(F3 a, F3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline F3 norm3(F3 a) { float inv = 1.0f / std::sqrt(dot3(a, a)); return muls(a, inv); }
static inline float maxc(F3 a) { return std::fmax(a.x, std::fmax(a.y, a.z)); }
static inline F3 lerp3(F3 a, F3 b, float t) { return add(a, muls(sub(b, a), t)); }
static inline float sq(float x) { return x * x; }

// sin/cos of 2*pi*t and atan2, from their Taylor series with range reduction
// (the CUDA pass uses the same polynomials so both sides round identically).
static void sincos_turns(float t, float* s, float* c) {
    float q = std::floor(t * 4.0f + 0.5f);
    float r = t - q * 0.25f;
    int iq = ((int)q) & 3;
    float x = r * 6.28318548f;
    float x2 = x * x;
    float ps = x + x * x2 * (-0.166666672f + x2 * (0.00833333377f + x2 * (-0.000198412701f + x2 * 2.75573188e-06f)));
    float pc = 1.0f + x2 * (-0.5f + x2 * (0.0416666679f + x2 * (-0.00138888892f + x2 * (2.48015876e-05f + x2 * -2.75573188e-07f))));
    if (iq == 0) { *s = ps; *c = pc; }
    else if (iq == 1) { *s = pc; *c = -ps; }
    else if (iq == 2) { *s = -ps; *c = -pc; }
    else { *s = -pc; *c = ps; }
}
static float atan_unit(float z) {
    float off = 0.0f;
    if (z > 0.414213568f) { z = (z - 1.0f) / (z + 1.0f); off = 0.785398185f; }
    float z2 = z * z;
    float p = 1.0f + z2 * (-0.333333343f + z2 * (0.200000003f + z2 * (-0.142857149f + z2 * (0.111111112f +
              z2 * (-0.0909090936f + z2 * (0.0769230798f + z2 * (-0.0666666701f + z2 * 0.0588235296f)))))));
    return off + z * p;
}
static float atan2_det(float y, float x) {
    float ax = std::fabs(x), ay = std::fabs(y);
    float mx = std::fmax(ax, ay), mn = std::fmin(ax, ay);
    if (mx == 0.0f) return 0.0f;
    float a = atan_unit(mn / mx);
    if (ay > ax) a = 1.57079637f - a;
    if (x < 0.0f) a = 3.14159274f - a;
    if (y < 0.0f) a = -a;
    return a;
}
static float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16, exp = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    if (exp == 0) { float f = (float)man * 5.96046448e-08f; return sign ? -f : f; }
    uint32_t bits = exp == 31 ? (sign | 0x7f800000u | (man << 13)) : (sign | ((exp + 112u) << 23) | (man << 13));
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// ------------------------------------------------------------- PCG32 ----
// O'Neill 2014, pcg32 XSH-RR with a 64-bit LCG (pcg_basic).
struct Pcg { uint64_t state, inc; };
static uint32_t pcg_next(Pcg& g) {
    uint64_t old = g.state;
    g.state = old * 6364136223846793005ULL + g.inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
static Pcg pcg_seed(uint64_t initstate, uint64_t initseq) {
    Pcg g{0u, (initseq << 1u) | 1u};
    pcg_next(g);
    g.state += initstate;
    pcg_next(g);
    return g;
}
static float pcg_uniform(Pcg& g) { return (float)(pcg_next(g) >> 8) * 5.96046448e-08f; }
static uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static uint64_t sample_initstate(uint64_t seed, uint32_t sample) {
    return mix64(seed + 0x9e3779b97f4a7c15ULL * ((uint64_t)sample + 1u));
}
// per-path start state: the pixel mixed into the sample's state (decorrelates the streams)
static uint64_t path_initstate(uint64_t seed, uint32_t sample, uint64_t pixel) {
    return mix64(sample_initstate(seed, sample) ^ mix64(pixel * 0x9e3779b97f4a7c15ULL + 0x632be59bd9b4e019ULL));
}

// -------------------------------------------------- reference BSDF ----
static const float kInvPi = 0.318309873f;
struct Surf { F3 base, f0, f90; float rough, ior; };

static F3 schlick_mix(F3 f0, F3 f90, float c) {            // utils.hlsl:40-42
    float x = 1.0f - c;
    float x2 = x * x;
    return lerp3(f0, f90, (x2 * x2) * x);
}
static F3 schlick_fresnel(F3 f0, F3 f90, float c, float ior) {  // utils.hlsl:44-51
    if (c < 0.0f) {
        float eta = 1.0f / ior;
        float s2 = eta * eta * (1.0f - c * c);
        c = std::sqrt(std::fmax(1.0f - s2, 0.0f));
    }
    return schlick_mix(f0, f90, c);
}
static void aniso_rough(float r, float* rx, float* ry) {  // utils.hlsl:54-59, anisotropy 0
    float aniso = std::sqrt(1.0f - 0.0f * 0.9f);
    float r2 = r * r;
    *rx = std::fmax(r2 / aniso, 0.001f);
    *ry = std::fmax(r2 * aniso, 0.001f);
}
static float ggx_ndf(F3 h, float rx, float ry) {  // utils.hlsl:62-65
    float a = sq(h.x / rx) + sq(h.y / ry) + sq(h.z);
    return kInvPi / (rx * ry * a * a);
}
static float ggx_g1(F3 v, float rx, float ry) {  // utils.hlsl:67-70
    float a = (sq(rx * v.x) + sq(ry * v.y)) / std::fmax(v.z * v.z, 0.0001f);
    return 2.0f / (1.0f + std::sqrt(1.0f + a));
}
static float ggx_vis_hc(F3 v, F3 l, float rx, float ry) {  // utils.hlsl:92-96
    float a = l.z * std::sqrt(sq(rx * v.x) + sq(ry * v.y) + sq(v.z));
    float b = v.z * std::sqrt(sq(rx * l.x) + sq(ry * l.y) + sq(l.z));
    return 0.5f / std::fmax(a + b, 0.0001f);
}
static F3 ggx_vndf_sample(F3 v, float rx, float ry, float u0, float u1) {  // utils.hlsl:98-116
    if (v.z < 0.0f) v = neg(v);
    F3 vh = norm3(f3(rx * v.x, ry * v.y, v.z));
    float ls = vh.x * vh.x + vh.y * vh.y;
    F3 t1v = ls > 0.0f ? divs(f3(-vh.y, vh.x, 0.0f), std::sqrt(ls)) : f3(1.0f, 0.0f, 0.0f);
    F3 t2v = cross3(vh, t1v);
    float r = std::sqrt(u0);
    float sp, cp;
    sincos_turns(u1, &sp, &cp);
    float t1 = r * cp, t2 = r * sp;
    float s = 0.5f * (1.0f + vh.z);
    t2 = (1.0f - s) * std::sqrt(1.0f - t1 * t1) + s * t2;
    F3 nh = add(add(smul(t1, t1v), smul(t2, t2v)), smul(std::sqrt(std::fmax(1.0f - t1 * t1 - t2 * t2, 0.0f)), vh));
    return norm3(f3(rx * nh.x, ry * nh.y, std::fmax(nh.z, 0.0f)));
}
static float ggx_vndf_pdf(F3 h, F3 v, float rx, float ry) {  // utils.hlsl:118-121
    return ggx_g1(v, rx, ry) * ggx_ndf(h, rx, ry) * std::fmax(dot3(h, v), 0.0f) / std::fmax(v.z, 0.0001f);
}
struct Frm { F3 x, y, z; };
static Frm make_frame(F3 n) {  // frame.hlsl:9-18
    Frm f;
    f.z = n;
    float sign = n.z > 0.0f ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    f.x = f3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f.y = f3(b, sign + n.y * n.y * a, -n.y);
    return f;
}
static F3 local_of(const Frm& f, F3 v) { return f3(dot3(v, f.x), dot3(v, f.y), dot3(v, f.z)); }
static F3 world_of(const Frm& f, F3 v) { return add(add(smul(v.x, f.x), smul(v.y, f.y)), smul(v.z, f.z)); }
static F3 eval_lit(F3 N, F3 T, F3 B, F3 V, F3 L, const Surf& s) {  // lit.hlsl:5-35
    F3 H = norm3(add(V, L));
    F3 lh = f3(dot3(H, T), dot3(H, B), dot3(H, N));
    F3 lv = f3(dot3(V, T), dot3(V, B), dot3(V, N));
    F3 ll = f3(dot3(L, T), dot3(L, B), dot3(L, N));
    if (lv.z <= 0.0f || ll.z <= 0.0f) return f3(0, 0, 0);
    F3 fr = schlick_fresnel(s.f0, s.f90, std::fmax(dot3(V, H), 0.0f), s.ior);
    F3 diffuse = muls(muls(mul(sub(f3(1, 1, 1), fr), s.base), kInvPi), std::fmax(ll.z, 0.0f));
    float rx, ry;
    aniso_rough(s.rough, &rx, &ry);
    float ndf = ggx_ndf(lh, rx, ry);
    float vis = ggx_vis_hc(lv, ll, rx, ry);
    F3 spec = muls(muls(muls(fr, ndf), vis), std::fmax(ll.z, 0.0f));
    return add(diffuse, spec);
}
static F3 sphere_sample(float u0, float u1) {  // sampling.hlsl:13-19
    float z = u1 * 2.0f - 1.0f;
    float r = std::sqrt(std::fmax(1.0f - z * z, 0.0f));
    float sp, cp;
    sincos_turns(u0, &sp, &cp);
    return f3(cp * r, sp * r, z);
}
static F3 cos_hemi_sample(float u0, float u1) {  // sampling.hlsl:24-28
    float r = std::sqrt(u1);
    float sp, cp;
    sincos_turns(u0, &sp, &cp);
    return f3(cp * r, sp * r, std::sqrt(std::fmax(1.0f - u1, 0.0f)));
}
static float spec_prob(const Surf& s, float ndotv) {
    F3 fn = schlick_mix(s.f0, s.f90, ndotv);
    float ws = fn.x + fn.y + fn.z;
    float wd = (1.0f - fn.x) * s.base.x + (1.0f - fn.y) * s.base.y + (1.0f - fn.z) * s.base.z;
    float p = ws / (ws + wd);
    return std::fmin(std::fmax(p, 0.1f), 0.9f);
}
static float mix_pdf(F3 lv, F3 ll, float rx, float ry, float ps) {
    if (ll.z <= 0.0f) return 0.0f;
    F3 h = norm3(add(lv, ll));
    float hv = std::fabs(dot3(h, lv));
    float pspec = hv > 0.0f ? ggx_vndf_pdf(h, lv, rx, ry) / (4.0f * hv) : 0.0f;
    return ps * pspec + (1.0f - ps) * (ll.z * kInvPi);
}

// ------------------------------------------------------------- scene ----
// tr: transparency of the any-hit rule (0 = opaque); na..nc: vertex normals where the scene has them (has_n)
struct Tri { F3 a, b, c; uint32_t prim, mat; float tr; F3 na, nb, nc; uint32_t has_n; };
struct BNode { float lo[3], hi[3]; uint32_t left_or_first, count; uint32_t axis; };  // count > 0: leaf

struct Scene {
    std::vector<Tri> tris;         // in BVH leaf order
    std::vector<BNode> nodes;
    std::vector<float> mats;       // 8 per material: base rgb, rough, f0 rgb, metallic
    uint32_t nmat = 0;
    // lights: 0 directional (a = direction, b = emission), 1 point/spot (a = position, b = emission,
    // bw = 1 / range^2, c = direction to the light, cw = cos_inner, dx = cos_outer), 2 rect (a = corner,
    // b = emission, bw = two_sided, c / d = edges, cw = area)
    struct Light { uint32_t kind; F3 a, b, c, d; float bw, cw, dx; };
    uint32_t nlights = 0;
    Light lights[8];
    uint32_t sky_kind = 0;
    F3 sky_color{0, 0, 0};
    uint32_t sw = 0, sh = 0;
    std::vector<uint16_t> texels;
    std::vector<float> ptab, aprob;   // sky: pdf per texel, alias keep probability
    std::vector<uint32_t> alias;
    float extent = 1.0f, offset = 0.0f;
    float box_lo[3] = {0, 0, 0}, box_inv[3] = {1, 1, 1};   // the radiance cache's position normalisation
    // two-level scenes: instances of geometries (each a Scene holding tris + BVH only)
    struct Inst {
        const struct Scene* geo;
        uint32_t material;          // every triangle's material, or UINT32_MAX
        float o2w[12], w2o[12];     // row-major 3x4
        uint32_t prim_base;
    };
    std::vector<Inst> inst;
    std::vector<float> trm;         // per material transparency (two-level scenes)
    float glo[3], ghi[3];           // a geometry's bounds over all its vertices
};

// binned SAH binary BVH (16 bins, leaves of up to 4 triangles)
struct BuildRef { float lo[3], hi[3], c[3]; uint32_t t; };
static double area(const float lo[3], const float hi[3]) {
    double d0 = std::max(0.0, (double)hi[0] - lo[0]), d1 = std::max(0.0, (double)hi[1] - lo[1]),
           d2 = std::max(0.0, (double)hi[2] - lo[2]);
    return 2.0 * (d0 * d1 + d1 * d2 + d2 * d0);
}
static uint32_t build_rec(Scene& S, std::vector<BuildRef>& refs, uint32_t b, uint32_t e) {
    uint32_t ni = (uint32_t)S.nodes.size();
    S.nodes.push_back(BNode{});
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = b; i < e; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], refs[i].lo[k]); hi[k] = std::max(hi[k], refs[i].hi[k]);
            clo[k] = std::min(clo[k], refs[i].c[k]); chi[k] = std::max(chi[k], refs[i].c[k]);
        }
    uint32_t n = e - b;
    auto make_leaf = [&]() {
        BNode& nd = S.nodes[ni];
        for (int k = 0; k < 3; ++k) { nd.lo[k] = lo[k]; nd.hi[k] = hi[k]; }
        nd.left_or_first = b;
        nd.count = n;
        return ni;
    };
    if (n <= 2) return make_leaf();
    const int NB = 16;
    double best = INFINITY;
    int ba = -1, bs = 0;
    for (int a = 0; a < 3; ++a) {
        float ext = chi[a] - clo[a];
        if (!(ext > 0.0f)) continue;
        uint32_t cnt[NB] = {0};
        float blo[NB][3], bhi[NB][3];
        for (int j = 0; j < NB; ++j)
            for (int k = 0; k < 3; ++k) { blo[j][k] = INFINITY; bhi[j][k] = -INFINITY; }
        for (uint32_t i = b; i < e; ++i) {
            int j = std::min(NB - 1, (int)((refs[i].c[a] - clo[a]) / ext * NB));
            cnt[j]++;
            for (int k = 0; k < 3; ++k) { blo[j][k] = std::min(blo[j][k], refs[i].lo[k]); bhi[j][k] = std::max(bhi[j][k], refs[i].hi[k]); }
        }
        for (int s = 1; s < NB; ++s) {
            float l0[3] = {INFINITY, INFINITY, INFINITY}, l1[3] = {-INFINITY, -INFINITY, -INFINITY};
            float r0[3] = {INFINITY, INFINITY, INFINITY}, r1[3] = {-INFINITY, -INFINITY, -INFINITY};
            uint32_t nl = 0, nr = 0;
            for (int j = 0; j < NB; ++j) {
                float* x0 = j < s ? l0 : r0;
                float* x1 = j < s ? l1 : r1;
                if (j < s) nl += cnt[j]; else nr += cnt[j];
                for (int k = 0; k < 3; ++k) { x0[k] = std::min(x0[k], blo[j][k]); x1[k] = std::max(x1[k], bhi[j][k]); }
            }
            if (!nl || !nr) continue;
            double c = area(l0, l1) * nl + area(r0, r1) * nr;
            if (c < best) { best = c; ba = a; bs = s; }
        }
    }
    uint32_t mid;
    if (ba < 0) {
        if (n <= 4) return make_leaf();
        mid = b + n / 2;
    } else {
        double leaf_cost = (double)n, split_cost = 0.5 + best / std::max(area(lo, hi), 1e-30);
        if (n <= 4 && leaf_cost <= split_cost) return make_leaf();
        float ext = chi[ba] - clo[ba];
        auto it = std::partition(refs.begin() + b, refs.begin() + e, [&](const BuildRef& r) {
            return std::min(NB - 1, (int)((r.c[ba] - clo[ba]) / ext * NB)) < bs;
        });
        mid = (uint32_t)(it - refs.begin());
        if (mid == b || mid == e) mid = b + n / 2;
    }
    int axis = 0;
    float ext0 = hi[0] - lo[0];
    if (hi[1] - lo[1] > ext0) { axis = 1; ext0 = hi[1] - lo[1]; }
    if (hi[2] - lo[2] > ext0) axis = 2;
    if (ba >= 0) axis = ba;
    build_rec(S, refs, b, mid);
    uint32_t right = build_rec(S, refs, mid, e);
    BNode& nd = S.nodes[ni];
    for (int k = 0; k < 3; ++k) { nd.lo[k] = lo[k]; nd.hi[k] = hi[k]; }
    nd.left_or_first = right;  // left child is ni + 1
    nd.count = 0;
    nd.axis = (uint32_t)axis;
    return ni;
}

// ------------------------------------------------------------ traversal ----
struct Ray {
    F3 o, d;
    float tmin, tmax;
    uint32_t oseed;   // opacity seed (the path's PCG32 word; 0 for the stage entry points)
    float id[3];
    float idc[3];     // reciprocals of the compressed-BVH box test: |d| below 1e-20 taken as +-1e-20
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
static float comp(F3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static Ray make_ray(F3 o, float tmin, F3 d, float tmax, uint32_t oseed = 0) {
    Ray r;
    r.o = o; r.d = d; r.tmin = tmin; r.tmax = tmax; r.oseed = oseed;
    for (int k = 0; k < 3; ++k) {
        float dk = comp(d, k);
        r.id[k] = 1.0f / dk;
        r.idc[k] = 1.0f / (std::fabs(dk) < 1e-20f ? std::copysign(1e-20f, dk) : dk);
    }
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = 0;
    float m = ax;
    if (ay > m) { kz = 1; m = ay; }
    if (az > m) kz = 2;
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    float dkz = comp(d, kz);
    if (dkz < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = comp(d, kx) / dkz;
    r.Sy = comp(d, ky) / dkz;
    r.Sz = 1.0f / dkz;
    return r;
}
// Woop, Benthin, Wald 2013 watertight test (fp32, double fallback on zero edges)
static bool tri_hit(const Ray& r, const Tri& t, float tbest, uint32_t best_prim, float& to, float& uo, float& vo,
                    uint32_t prim_base = 0) {
    F3 A = sub(t.a, r.o), B = sub(t.b, r.o), C = sub(t.c, r.o);
    float Akx = comp(A, r.kx), Aky = comp(A, r.ky), Akz = comp(A, r.kz);
    float Bkx = comp(B, r.kx), Bky = comp(B, r.ky), Bkz = comp(B, r.kz);
    float Ckx = comp(C, r.kx), Cky = comp(C, r.ky), Ckz = comp(C, r.kz);
    float Ax = Akx - r.Sx * Akz, Ay = Aky - r.Sy * Akz;
    float Bx = Bkx - r.Sx * Bkz, By = Bky - r.Sy * Bkz;
    float Cx = Ckx - r.Sx * Ckz, Cy = Cky - r.Sy * Ckz;
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
    float T = U * Az + V * Bz + W * Cz;
    float rcp = 1.0f / det;
    float tt = T * rcp;
    if (!(tt > r.tmin)) return false;
    if (!(tt < tbest || (tt == tbest && prim_base + t.prim < best_prim))) return false;
    to = tt; uo = U * rcp; vo = V * rcp;
    return true;
}
static bool box_hit(const Ray& r, const BNode& n, float tbest) {
    float tn = r.tmin, tf = INFINITY;
    const float o[3] = {r.o.x, r.o.y, r.o.z};
    const float d[3] = {r.d.x, r.d.y, r.d.z};
    for (int k = 0; k < 3; ++k) {
        if (d[k] == 0.0f) {  // parallel to the slab: inside it (boundary included) or never
            if (o[k] < n.lo[k] || o[k] > n.hi[k]) return false;
            continue;
        }
        float t0 = (n.lo[k] - o[k]) * r.id[k], t1 = (n.hi[k] - o[k]) * r.id[k];
        if (t0 > t1) std::swap(t0, t1);
        tn = std::fmax(tn, t0);
        tf = std::fmin(tf, t1);
    }
    // relative pad on both ends: rounding of the slab products never culls a
    // box that holds a hit at t <= tbest (ties at tbest included)
    float hi = std::fmin(tf, tbest);
    return tn - std::fabs(tn) * 9.5e-7f <= hi + std::fabs(hi) * 9.5e-7f;
}
struct Counts { uint64_t nodes = 0, tris = 0; };
// returns index into S.tris (leaf order) or UINT32_MAX
static uint32_t bits_of(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
// Rays that are traced (the device traversal's rule): origin and direction
// finite, direction not zero (a zero direction is skipped as a miss,
// rt_gbuffer.hlsl:13-15) and tmin <= tmax; every other ray is a miss.
static bool finite_bits(float x) { return (bits_of(x) & 0x7f800000u) != 0x7f800000u; }
static bool ray_traceable(const Ray& r) {
    bool fin = finite_bits(r.o.x) && finite_bits(r.o.y) && finite_bits(r.o.z) && finite_bits(r.d.x) &&
               finite_bits(r.d.y) && finite_bits(r.d.z);
    return fin && !(r.d.x == 0.0f && r.d.y == 0.0f && r.d.z == 0.0f) && r.tmin <= r.tmax;
}
// Stochastic-opacity uniform of a ray: the bits of its origin and direction
// combined as gen_opacity_random_for does (hits/rt_gbuffer.hlsl:14-19), with
// the path's PCG32 word as the seed, hashed by SplitMix64's finaliser.
static float opacity_random(const Ray& r) {
    uint32_t h = bits_of(r.o.x) ^ bits_of(r.o.y) ^ bits_of(r.o.z) ^ bits_of(r.d.x) ^ bits_of(r.d.y) ^ bits_of(r.d.z);
    uint64_t z = mix64(((uint64_t)h << 32) | (uint64_t)r.oseed);
    return (float)(uint32_t)(z >> 40) * 5.96046448e-08f;
}
// The any-hit rule (rt_gbuffer_hit.hlsl:20-35): a candidate on a triangle of
// transparency tr is ignored when the ray's uniform is below tr.
static bool keep_hit(const Ray& r, float tr) { return tr == 0.0f || !(opacity_random(r) < tr); }

// Closest / any hit in one BVH.  `r` is the ray in the BVH's space, `rw` the
// world ray (opacity decisions); `prim_base` makes primitive ids global;
// `trm` (two-level scenes) gives the transparency per effective material,
// otherwise the triangle's own.  Updates the best hit; true when any-hit found one.
struct Best { float t; uint32_t leaf, prim, inst; float u, v; };
static bool trace_bvh(const Scene& G, const Ray& r, const Ray& rw, bool any, uint32_t prim_base, uint32_t mat_override,
                      const float* trm, uint32_t inst, Best& b, Counts* cnt) {
    uint32_t stack[128];
    int sp = 0;
    if (ray_traceable(rw)) stack[sp++] = 0;
    while (sp) {
        uint32_t ni = stack[--sp];
        const BNode& n = G.nodes[ni];
        if (cnt) cnt->nodes++;
        if (!box_hit(r, n, b.t)) continue;
        if (n.count) {
            for (uint32_t i = 0; i < n.count; ++i) {
                const Tri& t = G.tris[n.left_or_first + i];
                if (cnt) cnt->tris++;
                float tt, u, v;
                if (!tri_hit(r, t, b.t, b.prim, tt, u, v, prim_base)) continue;
                float tr = trm ? trm[mat_override != UINT32_MAX ? mat_override : t.mat] : t.tr;
                if (!keep_hit(rw, tr)) continue;
                b.t = tt; b.leaf = n.left_or_first + i; b.prim = prim_base + t.prim; b.inst = inst; b.u = u; b.v = v;
                if (any) return true;
            }
        } else {
            uint32_t l = ni + 1, rr = n.left_or_first;
            bool neg = comp(r.d, (int)n.axis) < 0.0f;
            // push the far child first
            if (neg) { stack[sp++] = l; stack[sp++] = rr; } else { stack[sp++] = rr; stack[sp++] = l; }
        }
    }
    return false;
}

// Row-major 3x4 transforms in the GPU's operation order.
static F3 xf_point(const float* m, F3 p) {
    return f3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
              ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}
static F3 xf_dir(const float* m, F3 d) {
    return f3((m[0] * d.x + m[1] * d.y) + m[2] * d.z, (m[4] * d.x + m[5] * d.y) + m[6] * d.z,
              (m[8] * d.x + m[9] * d.y) + m[10] * d.z);
}
static F3 xf_normal(const float* m, F3 n) {  // transpose of the linear part
    return f3((m[0] * n.x + m[4] * n.y) + m[8] * n.z, (m[1] * n.x + m[5] * n.y) + m[9] * n.z,
              (m[2] * n.x + m[6] * n.y) + m[10] * n.z);
}

// Closest / any hit of a world ray.  Two-level scenes test every instance (no
// TLAS: the checker does not depend on one) with the ray moved into the
// instance's space; ties resolve to the lower global primitive id.  Returns the
// leaf index (in the instance's geometry for two-level scenes), inst_out the instance.
static uint32_t trace(const Scene& S, const Ray& r, bool any, float& to, float& uo, float& vo, Counts* cnt,
                      uint32_t* inst_out = nullptr) {
    Best b{r.tmax, UINT32_MAX, UINT32_MAX, UINT32_MAX, 0.0f, 0.0f};
    if (S.inst.empty()) {
        trace_bvh(S, r, r, any, 0, UINT32_MAX, nullptr, UINT32_MAX, b, cnt);
    } else {
        for (uint32_t i = 0; i < S.inst.size(); ++i) {
            const Scene::Inst& I = S.inst[i];
            Ray ro = make_ray(xf_point(I.w2o, r.o), r.tmin, xf_dir(I.w2o, r.d), r.tmax, r.oseed);
            if (trace_bvh(*I.geo, ro, r, any, I.prim_base, I.material, S.trm.empty() ? nullptr : S.trm.data(), i, b,
                          cnt))
                break;
        }
    }
    to = b.t; uo = b.u; vo = b.v;
    if (inst_out) *inst_out = b.inst;
    return b.leaf;
}

// Geometric normal (world, unit, not faced), first edge (world) and material of a hit.
static void hit_geom(const Scene& S, uint32_t leaf, uint32_t inst, F3& ng, F3& edge, uint32_t& mat) {
    const Tri& T = inst == UINT32_MAX ? S.tris[leaf] : S.inst[inst].geo->tris[leaf];
    ng = norm3(cross3(sub(T.b, T.a), sub(T.c, T.a)));
    edge = sub(T.b, T.a);
    mat = T.mat;
    if (inst != UINT32_MAX) {
        const Scene::Inst& I = S.inst[inst];
        ng = norm3(xf_normal(I.w2o, ng));
        edge = xf_dir(I.o2w, edge);
        if (I.material != UINT32_MAX) mat = I.material;
    }
    if (mat >= S.nmat) mat = 0;
}

// Shading normal of a hit on a triangle with vertex normals (hit.hlsl:55-71, 158): n0 + (n1 - n0) b1 +
// (n2 - n0) b2 normalised, b1 = v and b2 = 1 - u - v the weights of the second and third vertex; a zero
// interpolated normal keeps ng.  Single-level scenes only (a two-level hit keeps its geometric normal).
static F3 shade_normal(const Scene& S, uint32_t leaf, uint32_t inst, float u, float v, F3 ng) {
    if (inst != UINT32_MAX) return ng;
    const Tri& T = S.tris[leaf];
    if (!T.has_n) return ng;
    float b1 = v, b2 = 1.0f - u - v;
    F3 n = add(add(T.na, muls(sub(T.nb, T.na), b1)), muls(sub(T.nc, T.na), b2));
    return dot3(n, n) > 0.0f ? norm3(n) : ng;
}

// ------------------------------------------------------------------ sky ----
static F3 texel(const Scene& S, uint32_t i, uint32_t j) {
    const uint16_t* t = &S.texels[((size_t)i * S.sw + j) * 4];
    return f3(half_to_float(t[0]) * S.sky_color.x, half_to_float(t[1]) * S.sky_color.y, half_to_float(t[2]) * S.sky_color.z);
}
static void dir_texel(const Scene& S, F3 d, uint32_t& i, uint32_t& j, float& st) {
    float rxz = std::sqrt(d.x * d.x + d.z * d.z);
    float theta = atan2_det(rxz, d.y);
    float phi = atan2_det(d.z, d.x);
    float v = theta * kInvPi;
    float u = phi * (0.5f * kInvPi) + 0.5f;
    int ii = (int)std::floor(v * (float)S.sh), jj = (int)std::floor(u * (float)S.sw);
    ii = std::min(std::max(ii, 0), (int)S.sh - 1);
    jj = std::min(std::max(jj, 0), (int)S.sw - 1);
    i = (uint32_t)ii; j = (uint32_t)jj; st = rxz;
}
static const float kTwoPiSq = 19.7392082f;
static F3 sky_eval(const Scene& S, F3 d) {
    if (S.sky_kind == 0) return S.sky_color;
    uint32_t i, j; float st;
    dir_texel(S, d, i, j, st);
    return texel(S, i, j);
}
static float sky_pdf(const Scene& S, F3 d) {
    if (S.sky_kind == 0) return 0.0795774683f;
    uint32_t i, j; float st;
    dir_texel(S, d, i, j, st);
    if (!(st > 0.0f)) return 0.0f;
    return S.ptab[(size_t)i * S.sw + j] / (kTwoPiSq * st);
}
// Equirect sky: the alias table picks a texel (u0: entry, u1: keep or alias and,
// rescaled, the row position in the texel; u2: the column position).
static F3 sky_sample(const Scene& S, float u0, float u1, float u2, float& pdf, F3& le) {
    if (S.sky_kind == 0) { pdf = 0.0795774683f; le = S.sky_color; return sphere_sample(u0, u1); }
    const uint32_t n = S.sw * S.sh;
    uint32_t k = (uint32_t)(u0 * (float)n);
    k = k < n ? k : n - 1u;
    float keep = S.aprob[k];
    uint32_t t;
    float fy;
    if (u1 < keep) { t = k; fy = u1 / keep; }
    else { t = S.alias[k]; fy = (u1 - keep) / (1.0f - keep); }
    fy = std::fmin(std::fmax(fy, 0.0f), 0.99999994f);
    float fx = u2;
    uint32_t i = t / S.sw, j = t - i * S.sw;
    float st, ct, sp, cp;
    sincos_turns(((float)i + fy) / (2.0f * (float)S.sh), &st, &ct);
    sincos_turns(((float)j + fx) / (float)S.sw - 0.5f, &sp, &cp);
    F3 d = f3(st * cp, ct, st * sp);
    float p = S.ptab[(size_t)i * S.sw + j];
    pdf = (st > 0.0f && p > 0.0f) ? p / (kTwoPiSq * st) : 0.0f;
    le = texel(S, i, j);
    return d;
}
// Texel weights (r + g + b) sin(theta), pdf table, and the alias table (Walker's
// method, Vose's construction: small entries, taken from the back, borrow the
// excess of the last large one).
static void build_sky(Scene& S) {
    const uint32_t W = S.sw, H = S.sh;
    const size_t N = (size_t)W * H;
    S.ptab.assign(N, 0.0f);
    std::vector<double> w((size_t)H * W), rows(H);
    double total = 0.0;
    for (uint32_t i = 0; i < H; ++i) {
        float st, ct;
        sincos_turns(((float)i + 0.5f) / (2.0f * (float)H), &st, &ct);
        double rs = 0.0;
        for (uint32_t j = 0; j < W; ++j) {
            const uint16_t* t = &S.texels[((size_t)i * W + j) * 4];
            float lum = half_to_float(t[0]) + half_to_float(t[1]) + half_to_float(t[2]);
            double x = lum > 0.0f ? (double)lum * (double)st : 0.0;
            w[(size_t)i * W + j] = x;
            rs += x;
        }
        rows[i] = rs;
        total += rs;
    }
    for (size_t k = 0; k < N; ++k)
        S.ptab[k] = total > 0.0 ? (float)(w[k] * (double)W * (double)H / total) : 0.0f;
    S.aprob.assign(N, 1.0f);
    S.alias.assign(N, 0u);
    std::vector<double> q(N);
    std::vector<uint32_t> small, large;
    for (size_t k = 0; k < N; ++k) {
        q[k] = total > 0.0 ? w[k] * (double)N / total : 1.0;
        (q[k] < 1.0 ? small : large).push_back((uint32_t)k);
        S.alias[k] = (uint32_t)k;
    }
    while (!small.empty() && !large.empty()) {
        uint32_t sm = small.back();
        small.pop_back();
        uint32_t lg = large.back();
        S.aprob[sm] = (float)q[sm];
        S.alias[sm] = lg;
        q[lg] = (q[lg] + q[sm]) - 1.0;
        if (q[lg] < 1.0) {
            large.pop_back();
            small.push_back(lg);
        }
    }
}

// --------------------------------------------------------- wavefront ----
struct Cam { F3 pos, s, u, f; float tan_half, aspect; uint32_t w, h; };
static Cam make_cam(const float* c) {  // pos3 front3 up3 fov w h
    Cam k;
    k.pos = f3(c[0], c[1], c[2]);
    k.f = norm3(f3(c[3], c[4], c[5]));
    k.s = norm3(cross3(k.f, f3(c[6], c[7], c[8])));
    k.u = cross3(k.s, k.f);
    k.w = (uint32_t)c[10];
    k.h = (uint32_t)c[11];
    k.tan_half = (float)std::tan((double)c[9] * 3.14159265358979323846 / 360.0);
    k.aspect = (float)k.w / (float)k.h;
    return k;
}

struct Settings {
    uint32_t spp, max_seg, sample_offset, flags;
    uint64_t seed;
    float ray_length, t_min;
    // radiance cache: hits of segment cache_seg or later whose roughness is at least cache_rough (or that
    // reach the last segment) end in a query of the network with weights cache_w (0 / null: no cache)
    uint32_t cache_seg = 0;
    float cache_rough = 0.0f;
    const float* cache_w = nullptr;
};

// The cache network's output for raw inputs `raw` (defined with the network below).
static void cache_predict(const float* W, const float* raw, float y[3]);

// Raw inputs of a cache query at a path vertex: position normalised to the scene box, outgoing direction and
// normal as (theta / pi, phi / 2pi + 1/2), roughness, albedo, depth = bounce / 8 (the kernels' mlp_raw_inputs).
static void cache_raw_inputs(const Scene& S, F3 p, F3 wo, F3 n, float rough, F3 albedo, float depth, float* raw) {
    raw[0] = (p.x - S.box_lo[0]) * S.box_inv[0];
    raw[1] = (p.y - S.box_lo[1]) * S.box_inv[1];
    raw[2] = (p.z - S.box_lo[2]) * S.box_inv[2];
    raw[3] = atan2_det(std::sqrt(wo.x * wo.x + wo.z * wo.z), wo.y) * kInvPi;
    raw[4] = atan2_det(wo.z, wo.x) * (0.5f * kInvPi) + 0.5f;
    raw[5] = atan2_det(std::sqrt(n.x * n.x + n.z * n.z), n.y) * kInvPi;
    raw[6] = atan2_det(n.z, n.x) * (0.5f * kInvPi) + 0.5f;
    raw[7] = rough;
    raw[8] = albedo.x; raw[9] = albedo.y; raw[10] = albedo.z;
    raw[11] = depth;
}
enum { F_JITTER = 1, F_NO_SUN = 2, F_NO_SKY = 4, F_FIXED = 64 };

// F_FIXED (the library's BSM_PT_DETERMINISTIC, pt_device.h accum_fixed_add and pt_kernels.cu k_fold_fixed):
// a contribution value x > 0 as a 32.32 fixed-point integer, x * 2^32 rounded to nearest even (saturating);
// the pixel's sum of these is exact, so it does not depend on the order of the additions.
static uint64_t fixed32(float x) {
    if (!(x > 0.0f)) return 0;
    const float y = x * 4294967296.0f;
    if (y >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)std::nearbyint((double)y);
}

struct PathQ {  // one wavefront queue in the oracle (structure of arrays)
    std::vector<F3> o, d, thr;
    std::vector<float> tmin, tmax, lpdf;
    std::vector<uint32_t> pix, seg;
    std::vector<Pcg> rng;
    void clear() { o.clear(); d.clear(); thr.clear(); tmin.clear(); tmax.clear(); lpdf.clear(); pix.clear(); seg.clear(); rng.clear(); }
    size_t size() const { return o.size(); }
    void push(F3 oo, float tn, F3 dd, float tx, F3 t, float lp, uint32_t p, uint32_t s, Pcg g) {
        o.push_back(oo); tmin.push_back(tn); d.push_back(dd); tmax.push_back(tx); thr.push_back(t); lpdf.push_back(lp);
        pix.push_back(p); seg.push_back(s); rng.push_back(g);
    }
};
struct ShadowQ {
    std::vector<F3> o, d, c;
    std::vector<float> tmin, tmax;
    std::vector<uint32_t> pix, seed;
    void clear() { o.clear(); d.clear(); c.clear(); tmin.clear(); tmax.clear(); pix.clear(); seed.clear(); }
};

// Next-event sample of a light from P (point_light_eval, lights.hlsl:15-25;
// rect lights sampled uniformly by area): direction, shadow-ray length and the
// radiance arriving along the direction (before the BSDF).
static bool light_sample(const Scene::Light& L, F3 P, float u0, float u1, float ray_len, F3& dir, float& tmax, F3& e) {
    if (L.kind == 0) { dir = L.a; e = L.b; tmax = ray_len; return true; }
    F3 lvec = L.kind == 1 ? sub(L.a, P) : sub(add(add(L.a, muls(L.c, u0)), muls(L.d, u1)), P);
    float d2 = dot3(lvec, lvec);
    if (!(d2 > 0.0f)) return false;
    float dist = std::sqrt(d2);
    dir = divs(lvec, dist);
    tmax = std::fmin(dist, ray_len);
    if (L.kind == 1) {
        float x = d2 * L.bw;
        float att = std::fmin(std::fmax(1.0f - x * x, 0.0f), 1.0f) / std::fmax(d2, 0.001f);
        if (L.cw > L.dx) {
            float ct = std::fmin(std::fmax(dot3(dir, L.c), L.dx), L.cw);
            att = att * ((ct - L.dx) / std::fmax(L.cw - L.dx, 0.001f));
        }
        e = muls(L.b, att);
        return att > 0.0f;
    }
    F3 n = norm3(cross3(L.c, L.d));
    float cl = dot3(dir, n);  // the rectangle emits towards -n
    if (L.bw != 0.0f) cl = std::fabs(cl);
    if (!(cl > 0.0f)) return false;
    e = muls(L.b, cl * L.cw / d2);
    return true;
}

// Renders pixels [pix_begin, pix_end) of one camera; `acc` receives RGB sums
// (3 floats per pixel, indexed from pix_begin), or `fx` their 32.32 fixed-point
// sums (F_FIXED).
static void render_tile(const Scene& S, const Cam& K, const Settings& st, uint32_t pix_begin, uint32_t pix_end,
                        float* acc, uint64_t* fx, uint64_t* ext_cnt, uint64_t* sh_cnt) {
    PathQ q, nq;
    ShadowQ sq;
    auto add_px = [&](uint32_t pix, F3 c) {
        const size_t k = 3 * (size_t)(pix - pix_begin);
        if (fx) { fx[k] += fixed32(c.x); fx[k + 1] += fixed32(c.y); fx[k + 2] += fixed32(c.z); }
        else { acc[k] += c.x; acc[k + 1] += c.y; acc[k + 2] += c.z; }
    };
    for (uint32_t s = 0; s < st.spp; ++s) {
        q.clear();
        // camera (generate_camera_ray.hlsl:9-15)
        for (uint32_t p = pix_begin; p < pix_end; ++p) {
            uint32_t px = p % K.w, py = p / K.w;
            Pcg g = pcg_seed(path_initstate(st.seed, st.sample_offset + s, p), (uint64_t)p);
            float jx = 0.5f, jy = 0.5f;
            if (st.flags & F_JITTER) { jx = pcg_uniform(g); jy = pcg_uniform(g); }
            float uvx = ((float)px + jx) / (float)K.w;
            float uvy = ((float)py + jy) / (float)K.h;
            float ndx = uvx * 2.0f - 1.0f, ndy = 1.0f - uvy * 2.0f;
            F3 dl = norm3(f3(ndx * K.aspect * K.tan_half, ndy * K.tan_half, -1.0f));
            F3 dw = norm3(add(add(muls(K.s, dl.x), muls(K.u, dl.y)), muls(neg(K.f), dl.z)));
            q.push(K.pos, st.t_min, dw, st.ray_length, f3(1, 1, 1), 0.0f, p, 0, g);
        }
        for (uint32_t seg = 0; seg < st.max_seg && q.size(); ++seg) {
            ext_cnt[seg] += q.size();
            nq.clear();
            sq.clear();
            for (size_t i = 0; i < q.size(); ++i) {
                // extend
                Ray r = make_ray(q.o[i], q.tmin[i], q.d[i], q.tmax[i], (uint32_t)q.rng[i].state);
                float t, u, v;
                uint32_t hinst;
                uint32_t hit = trace(S, r, false, t, u, v, nullptr, &hinst);
                F3 d = q.d[i], thr = q.thr[i];
                if (hit == UINT32_MAX) {  // deferred_lighting_secondary.hlsl:23-29
                    F3 le = sky_eval(S, d);
                    float w = 1.0f;
                    if (seg > 0 && !(st.flags & F_NO_SKY)) {
                        float pb = q.lpdf[i], pl = sky_pdf(S, d);
                        float pb2 = pb * pb, pl2 = pl * pl;
                        w = pb2 + pl2 > 0.0f ? pb2 / (pb2 + pl2) : 1.0f;
                    }
                    F3 c = muls(mul(thr, le), w);
                    if (maxc(c) > 0.0f) add_px(q.pix[i], c);
                    continue;
                }
                // shade
                F3 ng, edge;
                uint32_t mat;
                hit_geom(S, hit, hinst, ng, edge, mat);
                if (dot3(ng, d) > 0.0f) ng = neg(ng);
                F3 N = shade_normal(S, hit, hinst, u, v, ng);
                if (dot3(N, d) > 0.0f) N = neg(N);
                F3 P = add(q.o[i], muls(d, t));
                const float* m = &S.mats[8 * (size_t)mat];
                Surf surf{f3(m[0], m[1], m[2]), f3(m[4], m[5], m[6]), f3(1, 1, 1), m[3], 1.5f};
                if (st.cache_w && seg >= st.cache_seg && (surf.rough >= st.cache_rough || seg + 1 >= st.max_seg)) {
                    // a cache query ends the path: throughput x max(prediction, 0), no NEE, no continuation
                    float raw[12], y[3];
                    cache_raw_inputs(S, P, neg(d), N, surf.rough, surf.base, (float)seg * 0.125f, raw);
                    cache_predict(st.cache_w, raw, y);
                    F3 c = mul(thr, f3(std::fmax(y[0], 0.0f), std::fmax(y[1], 0.0f), std::fmax(y[2], 0.0f)));
                    add_px(q.pix[i], c);
                    continue;
                }
                Frm fr = make_frame(N);
                F3 V = neg(d);
                Pcg g = q.rng[i];
                float us0 = pcg_uniform(g), us1 = pcg_uniform(g), us2 = pcg_uniform(g), ul = pcg_uniform(g),
                      ub0 = pcg_uniform(g), ub1 = pcg_uniform(g);
                F3 org = add(P, muls(ng, S.offset));
                float rx, ry;
                aniso_rough(surf.rough, &rx, &ry);
                F3 lv = local_of(fr, V);
                float ps = spec_prob(surf, lv.z);
                for (uint32_t l = 0; l < S.nlights; ++l) {  // deferred_lighting_secondary.hlsl:51-96
                    const Scene::Light& Lt = S.lights[l];
                    float ur0 = 0.0f, ur1 = 0.0f;
                    if (Lt.kind == 2) { ur0 = pcg_uniform(g); ur1 = pcg_uniform(g); }  // after the vertex's six
                    if (st.flags & F_NO_SUN) continue;
                    F3 L, e;
                    float smax;
                    if (!light_sample(Lt, P, ur0, ur1, st.ray_length, L, smax, e)) continue;
                    F3 f = eval_lit(N, fr.x, fr.y, V, L, surf);
                    F3 c = mul(mul(thr, e), f);
                    if (maxc(c) > 0.0f) {
                        sq.o.push_back(org); sq.tmin.push_back(st.t_min); sq.d.push_back(L);
                        sq.tmax.push_back(smax); sq.c.push_back(c); sq.pix.push_back(q.pix[i]);
                        sq.seed.push_back((uint32_t)g.state);
                    }
                }
                if (!(st.flags & F_NO_SKY)) {
                    float pl;
                    F3 le;
                    F3 L = sky_sample(S, us0, us1, us2, pl, le);
                    if (pl > 0.0f) {
                        F3 f = eval_lit(N, fr.x, fr.y, V, L, surf);
                        if (maxc(f) > 0.0f) {
                            F3 ll = local_of(fr, L);
                            float pb = mix_pdf(lv, ll, rx, ry, ps);
                            float pl2 = pl * pl, pb2 = pb * pb;
                            float w = pl2 / (pl2 + pb2);
                            F3 c = muls(mul(mul(thr, le), f), w / pl);
                            if (maxc(c) > 0.0f) {
                                sq.o.push_back(org); sq.tmin.push_back(st.t_min); sq.d.push_back(L);
                                sq.tmax.push_back(st.ray_length); sq.c.push_back(c); sq.pix.push_back(q.pix[i]);
                                sq.seed.push_back((uint32_t)g.state);
                            }
                        }
                    }
                }
                // sample_secondary_ray.hlsl:16-28 (termination) and :51-64 (weight)
                if (seg + 1 < st.max_seg && maxc(thr) >= 0.001f) {
                    F3 ll;
                    if (ul < ps) ll = [&] { F3 h = ggx_vndf_sample(lv, rx, ry, ub0, ub1); return sub(neg(lv), muls(h, 2.0f * dot3(neg(lv), h))); }();
                    else ll = cos_hemi_sample(ub0, ub1);
                    if (ll.z > 0.0f) {
                        F3 L = world_of(fr, ll);
                        float pdf = mix_pdf(lv, ll, rx, ry, ps);
                        F3 f = eval_lit(N, fr.x, fr.y, V, L, surf);
                        F3 w = pdf > 0.0f ? divs(f, pdf) : f3(0, 0, 0);
                        if (!std::isfinite(w.x) || !std::isfinite(w.y) || !std::isfinite(w.z)) w = f3(0, 0, 0);
                        F3 nt = mul(thr, w);
                        if (maxc(nt) > 0.0f) nq.push(org, st.t_min, L, st.ray_length, nt, pdf, q.pix[i], seg + 1, g);
                    }
                }
            }
            // shadow (any hit)
            sh_cnt[seg] += sq.o.size();
            for (size_t k = 0; k < sq.o.size(); ++k) {
                Ray r = make_ray(sq.o[k], sq.tmin[k], sq.d[k], sq.tmax[k], sq.seed[k]);
                float t, u, v;
                if (trace(S, r, true, t, u, v, nullptr) == UINT32_MAX) add_px(sq.pix[k], sq.c[k]);
            }
            std::swap(q, nq);
        }
    }
}

static int nthreads(int req) {
    int hc = (int)std::thread::hardware_concurrency();
    return req > 0 ? req : (hc > 0 ? hc : 1);
}

}  // namespace orc

using namespace orc;

// Triangles and the binary BVH of a mesh (a scene's or a two-level geometry's).
static void build_geometry(Scene* S, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                           const uint32_t* mat_ids, const float* normals = nullptr) {
    std::vector<BuildRef> refs(nt);
    std::vector<Tri> soup(nt);
    for (uint32_t t = 0; t < nt; ++t) {
        uint32_t v[3];
        for (int c = 0; c < 3; ++c) v[c] = idx ? idx[3 * t + c] : 3 * t + c;
        Tri& T = soup[t];
        T.a = f3(pos[3 * v[0]], pos[3 * v[0] + 1], pos[3 * v[0] + 2]);
        T.b = f3(pos[3 * v[1]], pos[3 * v[1] + 1], pos[3 * v[1] + 2]);
        T.c = f3(pos[3 * v[2]], pos[3 * v[2] + 1], pos[3 * v[2] + 2]);
        T.prim = t;
        T.mat = mat_ids ? mat_ids[t] : 0;
        T.tr = 0.0f;
        T.has_n = normals ? 1u : 0u;
        if (normals) {
            T.na = f3(normals[3 * v[0]], normals[3 * v[0] + 1], normals[3 * v[0] + 2]);
            T.nb = f3(normals[3 * v[1]], normals[3 * v[1] + 1], normals[3 * v[1] + 2]);
            T.nc = f3(normals[3 * v[2]], normals[3 * v[2] + 1], normals[3 * v[2] + 2]);
        }
        BuildRef& R = refs[t];
        const F3 vs[3] = {T.a, T.b, T.c};
        for (int k = 0; k < 3; ++k) {
            R.lo[k] = std::min({comp(vs[0], k), comp(vs[1], k), comp(vs[2], k)});
            R.hi[k] = std::max({comp(vs[0], k), comp(vs[1], k), comp(vs[2], k)});
            R.c[k] = 0.5f * (R.lo[k] + R.hi[k]);
        }
        R.t = t;
    }
    (void)nv;
    S->nodes.reserve(2 * (size_t)nt);
    build_rec(*S, refs, 0, nt);
    S->tris.resize(nt);
    for (uint32_t i = 0; i < nt; ++i) S->tris[i] = soup[refs[i].t];
}

// Materials (7 floats each: base rgb, roughness, metallic, opacity, blend mode),
// lights, sky and the ray offset of a scene with bounds lo / hi.
// IEEE half of a float, round to nearest even.
static uint16_t float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u, exp = (x >> 23) & 0xffu, man = x & 0x7fffffu;
    if (exp == 0xffu) return (uint16_t)(sign | 0x7c00u | (man ? 0x200u : 0u));
    int e = (int)exp - 112;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        man |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - e), h = man >> shift;
        uint32_t rem = man & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)e << 10) | (man >> 13), rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

// A cubemap (faces +X -X +Y -Y +Z -Z of size S) resampled to a 4S x 2S equirect
// map: texel-centre direction, the sky rotation, the standard cube face table,
// bilinear inside the face.
static void cube_to_equirect(const uint16_t* faces, uint32_t S, const float* xf, std::vector<uint16_t>& out) {
    const uint32_t W = 4 * S, H = 2 * S;
    out.assign((size_t)W * H * 4, 0);
    double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    bool any = false;
    for (int k = 0; k < 9; ++k) any = any || xf[k] != 0.0f;
    if (any)
        for (int k = 0; k < 9; ++k) R[k] = xf[k];
    const double pi = 3.14159265358979323846;
    for (uint32_t i = 0; i < H; ++i) {
        double th = pi * (i + 0.5) / H;
        for (uint32_t j = 0; j < W; ++j) {
            double ph = 2.0 * pi * ((j + 0.5) / W - 0.5);
            double d0[3] = {std::sin(th) * std::cos(ph), std::cos(th), std::sin(th) * std::sin(ph)};
            double d[3];
            for (int k = 0; k < 3; ++k) d[k] = R[3 * k] * d0[0] + R[3 * k + 1] * d0[1] + R[3 * k + 2] * d0[2];
            double ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
            int face;
            double sc, tc, ma;
            if (ax >= ay && ax >= az) { face = d[0] > 0 ? 0 : 1; ma = ax; sc = d[0] > 0 ? -d[2] : d[2]; tc = -d[1]; }
            else if (ay >= az) { face = d[1] > 0 ? 2 : 3; ma = ay; sc = d[0]; tc = d[1] > 0 ? d[2] : -d[2]; }
            else { face = d[2] > 0 ? 4 : 5; ma = az; sc = d[2] > 0 ? d[0] : -d[0]; tc = -d[1]; }
            double x = ((sc / ma + 1.0) * 0.5) * S - 0.5, y = ((tc / ma + 1.0) * 0.5) * S - 0.5;
            x = std::min(std::max(x, 0.0), (double)S - 1);
            y = std::min(std::max(y, 0.0), (double)S - 1);
            uint32_t x0 = (uint32_t)x, y0 = (uint32_t)y;
            uint32_t x1 = std::min(x0 + 1, S - 1), y1 = std::min(y0 + 1, S - 1);
            double fx = x - x0, fy = y - y0;
            const uint16_t* F = faces + (size_t)face * S * S * 4;
            for (int c = 0; c < 4; ++c) {
                auto at = [&](uint32_t xx, uint32_t yy) { return (double)half_to_float(F[((size_t)yy * S + xx) * 4 + c]); };
                double v = (at(x0, y0) * (1 - fx) + at(x1, y0) * fx) * (1 - fy) + (at(x0, y1) * (1 - fx) + at(x1, y1) * fx) * fy;
                out[((size_t)i * W + j) * 4 + c] = float_to_half((float)v);
            }
        }
    }
}

// Lights: 16 floats each, the first the kind.  0: direction, emission;
// 1: position, emission, range, direction to the light, cos_inner, cos_outer;
// 2: centre, axis x, axis y, width, height, emission, two_sided.
static bool setup_shading(Scene* S, const float* materials, uint32_t nm, const float* lights, uint32_t nl,
                          uint32_t sky_kind, const float* sky_color, uint32_t sky_w, uint32_t sky_h,
                          const uint16_t* sky_texels, const float* sky_xf, const float lo[3], const float hi[3]) {
    S->extent = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), std::max(hi[2] - lo[2], 1e-6f));
    S->offset = 2e-5f * S->extent;
    for (int k = 0; k < 3; ++k) {
        S->box_lo[k] = lo[k];
        S->box_inv[k] = 1.0f / std::max(hi[k] - lo[k], 1e-6f);
    }
    S->nmat = nm;
    S->mats.resize(8 * (size_t)nm);
    S->trm.assign(nm, 0.0f);
    for (uint32_t m = 0; m < nm; ++m) {
        const float* M = materials + 7 * (size_t)m;
        if (M[6] == 1.0f) S->trm[m] = M[5] < 0.01f ? 1.0f : 0.0f;   // ALPHA_TEST_OPACITY_THRESHOLD (utils.hlsl:38)
        if (M[6] == 2.0f) S->trm[m] = 1.0f - M[5];
        float* o = &S->mats[8 * (size_t)m];
        o[0] = M[0]; o[1] = M[1]; o[2] = M[2]; o[3] = M[3];
        for (int k = 0; k < 3; ++k) o[4 + k] = 0.04f + (M[k] - 0.04f) * M[4];  // lerp(0.04, base, metallic)
        o[7] = M[4];
    }
    if (nl > 8) return false;
    S->nlights = nl;
    for (uint32_t l = 0; l < nl; ++l) {
        const float* r = lights + 16 * (size_t)l;
        Scene::Light& L = S->lights[l];
        L = Scene::Light{};
        L.kind = (uint32_t)r[0];
        if (L.kind == 0) {
            L.a = norm3(f3(r[1], r[2], r[3]));
            L.b = f3(r[4], r[5], r[6]);
        } else if (L.kind == 1) {
            L.a = f3(r[1], r[2], r[3]);
            L.b = f3(r[4], r[5], r[6]);
            L.bw = 1.0f / (r[7] * r[7]);
            L.cw = r[11];
            L.dx = r[12];
            L.c = L.cw > L.dx ? norm3(f3(r[8], r[9], r[10])) : f3(0.0f, 0.0f, 1.0f);
        } else {
            F3 c = f3(r[1], r[2], r[3]), ax = f3(r[4], r[5], r[6]), ay = f3(r[7], r[8], r[9]);
            float w = r[10], h = r[11];
            L.a = sub(sub(c, muls(ax, 0.5f * w)), muls(ay, 0.5f * h));
            L.b = f3(r[12], r[13], r[14]);
            L.bw = r[15] != 0.0f ? 1.0f : 0.0f;
            L.c = muls(ax, w);
            L.d = muls(ay, h);
            L.cw = w * h;
        }
    }
    S->sky_kind = sky_kind == 2 ? 1 : sky_kind;
    S->sky_color = f3(sky_color[0], sky_color[1], sky_color[2]);
    if (sky_kind == 1 || sky_kind == 2) {
        if (!sky_texels || !sky_w || !sky_h) return false;
        if (sky_kind == 2) {  // cubemap: resampled to the equirect layout, as the library does on upload
            cube_to_equirect(sky_texels, sky_w, sky_xf, S->texels);
            S->sw = 4 * sky_w; S->sh = 2 * sky_w;
        } else {
            S->sw = sky_w; S->sh = sky_h;
            S->texels.assign(sky_texels, sky_texels + (size_t)sky_w * sky_h * 4);
        }
        build_sky(*S);
    }
    return true;
}

ORC_API int orc_scene_create(const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt, const uint32_t* mat_ids,
                             const float* materials, uint32_t nm, const float* lights, uint32_t nl, uint32_t sky_kind,
                             const float* sky_color, uint32_t sky_w, uint32_t sky_h, const uint16_t* sky_texels,
                             const float* sky_xf, const float* normals, void** out) {
    if (!pos || !nt || !materials || !nm || !out || nl > 8) return -1;
    Scene* S = new Scene();
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < nv; ++i)
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], pos[3 * i + k]); hi[k] = std::max(hi[k], pos[3 * i + k]); }
    build_geometry(S, pos, nv, idx, nt, mat_ids, normals);
    if (!setup_shading(S, materials, nm, lights, nl, sky_kind, sky_color, sky_w, sky_h, sky_texels, sky_xf, lo, hi)) {
        delete S;
        return -1;
    }
    for (Tri& T : S->tris) T.tr = T.mat < nm ? S->trm[T.mat] : 0.0f;
    S->trm.clear();  // single-level: the triangles carry their transparency
    *out = S;
    return 0;
}

// A geometry of two-level scenes: triangles and BVH in object space.
ORC_API int orc_geometry_create(const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                                const uint32_t* mat_ids, void** out) {
    if (!pos || !nt || !out) return -1;
    Scene* G = new Scene();
    for (int k = 0; k < 3; ++k) { G->glo[k] = INFINITY; G->ghi[k] = -INFINITY; }
    for (uint32_t i = 0; i < nv; ++i)
        for (int k = 0; k < 3; ++k) {
            G->glo[k] = std::min(G->glo[k], pos[3 * i + k]);
            G->ghi[k] = std::max(G->ghi[k], pos[3 * i + k]);
        }
    build_geometry(G, pos, nv, idx, nt, mat_ids);
    *out = G;
    return 0;
}

// World-to-object transform: the inverse of the row-major 3x4 object-to-world
// transform in double (cofactors, first-row determinant), rounded to float.
static bool invert_affine(const float* m, float* inv) {
    double L00 = m[0], L01 = m[1], L02 = m[2], t0 = m[3];
    double L10 = m[4], L11 = m[5], L12 = m[6], t1 = m[7];
    double L20 = m[8], L21 = m[9], L22 = m[10], t2 = m[11];
    double c00 = L11 * L22 - L12 * L21, c01 = L02 * L21 - L01 * L22, c02 = L01 * L12 - L02 * L11;
    double c10 = L12 * L20 - L10 * L22, c11 = L00 * L22 - L02 * L20, c12 = L02 * L10 - L00 * L12;
    double c20 = L10 * L21 - L11 * L20, c21 = L01 * L20 - L00 * L21, c22 = L00 * L11 - L01 * L10;
    double det = L00 * c00 + L01 * c10 + L02 * c20;
    if (!std::isfinite(det) || !(std::fabs(det) > 1e-30)) return false;
    double r[9] = {c00 / det, c01 / det, c02 / det, c10 / det, c11 / det, c12 / det, c20 / det, c21 / det, c22 / det};
    for (int i = 0; i < 3; ++i) {
        inv[4 * i] = (float)r[3 * i];
        inv[4 * i + 1] = (float)r[3 * i + 1];
        inv[4 * i + 2] = (float)r[3 * i + 2];
        inv[4 * i + 3] = (float)(-(r[3 * i] * t0 + r[3 * i + 1] * t1 + r[3 * i + 2] * t2));
    }
    return true;
}

// An instance's world box: the transformed corners of the geometry's box in
// double, padded by 1e-5 of the coordinates' magnitude, rounded outward (the
// scene bounds, hence the ray offset, come from these boxes).
static void instance_world_box(const float* m, const float glo[3], const float ghi[3], float lo[3], float hi[3]) {
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
        double p[3] = {(c & 1) ? ghi[0] : glo[0], (c & 2) ? ghi[1] : glo[1], (c & 4) ? ghi[2] : glo[2]};
        for (int k = 0; k < 3; ++k) {
            double w = (double)m[4 * k] * p[0] + (double)m[4 * k + 1] * p[1] + (double)m[4 * k + 2] * p[2] +
                       (double)m[4 * k + 3];
            mn[k] = std::min(mn[k], w);
            mx[k] = std::max(mx[k], w);
        }
    }
    double mag = 0.0;
    for (int k = 0; k < 3; ++k) mag = std::max(mag, std::max(std::fabs(mn[k]), std::fabs(mx[k])));
    double pad = 1e-5 * mag + 1e-30;
    for (int k = 0; k < 3; ++k) {
        float l = (float)(mn[k] - pad), h = (float)(mx[k] + pad);
        while ((double)l > mn[k] - pad) l = std::nextafter(l, -INFINITY);
        while ((double)h < mx[k] + pad) h = std::nextafter(h, INFINITY);
        lo[k] = l;
        hi[k] = h;
    }
}

// A two-level scene over geometries: instance i uses geometry inst_geo[i],
// material inst_mat[i] (UINT32_MAX: the geometry's ids) and the object-to-world
// transform inst_xf[12 i .. 12 i + 11].
ORC_API int orc_scene_create_instanced(void* const* geoms, uint32_t ng, const uint32_t* inst_geo,
                                       const uint32_t* inst_mat, const float* inst_xf, uint32_t ni,
                                       const float* materials, uint32_t nm, const float* lights, uint32_t nl,
                                       uint32_t sky_kind, const float* sky_color, uint32_t sky_w, uint32_t sky_h,
                                       const uint16_t* sky_texels, const float* sky_xf, void** out) {
    if (!geoms || !ni || !materials || !nm || !out || nl > 8) return -1;
    Scene* S = new Scene();
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t prim_base = 0;
    for (uint32_t i = 0; i < ni; ++i) {
        if (inst_geo[i] >= ng) { delete S; return -1; }
        const Scene* G = (const Scene*)geoms[inst_geo[i]];
        Scene::Inst I;
        I.geo = G;
        I.material = inst_mat[i];
        std::memcpy(I.o2w, inst_xf + 12 * (size_t)i, sizeof(I.o2w));
        if (!invert_affine(I.o2w, I.w2o)) { delete S; return -1; }
        I.prim_base = prim_base;
        prim_base += (uint32_t)G->tris.size();
        float bl[3], bh[3];
        instance_world_box(I.o2w, G->glo, G->ghi, bl, bh);
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], bl[k]); hi[k] = std::max(hi[k], bh[k]); }
        S->inst.push_back(I);
    }
    if (!setup_shading(S, materials, nm, lights, nl, sky_kind, sky_color, sky_w, sky_h, sky_texels, sky_xf, lo, hi)) {
        delete S;
        return -1;
    }
    bool any = false;
    for (float t : S->trm) any = any || t != 0.0f;
    if (!any) S->trm.clear();
    *out = S;
    return 0;
}

ORC_API void orc_scene_destroy(void* s) { delete (Scene*)s; }

// rays: n x 8 floats; hits: n x 4 u32 (t bits, prim, u bits, v bits)
ORC_API int orc_trace(void* sp, const float* rays, uint32_t n, uint32_t* hits, int any, int threads,
                      uint32_t* counts) {
    const Scene& S = *(Scene*)sp;
    int nt = nthreads(threads);
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        while (true) {
            uint32_t b = next.fetch_add(4096);
            if (b >= n) break;
            uint32_t e = std::min(n, b + 4096);
            for (uint32_t i = b; i < e; ++i) {
                const float* R = rays + 8 * (size_t)i;
                Ray r = make_ray(f3(R[0], R[1], R[2]), R[3], f3(R[4], R[5], R[6]), R[7]);
                float t, u, v;
                Counts c;
                uint32_t hi;
                uint32_t h = trace(S, r, any != 0, t, u, v, counts ? &c : nullptr, &hi);
                uint32_t* H = hits + 4 * (size_t)i;
                std::memcpy(&H[0], &t, 4);
                H[1] = h == UINT32_MAX ? UINT32_MAX
                                       : (hi == UINT32_MAX ? S.tris[h].prim : S.inst[hi].prim_base + S.inst[hi].geo->tris[h].prim);
                std::memcpy(&H[2], &u, 4);
                std::memcpy(&H[3], &v, 4);
                if (counts) { counts[2 * (size_t)i] = (uint32_t)c.nodes; counts[2 * (size_t)i + 1] = (uint32_t)c.tris; }
            }
        }
    };
    std::vector<std::thread> ts;
    for (int k = 1; k < nt; ++k) ts.emplace_back(work);
    work();
    for (auto& t : ts) t.join();
    return 0;
}

// camera: pos3 front3 up3 fov w h (12 floats); settings: spp, max_seg, sample_offset, flags (u32),
// seed (u64), ray_length, t_min.  Renders rows [row_begin, row_end); out = w x (rows) x 4 mean RGBA.
// stats: [16] extend rays per segment, [16] shadow rays per segment.
static int render_rows(void* sp, const float* camera, const Settings& st, uint32_t row_begin, uint32_t row_end,
                       float* out, uint64_t* stats, int threads, double* seconds);

ORC_API int orc_render(void* sp, const float* camera, uint32_t spp, uint32_t max_seg, uint32_t sample_offset,
                       uint32_t flags, uint64_t seed, float ray_length, float t_min, uint32_t row_begin,
                       uint32_t row_end, float* out, uint64_t* stats, int threads, double* seconds) {
    Settings st{spp, max_seg, sample_offset, flags, seed, ray_length, t_min};
    return render_rows(sp, camera, st, row_begin, row_end, out, stats, threads, seconds);
}

// The cached pass (bsm_render_cached without its training step): paths end in a query of the network with
// weights W (kMlpParams floats, rounded to bfloat16 as the kernels' copies are) at segment cache_seg.
ORC_API int orc_render_cached(void* sp, const float* camera, uint32_t spp, uint32_t max_seg, uint32_t flags,
                              uint64_t seed, float ray_length, float t_min, const float* W, uint32_t cache_seg,
                              float cache_rough, uint32_t row_begin, uint32_t row_end, float* out, uint64_t* stats,
                              int threads) {
    if (!W || cache_seg == 0 || cache_seg >= max_seg) return -1;
    Settings st{spp, max_seg, 0, flags, seed, ray_length, t_min};
    st.cache_seg = cache_seg;
    st.cache_rough = cache_rough;
    st.cache_w = W;
    return render_rows(sp, camera, st, row_begin, row_end, out, stats, threads, nullptr);
}

static int render_rows(void* sp, const float* camera, const Settings& st, uint32_t row_begin, uint32_t row_end,
                       float* out, uint64_t* stats, int threads, double* seconds) {
    const Scene& S = *(Scene*)sp;
    Cam K = make_cam(camera);
    const uint32_t spp = st.spp, max_seg = st.max_seg;
    if (row_end > K.h || row_begin >= row_end || max_seg == 0 || max_seg > 16 || spp == 0) return -1;
    uint32_t p0 = row_begin * K.w, p1 = row_end * K.w;
    const bool fixed = (st.flags & F_FIXED) != 0;
    std::vector<float> acc(fixed ? 0 : 3 * (size_t)(p1 - p0), 0.0f);
    std::vector<uint64_t> fxs(fixed ? 3 * (size_t)(p1 - p0) : 0, 0);
    const uint32_t tile = 256;  // 16 x 16 pixels worth of paths per task
    uint32_t ntiles = (p1 - p0 + tile - 1) / tile;
    std::atomic<uint32_t> next{0};
    int nt = nthreads(threads);
    std::vector<std::vector<uint64_t>> ext(nt, std::vector<uint64_t>(16, 0)), sh(nt, std::vector<uint64_t>(16, 0));
    auto t0 = std::chrono::steady_clock::now();
    auto work = [&](int id) {
        while (true) {
            uint32_t k = next.fetch_add(1);
            if (k >= ntiles) break;
            uint32_t b = p0 + k * tile, e = std::min(p1, b + tile);
            render_tile(S, K, st, b, e, fixed ? nullptr : acc.data() + 3 * (size_t)(b - p0),
                        fixed ? fxs.data() + 3 * (size_t)(b - p0) : nullptr, ext[id].data(), sh[id].data());
        }
    };
    std::vector<std::thread> ts;
    for (int k = 1; k < nt; ++k) ts.emplace_back(work, k);
    work(0);
    for (auto& t : ts) t.join();
    double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (seconds) *seconds = sec;
    float inv = 1.0f / (float)spp;
    for (size_t p = 0; p < (size_t)(p1 - p0); ++p) {
        for (int c = 0; c < 3; ++c) {
            // F_FIXED: the sum to FP32 as the library folds it (double, then float), then the mean
            const float sum = fixed ? (float)((double)fxs[3 * p + c] * 0x1p-32) : acc[3 * p + c];
            out[4 * p + c] = sum * inv;
        }
        out[4 * p + 3] = 1.0f;
    }
    if (stats) {
        for (int s = 0; s < 32; ++s) stats[s] = 0;
        for (int k = 0; k < nt; ++k)
            for (int s = 0; s < 16; ++s) { stats[s] += ext[k][s]; stats[16 + s] += sh[k][s]; }
    }
    return 0;
}

// ---- primary-hit outputs: G-buffer packing and reverse-Z depth ----
// pack.hlsl:6-8: 32 bits as two 16-bit fractions of 65536.
static void unorm16x2(uint32_t x, float* o) {
    o[0] = (float)(x & 0xffffu) / 65536.0f;
    o[1] = (float)(x >> 16) / 65536.0f;
}
// pack.hlsl:14-16: 11/11/10 bits, truncated.
static uint32_t rg11b10(F3 c) {
    return (uint32_t)(c.x * 2047.0f) | ((uint32_t)(c.y * 2047.0f) << 11) | ((uint32_t)(c.z * 1023.0f) << 22);
}
// pack.hlsl:83-93: octahedral encoding (L1-normalise, fold the lower half).
static void octahedral(F3 n, float* o) {
    float l1 = std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z);
    n = divs(n, l1);
    if (n.z >= 0.0f) {
        o[0] = n.x;
        o[1] = n.y;
    } else {
        o[0] = (1.0f - std::fabs(n.y)) * (n.x >= 0.0f ? 1.0f : -1.0f);
        o[1] = (1.0f - std::fabs(n.x)) * (n.y >= 0.0f ? 1.0f : -1.0f);
    }
}
// renderer/gbuffer.hlsl:18-31 (lit model, f90 = 1, anisotropy 0, ior 1.5) with
// pack_normal_and_tangent (pack.hlsl:113-121).  g: 4 x float4.
static void gbuffer_pack(F3 N, F3 T, F3 base, F3 f0, float rough, float* g) {
    g[0] = base.x; g[1] = base.y; g[2] = base.z; g[3] = 1.0f;
    float oc[2];
    octahedral(N, oc);
    Frm fr = make_frame(N);
    float px = dot3(T, fr.x), py = dot3(T, fr.y);
    float l1 = std::fabs(px) + std::fabs(py);
    px = px / l1;
    py = py / l1;
    float qx = px * 0.5f + 0.5f;
    g[4] = oc[0]; g[5] = oc[1]; g[6] = py < 0.0f ? -qx : qx; g[7] = rough;
    unorm16x2(rg11b10(f0), g + 8);
    unorm16x2(rg11b10(f3(1.0f, 1.0f, 1.0f)), g + 10);
    g[12] = 0.0f; g[13] = 1.0f / 1.5f; g[14] = 0.0f; g[15] = 1.0f / 256.0f;
}
// pt_depth.hlsl:13-15 with perspective_reverse_z (math.cpp:5-11): clip z / w.
static float rz_depth(F3 eye, F3 f, F3 P, float near_z, float far_z) {
    float inv = 1.0f / (far_z - near_z);
    float m22 = near_z * inv;
    float m32 = near_z * far_z * inv;
    float zv = -dot3(f, sub(P, eye));
    return (m22 * zv + m32) / -zv;
}

// One pixel-centre ray per pixel (generate_camera_ray.hlsl:9-15) and its closest
// hit (rt_gbuffer.hlsl:17-35): depth (w*h), G-buffer planes gb (4 x w*h float4,
// plane-major), hit positions (w*h float4; (direction, -1) on a miss).
ORC_API int orc_primary(void* sp, const float* camera, float ray_length, float t_min, float near_z, float far_z,
                        uint64_t seed, uint32_t sample_offset, float* depth, float* gb, float* hitpos, int threads) {
    const Scene& S = *(Scene*)sp;
    Cam K = make_cam(camera);
    const uint32_t npix = K.w * K.h;
    int nt = nthreads(threads);
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        while (true) {
            uint32_t b = next.fetch_add(1024);
            if (b >= npix) break;
            uint32_t e = std::min(npix, b + 1024);
            for (uint32_t p = b; p < e; ++p) {
                uint32_t px = p % K.w, py = p / K.w;
                float uvx = ((float)px + 0.5f) / (float)K.w;
                float uvy = ((float)py + 0.5f) / (float)K.h;
                float ndx = uvx * 2.0f - 1.0f, ndy = 1.0f - uvy * 2.0f;
                F3 dl = norm3(f3(ndx * K.aspect * K.tan_half, ndy * K.tan_half, -1.0f));
                F3 dw = norm3(add(add(muls(K.s, dl.x), muls(K.u, dl.y)), muls(neg(K.f), dl.z)));
                // opacity decisions of sample 0 of an unjittered render
                Pcg pg = pcg_seed(path_initstate(seed, sample_offset, p), (uint64_t)p);
                Ray r = make_ray(K.pos, t_min, dw, ray_length, (uint32_t)pg.state);
                float t, u, v;
                uint32_t hi;
                uint32_t h = trace(S, r, false, t, u, v, nullptr, &hi);
                float g[16] = {0};
                float z = 0.0f, hp[4] = {dw.x, dw.y, dw.z, -1.0f};
                if (h != UINT32_MAX) {
                    F3 ng, edge;
                    uint32_t mi;
                    hit_geom(S, h, hi, ng, edge, mi);
                    if (dot3(ng, dw) > 0.0f) ng = neg(ng);
                    ng = shade_normal(S, h, hi, u, v, ng);
                    if (dot3(ng, dw) > 0.0f) ng = neg(ng);
                    F3 tan = norm3(edge);
                    const float* m = S.mats.data() + 8 * (size_t)mi;
                    gbuffer_pack(ng, tan, f3(m[0], m[1], m[2]), f3(m[4], m[5], m[6]), m[3], g);
                    F3 P = add(K.pos, muls(dw, t));
                    z = rz_depth(K.pos, K.f, P, near_z, far_z);
                    hp[0] = P.x; hp[1] = P.y; hp[2] = P.z; hp[3] = t;
                }
                if (depth) depth[p] = z;
                if (gb)
                    for (int k = 0; k < 4; ++k) std::memcpy(gb + 4 * ((size_t)k * npix + p), g + 4 * k, 16);
                if (hitpos) std::memcpy(hitpos + 4 * (size_t)p, hp, 16);
            }
        }
    };
    std::vector<std::thread> ts;
    for (int k = 1; k < nt; ++k) ts.emplace_back(work);
    work();
    for (auto& t : ts) t.join();
    return 0;
}

// Building blocks exposed for the unit tests (known-answer checks).
ORC_API void orc_pcg32(uint64_t initstate, uint64_t initseq, uint32_t n, uint32_t* out) {
    Pcg g = pcg_seed(initstate, initseq);
    for (uint32_t i = 0; i < n; ++i) out[i] = pcg_next(g);
}
ORC_API void orc_sincos_turns(const float* t, uint32_t n, float* s, float* c) {
    for (uint32_t i = 0; i < n; ++i) sincos_turns(t[i], &s[i], &c[i]);
}
ORC_API void orc_atan2(const float* y, const float* x, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = atan2_det(y[i], x[i]);
}
// in: N3 V3 L3 base3 f0_3 roughness (16 floats); out: diffuse+specular (3)
ORC_API void orc_eval_lit(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 16 * (size_t)i;
        F3 N = f3(a[0], a[1], a[2]), V = f3(a[3], a[4], a[5]), L = f3(a[6], a[7], a[8]);
        Surf s{f3(a[9], a[10], a[11]), f3(a[12], a[13], a[14]), f3(1, 1, 1), a[15], 1.5f};
        Frm fr = make_frame(N);
        F3 r = eval_lit(N, fr.x, fr.y, V, L, s);
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
}
// in: V3 (local) rx ry u0 u1 (7 floats); out: h (3) and pdf of h (1)
ORC_API void orc_vndf(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 7 * (size_t)i;
        F3 v = f3(a[0], a[1], a[2]);
        F3 h = ggx_vndf_sample(v, a[3], a[4], a[5], a[6]);
        out[4 * i] = h.x; out[4 * i + 1] = h.y; out[4 * i + 2] = h.z;
        out[4 * i + 3] = ggx_vndf_pdf(h, v, a[3], a[4]);
    }
}
// in: N3; out: frame x3 y3
ORC_API void orc_frame(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        Frm f = make_frame(f3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
        float* o = out + 6 * (size_t)i;
        o[0] = f.x.x; o[1] = f.x.y; o[2] = f.x.z; o[3] = f.y.x; o[4] = f.y.y; o[5] = f.y.z;
    }
}
// in: V3 N3 T3 base3 f0_3 roughness (16 floats); out: the packed G-buffer (16 floats).
// V is unused, as in pack_surface_to_gbuffer.
ORC_API void orc_gbuffer_pack(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) {
        const float* a = in + 16 * (size_t)i;
        gbuffer_pack(f3(a[3], a[4], a[5]), f3(a[6], a[7], a[8]), f3(a[9], a[10], a[11]), f3(a[12], a[13], a[14]),
                     a[15], out + 16 * (size_t)i);
    }
}
// Sky samples for the unit tests: u (n x 3 uniforms) -> direction, pdf, and the
// pdf the sky reports for that direction (n x 5).
ORC_API void orc_sky_sample(void* sp, const float* u, uint32_t n, float* out) {
    const Scene& S = *(const Scene*)sp;
    for (uint32_t i = 0; i < n; ++i) {
        float pdf;
        F3 le;
        F3 d = sky_sample(S, u[3 * i], u[3 * i + 1], u[3 * i + 2], pdf, le);
        float* o = out + 5 * (size_t)i;
        o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = pdf; o[4] = sky_pdf(S, d);
    }
}

ORC_API uint32_t orc_scene_bvh_nodes(void* sp) { return (uint32_t)((Scene*)sp)->nodes.size(); }

// The next-event sample of one light (a 16-float row as the scene takes it) from n points P (3 floats each),
// with the uniforms (u0, u1) of rect lights: out 8 floats per point = arriving radiance (3), direction to the
// light (3), shadow-ray length, 1 when the light reaches P.  The render's own light_sample.
ORC_API int orc_light_eval(const float* row, const float* P, const float* u, uint32_t n, float ray_len, float* out) {
    Scene S;
    const float mat[7] = {0.5f, 0.5f, 0.5f, 0.5f, 0.0f, 1.0f, 0.0f};
    const float col[3] = {0.0f, 0.0f, 0.0f}, lo[3] = {0.0f, 0.0f, 0.0f}, hi[3] = {1.0f, 1.0f, 1.0f};
    if (!setup_shading(&S, mat, 1, row, 1, 0, col, 0, 0, nullptr, nullptr, lo, hi)) return 1;
    for (uint32_t i = 0; i < n; ++i) {
        F3 dir{0, 0, 0}, e{0, 0, 0};
        float tmax = 0.0f;
        bool lit = light_sample(S.lights[0], f3(P[3 * i], P[3 * i + 1], P[3 * i + 2]), u ? u[2 * i] : 0.0f,
                                u ? u[2 * i + 1] : 0.0f, ray_len, dir, tmax, e);
        float* o = out + 8 * (size_t)i;
        o[0] = e.x; o[1] = e.y; o[2] = e.z; o[3] = dir.x; o[4] = dir.y; o[5] = dir.z; o[6] = tmax;
        o[7] = lit ? 1.0f : 0.0f;
    }
    return 0;
}

// ============================================ compressed-BVH traversal ====
// Restatement of the product's single-ray traversal of its compressed 8-wide
// BVH, used to count the nodes visited and triangles tested per ray on the
// product's own tree (the traversal-bytes figure: 80 B per node, 48 B per
// triangle) and to check that the quantised boxes never cull a hit.  Layout
// of one 80-byte node: frame origin p (3 x f32), biased exponents e (3 x u8),
// internal-child mask, child_base, tri_base, a 16-bit triangle mask (bits
// 2s and 2s + 1: leaf slot s holds a first / a second triangle, triangles
// stored from tri_base in slot order) and 6 pad bytes, then the low planes
// x/y/z and the high planes x/y/z, 8 bytes each.  A triangle is 48 bytes:
// v0, prim, v1, material, v2, transparency bits.
//
// Arithmetic, in this order, as the device kernel evaluates it: per axis the
// slab scale s = 2^(e-127) / d and offset a = (p - o) / d - 2^23 s (a component
// d below 1e-20 in magnitude taken as +-1e-20, as the device does); the plane
// of byte q is at fma(2^23 + q, s, a) (near) or fma(2^23 + q, s PAD, a PAD)
// (far), PAD = 1.00000095; a child is hit when max(near x/y/z, tmin) <=
// min(far x/y/z, t_best).  Children are visited nearest-octant first
// (descending slot ^ (7 ^ octant)), the hit triangles in ascending index,
// all of a node's triangles before its next child.
namespace orc {
struct CwNodeO {
    float p[3];
    uint8_t e[3], imask;
    uint32_t child_base, tri_base;
    uint16_t tri_mask;
    uint8_t pad[6];
    uint8_t qlo[3][8], qhi[3][8];
};
static_assert(sizeof(CwNodeO) == 80, "node layout");
struct CwTriO { float v0[3]; uint32_t prim; float v1[3]; uint32_t mat; float v2[3]; uint32_t tr; };
static_assert(sizeof(CwTriO) == 48, "triangle layout");

static float pow2_biased(uint8_t e) { uint32_t u = (uint32_t)e << 23; float f; std::memcpy(&f, &u, 4); return f; }

// Hit bits of node `n`: internal children at bit 24 + (slot ^ key), the
// triangles of a hit leaf slot s at its tri_mask bits 2s, 2s + 1.
static uint32_t cw_node_hits(const Ray& r, const CwNodeO& n, uint32_t key, float tbest) {
    const float PAD = 1.00000095f;
    float o[3] = {r.o.x, r.o.y, r.o.z};
    float s[3], a[3], sf[3], af[3];
    for (int k = 0; k < 3; ++k) {
        s[k] = pow2_biased(n.e[k]) * r.idc[k];
        a[k] = (n.p[k] - o[k]) * r.idc[k];
        a[k] = a[k] - 8388608.0f * s[k];
        sf[k] = s[k] * PAD;
        af[k] = a[k] * PAD;
    }
    uint32_t hits = 0;
    for (int c = 0; c < 8; ++c) {
        bool inner = (n.imask >> c) & 1u;
        uint32_t tm = ((uint32_t)n.tri_mask >> (2 * c)) & 3u;
        if (!inner && tm == 0u) continue;   // an empty slot
        float tnear[3], tfar[3];
        for (int k = 0; k < 3; ++k) {
            bool neg = r.idc[k] < 0.0f;
            float qn = 8388608.0f + (float)(neg ? n.qhi[k][c] : n.qlo[k][c]);
            float qf = 8388608.0f + (float)(neg ? n.qlo[k][c] : n.qhi[k][c]);
            tnear[k] = std::fmaf(qn, s[k], a[k]);
            tfar[k] = std::fmaf(qf, sf[k], af[k]);
        }
        float tn = std::fmax(std::fmax(tnear[0], tnear[1]), std::fmax(tnear[2], r.tmin));
        float tf = std::fmin(std::fmin(tfar[0], tfar[1]), std::fmin(tfar[2], tbest));
        if (!(tn <= tf)) continue;
        if (inner) hits |= 1u << (24 + ((uint32_t)c ^ key));
        else hits |= tm << (2 * c);
    }
    return hits;
}

static uint32_t cw_trace(const CwNodeO* nodes, const CwTriO* tris, const Ray& r, bool any, float& to, float& uo,
                         float& vo, uint32_t& prim_out, Counts* cnt) {
    uint32_t oct = (r.idc[0] < 0.0f ? 1u : 0u) | (r.idc[1] < 0.0f ? 2u : 0u) | (r.idc[2] < 0.0f ? 4u : 0u);
    uint32_t key = 7u ^ oct;
    float tbest = r.tmax, bu = 0.0f, bv = 0.0f;
    uint32_t best_leaf = UINT32_MAX, best_prim = UINT32_MAX;
    struct Group { uint32_t base, bits, mask; };
    std::vector<Group> stack;
    Group G{0u, ray_traceable(r) ? (0x80000000u | (1u << (7u ^ key))) : 0u, 0u};  // the root: slot 7 ^ key of a virtual parent
    Group T{0u, 0u, 0u};
    while (true) {
        while (T.bits) {
            uint32_t bit = (uint32_t)__builtin_ctz(T.bits);
            T.bits &= T.bits - 1u;
            uint32_t ti = T.base + (uint32_t)__builtin_popcount(T.mask & ((1u << bit) - 1u));
            const CwTriO& ct = tris[ti];
            if (cnt) cnt->tris++;
            Tri t;
            t.a = f3(ct.v0[0], ct.v0[1], ct.v0[2]);
            t.b = f3(ct.v1[0], ct.v1[1], ct.v1[2]);
            t.c = f3(ct.v2[0], ct.v2[1], ct.v2[2]);
            t.prim = ct.prim;
            t.mat = ct.mat;
            std::memcpy(&t.tr, &ct.tr, 4);
            float tt, u, v;
            if (!tri_hit(r, t, tbest, best_prim, tt, u, v)) continue;
            if (!keep_hit(r, t.tr)) continue;
            tbest = tt; best_leaf = ti; best_prim = t.prim; bu = u; bv = v;
            if (any) { to = tt; uo = u; vo = v; prim_out = t.prim; return ti; }
        }
        if ((G.bits & 0xff000000u) == 0u) {
            if (stack.empty()) break;
            G = stack.back();
            stack.pop_back();
        }
        uint32_t bit = 31u - (uint32_t)__builtin_clz(G.bits & 0xff000000u);
        G.bits &= ~(1u << bit);
        uint32_t slot = (bit - 24u) ^ key;
        uint32_t ni = G.base + (uint32_t)__builtin_popcount(G.bits & 0xffu & ((1u << slot) - 1u));
        if (G.bits & 0xff000000u) stack.push_back(G);
        if (cnt) cnt->nodes++;
        const CwNodeO& n = nodes[ni];
        uint32_t h = cw_node_hits(r, n, key, tbest);
        G = Group{n.child_base, (h & 0xff000000u) | n.imask, 0u};
        T = Group{n.tri_base, h & 0x0000ffffu, n.tri_mask};
    }
    to = tbest; uo = bu; vo = bv;
    prim_out = best_prim;
    return best_leaf;
}
}  // namespace orc

// rays: n x 8 floats (origin, tmin, direction, tmax); hits: n x 4 words (t bits,
// primitive id or 0xffffffff, u bits, v bits); counts (optional): n x 2 (nodes
// visited, triangles tested).
ORC_API int orc_cwbvh_trace(const void* nodes, uint64_t num_nodes, const void* tris, uint64_t num_tris,
                            const float* rays, uint32_t n, int any, uint32_t* hits, uint32_t* counts, int threads) {
    if (!nodes || !tris || num_nodes == 0) return -1;
    const CwNodeO* N = (const CwNodeO*)nodes;
    const CwTriO* T = (const CwTriO*)tris;
    (void)num_tris;
    int nt = nthreads(threads);
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        while (true) {
            uint32_t b = next.fetch_add(1024);
            if (b >= n) break;
            uint32_t e = std::min(n, b + 1024);
            for (uint32_t i = b; i < e; ++i) {
                const float* R = rays + 8 * (size_t)i;
                Ray r = make_ray(f3(R[0], R[1], R[2]), R[3], f3(R[4], R[5], R[6]), R[7]);
                float t, u, v;
                uint32_t prim;
                Counts c;
                cw_trace(N, T, r, any != 0, t, u, v, prim, counts ? &c : nullptr);
                uint32_t* H = hits + 4 * (size_t)i;
                std::memcpy(&H[0], &t, 4);
                H[1] = prim;
                std::memcpy(&H[2], &u, 4);
                std::memcpy(&H[3], &v, 4);
                if (counts) { counts[2 * (size_t)i] = (uint32_t)c.nodes; counts[2 * (size_t)i + 1] = (uint32_t)c.tris; }
            }
        }
    };
    std::vector<std::thread> ts;
    for (int k = 1; k < nt; ++k) ts.emplace_back(work);
    work();
    for (auto& t : ts) t.join();
    return 0;
}

// ===================================================== radiance-cache MLP ====
// CPU restatement of the cache network (64 encoded inputs, 4 hidden ReLU
// layers of 64, 3 outputs, no biases) with the same rounding points as the
// tensor-core kernels when `bf16` is set: encoded features, hidden
// activations, weights and back-propagated gradients are rounded to bfloat16
// (round to nearest even) before each product; sums are fp32.  With `bf16`
// clear it is plain fp32 (used for finite-difference checks).
namespace orc {
static float bf16r(float x, bool on) {
    if (!on) return x;
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
static float mlp_feature(const float* raw, int f) {
    if (f < 56) {
        int d = f >> 3, k = (f & 7) >> 1;
        float s, c;
        sincos_turns(raw[d] * (float)(1 << k) * 0.5f, &s, &c);
        return (f & 1) ? c : s;
    }
    int r = f - 56;
    if (r < 5) return raw[7 + r];
    return r == 5 ? 1.0f : 0.0f;
}
constexpr int kP = 4 * 4096 + 8 * 64;
struct MlpAct { float e[64], a[4][64], y[8]; };
static void mlp_fwd(const float* W, const float* raw, bool bf, MlpAct& A) {
    for (int f = 0; f < 64; ++f) A.e[f] = bf16r(mlp_feature(raw, f), bf);
    const float* in = A.e;
    for (int l = 0; l < 4; ++l) {
        const float* Wl = W + l * 4096;
        for (int o = 0; o < 64; ++o) {
            float z = 0.0f;
            for (int i = 0; i < 64; ++i) z += bf16r(Wl[o * 64 + i], bf) * in[i];
            A.a[l][o] = bf16r(std::fmax(z, 0.0f), bf);
        }
        in = A.a[l];
    }
    const float* W4 = W + 4 * 4096;
    for (int o = 0; o < 8; ++o) {
        float z = 0.0f;
        for (int i = 0; i < 64; ++i) z += bf16r(W4[o * 64 + i], bf) * in[i];
        A.y[o] = o < 3 ? z : 0.0f;
    }
}
static void cache_predict(const float* W, const float* raw, float y[3]) {
    MlpAct A;
    mlp_fwd(W, raw, true, A);
    for (int c = 0; c < 3; ++c) y[c] = A.y[c];
}
}  // namespace orc

// samples: n x 16 floats (raw 12, target 3, pad); out: n x 3
ORC_API void orc_mlp_forward(const float* W, const float* samples, uint32_t n, float* out, int bf16) {
    for (uint32_t s = 0; s < n; ++s) {
        orc::MlpAct A;
        orc::mlp_fwd(W, samples + 16 * (size_t)s, bf16 != 0, A);
        for (int c = 0; c < 3; ++c) out[3 * (size_t)s + c] = A.y[c];
    }
}

// Gradient of the mean relative L2 loss  mean_{s,c} (y - t)^2 / (y^2 + 0.01)  (the y^2 in the
// denominator is held constant, as in the kernels); returns the loss.
ORC_API float orc_mlp_gradient(const float* W, const float* samples, uint32_t n, float* dW, int bf16) {
    const bool bf = bf16 != 0;
    for (int i = 0; i < orc::kP; ++i) dW[i] = 0.0f;
    double loss = 0.0;
    const float inv = 1.0f / (3.0f * (float)n);
    for (uint32_t s = 0; s < n; ++s) {
        const float* S = samples + 16 * (size_t)s;
        orc::MlpAct A;
        orc::mlp_fwd(W, S, bf, A);
        float gy[8] = {0};
        for (int c = 0; c < 3; ++c) {
            float d = A.y[c] - S[12 + c], den = A.y[c] * A.y[c] + 0.01f;
            loss += (double)(d * d / den * inv);
            gy[c] = orc::bf16r(2.0f * d / den * inv, bf);
        }
        // output layer
        const float* W4 = W + 4 * 4096;
        float* dW4 = dW + 4 * 4096;
        float g[64];
        for (int i = 0; i < 64; ++i) {
            float acc = 0.0f;
            for (int o = 0; o < 8; ++o) {
                dW4[o * 64 + i] += gy[o] * A.a[3][i];
                acc += orc::bf16r(W4[o * 64 + i], bf) * gy[o];
            }
            g[i] = acc;
        }
        for (int l = 3; l >= 0; --l) {
            float gz[64];
            for (int i = 0; i < 64; ++i) gz[i] = orc::bf16r(A.a[l][i] > 0.0f ? g[i] : 0.0f, bf);
            const float* prev = l > 0 ? A.a[l - 1] : A.e;
            const float* Wl = W + l * 4096;
            float* dWl = dW + l * 4096;
            for (int o = 0; o < 64; ++o)
                for (int i = 0; i < 64; ++i) dWl[o * 64 + i] += gz[o] * prev[i];
            if (l > 0) {
                for (int i = 0; i < 64; ++i) {
                    float acc = 0.0f;
                    for (int o = 0; o < 64; ++o) acc += orc::bf16r(Wl[o * 64 + i], bf) * gz[o];
                    g[i] = acc;
                }
            }
        }
    }
    return (float)loss;
}

// One Adam step (beta1 0.9, beta2 0.99, eps 1e-8) at 1-based step t; padded output rows stay zero.
ORC_API void orc_mlp_adam(float* W, const float* dW, float* m, float* v, float lr, int t) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    float bc1 = 1.0f - std::pow(b1, (float)t), bc2 = 1.0f - std::pow(b2, (float)t);
    for (int i = 0; i < orc::kP; ++i) {
        float g = dW[i];
        m[i] = b1 * m[i] + (1.0f - b1) * g;
        v[i] = b2 * v[i] + (1.0f - b2) * g * g;
        float mh = m[i] / bc1, vh = v[i] / bc2;
        float w = W[i] - lr * mh / (std::sqrt(vh) + eps);
        if (i >= 4 * 4096 + 3 * 64) w = 0.0f;
        W[i] = w;
    }
}
