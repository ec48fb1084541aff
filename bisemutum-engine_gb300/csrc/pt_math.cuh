// pt_math.cuh — vector math, deterministic transcendental functions and the
// PCG32 generator shared by the device kernels and the host-side setup code.
//
// Every function here is built only from IEEE-754 single-precision +, -, *, /
// and sqrt (all correctly rounded on sm_103a when compiled with --fmad=false,
// -prec-div=true, -prec-sqrt=true, and on the host with -ffp-contract=off).
// That makes a path's arithmetic reproducible bit for bit on any IEEE machine,
// which is what lets a CPU build of the same stages check primitive ids and
// path decisions exactly.  The sine/cosine and arctangent below are written
// from their Taylor series with a quadrant / octant range reduction; they do
// not use the CUDA math library.
#pragma once

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#include <cuda_runtime.h>
#define BSM_HD __host__ __device__ __forceinline__
#else
#include <vector_types.h>
#define BSM_HD static inline
#endif

namespace bsm {

// Constants as the reference declares them (bisemutum/shaders/core/utils/math.hlsl:3-10):
// PI is the float nearest 3.14159265359, INV_PI is 1/PI evaluated in float.
#define BSM_PI 3.14159265359f
#define BSM_TWO_PI (2.0f * 3.14159265359f)
#define BSM_INV_PI 0.318309873f
#define BSM_INV_FOUR_PI 0.0795774683f

// bit pattern of a float (memcpy: defined on the host, one move on the device)
BSM_HD uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

struct V3 { float x, y, z; };

BSM_HD V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
BSM_HD V3 v3s(float s) { return v3(s, s, s); }
BSM_HD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
BSM_HD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
BSM_HD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
BSM_HD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
BSM_HD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
BSM_HD V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
BSM_HD V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
BSM_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
BSM_HD V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
BSM_HD float fmax3(float a, float b, float c) { return fmaxf(a, fmaxf(b, c)); }
BSM_HD float max_comp(V3 a) { return fmax3(a.x, a.y, a.z); }
// normalize(v) = v * (1 / |v|): one IEEE division and one IEEE square root.
BSM_HD V3 normalize(V3 a) {
    float inv = 1.0f / sqrtf(dot(a, a));
    return a * inv;
}
// HLSL lerp(a, b, t) = a + t * (b - a).
BSM_HD V3 lerp(V3 a, V3 b, float t) { return a + (b - a) * t; }
// HLSL reflect(i, n) = i - 2 dot(i, n) n.
BSM_HD V3 reflect(V3 i, V3 n) { return i - n * (2.0f * dot(i, n)); }

BSM_HD float pow2(float x) { return x * x; }
BSM_HD float pow5(float x) { float x2 = x * x; return (x2 * x2) * x; }

// sin(2*pi*t) and cos(2*pi*t) for t in "turns".  Range reduction to the
// nearest quarter turn (exact for |t| < 2^22), then Taylor polynomials of
// degree 9 (sine) and 10 (cosine) on |x| <= pi/4, whose truncation error is
// below 2e-9.
BSM_HD void sincos_turns(float t, float* s, float* c) {
    float q = floorf(t * 4.0f + 0.5f);
    float r = t - q * 0.25f;
    int iq = ((int)q) & 3;
    float x = r * 6.28318548f;
    float x2 = x * x;
    float ps = x + x * x2 * (-0.166666672f + x2 * (0.00833333377f + x2 * (-0.000198412701f + x2 * 2.75573188e-06f)));
    float pc = 1.0f + x2 * (-0.5f + x2 * (0.0416666679f + x2 * (-0.00138888892f + x2 * (2.48015876e-05f + x2 * -2.75573188e-07f))));
    float sv, cv;
    if (iq == 0) { sv = ps; cv = pc; }
    else if (iq == 1) { sv = pc; cv = -ps; }
    else if (iq == 2) { sv = -ps; cv = -pc; }
    else { sv = -pc; cv = ps; }
    *s = sv; *c = cv;
}

// atan(z) for z in [0, 1]: z <= tan(pi/8) uses the Taylor series directly
// (degree 17, truncation < 3e-9), larger z uses atan(z) = pi/4 + atan((z-1)/(z+1)).
BSM_HD float atan_unit(float z) {
    float off = 0.0f;
    if (z > 0.414213568f) { z = (z - 1.0f) / (z + 1.0f); off = 0.785398185f; }
    float z2 = z * z;
    float p = 1.0f + z2 * (-0.333333343f + z2 * (0.200000003f + z2 * (-0.142857149f + z2 * (0.111111112f +
              z2 * (-0.0909090936f + z2 * (0.0769230798f + z2 * (-0.0666666701f + z2 * 0.0588235296f)))))));
    return off + z * p;
}
// atan2(y, x) in radians, in [-pi, pi].
BSM_HD float atan2_det(float y, float x) {
    float ax = fabsf(x), ay = fabsf(y);
    float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    if (mx == 0.0f) return 0.0f;
    float a = atan_unit(mn / mx);
    if (ay > ax) a = 1.57079637f - a;
    if (x < 0.0f) a = 3.14159274f - a;
    if (y < 0.0f) a = -a;
    return a;
}

// IEEE binary16 -> binary32 (exact).
BSM_HD float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1fu;
    uint32_t man = h & 0x3ffu;
    float f;
    if (exp == 0) {
        f = (float)man * 5.96046448e-08f;  // man * 2^-24
        if (sign) f = -f;
        return f;
    }
    uint32_t bits;
    if (exp == 31) bits = sign | 0x7f800000u | (man << 13);
    else bits = sign | ((exp + 112u) << 23) | (man << 13);
    union { uint32_t u; float f; } cv; cv.u = bits;
    return cv.f;
}

// ---- PCG32 (O'Neill 2014, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation"): 64-bit LCG
// state, XSH-RR output.  One stream per pixel (the increment), one starting
// state per sample. ----
struct Pcg { uint64_t state; uint64_t inc; };

BSM_HD uint32_t pcg_next(Pcg& g) {
    uint64_t old = g.state;
    g.state = old * 6364136223846793005ULL + g.inc;
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}
BSM_HD Pcg pcg_seed(uint64_t initstate, uint64_t initseq) {
    Pcg g; g.state = 0u; g.inc = (initseq << 1u) | 1u;
    pcg_next(g);
    g.state += initstate;
    pcg_next(g);
    return g;
}
// Uniform float in [0, 1) from the top 24 bits.
BSM_HD float pcg_uniform(Pcg& g) { return (float)(pcg_next(g) >> 8) * 5.96046448e-08f; }

// SplitMix64 finaliser (Steele, Lea, Flood 2014) used to derive a sample's
// starting state from the scene seed and the sample index.
BSM_HD uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
BSM_HD uint64_t sample_initstate(uint64_t seed, uint32_t sample) {
    return mix64(seed + 0x9e3779b97f4a7c15ULL * ((uint64_t)sample + 1u));
}
// Start state of the PCG32 stream of one (pixel, sample) path.  Streams that
// share a start state and differ only in their increments are correlated at
// some draws (measured: correlation 0.16 between pixels 32 apart at the 36th
// draw), so the pixel is mixed into the state as well.
BSM_HD uint64_t path_initstate(uint64_t seed, uint32_t sample, uint64_t pixel) {
    return mix64(sample_initstate(seed, sample) ^ mix64(pixel * 0x9e3779b97f4a7c15ULL + 0x632be59bd9b4e019ULL));
}

// Per-ray uniform of the stochastic-opacity test.  As the reference's
// gen_opacity_random_for (renderer/raytracing/hits/rt_gbuffer.hlsl:14-19) it
// combines the bits of the ray's origin and direction with a seed (there: the
// frame index; here: the path's PCG32 state, which differs per sample and
// bounce), then hashes them: SplitMix64's finaliser, top 24 bits as [0, 1).
BSM_HD float opacity_random(float ox, float oy, float oz, float dx, float dy, float dz, uint32_t seed) {
    uint32_t h = f2u(ox) ^ f2u(oy) ^ f2u(oz) ^ f2u(dx) ^ f2u(dy) ^ f2u(dz);
    uint64_t z = mix64(((uint64_t)h << 32) | (uint64_t)seed);
    return (float)(uint32_t)(z >> 40) * 5.96046448e-08f;
}

}  // namespace bsm
