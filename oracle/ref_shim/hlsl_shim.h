// hlsl_shim.h — TEST INFRASTRUCTURE: the subset of HLSL that the reference's
// material / frame / sampling / G-buffer packing shader code uses, as C++ types
// and functions, so that it compiles unmodified (apart from out/inout
// parameters turned into references by oracle/build.py) with g++ and produces
// golden vectors.  Swizzles (.xy of float3, .yx of float2, .xy/.zw/.xyz of
// float4) read, and two-component ones write, through a union.  Semantics
// follow the HLSL intrinsic definitions: componentwise vector ops,
// lerp(a, b, t) = a + t * (b - a), saturate = clamp to [0, 1],
// reflect(i, n) = i - 2 * n * dot(i, n).
#pragma once
#include <cmath>
#include <cstdint>

typedef uint32_t uint;

struct bool3 { bool x, y, z; };
struct bool4 { bool x, y, z, w; };

struct float2;
// Two-component swizzle of an N-float vector (reads and writes, e.g. n.xy = ...).
template <int N, int A, int B>
struct Swizzle2 {
    float v[N];
    inline operator float2() const;
    inline Swizzle2& operator=(const float2& o);
};

struct float2 {
    union {
        struct { float x, y; };
        Swizzle2<2, 1, 0> yx;
    };
    float2() { x = 0; y = 0; }
    float2(double s) { x = (float)s; y = (float)s; }
    float2(float a, float b) { x = a; y = b; }
    float2(const float2& o) { x = o.x; y = o.y; }
    float2& operator=(const float2& o) { x = o.x; y = o.y; return *this; }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
template <int N, int A, int B>
inline Swizzle2<N, A, B>::operator float2() const { return float2(v[A], v[B]); }
template <int N, int A, int B>
inline Swizzle2<N, A, B>& Swizzle2<N, A, B>::operator=(const float2& o) { v[A] = o.x; v[B] = o.y; return *this; }

struct float3 {
    union {
        struct { float x, y, z; };
        Swizzle2<3, 0, 1> xy;
    };
    float3() { x = 0; y = 0; z = 0; }
    float3(double s) { x = (float)s; y = (float)s; z = (float)s; }
    float3(float a, float b, float c) { x = a; y = b; z = c; }
    float3(float2 v, float c) { x = v.x; y = v.y; z = c; }
    float3(const float3& o) { x = o.x; y = o.y; z = o.z; }
    float3& operator=(const float3& o) { x = o.x; y = o.y; z = o.z; return *this; }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};
struct uint2 {
    uint x, y;
    explicit uint2(float2 f) : x((uint)f.x), y((uint)f.y) {}
};

// Three-component read swizzle of a float4 (.xyz).
template <int A, int B, int C>
struct Swizzle3 {
    float v[4];
    operator float3() const { return float3(v[A], v[B], v[C]); }
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        Swizzle2<4, 0, 1> xy;
        Swizzle2<4, 2, 3> zw;
        Swizzle3<0, 1, 2> xyz;
    };
    float4() { x = 0; y = 0; z = 0; w = 0; }
    float4(double s) { x = (float)s; y = (float)s; z = (float)s; w = (float)s; }
    float4(float a, float b, float c, float d) { x = a; y = b; z = c; w = d; }
    float4(float3 v, float d) { x = v.x; y = v.y; z = v.z; w = d; }
    float4(float2 a, float2 b) { x = a.x; y = a.y; z = b.x; w = b.y; }
    float4(const float4& o) { x = o.x; y = o.y; z = o.z; w = o.w; }
    float4& operator=(const float4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};

#define SHIM_V3OP(op)                                                                                     \
    inline float3 operator op(float3 a, float3 b) { return float3(a.x op b.x, a.y op b.y, a.z op b.z); } \
    inline float3 operator op(float3 a, float s) { return float3(a.x op s, a.y op s, a.z op s); }       \
    inline float3 operator op(float s, float3 a) { return float3(s op a.x, s op a.y, s op a.z); }
SHIM_V3OP(+) SHIM_V3OP(-) SHIM_V3OP(*) SHIM_V3OP(/)
#define SHIM_V4OP(op)                                                                                                \
    inline float4 operator op(float4 a, float4 b) { return float4(a.x op b.x, a.y op b.y, a.z op b.z, a.w op b.w); } \
    inline float4 operator op(float4 a, float s) { return float4(a.x op s, a.y op s, a.z op s, a.w op s); }         \
    inline float4 operator op(float s, float4 a) { return float4(s op a.x, s op a.y, s op a.z, s op a.w); }
SHIM_V4OP(+) SHIM_V4OP(-) SHIM_V4OP(*) SHIM_V4OP(/)
#define SHIM_V2OP(op)                                                                       \
    inline float2 operator op(float2 a, float2 b) { return float2(a.x op b.x, a.y op b.y); } \
    inline float2 operator op(float2 a, float s) { return float2(a.x op s, a.y op s); }
SHIM_V2OP(+) SHIM_V2OP(-) SHIM_V2OP(*) SHIM_V2OP(/)
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
inline float2 operator-(double s, float2 a) { return float2((float)s - a.x, (float)s - a.y); }
inline float3& operator/=(float3& a, float s) { a = a / s; return a; }
inline float2& operator/=(float2& a, float s) { a = a / s; return a; }
inline float4 operator-(float4 a) { return float4(-a.x, -a.y, -a.z, -a.w); }
inline float3 operator/(double s, float3 a) { return float3((float)s / a.x, (float)s / a.y, (float)s / a.z); }
inline float4 operator/(double s, float4 a) { return float4((float)s / a.x, (float)s / a.y, (float)s / a.z, (float)s / a.w); }
inline bool3 operator<(float3 a, double s) { return bool3{a.x < s, a.y < s, a.z < s}; }
inline bool4 operator<(float4 a, double s) { return bool4{a.x < s, a.y < s, a.z < s, a.w < s}; }

struct float2x2 {
    float2 r[2];
    float2x2(float a, float b, float c, float d) { r[0] = float2(a, b); r[1] = float2(c, d); }
    float2& operator[](int i) { return r[i]; }
    const float2& operator[](int i) const { return r[i]; }
};
struct float3x3 {
    float3 r[3];
    float3x3(float a, float b, float c, float d, float e, float f, float g, float h, float i) {
        r[0] = float3(a, b, c); r[1] = float3(d, e, f); r[2] = float3(g, h, i);
    }
    float3& operator[](int i) { return r[i]; }
    const float3& operator[](int i) const { return r[i]; }
};
struct float4x4 {
    float4 r[4];
    float4& operator[](int i) { return r[i]; }
    const float4& operator[](int i) const { return r[i]; }
};
inline float determinant(const float2x2& m) { return m[0][0] * m[1][1] - m[0][1] * m[1][0]; }
inline float determinant(const float3x3& m) {
    return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}

inline float max(float a, float b) { return a > b ? a : b; }
inline float max(float a, double b) { return max(a, (float)b); }
inline float max(double a, float b) { return max((float)a, b); }
inline float max(double a, double b) { return max((float)a, (float)b); }
inline float min(float a, float b) { return a < b ? a : b; }
inline float min(float a, double b) { return min(a, (float)b); }
inline float min(double a, double b) { return min((float)a, (float)b); }
inline float3 max(float3 a, float3 b) { return float3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline float4 max(float4 a, float4 b) { return float4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
inline float clamp(float x, double lo, double hi) { return min(max(x, (float)lo), (float)hi); }
inline float saturate(float x) { return min(max(x, 0.0f), 1.0f); }
inline float abs(float a) { return std::fabs(a); }
inline float2 abs(float2 a) { return float2(std::fabs(a.x), std::fabs(a.y)); }
inline float3 abs(float3 a) { return float3(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }
inline float4 abs(float4 a) { return float4(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z), std::fabs(a.w)); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float3 normalize(float3 a) { return a / std::sqrt(dot(a, a)); }
inline float lerp(float a, float b, float t) { return a + t * (b - a); }
inline float3 lerp(float3 a, float3 b, float t) { return a + t * (b - a); }
inline float3 lerp(float3 a, float b, bool3 t) {
    return float3(t.x ? b : a.x, t.y ? b : a.y, t.z ? b : a.z);
}
inline float4 lerp(float4 a, float4 b, float t) { return a + t * (b - a); }
inline float4 lerp(float4 a, float b, bool4 t) {
    return float4(t.x ? b : a.x, t.y ? b : a.y, t.z ? b : a.z, t.w ? b : a.w);
}
inline float3 reflect(float3 i, float3 n) { return i - 2.0f * n * dot(i, n); }
