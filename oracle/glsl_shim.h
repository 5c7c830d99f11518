// glsl_shim.h — ORACLE: test infrastructure only.
//
// The GLSL types, built-ins and ray-tracing environment that the reference's
// rtcommon.glsl, restir.glsl, rt.rgen and tonemap.frag use, in C++, so that those shader
// files compile as C++ (after the textual rewrites of make_ref_shade.py) and
// serve as the reference's own code for the shading oracle.  Every
// operation is one FP32 operation as GLSL defines it (dot and matrix
// products summed left to right; normalize(v) = v / length(v);
// reflect(i, n) = i - 2 dot(n, i) n; mix(x, y, a) = x (1 - a) + y a).  sin,
// cos, pow and exp, which GLSL leaves to the implementation, are the
// restatement's own (shade_oracle.c), as are the scene tracer behind
// traceRayEXT and the filtering of the material textures.  Compile with
// -ffp-contract=off.
#pragma once

#include <cmath>
#include <cstdint>

#include "shade_oracle.h"

typedef unsigned int uint;

struct vec4;
struct uvec2 {
    uint x, y;
};
struct uvec3 {
    uint x, y, z;
    uvec2 xy;
};

struct vec2 {
    float x, y;
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(const uvec2& u) : x((float)u.x), y((float)u.y) {}
    explicit vec2(const uvec3& u) : x((float)u.x), y((float)u.y) {}
};

struct vec3 {
    union { float x; float r; };
    union { float y; float g; };
    union { float z; float b; };
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b_, float c) : x(a), y(b_), z(c) {}
    explicit vec3(const vec4& v);
};

// swizzles of a vec4: read as a vector, assigned component by component
template <int A, int B>
struct sw2 {
    float v[4];
    operator vec2() const { return vec2(v[A], v[B]); }
    sw2& operator=(vec2 o) {
        v[A] = o.x;
        v[B] = o.y;
        return *this;
    }
};
template <int A, int B, int C>
struct sw3 {
    float v[4];
    operator vec3() const { return vec3(v[A], v[B], v[C]); }
    sw3& operator=(vec3 o) {
        v[A] = o.x;
        v[B] = o.y;
        v[C] = o.z;
        return *this;
    }
    sw3& operator/=(float s) {
        v[A] = v[A] / s;
        v[B] = v[B] / s;
        v[C] = v[C] / s;
        return *this;
    }
};

// (an anonymous struct inside the union: a GNU extension g++ accepts)
struct vec4 {
    union {
        struct {
            float x, y, z, w;
        };
        struct {
            float r, g, b, a;
        };
        float c[4];
        sw2<0, 1> xy;
        sw3<0, 1, 2> xyz;
        sw3<0, 1, 2> rgb;
    };
    vec4() { c[0] = c[1] = c[2] = c[3] = 0.0f; }
    vec4(float a, float b, float c_, float d) {
        c[0] = a;
        c[1] = b;
        c[2] = c_;
        c[3] = d;
    }
    vec4(vec3 v, float d) : vec4(v.x, v.y, v.z, d) {}
    vec4(vec2 v, float c_, float d) : vec4(v.x, v.y, c_, d) {}
    vec4(const vec4& o) : vec4(o.c[0], o.c[1], o.c[2], o.c[3]) {}
    vec4& operator=(const vec4& o) {
        for (int k = 0; k < 4; ++k) c[k] = o.c[k];
        return *this;
    }
};
inline vec3::vec3(const vec4& v) : x(v.c[0]), y(v.c[1]), z(v.c[2]) {}

struct ivec2 {
    int x, y;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const uvec2& u) : x((int)u.x), y((int)u.y) {}
    explicit ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
};
struct ivec3 {
    int x, y, z;
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
};
struct bvec2 {
    bool x, y;
};
struct bvec3 {
    bool x, y, z;
};

struct mat3 {
    vec3 col[3];
    mat3(vec3 a, vec3 b, vec3 c) : col{a, b, c} {}
};
struct mat4 {
    float m[4][4];  // m[column][row], as GLSL stores it
};

// ---- vector arithmetic ------------------------------------------------------
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator+(vec2 a, float s) { return vec2(a.x + s, a.y + s); }
inline vec2 operator-(vec2 a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, vec3 a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator+(float s, vec3 a) { return vec3(s + a.x, s + a.y, s + a.z); }
inline vec3 operator-(float s, vec3 a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3 operator-(vec3 a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }
inline vec3 operator+(vec3 a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3& operator+=(vec3& a, vec3 b) { return a = a + b; }
inline vec3& operator*=(vec3& a, vec3 b) { return a = a * b; }
inline vec3& operator/=(vec3& a, float s) { return a = a / s; }

inline vec3 operator*(const mat3& m, vec3 v) { return m.col[0] * v.x + m.col[1] * v.y + m.col[2] * v.z; }
inline vec4 operator*(const mat4& m, const vec4& v) {
    float r[4];
    for (int i = 0; i < 4; ++i) r[i] = m.m[0][i] * v.c[0] + m.m[1][i] * v.c[1] + m.m[2][i] * v.c[2] + m.m[3][i] * v.c[3];
    return vec4(r[0], r[1], r[2], r[3]);
}

// ---- built-ins ----------------------------------------------------------------
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(vec3 a, vec3 b) { return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float length(vec3 a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(vec3 a) { return a / length(a); }
inline vec3 reflect(vec3 i, vec3 n) { return i - 2.0f * dot(n, i) * n; }
inline vec3 mix(vec3 x, vec3 y, float a) { return x * (1.0f - a) + y * a; }

inline float sqrt(float a) { return std::sqrt(a); }
inline float abs(float a) { return std::fabs(a); }
inline float sin(float a) { return orc_sh_sin(a); }
inline float cos(float a) { return orc_sh_cos(a); }
inline float pow(float a, float b) { return orc_sh_pow(a, b); }
inline float exp(float a) { return orc_sh_exp(a); }
inline vec3 pow(vec3 a, vec3 b) { return vec3(pow(a.x, b.x), pow(a.y, b.y), pow(a.z, b.z)); }
inline vec3 exp(vec3 a) { return vec3(exp(a.x), exp(a.y), exp(a.z)); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline vec3 min(vec3 a, vec3 b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(vec3 a, vec3 b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

inline bvec2 greaterThan(vec2 a, vec2 b) { return bvec2{a.x > b.x, a.y > b.y}; }
inline bvec2 lessThan(vec2 a, vec2 b) { return bvec2{a.x < b.x, a.y < b.y}; }
inline bvec3 greaterThan(vec3 a, vec3 b) { return bvec3{a.x > b.x, a.y > b.y, a.z > b.z}; }
inline bool all(bvec2 v) { return v.x && v.y; }
inline bool any(bvec3 v) { return v.x || v.y || v.z; }

// ---- resources --------------------------------------------------------------
// RGBA float images read at their nearest texel with repeat addressing (the
// G-buffer sampler of rt.cpp:449-450, vulkan.cpp:522-531), or RGBA8 sRGB
// material textures (`texels`: rt.cpp:439-447's images and linear sampler)
// through the restatement's texture()
struct sampler2D {
    const float* data;
    int w, h;
    const unsigned char* texels = nullptr;
};
struct image2D {
    float* data;
    int w, h;
};
inline vec4 texture(const sampler2D& s, vec2 uv) {
    if (s.texels) {
        float o[4];
        orc_sh_texture(s.w, s.h, s.texels, uv.x, uv.y, o);
        return vec4(o[0], o[1], o[2], o[3]);
    }
    if (!s.data) return vec4();
    const int i = ((int)std::floor(uv.x * (float)s.w) % s.w + s.w) % s.w;
    const int j = ((int)std::floor(uv.y * (float)s.h) % s.h + s.h) % s.h;
    const float* p = s.data + 4 * ((int64_t)j * s.w + i);
    return vec4(p[0], p[1], p[2], p[3]);
}
inline vec4 imageLoad(const image2D& im, ivec2 p) {
    const float* q = im.data + 4 * ((int64_t)p.y * im.w + p.x);
    return vec4(q[0], q[1], q[2], q[3]);
}
inline void imageStore(const image2D& im, ivec2 p, const vec4& v) {
    float* q = im.data + 4 * ((int64_t)p.y * im.w + p.x);
    for (int k = 0; k < 4; ++k) q[k] = v.c[k];
}

struct accelerationStructureEXT {};
const uint gl_RayFlagsOpaqueEXT = 1u, gl_RayFlagsTerminateOnFirstHitEXT = 4u,
           gl_RayFlagsSkipClosestHitShaderEXT = 8u;
inline uvec3 gl_LaunchIDEXT, gl_LaunchSizeEXT;
inline uint64_t g_clock;
inline uint64_t clockARB() { return g_clock; }
// defined by the wrapper, after the shader's payload
void traceRayEXT(accelerationStructureEXT, uint flags, uint cull, uint sbt_off, uint sbt_stride, uint miss, vec3 o,
                 float tmin, vec3 d, float tmax, int payload_location);
