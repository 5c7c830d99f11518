// shade.cu — the reference's path tracer (src/shaders/rt/rt.rgen,
// rtcommon.glsl, restir.glsl, tonemap.frag) as CUDA kernels over the
// closest-point engine's BVH, into a headless image buffer.
//
// One thread renders one pixel: the shader's per-pixel random stream (TEA
// seed, then one linear congruential sequence through every sample and
// bounce) and ReSTIR's per-pixel reservoir run sequentially through the
// pixel's samples, so they stay in registers.  Each bounce traces its ray
// through the scene's wide BVH with ray_walk (raywalk.cuh): the nearest
// Möller–Trumbore hit, ties to the least triangle index, equal to a brute
// force over every triangle bit for bit.  Shading follows the shader's
// operations in its order: the five integrators (direct lighting, material
// sampling, MIS with the power heuristic, ReSTIR direct-only, ReSTIR with
// temporal reuse), Blinn-Phong and GGX, uniform light sampling with the
// brute-force light pdf, Russian roulette, frame accumulation and the debug
// views of the previous frame's buffers.
//
// This file is compiled with -fmad=false: no multiply-add contraction, every
// FP32 expression rounds as written, left to right, as the shader's
// operations do.  sin, cos, pow and exp are the engine's own routines
// (Cody-Waite reduction with Taylor polynomials; 2^(y log2 x) through the
// atanh and exponential series), evaluated in FP64 and rounded once — what
// GLSL leaves to the implementation is fixed here so that a CPU restatement
// can reproduce a frame exactly.  Where the shader reads the clock for the
// pixel seed (rt.rgen:569) the caller's seed stands in.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "handles.cuh"
#include "raywalk.cuh"

namespace cpq {
namespace {

// The routines many call sites share — the scene tracer, sin / cos / pow /
// exp, the materials and the light sampling — stay out of line: a pixel's
// warp diverges across integrators, bounces and materials, and one copy of
// each keeps the kernel's hot code in the instruction cache (inlined, the
// kernel stalls mostly on instruction fetch).  Calls round nothing
// differently: every operation is the same, and this file has no multiply-add
// contraction.
#ifndef CPQ_SHADE_INLINE
#define SH_CALL __noinline__
#else
#define SH_CALL
#endif

constexpr float kPi = 3.141592f;          // rtcommon.glsl:6 (the shader's truncated constant)
constexpr float kLargeDist = 10000000.0f;  // rtcommon.glsl:7
constexpr float kEps = 0.00001f;           // rtcommon.glsl:8

struct v3 {
    float x, y, z;
};
__device__ __forceinline__ v3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ v3 ld(const float* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ v3 mulv(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ v3 divs(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length3(v3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ v3 normalize3(v3 a) { return divs(a, length3(a)); }
// GLSL reflect: I - 2 dot(N, I) N
__device__ __forceinline__ v3 reflect3(v3 i, v3 n) { return sub(i, scl(n, 2.0f * dot(n, i))); }
// x*a + y*b + z*c, summed left to right (a matrix-vector product's order)
__device__ __forceinline__ v3 comb(v3 a, float x, v3 b, float y, v3 c, float z) {
    return mk(a.x * x + b.x * y + c.x * z, a.y * x + b.y * y + c.y * z, a.z * x + b.z * y + c.z * z);
}
__device__ __forceinline__ bool any_pos(v3 a) { return a.x > 0.0f || a.y > 0.0f || a.z > 0.0f; }

// ---- sin, cos, pow, exp ----------------------------------------------------

// sin and cos: Cody-Waite reduction by pi/2 in FP64 (one multiply, one
// round-to-nearest-integer, one multiply and one subtract), then the Taylor
// polynomials of sin (to r^9) and cos (to r^10) on |r| <= pi/4 in FP32
// Horner form: truncation below 2e-9 absolute, within about an ulp.
__device__ SH_CALL void sh_sincos(float x, float* s, float* c) {
    const double kTwoOverPi = 0.63661977236758134308;
    const double kPiOver2 = 1.57079632679489661923;
    const double k = nearbyint((double)x * kTwoOverPi);
    const double kp = k * kPiOver2;
    const float r = (float)((double)x - kp);
    const float z = r * r;
    const float sp = r + r * z * (-1.0f / 6.0f + z * (1.0f / 120.0f + z * (-1.0f / 5040.0f + z * (1.0f / 362880.0f))));
    const float cp =
        1.0f + z * (-0.5f + z * (1.0f / 24.0f + z * (-1.0f / 720.0f + z * (1.0f / 40320.0f + z * (-1.0f / 3628800.0f)))));
    switch (((long long)k) & 3) {
        case 0: *s = sp; *c = cp; break;
        case 1: *s = cp; *c = -sp; break;
        case 2: *s = -sp; *c = -cp; break;
        default: *s = -cp; *c = sp; break;
    }
}

constexpr double kLn2 = 0.69314718055994530942;
constexpr double kInvLn2 = 1.44269504088896340736;

// 1 / j! for j = 0..10, each the correctly rounded quotient
__constant__ double c_inv_fact[11] = {1.0,        1.0,         1.0 / 2.0,      1.0 / 6.0,
                                      1.0 / 24.0, 1.0 / 120.0, 1.0 / 720.0,    1.0 / 5040.0,
                                      1.0 / 40320.0, 1.0 / 362880.0, 1.0 / 3628800.0};
// 1 / j for odd j = 1..15
__constant__ double c_inv_odd[8] = {1.0,        1.0 / 3.0,  1.0 / 5.0,  1.0 / 7.0,
                                    1.0 / 9.0,  1.0 / 11.0, 1.0 / 13.0, 1.0 / 15.0};

// 2^k for an integer |k| <= 1022, from its bits
__device__ __forceinline__ double sh_pow2i(int k) { return __longlong_as_double((long long)(k + 1023) << 52); }

// 1 / d in FP64 for d in [1.7, 2.5] without a division: the FP32 quotient
// (relative error below 2^-23) refined by two Newton steps r += r (1 - d r),
// each two fused multiply-adds that square the error (below 2^-52 after).
__device__ __forceinline__ double sh_rcp_d(double d) {
    double r = (double)(1.0f / (float)d);
    double e = fma(-d, r, 1.0);
    r = fma(r, e, r);
    e = fma(-d, r, 1.0);
    return fma(r, e, r);
}

// 2^t in FP64: 2^k e^((t - k) ln 2), k the nearest integer to t, the
// exponential's Taylor series to degree 10 (|(t - k) ln 2| <= 0.35:
// truncation below 2.2e-13 relative) in fused multiply-adds, scaled exactly.
__device__ SH_CALL double sh_exp2_d(double t) {
    if (t > 200.0) return INFINITY;
    if (t < -200.0) return 0.0;
    const double k = nearbyint(t);
    const double g = (t - k) * kLn2;
    double p = c_inv_fact[10];
    for (int j = 9; j >= 0; --j) p = fma(g, p, c_inv_fact[j]);
    return p * sh_pow2i((int)k);
}

// pow(x, y) for x >= 0: 2^(y log2 x) in FP64, rounded once.  log2 x = e +
// ln(m) / ln 2 with x = m 2^e, m in [sqrt(1/2), sqrt(2)), and ln m =
// 2 atanh(s), s = (m - 1) / (m + 1) (the quotient through sh_rcp_d), summed
// to s^15 in fused multiply-adds.
__device__ SH_CALL float sh_pow(float xf, float yf) {
    if (xf != xf || yf != yf) return NAN;
    if (xf < 0.0f) return NAN;
    if (xf == 0.0f) return yf > 0.0f ? 0.0f : (yf == 0.0f ? 1.0f : INFINITY);
    if (yf == 0.0f || xf == 1.0f) return 1.0f;
    if (isinf(xf)) return yf > 0.0f ? INFINITY : 0.0f;
    // exact cases: x^1 = x, x^(1/2) the correctly rounded square root, and a
    // small positive integer power as FP64 products (square and multiply,
    // at most 12 roundings of 2^-53), rounded once
    if (yf == 1.0f) return xf;
    if (yf == 0.5f) return sqrtf(xf);
    if (yf > 1.0f && yf <= 64.0f && yf == floorf(yf)) {
        int n = (int)yf;
        double b = (double)xf, r = 1.0;
        for (;;) {
            if (n & 1) r = r * b;
            n >>= 1;
            if (n == 0) break;
            b = b * b;
        }
        return (float)r;
    }
    int e;
    double m = frexp((double)xf, &e);  // m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) * sh_rcp_d(m + 1.0);
    const double s2 = s * s;
    double series = c_inv_odd[7];
    for (int j = 6; j >= 0; --j) series = fma(s2, series, c_inv_odd[j]);
    const double lnm = 2.0 * s * series;
    const double t = (double)yf * fma(lnm, kInvLn2, (double)e);
    return (float)sh_exp2_d(t);
}

// e^x = 2^(x / ln 2) in FP64, rounded once
__device__ float sh_exp(float x) {
    if (x != x) return NAN;
    return (float)sh_exp2_d((double)x * kInvLn2);
}

// ---- random numbers (rtcommon.glsl:99-139) ----------------------------------

// TEA with 16 cycles and the shader's key: a hash of (pixel, seed)
__device__ uint32_t sh_tea(uint32_t v0, uint32_t v1) {
    uint32_t s0 = 0;
    for (int n = 0; n < 16; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
// linear congruential step (Numerical Recipes constants), low 24 bits out
__device__ __forceinline__ uint32_t sh_lcg(uint32_t* prev) {
    *prev = 1664525u * *prev + 1013904223u;
    return *prev & 0x00FFFFFFu;
}
__device__ __forceinline__ float sh_randf(uint32_t* prev) { return (float)sh_lcg(prev) / (float)0x01000000; }
__device__ __forceinline__ uint32_t sh_randu(uint32_t* prev, uint32_t a, uint32_t b) {
    return sh_lcg(prev) % (b - a) + a;
}
// base-2 radical inverse by bit reversal
__device__ float sh_radical_inverse(uint32_t bits) {
    bits = (bits << 16) | (bits >> 16);
    bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
    bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
    bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
    bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
    return (float)bits * 2.3283064365386963e-10f;
}

// ---- samplers (rtcommon.glsl:153-179) ----------------------------------------

// cos^exponent lobe about z
__device__ v3 cospow_hemisphere(float exponent, uint32_t* seed, v3 x, v3 y, v3 z) {
    const float phi = 2.0f * kPi * sh_randf(seed);
    const float cos_t = sh_pow(sh_randf(seed), 1.0f / (exponent + 1.0f));
    const float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float sp, cp;
    sh_sincos(phi, &sp, &cp);
    return comb(x, cp * sin_t, y, sp * sin_t, z, cos_t);
}
// uniform point on a triangle, as barycentrics
__device__ v3 triangle_sample(uint32_t* seed) {
    const float u = sqrtf(sh_randf(seed));
    const float v = sh_randf(seed);
    const float a = u * (1.0f - v);
    const float b = u * v;
    return mk(a, b, 1.0f - a - b);
}

// ---- triangles, boxes, frames (rtcommon.glsl:181-251) ------------------------

// the shader's triangle_hit: |det| < EPS misses, u and v in range, t >= 0
__device__ bool triangle_hit(v3 o, v3 d, v3 pa, v3 pb, v3 pc, v3* hitp) {
    const v3 e1 = sub(pb, pa);
    const v3 e2 = sub(pc, pa);
    const v3 p = cross(d, e2);
    const float det = dot(e1, p);
    if (fabsf(det) < kEps) return false;
    const float inv = 1.0f / det;
    const v3 s = sub(o, pa);
    const float u = dot(s, p) * inv;
    if (u < 0.0f || u > 1.0f) return false;
    const v3 q = cross(s, e1);
    const float v = dot(d, q) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    const float t = dot(e2, q) * inv;
    *hitp = add(o, scl(d, t));
    return t >= 0.0f;
}
// solid-angle pdf of d from o under uniform area sampling of the triangle
__device__ SH_CALL float triangle_pdf(v3 o, v3 d, v3 v0, v3 v1, v3 v2) {
    v3 hitp;
    if (triangle_hit(o, d, v0, v1, v2, &hitp)) {
        const float a = 2.0f / length3(cross(sub(v1, v0), sub(v2, v0)));
        const v3 dist = sub(hitp, o);
        const v3 n = normalize3(cross(sub(v1, v0), sub(v2, v0)));
        const float g = dot(dist, dist) / fabsf(dot(n, d));
        return a * g;
    }
    return 0.0f;
}
__device__ void make_tanspace(v3 n, v3* t, v3* b) {
    if (fabsf(n.x) > fabsf(n.y))
        *t = divs(mk(n.z, 0.0f, -n.x), sqrtf(n.x * n.x + n.z * n.z));
    else
        *t = divs(mk(0.0f, -n.z, n.y), sqrtf(n.y * n.y + n.z * n.z));
    *b = cross(n, *t);
}
__device__ __forceinline__ float power_heuristic(float a, float b) { return a * a / (a * a + b * b); }
__device__ __forceinline__ float luma(v3 c) { return 0.299f * c.x + 0.587f * c.y + 0.114f * c.z; }
// slab test, t >= 0; min and max ignore a NaN operand
__device__ bool hit_bbox(v3 o, v3 d, v3 bmin, v3 bmax) {
    const v3 inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    const v3 t0 = mulv(sub(bmin, o), inv);
    const v3 t1 = mulv(sub(bmax, o), inv);
    const v3 tn = mk(fminf(t0.x, t1.x), fminf(t0.y, t1.y), fminf(t0.z, t1.z));
    const v3 tf = mk(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y), fmaxf(t0.z, t1.z));
    const float near_max = fmaxf(fmaxf(tn.x, tn.y), fmaxf(tn.z, 0.0f));
    const float far_min = fminf(fminf(tf.x, tf.y), tf.z);
    return near_max <= far_min;
}

// ---- materials (rtcommon.glsl:253-369) ---------------------------------------

struct MatInfo {
    v3 albedo, emissive;
    float roughness;
    bool use_tanspace;  // the object has a normal texture
    v3 tn;              // its tangent-space normal at the hit
};
struct ShadeInfo {
    v3 wo, t, b, n;
};

// normalised Blinn-Phong lobe, exponent 1 / roughness, as a pdf over wi
__device__ float bp_pdf(const MatInfo& m, const ShadeInfo& sh, v3 wi) {
    const float o_dn = dot(neg(sh.wo), sh.n);
    const float i_dn = dot(wi, sh.n);
    if (o_dn <= 0.0f || i_dn <= 0.0f) return 0.0f;
    const float ex = 1.0f / m.roughness;
    const v3 h = normalize3(sub(wi, sh.wo));
    const float cosine = fmaxf(dot(h, sh.n), 0.0f);
    const float n_pdf = (ex + 1.0f) / (2.0f * kPi) * sh_pow(cosine, ex);
    return n_pdf / (4.0f * dot(neg(sh.wo), h));
}
__device__ v3 bp_eval(const MatInfo& m, const ShadeInfo& sh, v3 wi) { return scl(m.albedo, bp_pdf(m, sh, wi)); }
__device__ bool bp_sample(uint32_t* seed, const MatInfo& m, const ShadeInfo& sh, v3* wi) {
    const float ex = 1.0f / m.roughness;
    const v3 h = cospow_hemisphere(ex, seed, sh.t, sh.b, sh.n);
    *wi = reflect3(sh.wo, h);
    return dot(*wi, sh.n) > 0.0f;
}
// GGX with Schlick Fresnel and the Smith joint visibility; a2 = roughness^2
__device__ v3 ggx_f(v3 r0, float i_dn) {
    const float c5 = sh_pow(1.0f - i_dn, 5.0f);
    return mk(r0.x + (1.0f - r0.x) * c5, r0.y + (1.0f - r0.y) * c5, r0.z + (1.0f - r0.z) * c5);
}
__device__ float ggx_g(float o_dn, float i_dn, float a2) {
    const float sq0 = sqrtf(a2 + (1.0f - a2) * i_dn * i_dn);
    const float sq1 = sqrtf(a2 + (1.0f - a2) * o_dn * o_dn);
    return 2.0f * o_dn * i_dn / (o_dn * sq0 + i_dn * sq1);
}
__device__ float ggx_d(float n_dh, float a2) {
    const float b = n_dh * n_dh * (a2 - 1.0f) + 1.0f;
    return a2 / (kPi * b * b);
}
__device__ float ggx_pdf(const MatInfo& m, const ShadeInfo& sh, v3 wi) {
    const float o_dn = dot(neg(sh.wo), sh.n);
    const float i_dn = dot(wi, sh.n);
    if (o_dn <= 0.0f || i_dn <= 0.0f) return 0.0f;
    const v3 h = normalize3(sub(wi, sh.wo));
    const float n_dh = fmaxf(dot(h, sh.n), 0.0f);
    const float o_dh = fmaxf(dot(wi, h), 0.0f);
    const float a2 = m.roughness * m.roughness;
    return ggx_d(n_dh, a2) * n_dh / (4.0f * o_dh);
}
__device__ v3 ggx_eval(const MatInfo& m, const ShadeInfo& sh, v3 wi) {
    const float o_dn = dot(neg(sh.wo), sh.n);
    const float i_dn = dot(wi, sh.n);
    if (o_dn <= 0.0f || i_dn <= 0.0f) return mk(0.0f, 0.0f, 0.0f);
    const v3 h = normalize3(sub(wi, sh.wo));
    const float n_dh = fmaxf(dot(h, sh.n), 0.0f);
    const float a2 = m.roughness * m.roughness;
    const v3 f = ggx_f(m.albedo, i_dn);
    const float d = ggx_d(n_dh, a2);
    const float g = ggx_g(o_dn, i_dn, a2);
    const float den = 4.0f * o_dn;
    return mk(f.x * d * g / den, f.y * d * g / den, f.z * d * g / den);
}
__device__ bool ggx_sample(uint32_t* seed, const MatInfo& m, const ShadeInfo& sh, v3* wi) {
    const float a2 = m.roughness * m.roughness;
    const float xi_x = sh_randf(seed);
    const float xi_y = sh_randf(seed);
    const float phi = 2.0f * kPi * xi_x;
    const float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (a2 - 1.0f) * xi_y));
    const float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float sp, cp;
    sh_sincos(phi, &sp, &cp);
    const v3 h = comb(sh.t, cp * sin_t, sh.b, sp * sin_t, sh.n, cos_t);
    *wi = reflect3(sh.wo, h);
    return dot(*wi, sh.n) > 0.0f;
}
__device__ SH_CALL float mat_pdf(int brdf, const MatInfo& m, const ShadeInfo& sh, v3 wi) {
    return brdf == 0 ? bp_pdf(m, sh, wi) : ggx_pdf(m, sh, wi);
}
__device__ SH_CALL v3 mat_eval(int brdf, const MatInfo& m, const ShadeInfo& sh, v3 wi) {
    return brdf == 0 ? bp_eval(m, sh, wi) : ggx_eval(m, sh, wi);
}
__device__ SH_CALL bool mat_sample(int brdf, uint32_t* seed, const MatInfo& m, const ShadeInfo& sh, v3* wi) {
    return brdf == 0 ? bp_sample(seed, m, sh, wi) : ggx_sample(seed, m, sh, wi);
}

// ---- scene -------------------------------------------------------------------

// A light: an object with an emission component above zero, its triangle
// range and world box (rt.cpp:47-58).
struct LightRec {
    int32_t obj;
    int32_t count;
    int64_t first;
    float bmin[3], bmax[3];
};

struct ShadeArgs {
    const void* nodes;     // the scene's wide BVH (world-space triangles)
    const TriRec* recs;
    int32_t root;
    const float* verts;    // nt x 9
    const float* normals;  // nt x 9
    const int32_t* obj;    // nt
    const float* albedo;   // nobj x 3
    const float* emissive; // nobj x 3
    const float* metal_rough;  // nobj x 2
    // textures (all NULL / 0 without): per-vertex (u, v) and tangents
    // (xyz, w), per object the texture index of each factor, and the
    // decoded (linear) texels of every texture
    const float* texcoords;   // nt x 6
    const float* tangents;    // nt x 12
    const int32_t* obj_tex;   // nobj x 4: albedo, emissive, metal_rough, normal, or -1
    const int32_t* tex_size;  // ntex x 2: width, height
    const int64_t* tex_off;   // ntex + 1 texel offsets
    const float4* texels;
    const LightRec* lights;
    uint32_t n_lights;
    cp_shade_camera cam;
    cp_shade_params p;
    float prev_pv[16];
    int has_pv;
    const float* prev_gbuf;
    const cp_shade_reservoir* prev_res;
    cp_shade_reservoir* out_res;
    float* image;
    float* gbuf;
    uint32_t* status;
};

struct HitRec {
    bool hit;
    int32_t tri;
    float u, v;
};

// The scene tracer: the nearest hit with t in [tmin, tmax] (ties to the
// least triangle index), or with `any` whether there is one.
template <int K>
__device__ SH_CALL HitRec trace(const ShadeArgs& a, v3 o, v3 d, float tmin, float tmax, bool any, int32_t* stack) {
    float bt = INFINITY, bu = 0.0f, bv = 0.0f;
    int bidx = INT_MAX;
    const bool found = raywalk::ray_walk<K>(static_cast<const WideNode<K>*>(a.nodes), a.recs, a.root, o.x, o.y, o.z,
                                            d.x, d.y, d.z, tmin, tmax, 0.0f, any, stack, a.status, bt, bidx, bu, bv);
    HitRec h;
    h.hit = found;
    h.tri = found ? bidx : -1;
    h.u = found ? bu : 0.0f;
    h.v = found ? bv : 0.0f;
    return h;
}

__device__ __forceinline__ v3 vert(const ShadeArgs& a, int64_t t, int j) { return ld(a.verts + 9 * t + 3 * j); }
__device__ __forceinline__ v3 nrm(const ShadeArgs& a, int64_t t, int j) { return ld(a.normals + 9 * t + 3 * j); }

// visibility(a, b): whether something lies between (rt.rgen:271-289)
template <int K>
__device__ bool occluded(const ShadeArgs& a, v3 pa, v3 pb, int32_t* stack) {
    const v3 dir = sub(pb, pa);
    const float d = length3(dir);
    return trace<K>(a, pa, divs(dir, d), kEps, d - kEps, true, stack).hit;
}

// ---- textures (rt.rgen:97-129; images RGBA8 sRGB, linear filter, repeat) ----

// x mod 1 in [0, 1); NaN, the infinities and a difference that rounds up to
// 1 give 0
__device__ __forceinline__ float wrap01(float x) {
    float f = x - floorf(x);
    if (!(f >= 0.0f && f < 1.0f)) f = 0.0f;
    return f;
}
// the engine's texture(): bilinear blend at level 0 of the four decoded
// texels around (u mod 1) w - 1/2, (v mod 1) h - 1/2, neighbours wrapping
// around the edges; the same operations in the same order as the
// restatement
__device__ SH_CALL float4 tex_sample(const ShadeArgs& a, int32_t tex, float u, float v) {
    const int32_t w = a.tex_size[2 * tex], h = a.tex_size[2 * tex + 1];
    const float4* t = a.texels + a.tex_off[tex];
    const float fx = wrap01(u) * (float)w - 0.5f, fy = wrap01(v) * (float)h - 0.5f;
    const float x0 = floorf(fx), y0 = floorf(fy);
    const float ax = fx - x0, ay = fy - y0;
    int i0 = (int)x0, j0 = (int)y0;  // in [-1, w - 1] and [-1, h - 1]
    if (i0 < 0) i0 = w - 1;
    if (j0 < 0) j0 = h - 1;
    const int i1 = i0 + 1 == w ? 0 : i0 + 1, j1 = j0 + 1 == h ? 0 : j0 + 1;
    const float4 t00 = t[(int64_t)j0 * w + i0], t10 = t[(int64_t)j0 * w + i1];
    const float4 t01 = t[(int64_t)j1 * w + i0], t11 = t[(int64_t)j1 * w + i1];
    const float bx = 1.0f - ax, by = 1.0f - ay;
    float4 r;
    r.x = (t00.x * bx + t10.x * ax) * by + (t01.x * bx + t11.x * ax) * ay;
    r.y = (t00.y * bx + t10.y * ax) * by + (t01.y * bx + t11.y * ax) * ay;
    r.z = (t00.z * bx + t10.z * ax) * by + (t01.z * bx + t11.z * ax) * ay;
    r.w = (t00.w * bx + t10.w * ax) * by + (t01.w * bx + t11.w * ax) * ay;
    return r;
}
__device__ __forceinline__ int32_t obj_tex(const ShadeArgs& a, int32_t o, int k) {
    return a.obj_tex ? a.obj_tex[4 * o + k] : -1;
}
__device__ __forceinline__ float tcd(const ShadeArgs& a, int64_t t, int j, int k) {
    return a.texcoords ? a.texcoords[6 * t + 2 * j + k] : 0.0f;
}
__device__ __forceinline__ v3 tng(const ShadeArgs& a, int64_t t, int j) {
    if (!a.tangents) return mk(0.0f, 0.0f, 0.0f);
    const float* q = a.tangents + 12 * t + 4 * j;
    return scl(ld(q), q[3]);
}

struct HitInfo {
    v3 pos, normal;
    float tc[2];           // texture coordinates (scenes with textures)
    int32_t tri;           // for the tangent, which only a normal map reads
    float bx, by, bz;
};
// interpolated world position, unit normal and texture coordinates at a hit
// (rt.rgen:62-95; identity model matrices for world-space triangles); the
// unit tangent comes from hit_tangent where a normal map needs it
__device__ HitInfo make_hit_info(const ShadeArgs& a, const HitRec& h) {
    const float bx = 1.0f - h.u - h.v, by = h.u, bz = h.v;
    HitInfo r;
    r.normal = normalize3(comb(nrm(a, h.tri, 0), bx, nrm(a, h.tri, 1), by, nrm(a, h.tri, 2), bz));
    r.pos = comb(vert(a, h.tri, 0), bx, vert(a, h.tri, 1), by, vert(a, h.tri, 2), bz);
    r.tc[0] = r.tc[1] = 0.0f;
    if (a.obj_tex)
        for (int k = 0; k < 2; ++k)
            r.tc[k] = tcd(a, h.tri, 0, k) * bx + tcd(a, h.tri, 1, k) * by + tcd(a, h.tri, 2, k) * bz;
    r.tri = h.tri;
    r.bx = bx;
    r.by = by;
    r.bz = bz;
    return r;
}
__device__ __forceinline__ v3 hit_tangent(const ShadeArgs& a, const HitInfo& h) {
    return normalize3(comb(tng(a, h.tri, 0), h.bx, tng(a, h.tri, 1), h.by, tng(a, h.tri, 2), h.bz));
}
// material of the hit object at texture coordinates tc: each factor, or its
// texture where the object has one (rt.rgen:97-129)
__device__ MatInfo make_mat_info(const ShadeArgs& a, int32_t o, const float* tc) {
    MatInfo m;
    m.albedo = ld(a.albedo + 3 * o);
    if (obj_tex(a, o, 0) >= 0) {
        const float4 t = tex_sample(a, obj_tex(a, o, 0), tc[0], tc[1]);
        m.albedo = mk(t.x, t.y, t.z);
    }
    m.emissive = ld(a.emissive + 3 * o);
    if (obj_tex(a, o, 1) >= 0) {
        const float4 t = tex_sample(a, obj_tex(a, o, 1), tc[0], tc[1]);
        m.emissive = mk(t.x, t.y, t.z);
    }
    float metal = a.metal_rough[2 * o], rough = a.metal_rough[2 * o + 1];
    if (obj_tex(a, o, 2) >= 0) {
        const float4 t = tex_sample(a, obj_tex(a, o, 2), tc[0], tc[1]);
        metal = t.x;
        rough = t.y;
    }
    m.roughness = rough;
    if (a.p.use_metalness)  // mix(vec3(0.04), albedo, metal)
        m.albedo = mk(0.04f * (1.0f - metal) + m.albedo.x * metal, 0.04f * (1.0f - metal) + m.albedo.y * metal,
                      0.04f * (1.0f - metal) + m.albedo.z * metal);
    m.use_tanspace = obj_tex(a, o, 3) >= 0;
    m.tn = mk(0.0f, 0.0f, 0.0f);
    if (m.use_tanspace) {  // texture(...).xyz * 2.0 - 1.0
        const float4 t = tex_sample(a, obj_tex(a, o, 3), tc[0], tc[1]);
        m.tn = mk(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f);
    }
    return m;
}
// shading frame facing the incoming ray, the normal bent by the normal map
// when it is on (rt.rgen:131-148)
__device__ ShadeInfo make_shade_info(const ShadeArgs& a, v3 wo, const HitInfo& hit, const MatInfo& m) {
    ShadeInfo sh;
    sh.wo = wo;
    v3 normal = hit.normal;
    if (dot(sh.wo, normal) > 0.0f) normal = neg(normal);
    sh.n = normal;
    if (m.use_tanspace && a.p.use_normal_map == 1) {  // N = normalize(mat3(T, B, N) * tn)
        sh.t = hit_tangent(a, hit);
        sh.b = cross(sh.n, sh.t);
        sh.n = normalize3(add(add(scl(sh.t, m.tn.x), scl(sh.b, m.tn.y)), scl(sh.n, m.tn.z)));
    }
    make_tanspace(sh.n, &sh.t, &sh.b);
    return sh;
}

struct LightSample {
    v3 pos, normal, emissive;
    float pdf;
};
// a point on a uniformly chosen triangle of a uniformly chosen light (rt.rgen:150-194)
__device__ SH_CALL LightSample light_sample(const ShadeArgs& a, uint32_t* seed, v3 p) {
    const uint32_t li = sh_randu(seed, 0, a.n_lights);
    const LightRec& L = a.lights[li];
    const uint32_t n_tris = (uint32_t)L.count;
    const uint32_t ti = sh_randu(seed, 0, n_tris);
    const int64_t t = L.first + ti;
    const v3 v0 = vert(a, t, 0), v1 = vert(a, t, 1), v2 = vert(a, t, 2);
    const v3 bary = triangle_sample(seed);
    LightSample r;
    r.pos = comb(v0, bary.x, v1, bary.y, v2, bary.z);
    r.emissive = ld(a.emissive + 3 * L.obj);
    if (obj_tex(a, L.obj, 1) >= 0) {
        // the shader's coordinates: u interpolated, v vertex 1's at every
        // corner (rt.rgen:175)
        const float tu = tcd(a, t, 0, 0) * bary.x + tcd(a, t, 1, 0) * bary.y + tcd(a, t, 2, 0) * bary.z;
        const float tv = tcd(a, t, 1, 1) * bary.x + tcd(a, t, 1, 1) * bary.y + tcd(a, t, 1, 1) * bary.z;
        const float4 e = tex_sample(a, obj_tex(a, L.obj, 1), tu, tv);
        r.emissive = mk(e.x, e.y, e.z);
    }
    const v3 narea = cross(sub(v1, v0), sub(v2, v0));
    const float ar = 2.0f / length3(narea);
    const v3 dist = sub(r.pos, p);
    const v3 n = normalize3(narea);
    const v3 d = normalize3(dist);
    const float g = dot(dist, dist) / fabsf(dot(n, d));
    r.normal = n;
    r.pdf = ar * g / (float)(n_tris * a.n_lights);
    return r;
}
// direction to a uniform point on a uniformly chosen light triangle (rt.rgen:196-220)
__device__ SH_CALL v3 light_sample_dir(const ShadeArgs& a, uint32_t* seed, v3 p) {
    const uint32_t li = sh_randu(seed, 0, a.n_lights);
    const LightRec& L = a.lights[li];
    const uint32_t ti = sh_randu(seed, 0, (uint32_t)L.count);
    const int64_t t = L.first + ti;
    const v3 bary = triangle_sample(seed);
    const v3 pt = comb(vert(a, t, 0), bary.x, vert(a, t, 1), bary.y, vert(a, t, 2), bary.z);
    return normalize3(sub(pt, p));
}
// brute-force solid-angle pdf of light sampling for direction d (rt.rgen:222-255)
__device__ SH_CALL float light_pdf(const ShadeArgs& a, v3 p, v3 d) {
    float oacc = 0.0f;
    for (uint32_t l = 0; l < a.n_lights; ++l) {
        const LightRec& L = a.lights[l];
        float tacc = 0.0f;
        if (!hit_bbox(p, d, ld(L.bmin), ld(L.bmax))) continue;
        for (int64_t t = L.first; t < L.first + L.count; ++t)
            tacc += triangle_pdf(p, d, vert(a, t, 0), vert(a, t, 1), vert(a, t, 2));
        oacc += tacc / (float)L.count;
    }
    return oacc / (float)a.n_lights;
}

struct TraceInfo {
    v3 o, d, acc, throughput;
    int depth;
    float mis;
};

// emission of what the ray hits first, or the environment (rt.rgen:291-299)
template <int K>
__device__ v3 direct_light(const ShadeArgs& a, v3 o, v3 d, int32_t* stack) {
    const HitRec h = trace<K>(a, o, d, kEps, kLargeDist, false, stack);
    if (!h.hit) return ld(a.p.env);
    const int32_t ob = a.obj[h.tri];
    if (obj_tex(a, ob, 1) < 0) return ld(a.emissive + 3 * ob);  // mat_info's emission, the factor
    const HitInfo hit = make_hit_info(a, h);
    return make_mat_info(a, ob, hit.tc).emissive;
}

// rt.rgen:301-355
template <int K>
__device__ void integrate_mis(const ShadeArgs& a, uint32_t* seed, TraceInfo& tr, const HitInfo& hit,
                              const MatInfo& m, const ShadeInfo& sh, int32_t* stack) {
    const int brdf = a.p.brdf;
    if (any_pos(m.emissive)) {
        tr.acc = add(tr.acc, mulv(scl(tr.throughput, tr.mis), m.emissive));
        tr.depth = a.p.max_depth;
        return;
    }
    tr.o = hit.pos;
    if (m.roughness == 0.0f) {
        tr.d = reflect3(sh.wo, sh.n);
        tr.throughput = mulv(tr.throughput, m.albedo);
        tr.mis = 1.0f;
        return;
    }
    const v3 wi_light = light_sample_dir(a, seed, hit.pos);
    const float pdf_l = light_pdf(a, hit.pos, wi_light);
    if (pdf_l != 0.0f) {
        const float pdf_m = mat_pdf(brdf, m, sh, wi_light);
        const v3 atten = mat_eval(brdf, m, sh, wi_light);
        const v3 weight = scl(divs(atten, pdf_l), power_heuristic(pdf_l, pdf_m));
        tr.acc = add(tr.acc, mulv(mulv(tr.throughput, weight), direct_light<K>(a, hit.pos, wi_light, stack)));
    }
    v3 wi;
    if (!mat_sample(brdf, seed, m, sh, &wi)) {
        tr.depth = a.p.max_depth;
        return;
    }
    const float pdf_m = mat_pdf(brdf, m, sh, wi);
    if (pdf_m != 0.0f) {
        const float pdf_l2 = light_pdf(a, hit.pos, wi);
        const v3 atten = mat_eval(brdf, m, sh, wi);
        tr.throughput = mulv(tr.throughput, divs(atten, pdf_m));
        tr.mis = power_heuristic(pdf_m, pdf_l2);
    } else {
        tr.depth = a.p.max_depth;
        return;
    }
    tr.d = wi;
}

// rt.rgen:357-390
__device__ void integrate_mats(const ShadeArgs& a, uint32_t* seed, TraceInfo& tr, const HitInfo& hit,
                               const MatInfo& m, const ShadeInfo& sh) {
    const int brdf = a.p.brdf;
    if (any_pos(m.emissive)) {
        tr.acc = add(tr.acc, mulv(m.emissive, tr.throughput));
        tr.depth = a.p.max_depth;
        return;
    }
    tr.o = hit.pos;
    if (m.roughness == 0.0f) {
        tr.d = reflect3(sh.wo, sh.n);
        tr.throughput = mulv(tr.throughput, m.albedo);
        return;
    }
    v3 wi;
    if (!mat_sample(brdf, seed, m, sh, &wi)) {
        tr.depth = a.p.max_depth;
        return;
    }
    const float pdf = mat_pdf(brdf, m, sh, wi);
    const v3 atten = mat_eval(brdf, m, sh, wi);
    if (pdf != 0.0f) {
        tr.throughput = mulv(tr.throughput, divs(atten, pdf));
    } else {
        tr.depth = a.p.max_depth;
        return;
    }
    tr.d = wi;
}

// rt.rgen:392-412
template <int K>
__device__ void integrate_direct(const ShadeArgs& a, uint32_t* seed, TraceInfo& tr, const HitInfo& hit,
                                 const MatInfo& m, const ShadeInfo& sh, int32_t* stack) {
    tr.depth = a.p.max_depth;
    if (any_pos(m.emissive)) {
        tr.acc = add(tr.acc, m.emissive);
        return;
    }
    if (m.roughness != 0.0f) {
        const LightSample L = light_sample(a, seed, hit.pos);
        const v3 wi = normalize3(sub(L.pos, hit.pos));
        const v3 atten = mat_eval(a.p.brdf, m, sh, wi);
        if (L.pdf != 0.0f) {
            const float shadow = occluded<K>(a, hit.pos, L.pos, stack) ? 0.0f : 1.0f;
            tr.acc = add(tr.acc, scl(mulv(divs(atten, L.pdf), L.emissive), shadow));
        }
    }
}

// ---- ReSTIR (restir.glsl; rt.rgen:414-548) -------------------------------------

struct Reservoir {
    v3 pos, normal, emissive;
    float w_sum, w;
    uint32_t n_seen;
};
__device__ Reservoir res_new() {
    Reservoir r;
    r.pos = r.normal = r.emissive = mk(0.0f, 0.0f, 0.0f);
    r.w_sum = r.w = 0.0f;
    r.n_seen = 0;
    return r;
}
__device__ Reservoir res_load(const cp_shade_reservoir& o) {
    Reservoir r;
    r.pos = ld(o.pos);
    r.normal = ld(o.normal);
    r.emissive = ld(o.emissive);
    r.w_sum = o.w_sum;
    r.w = o.w;
    r.n_seen = o.n_seen;
    return r;
}
__device__ void res_store(const Reservoir& r, cp_shade_reservoir& o) {
    o.pos[0] = r.pos.x; o.pos[1] = r.pos.y; o.pos[2] = r.pos.z;
    o.normal[0] = r.normal.x; o.normal[1] = r.normal.y; o.normal[2] = r.normal.z;
    o.emissive[0] = r.emissive.x; o.emissive[1] = r.emissive.y; o.emissive[2] = r.emissive.z;
    o.w_sum = r.w_sum;
    o.w = r.w;
    o.n_seen = r.n_seen;
}

// A point projected into the previous frame (rt.rgen:459-461, 648-650): false
// unless it lands inside the image; then uv holds its image coordinates and g
// the previous first-hit buffer's nearest texel (repeat addressing; zeros
// without a buffer).
__device__ bool prev_texel(const ShadeArgs& a, v3 pos, float uv[2], float g[9]) {
    float pp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (a.has_pv) {
        const float* M = a.prev_pv;
        for (int i = 0; i < 4; ++i) pp[i] = M[4 * i] * pos.x + M[4 * i + 1] * pos.y + M[4 * i + 2] * pos.z + M[4 * i + 3];
    }
    pp[0] = pp[0] / pp[3];
    pp[1] = pp[1] / pp[3];
    pp[0] = (pp[0] + 1.0f) * 0.5f;
    pp[1] = (pp[1] + 1.0f) * 0.5f;
    if (!(pp[0] > 0.0f && pp[1] > 0.0f && pp[0] < 1.0f && pp[1] < 1.0f)) return false;
    const int W = a.cam.width, H = a.cam.height;
    const int tx = (int)floorf(pp[0] * (float)W) % W, ty = (int)floorf(pp[1] * (float)H) % H;
    for (int k = 0; k < 9; ++k) g[k] = a.prev_gbuf ? a.prev_gbuf[9 * ((int64_t)ty * W + tx) + k] : 0.0f;
    uv[0] = pp[0];
    uv[1] = pp[1];
    return true;
}

// The previous frame's reservoir for a hit whose reprojected first hit agrees
// in position, albedo and normal (rt.rgen:457-479); false where the shader
// leaves the reuse.
__device__ bool temporal_reservoir(const ShadeArgs& a, const HitInfo& hit, const MatInfo& m, const ShadeInfo& sh,
                                   Reservoir* prev) {
    float pp[2], g[9];
    if (!prev_texel(a, hit.pos, pp, g)) return false;
    const int W = a.cam.width, H = a.cam.height;
    const v3 pd = sub(ld(g), hit.pos);
    if (dot(pd, pd) > 0.01f) return false;
    const v3 ad = sub(ld(g + 6), m.albedo);
    if (dot(ad, ad) > 0.01f) return false;
    if (dot(ld(g + 3), sh.n) < 0.5f) return false;
    int fx = (int)(pp[0] * (float)W), fy = (int)(pp[1] * (float)H);
    fx = fx < W ? fx : W - 1;
    fy = fy < H ? fy : H - 1;
    *prev = a.prev_res ? res_load(a.prev_res[(int64_t)fy * W + fx]) : res_new();
    return true;
}

__device__ void res_update(uint32_t* seed, Reservoir& r, float weight, v3 pos, v3 normal, v3 emissive) {
    r.n_seen++;
    r.w_sum += weight;
    if (sh_randf(seed) < weight / r.w_sum) {
        r.pos = pos;
        r.normal = normal;
        r.emissive = emissive;
    }
}

__device__ float update_weight(const ShadeArgs& a, Reservoir& r, const HitInfo& hit, const MatInfo& m,
                               const ShadeInfo& sh) {
    if (r.n_seen == 0) {
        r.w = 0.0f;
        return 0.0f;
    }
    const v3 dir = sub(r.pos, hit.pos);
    const v3 wi = normalize3(dir);
    const v3 atten = mat_eval(a.p.brdf, m, sh, wi);
    const float g = fabsf(dot(r.normal, wi)) / dot(dir, dir);
    const v3 contrib = mulv(scl(atten, g), r.emissive);
    const float p_hat = luma(contrib);
    r.w = (1.0f / p_hat) * (r.w_sum / (float)r.n_seen);
    if (p_hat == 0.0f) r.w = 0.0f;
    return p_hat;
}

// rt.rgen:425-507: candidates, then reuse of the previous frame's reservoir
// (first sample, temporal reuse on) or of this pixel's previous sample
template <int K>
__device__ void reservoir_sample(const ShadeArgs& a, uint32_t* seed, TraceInfo& tr, const HitInfo& hit,
                                 const MatInfo& m, const ShadeInfo& sh, Reservoir& prev, bool first, int32_t* stack) {
    Reservoir nr = res_new();
    for (int i = 0; i < a.p.new_samples; ++i) {
        const LightSample L = light_sample(a, seed, hit.pos);
        const v3 wi = normalize3(sub(L.pos, hit.pos));
        const v3 atten = mat_eval(a.p.brdf, m, sh, wi);
        const v3 contrib = divs(mulv(atten, L.emissive), L.pdf);
        res_update(seed, nr, luma(contrib), L.pos, L.normal, L.emissive);
    }
    const float new_p = update_weight(a, nr, hit, m, sh);
    if (new_p != 0.0f && occluded<K>(a, hit.pos, nr.pos, stack)) nr.w = 0.0f;
    if (!(first && a.p.use_temporal && !temporal_reservoir(a, hit, m, sh, &prev))) {
        Reservoir tres = res_new();
        res_update(seed, tres, new_p * nr.w * (float)nr.n_seen, nr.pos, nr.normal, nr.emissive);
        const float old_p = update_weight(a, prev, hit, m, sh);
        const uint32_t cap = (uint32_t)a.p.temporal_multiplier * nr.n_seen;
        prev.n_seen = cap < prev.n_seen ? cap : prev.n_seen;
        res_update(seed, tres, old_p * prev.w * (float)prev.n_seen, prev.pos, prev.normal, prev.emissive);
        tres.n_seen = nr.n_seen + prev.n_seen;
        (void)update_weight(a, tres, hit, m, sh);
        nr = tres;
    }
    if (nr.w != 0.0f) {
        const v3 dir = sub(nr.pos, hit.pos);
        const v3 wi = normalize3(dir);
        const v3 atten = mat_eval(a.p.brdf, m, sh, wi);
        const v3 contrib = mulv(atten, nr.emissive);
        const float g = fabsf(dot(nr.normal, wi)) / dot(dir, dir);
        tr.acc = add(tr.acc, scl(scl(contrib, nr.w), g));
    }
    prev = nr;
}

// rt.rgen:509-548
template <int K>
__device__ void integrate_restir(const ShadeArgs& a, uint32_t* seed, TraceInfo& tr, const HitInfo& hit,
                                 const MatInfo& m, const ShadeInfo& sh, bool d_only, Reservoir& prev, bool first,
                                 int32_t* stack) {
    const int brdf = a.p.brdf;
    if (any_pos(m.emissive)) {
        tr.acc = add(tr.acc, scl(mulv(m.emissive, tr.throughput), tr.mis));
        tr.depth = a.p.max_depth;
        return;
    }
    tr.o = hit.pos;
    if (m.roughness == 0.0f) {
        tr.d = reflect3(sh.wo, sh.n);
        tr.throughput = mulv(tr.throughput, m.albedo);
        tr.mis = 1.0f;
    } else {
        if (tr.depth == 0) reservoir_sample<K>(a, seed, tr, hit, m, sh, prev, first, stack);
        v3 wi;
        if (!mat_sample(brdf, seed, m, sh, &wi)) {
            tr.depth = a.p.max_depth;
            return;
        }
        const float pdf = mat_pdf(brdf, m, sh, wi);
        if (pdf != 0.0f) {
            const v3 atten = mat_eval(brdf, m, sh, wi);
            tr.throughput = mulv(tr.throughput, divs(atten, pdf));
            tr.mis = tr.depth == 0 ? 0.0f : 1.0f;
        } else {
            tr.depth = a.p.max_depth;
            return;
        }
        tr.d = wi;
    }
    if (d_only) tr.depth = a.p.max_depth;
}

// camera ray of sample s through pixel (x, y) (rt.rgen:550-565); the camera
// frame stands for the inverse view and projection, row 0 at the top
__device__ v3 camera_ray(const cp_shade_camera& cam, const cp_shade_params& p, uint32_t* seed, int s, int x, int y) {
    float jx, jy;
    if (p.qmc == 0) {
        if (p.frame == 0) {
            jx = 0.5f;
            jy = 0.5f;
        } else {
            jx = sh_randf(seed);
            jy = sh_randf(seed);
        }
    } else {
        const uint32_t i = (uint32_t)(s + p.samples * p.frame), n = (uint32_t)(p.samples * p.max_frame);
        jx = (float)i / (float)n;
        jy = sh_radical_inverse(i);
    }
    const float ux = ((float)x + jx) / (float)cam.width;
    const float uy = ((float)y + jy) / (float)cam.height;
    const float nx = ux * 2.0f - 1.0f, ny = uy * 2.0f - 1.0f;
    const v3 r = ld(cam.right), u = ld(cam.up), f = ld(cam.fwd);
    const float sx = nx * (cam.tan_half_y * cam.aspect), sy = -(ny * cam.tan_half_y);
    return normalize3(comb(r, sx, u, sy, f, 1.0f));
}

// rt.rgen:567-677, one thread per pixel; blocks of 16 x 16 pixels; one
// kernel per integrator (kIntegrator), so a launch's instruction stream
// holds only its own integrator's code and spills less.  Eight blocks per SM
// (32 registers a thread, the rest spilled to local memory that stays in
// L1): a warp's paths diverge across bounces, materials and ray walks, and
// it is the number of resident warps, not the spills, that sets the pace.
// The 1920 x 1440 MIS frame, one kernel for all integrators: 395 ms at 2
// blocks per SM (128 registers), 321 ms at 4, 287 ms at 5, 281 ms at 6, 286
// ms at 8 (239 ms at 6 with pow's exact cases); one kernel per integrator:
// 236 ms at 4, 207 at 5, 194 at 6, 188 at 7 and 8 (ReSTIR 262, 236, 223,
// 217, 217).
template <int K, int kIntegrator>
__global__ void __launch_bounds__(256, 8) k_shade(ShadeArgs a) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15);
    const int y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= a.cam.width || y >= a.cam.height) return;
    int32_t stack[raywalk::kRayStack];
    const cp_shade_params& p = a.p;
    uint32_t seed = sh_tea((uint32_t)(y * a.cam.width + x), p.seed);
    v3 acc = mk(0.0f, 0.0f, 0.0f);
    const v3 eye = ld(a.cam.eye);
    v3 g_pos = mk(0, 0, 0), g_norm = mk(0, 0, 0), g_alb = mk(0, 0, 0);
    Reservoir prev = res_new();
    for (int smp = 0; smp < p.samples; ++smp) {
        TraceInfo tr;
        tr.o = eye;
        tr.d = camera_ray(a.cam, p, &seed, smp, x, y);
        tr.acc = mk(0, 0, 0);
        tr.throughput = mk(1, 1, 1);
        tr.depth = 0;
        tr.mis = 1.0f;
        for (; tr.depth < p.max_depth; tr.depth++) {
            const HitRec h = trace<K>(a, tr.o, tr.d, kEps, kLargeDist, false, stack);
            if (!h.hit) {
                if (tr.depth == 0)
                    tr.acc = ld(p.clear);
                else
                    tr.acc = add(tr.acc, mulv(ld(p.env), tr.throughput));
                break;
            }
            const HitInfo hit = make_hit_info(a, h);
            const MatInfo m = make_mat_info(a, a.obj[h.tri], hit.tc);
            const ShadeInfo sh = make_shade_info(a, tr.d, hit, m);
            if (smp == 0 && tr.depth == 0) {
                g_pos = hit.pos;
                g_norm = sh.n;
                g_alb = m.albedo;
            }
            if constexpr (kIntegrator == 0) integrate_direct<K>(a, &seed, tr, hit, m, sh, stack);
            else if constexpr (kIntegrator == 1) integrate_mats(a, &seed, tr, hit, m, sh);
            else if constexpr (kIntegrator == 2) integrate_mis<K>(a, &seed, tr, hit, m, sh, stack);
            else if constexpr (kIntegrator == 3)
                integrate_restir<K>(a, &seed, tr, hit, m, sh, true, prev, smp == 0, stack);
            else
                integrate_restir<K>(a, &seed, tr, hit, m, sh, false, prev, smp == 0, stack);
            if (p.use_rr) {
                const float pc =
                    fminf(fmaxf(tr.throughput.x, fmaxf(tr.throughput.y, tr.throughput.z)) + 0.001f, 0.95f);
                if (sh_randf(&seed) >= pc) break;
                tr.throughput = divs(tr.throughput, pc);
            }
        }
        acc = add(acc, tr.acc);
    }
    const int64_t pix = (int64_t)y * a.cam.width + x;
    if (kIntegrator >= 3 && a.out_res) res_store(prev, a.out_res[pix]);
    const v3 avg = divs(acc, (float)p.samples);
    float* out = a.image + 3 * pix;
    if (p.frame > 0) {  // mix(old, avg, 1 / (frame + 1))
        const float w = 1.0f / (float)(p.frame + 1);
        out[0] = out[0] * (1.0f - w) + avg.x * w;
        out[1] = out[1] * (1.0f - w) + avg.y * w;
        out[2] = out[2] * (1.0f - w) + avg.z * w;
    } else {
        out[0] = avg.x;
        out[1] = avg.y;
        out[2] = avg.z;
    }
    if (p.debug_view > 0) {  // the previous frame's buffers, reprojected (rt.rgen:647-671)
        float uv[2], g[9];
        if (dot(g_norm, g_norm) > 0.5f && prev_texel(a, g_pos, uv, g)) {
            if (p.debug_view <= 3)
                for (int k = 0; k < 3; ++k) out[k] = g[3 * (p.debug_view - 1) + k];
        } else {
            out[0] = out[1] = out[2] = 0.0f;
        }
    }
    if (a.gbuf) {
        float* gb = a.gbuf + 9 * pix;
        const float g[9] = {g_pos.x, g_pos.y, g_pos.z, g_norm.x, g_norm.y, g_norm.z, g_alb.x, g_alb.y, g_alb.z};
        for (int k = 0; k < 9; ++k) gb[k] = g[k];
    }
}

// ---- tone mapping (tonemap.frag) ---------------------------------------------

// Hable's filmic curve with the shader's constants (tonemap.frag:16-25)
__device__ float filmic(float c) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((c * (A * c + C * B) + D * E) / (c * (A * c + B) + D * F)) - E / F;
}
// type 0 filmic (tonemap.frag:27-31), 1 exponential (:33-37), 2 none
__global__ void k_tonemap(int type, float exposure, float gamma, int64_t n, const float* __restrict__ in,
                          float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c = in[i];
    float r = c;
    if (type == 0) {
        const float w = 1.0f / filmic(11.2f);
        r = sh_pow(filmic(c * exposure) * w, 1.0f / gamma);
    } else if (type == 1) {
        r = sh_pow(1.0f - sh_exp(-c * exposure), 1.0f / gamma);
    }
    out[i] = r;
}

// ---- host side -------------------------------------------------------------------

__global__ void k_soup_indices(int32_t* tris, int64_t nt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3 * nt) tris[i] = (int32_t)i;
}

}  // namespace
}  // namespace cpq

struct cp_shade_scene {
    cp_mesh* mesh = nullptr;   // BVH over the world-space triangles, in scene order
    int64_t nt = 0;
    int32_t nobj = 0;
    float* verts = nullptr;    // device copies
    float* normals = nullptr;
    int32_t* obj = nullptr;
    float* albedo = nullptr;
    float* emissive = nullptr;
    float* metal_rough = nullptr;
    cpq::LightRec* lights = nullptr;
    uint32_t n_lights = 0;
    // textures (cp_shade_scene_textures)
    float* texcoords = nullptr;
    float* tangents = nullptr;
    int32_t* obj_tex = nullptr;
    int32_t* tex_size = nullptr;
    int64_t* tex_off = nullptr;
    float4* texels = nullptr;
    int32_t ntex = 0;
};

namespace {

void free_scene(cp_shade_scene* s) {
    if (!s) return;
    cp_mesh_destroy(s->mesh);
    cudaFree(s->verts);
    cudaFree(s->normals);
    cudaFree(s->obj);
    cudaFree(s->albedo);
    cudaFree(s->emissive);
    cudaFree(s->metal_rough);
    cudaFree(s->lights);
    cudaFree(s->texcoords);
    cudaFree(s->tangents);
    cudaFree(s->obj_tex);
    cudaFree(s->tex_size);
    cudaFree(s->tex_off);
    cudaFree(s->texels);
    delete s;
}

template <typename T>
cudaError_t dev_copy(T** dst, const T* src, size_t count, cudaStream_t st) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return e;
    return count ? cudaMemcpyAsync(*dst, src, sizeof(T) * count, cudaMemcpyDeviceToDevice, st) : cudaSuccess;
}

}  // namespace

extern "C" CP_API cp_status cp_shade_scene_create(const float* verts, const float* normals, const int32_t* obj,
                                                  int64_t nt, const float* albedo, const float* emissive,
                                                  const float* metal_rough, int32_t nobj, cp_stream_t stream,
                                                  cp_shade_scene** out) {
    using namespace cpq;
    if (!out) return set_error(CP_ERROR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (!verts || !normals || !obj || !albedo || !emissive || !metal_rough)
        return set_error(CP_ERROR_INVALID_VALUE, "a scene array is NULL");
    if (nt <= 0 || nobj <= 0) return set_error(CP_ERROR_INVALID_VALUE, "a scene needs a triangle and an object");
    if (nt > (int64_t(1) << 27) - 1) return set_error(CP_ERROR_NOT_SUPPORTED, "more than 2^27 - 1 triangles");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cp_shade_scene* s = new (std::nothrow) cp_shade_scene();
    if (!s) return set_error(CP_ERROR_OUT_OF_MEMORY, "host allocation of the handle failed");
    s->nt = nt;
    s->nobj = nobj;
    auto cuda_fail = [&](cudaError_t e, const char* what) {
        free_scene(s);
        return set_error(e == cudaErrorMemoryAllocation ? CP_ERROR_OUT_OF_MEMORY : CP_ERROR_CUDA,
                         std::string("cp_shade_scene_create: ") + what + ": " + cudaGetErrorString(e));
    };
    // the objects and emissions on the host: validation and the light list
    std::vector<int32_t> h_obj((size_t)nt);
    std::vector<float> h_em((size_t)nobj * 3), h_v((size_t)nt * 9);
    cudaError_t e = cudaMemcpyAsync(h_obj.data(), obj, sizeof(int32_t) * nt, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_em.data(), emissive, sizeof(float) * 3 * nobj, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_v.data(), verts, sizeof(float) * 9 * nt, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "reading the scene");
    for (int64_t t = 0; t < nt; ++t)
        if (h_obj[t] < 0 || h_obj[t] >= nobj) {
            free_scene(s);
            return set_error(CP_ERROR_INVALID_VALUE, "triangle " + std::to_string(t) + " names object " +
                                                         std::to_string(h_obj[t]) + " of " + std::to_string(nobj));
        }
    // every object with an emission component above zero, in object order,
    // with its (contiguous) triangle range and world box (rt.cpp:47-58)
    std::vector<LightRec> lights;
    for (int32_t o = 0; o < nobj; ++o) {
        if (!(h_em[3 * o] > 0.0f || h_em[3 * o + 1] > 0.0f || h_em[3 * o + 2] > 0.0f)) continue;
        int64_t first = -1, count = 0;
        for (int64_t t = 0; t < nt; ++t) {
            if (h_obj[t] != o) continue;
            if (first < 0) first = t;
            if (t != first + count) {
                free_scene(s);
                return set_error(CP_ERROR_INVALID_VALUE,
                                 "the triangles of light object " + std::to_string(o) + " are not contiguous");
            }
            ++count;
        }
        if (count == 0) continue;
        if (count > INT32_MAX) {
            free_scene(s);
            return set_error(CP_ERROR_NOT_SUPPORTED, "a light with more than 2^31 - 1 triangles");
        }
        LightRec r;
        r.obj = o;
        r.count = (int32_t)count;
        r.first = first;
        for (int k = 0; k < 3; ++k) {
            r.bmin[k] = INFINITY;
            r.bmax[k] = -INFINITY;
        }
        for (int64_t t = first; t < first + count; ++t)
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    r.bmin[k] = fminf(r.bmin[k], h_v[9 * t + 3 * j + k]);
                    r.bmax[k] = fmaxf(r.bmax[k], h_v[9 * t + 3 * j + k]);
                }
        lights.push_back(r);
    }
    s->n_lights = (uint32_t)lights.size();
    e = dev_copy(&s->verts, verts, (size_t)nt * 9, st);
    if (e == cudaSuccess) e = dev_copy(&s->normals, normals, (size_t)nt * 9, st);
    if (e == cudaSuccess) e = dev_copy(&s->obj, obj, (size_t)nt, st);
    if (e == cudaSuccess) e = dev_copy(&s->albedo, albedo, (size_t)nobj * 3, st);
    if (e == cudaSuccess) e = dev_copy(&s->emissive, emissive, (size_t)nobj * 3, st);
    if (e == cudaSuccess) e = dev_copy(&s->metal_rough, metal_rough, (size_t)nobj * 2, st);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&s->lights), sizeof(LightRec) * (lights.size() + 1));
    if (e == cudaSuccess && !lights.empty())
        e = cudaMemcpyAsync(s->lights, lights.data(), sizeof(LightRec) * lights.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "device copies");
    // the BVH: a triangle soup over the 3 nt vertices, triangle t = (3t, 3t+1, 3t+2)
    int32_t* tris = nullptr;
    e = cudaMalloc(reinterpret_cast<void**>(&tris), sizeof(int32_t) * 3 * nt);
    if (e != cudaSuccess) return cuda_fail(e, "index allocation");
    k_soup_indices<<<(unsigned)((3 * nt + 255) / 256), 256, 0, st>>>(tris, nt);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        cudaFree(tris);
        return cuda_fail(e, "index kernel");
    }
    cp_build_opts bo;
    cp_build_opts_default(&bo);
    bo.branching = 4;
    bo.leaf_size = 4;
    cp_status cs = cp_mesh_create(s->verts, 3 * nt, 12, tris, nt, &bo, stream, &s->mesh);
    cudaStreamSynchronize(st);
    cudaFree(tris);
    if (cs != CP_SUCCESS) {
        free_scene(s);
        return cs;
    }
    *out = s;
    return CP_SUCCESS;
}

namespace {
// RGBA8 texels to linear floats: sRGB colour through the engine's pow, alpha
// as stored / 255 (the decode of an R8G8B8A8_SRGB image; the restatement
// decodes each texel the same way)
__global__ void k_srgb_decode(const uint8_t* __restrict__ in, int64_t n, float4* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float c[3];
    for (int k = 0; k < 3; ++k) {
        const float x = (float)in[4 * i + k] / 255.0f;
        c[k] = x <= 0.04045f ? x / 12.92f : cpq::sh_pow((x + 0.055f) / 1.055f, 2.4f);
    }
    out[i] = make_float4(c[0], c[1], c[2], (float)in[4 * i + 3] / 255.0f);
}
}  // namespace

extern "C" CP_API cp_status cp_shade_scene_textures(cp_shade_scene* s, const float* texcoords, const float* tangents,
                                                    int32_t ntex, const int32_t* tex_size, const uint8_t* texels,
                                                    const int32_t* obj_tex, cp_stream_t stream) {
    using namespace cpq;
    if (!s) return set_error(CP_ERROR_INVALID_VALUE, "scene is NULL");
    if (ntex < 0) return set_error(CP_ERROR_INVALID_VALUE, "negative texture count");
    if (ntex > 0 && (!tex_size || !texels)) return set_error(CP_ERROR_INVALID_VALUE, "texture sizes or texels are NULL");
    // host checks first: every texture index an object names, every size
    std::vector<int64_t> off((size_t)ntex + 1, 0);
    for (int32_t k = 0; k < ntex; ++k) {
        const int64_t w = tex_size[2 * k], h = tex_size[2 * k + 1];
        if (w <= 0 || h <= 0 || w > (int64_t(1) << 20) || h > (int64_t(1) << 20))
            return set_error(CP_ERROR_INVALID_VALUE, "texture " + std::to_string(k) + " has a size outside 1..2^20");
        off[k + 1] = off[k] + w * h;
    }
    // the decode kernel reads the texels: they must be device memory
    if (ntex > 0) {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, texels) != cudaSuccess ||
            (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)) {
            cudaGetLastError();
            return set_error(CP_ERROR_INVALID_VALUE, "cp_shade_scene_textures: texels must be device memory");
        }
    }
    if (obj_tex)
        for (int64_t i = 0; i < 4 * (int64_t)s->nobj; ++i)
            if (obj_tex[i] < -1 || obj_tex[i] >= ntex)
                return set_error(CP_ERROR_INVALID_VALUE, "object " + std::to_string(i / 4) + " names texture " +
                                                             std::to_string(obj_tex[i]) + " of " + std::to_string(ntex));
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // the new arrays replace the old ones only when all are in place
    cp_shade_scene t;
    auto drop = [&]() {
        cudaFree(t.texcoords);
        cudaFree(t.tangents);
        cudaFree(t.obj_tex);
        cudaFree(t.tex_size);
        cudaFree(t.tex_off);
        cudaFree(t.texels);
    };
    cudaError_t e = cudaSuccess;
    if (texcoords) e = dev_copy(&t.texcoords, texcoords, (size_t)s->nt * 6, st);
    if (e == cudaSuccess && tangents) e = dev_copy(&t.tangents, tangents, (size_t)s->nt * 12, st);
    if (e == cudaSuccess && obj_tex) {
        e = cudaMalloc(reinterpret_cast<void**>(&t.obj_tex), sizeof(int32_t) * 4 * s->nobj);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(t.obj_tex, obj_tex, sizeof(int32_t) * 4 * s->nobj, cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess && ntex > 0) {
        e = cudaMalloc(reinterpret_cast<void**>(&t.tex_size), sizeof(int32_t) * 2 * ntex);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(t.tex_size, tex_size, sizeof(int32_t) * 2 * ntex, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t.tex_off), sizeof(int64_t) * (ntex + 1));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(t.tex_off, off.data(), sizeof(int64_t) * (ntex + 1), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t.texels), sizeof(float4) * off[ntex]);
        if (e == cudaSuccess) {
            k_srgb_decode<<<(unsigned)((off[ntex] + 255) / 256), 256, 0, st>>>(texels, off[ntex], t.texels);
            note_launch();
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        drop();
        t = cp_shade_scene();
        return set_error(e == cudaErrorMemoryAllocation ? CP_ERROR_OUT_OF_MEMORY : CP_ERROR_CUDA,
                         std::string("cp_shade_scene_textures: ") + cudaGetErrorString(e));
    }
    std::swap(s->texcoords, t.texcoords);
    std::swap(s->tangents, t.tangents);
    std::swap(s->obj_tex, t.obj_tex);
    std::swap(s->tex_size, t.tex_size);
    std::swap(s->tex_off, t.tex_off);
    std::swap(s->texels, t.texels);
    s->ntex = ntex;
    drop();  // the previous arrays
    t = cp_shade_scene();
    return CP_SUCCESS;
}

extern "C" CP_API cp_status cp_shade_scene_destroy(cp_shade_scene* s) {
    free_scene(s);
    return CP_SUCCESS;
}

extern "C" CP_API cp_status cp_shade_scene_lights(const cp_shade_scene* s, int32_t* n_lights) {
    if (!s || !n_lights) return cpq::set_error(CP_ERROR_INVALID_VALUE, "scene or out is NULL");
    *n_lights = (int32_t)s->n_lights;
    return CP_SUCCESS;
}

extern "C" CP_API cp_status cp_shade_render(const cp_shade_scene* s, const cp_shade_camera* cam,
                                            const cp_shade_params* p, float* image, float* gbuf,
                                            const float* prev_pv, const float* prev_gbuf,
                                            const cp_shade_reservoir* prev_res, cp_shade_reservoir* out_res,
                                            cp_stream_t stream) {
    using namespace cpq;
    if (!s || !cam || !p || !image) return set_error(CP_ERROR_INVALID_VALUE, "scene, camera, params or image is NULL");
    if (cam->width <= 0 || cam->height <= 0 || p->samples <= 0 || p->max_depth < 0)
        return set_error(CP_ERROR_INVALID_VALUE, "image size, samples and depth must be positive");
    if ((int64_t)cam->width * cam->height > INT32_MAX)
        return set_error(CP_ERROR_NOT_SUPPORTED, "more than 2^31 - 1 pixels");
    if (p->integrator < 0 || p->integrator > 4 || p->brdf < 0 || p->brdf > 1)
        return set_error(CP_ERROR_INVALID_VALUE, "integrator must be 0..4 and brdf 0..1");
    if (p->qmc && p->max_frame <= 0) return set_error(CP_ERROR_INVALID_VALUE, "qmc needs max_frame > 0");
    // every integrator but material sampling samples lights
    if (s->n_lights == 0 && p->integrator != 1)
        return set_error(CP_ERROR_INVALID_VALUE, "the scene has no light (an object with emission above zero)");
    cp_mesh_info_t mi;
    cp_status cs = cp_mesh_info(s->mesh, &mi);
    if (cs != CP_SUCCESS) return cs;
    ShadeArgs a;
    std::memset(&a, 0, sizeof a);
    const Bvh& b = s->mesh->bvh;
    a.nodes = b.nodes;
    a.recs = b.recs;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(&a.root, b.wide_root, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_error(CP_ERROR_CUDA, std::string("cp_shade_render: ") + cudaGetErrorString(e));
    a.verts = s->verts;
    a.normals = s->normals;
    a.obj = s->obj;
    a.albedo = s->albedo;
    a.emissive = s->emissive;
    a.metal_rough = s->metal_rough;
    a.texcoords = s->texcoords;
    a.tangents = s->tangents;
    a.obj_tex = s->obj_tex;
    a.tex_size = s->tex_size;
    a.tex_off = s->tex_off;
    a.texels = s->texels;
    a.lights = s->lights;
    a.n_lights = s->n_lights;
    a.cam = *cam;
    a.p = *p;
    if (prev_pv) {
        std::memcpy(a.prev_pv, prev_pv, sizeof a.prev_pv);
        a.has_pv = 1;
    }
    a.prev_gbuf = prev_gbuf;
    a.prev_res = prev_res;
    a.out_res = out_res;
    a.image = image;
    a.gbuf = gbuf;
    a.status = b.status;
    const dim3 grid((unsigned)((cam->width + 15) / 16), (unsigned)((cam->height + 15) / 16));
    // one kernel per integrator: a launch's instruction stream holds only its
    // own integrator's code
    switch (p->integrator) {
        case 0: k_shade<4, 0><<<grid, 256, 0, st>>>(a); break;
        case 1: k_shade<4, 1><<<grid, 256, 0, st>>>(a); break;
        case 2: k_shade<4, 2><<<grid, 256, 0, st>>>(a); break;
        case 3: k_shade<4, 3><<<grid, 256, 0, st>>>(a); break;
        default: k_shade<4, 4><<<grid, 256, 0, st>>>(a); break;
    }
    note_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CP_ERROR_CUDA, std::string("cp_shade_render: ") + cudaGetErrorString(e));
    return CP_SUCCESS;
}

extern "C" CP_API cp_status cp_shade_tonemap(int32_t type, float exposure, float gamma, int64_t n, const float* in,
                                             float* out, cp_stream_t stream) {
    using namespace cpq;
    if (type < 0 || type > 2 || n < 0) return set_error(CP_ERROR_INVALID_VALUE, "tone map type 0..2, n >= 0");
    if (n == 0) return CP_SUCCESS;
    if (!in || !out) return set_error(CP_ERROR_INVALID_VALUE, "in or out is NULL");
    k_tonemap<<<(unsigned)((n + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(type, exposure, gamma,
                                                                                                n, in, out);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CP_ERROR_CUDA, std::string("cp_shade_tonemap: ") + cudaGetErrorString(e));
    return CP_SUCCESS;
}
