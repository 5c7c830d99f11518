/*
 * shade_oracle.c — ORACLE: test infrastructure only (see shade_oracle.h).
 *
 * FP32 restatement of the reference's shading math, compiled like the rest
 * of the oracle without fast-math and with -ffp-contract=off: every float
 * expression rounds as written, in the shader's left-to-right order.  Each
 * function names the shader lines it restates.
 */
#define _POSIX_C_SOURCE 200809L
#include "shade_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define SH_PI 3.141592f        /* rtcommon.glsl:6 (the shader's truncated constant) */
#define SH_LARGE_DIST 10000000.0f /* rtcommon.glsl:7 */
#define SH_EPS 0.00001f        /* rtcommon.glsl:8 */

typedef struct {
    float x, y, z;
} v3;

static inline v3 mk(float x, float y, float z) {
    v3 r = {x, y, z};
    return r;
}
static inline v3 ld(const float* p) { return mk(p[0], p[1], p[2]); }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scl(v3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 mulv(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 divs(v3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
static inline v3 neg(v3 a) { return mk(-a.x, -a.y, -a.z); }
static inline float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float length3(v3 a) { return sqrtf(dot(a, a)); }
static inline v3 normalize3(v3 a) { return divs(a, length3(a)); }
/* GLSL reflect: I - 2 dot(N, I) N */
static inline v3 reflect3(v3 i, v3 n) { return sub(i, scl(n, 2.0f * dot(n, i))); }
/* x*a + y*b + z*c, summed left to right */
static inline v3 comb(v3 a, float x, v3 b, float y, v3 c, float z) {
    return add(add(scl(a, x), scl(b, y)), scl(c, z));
}
static inline int any_pos(v3 a) { return a.x > 0.0f || a.y > 0.0f || a.z > 0.0f; }

/* ===================================================================== */
/* sin, cos, pow                                                          */
/* ===================================================================== */

/* sin and cos of a float: Cody-Waite reduction by pi/2 in FP64 (one
 * multiply, one round-to-nearest-integer, one multiply-subtract written as
 * two operations), then the Taylor polynomials of sin (to r^9) and cos (to
 * r^10) on |r| <= pi/4 in FP32 Horner form; the truncation error is below
 * 2e-9 absolute, so the result is within about an ulp. */
static void sh_sincos(float x, float* s, float* c) {
    const double kTwoOverPi = 0.63661977236758134308;
    const double kPiOver2 = 1.57079632679489661923;
    const double k = nearbyint((double)x * kTwoOverPi);
    const double kp = k * kPiOver2;
    const float r = (float)((double)x - kp);
    const float z = r * r;
    const float sp = r + r * z * (-1.0f / 6.0f + z * (1.0f / 120.0f + z * (-1.0f / 5040.0f + z * (1.0f / 362880.0f))));
    const float cp =
        1.0f + z * (-0.5f + z * (1.0f / 24.0f + z * (-1.0f / 720.0f + z * (1.0f / 40320.0f + z * (-1.0f / 3628800.0f)))));
    const long q = ((long)k) & 3;
    switch (q) {
        case 0: *s = sp; *c = cp; break;
        case 1: *s = cp; *c = -sp; break;
        case 2: *s = -sp; *c = -cp; break;
        default: *s = -cp; *c = sp; break;
    }
}
static inline float sh_sin(float x) {
    float s, c;
    sh_sincos(x, &s, &c);
    return s;
}
static inline float sh_cos(float x) {
    float s, c;
    sh_sincos(x, &s, &c);
    return c;
}

/* pow(x, y) for x >= 0: 2^(y log2 x) in FP64, rounded once to FP32.
 * log2 x = e + ln(m) / ln 2 with x = m 2^e, m in [sqrt(1/2), sqrt(2)), and
 * ln m = 2 atanh(s), s = (m - 1) / (m + 1), |s| < 0.172, summed to s^15;
 * 2^t = 2^k e^(f ln 2), k = nearest integer to t, |f| <= 1/2, Taylor to
 * degree 10.  The series truncate below 3e-13 relative.  The divisions are
 * a multiply by 1/ln 2 and a Newton reciprocal, and the polynomials are
 * fused multiply-adds (fma() rounds once, as the GPU's does), so the GPU
 * kernels evaluate the same operations on their FP64 pipe, which on GB300
 * has 1/64 of the FP32 rate. */
static const double kLn2 = 0.69314718055994530942;
static const double kInvLn2 = 1.44269504088896340736;

/* 2^k for an integer |k| <= 1022, from its bits */
static double sh_pow2i(int k) {
    const uint64_t u = (uint64_t)(k + 1023) << 52;
    double d;
    memcpy(&d, &u, sizeof d);
    return d;
}

/* 1 / d for d in [1.7, 2.5] without a division: the FP32 quotient (relative
 * error below 2^-23) refined by two Newton steps r += r (1 - d r), each two
 * fused multiply-adds that square the error (below 2^-52 after). */
static double sh_rcp_d(double d) {
    double r = (double)(1.0f / (float)d);
    double e = fma(-d, r, 1.0);
    r = fma(r, e, r);
    e = fma(-d, r, 1.0);
    return fma(r, e, r);
}

/* 2^t in FP64: 2^k e^((t - k) ln 2), k the nearest integer to t, the
 * exponential's Taylor series to degree 10 (|(t - k) ln 2| <= 0.35),
 * scaled exactly */
static double sh_exp2_d(double t) {
    static const double kInvFact[11] = {1.0,         1.0,          1.0 / 2.0,      1.0 / 6.0,
                                        1.0 / 24.0,  1.0 / 120.0,  1.0 / 720.0,    1.0 / 5040.0,
                                        1.0 / 40320.0, 1.0 / 362880.0, 1.0 / 3628800.0};
    if (t > 200.0) return INFINITY;
    if (t < -200.0) return 0.0;
    const double k = nearbyint(t);
    const double g = (t - k) * kLn2;
    double p = kInvFact[10];
    for (int j = 9; j >= 0; --j) p = fma(g, p, kInvFact[j]);
    return p * sh_pow2i((int)k);
}

static float sh_pow(float xf, float yf) {
    static const double kInvOdd[8] = {1.0,       1.0 / 3.0,  1.0 / 5.0,  1.0 / 7.0,
                                      1.0 / 9.0, 1.0 / 11.0, 1.0 / 13.0, 1.0 / 15.0};
    if (xf != xf || yf != yf) return NAN;
    if (xf < 0.0f) return NAN;
    if (xf == 0.0f) return yf > 0.0f ? 0.0f : (yf == 0.0f ? 1.0f : INFINITY);
    if (yf == 0.0f || xf == 1.0f) return 1.0f;
    if (isinf(xf)) return yf > 0.0f ? INFINITY : 0.0f;
    /* exact cases: x^1 = x, x^(1/2) the correctly rounded square root, and a
     * small positive integer power as FP64 products (square and multiply,
     * at most 12 roundings of 2^-53), rounded once */
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
    double m = frexp((double)xf, &e); /* m in [0.5, 1) */
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) * sh_rcp_d(m + 1.0);
    const double s2 = s * s;
    double series = kInvOdd[7];
    for (int j = 6; j >= 0; --j) series = fma(s2, series, kInvOdd[j]);
    const double lnm = 2.0 * s * series;
    const double t = (double)yf * fma(lnm, kInvLn2, (double)e);
    return (float)sh_exp2_d(t);
}

/* e^x = 2^(x / ln 2) in FP64, rounded once */
static float sh_exp(float x) {
    if (x != x) return NAN;
    return (float)sh_exp2_d((double)x * kInvLn2);
}

/* ===================================================================== */
/* random numbers (rtcommon.glsl:99-139)                                  */
/* ===================================================================== */

/* TEA (Wheeler and Needham) with 16 cycles and the key the shader uses, as
 * a hash of (pixel, frame) into a seed (rtcommon.glsl:99-109). */
static uint32_t sh_tea(uint32_t v0, uint32_t v1) {
    uint32_t s0 = 0;
    for (int n = 0; n < 16; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

/* linear congruential step with the Numerical Recipes constants, low 24
 * bits out (rtcommon.glsl:111-116) */
static inline uint32_t sh_lcg(uint32_t* prev) {
    *prev = 1664525u * *prev + 1013904223u;
    return *prev & 0x00FFFFFFu;
}
static inline float sh_randf(uint32_t* prev) { return (float)sh_lcg(prev) / (float)0x01000000; }
static inline uint32_t sh_randu(uint32_t* prev, uint32_t a, uint32_t b) { return sh_lcg(prev) % (b - a) + a; }

/* Van der Corput radical inverse in base 2 by bit reversal (rtcommon.glsl:128-135) */
static float sh_radical_inverse(uint32_t bits) {
    bits = (bits << 16) | (bits >> 16);
    bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
    bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
    bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
    bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
    return (float)bits * 2.3283064365386963e-10f;
}

/* ===================================================================== */
/* samplers (rtcommon.glsl:141-179)                                       */
/* ===================================================================== */

/* cos(theta) uniform in [0, 1] about the frame's y axis (rtcommon.glsl:141-151) */
static v3 uniform_hemisphere(uint32_t* seed, v3 x, v3 y, v3 z) {
    const float xi1 = sh_randf(seed);
    const float xi2 = sh_randf(seed);
    const float costheta = xi1;
    const float sintheta = sqrtf(1.0f - costheta * costheta);
    const float phi = 2.0f * SH_PI * xi2;
    float sp, cp;
    sh_sincos(phi, &sp, &cp);
    return comb(x, sintheta * cp, y, costheta, z, sintheta * sp);
}

/* cosine-weighted about z (rtcommon.glsl:153-160) */
static v3 cosine_hemisphere(uint32_t* seed, v3 x, v3 y, v3 z) {
    const float phi = sh_randf(seed);
    const float cos_t2 = sh_randf(seed);
    const float sin_t = sqrtf(1.0f - cos_t2);
    const float ang = 2.0f * SH_PI * phi;
    float sp, cp;
    sh_sincos(ang, &sp, &cp);
    return comb(x, cp * sin_t, y, sp * sin_t, z, sqrtf(cos_t2));
}

/* cos^exponent lobe about z (rtcommon.glsl:162-169) */
static v3 cospow_hemisphere(float exponent, uint32_t* seed, v3 x, v3 y, v3 z) {
    const float phi = 2.0f * SH_PI * sh_randf(seed);
    const float cos_t = sh_pow(sh_randf(seed), 1.0f / (exponent + 1.0f));
    const float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float sp, cp;
    sh_sincos(phi, &sp, &cp);
    return comb(x, cp * sin_t, y, sp * sin_t, z, cos_t);
}

/* uniform point on a triangle, as barycentrics (rtcommon.glsl:173-179) */
static v3 triangle_sample(uint32_t* seed) {
    const float u = sqrtf(sh_randf(seed));
    const float v = sh_randf(seed);
    const float a = u * (1.0f - v);
    const float b = u * v;
    return mk(a, b, 1.0f - a - b);
}

/* ===================================================================== */
/* triangles, boxes, frames (rtcommon.glsl:181-251)                      */
/* ===================================================================== */

/* the shader's Möller-Trumbore: |det| < EPS misses, u and v in range, t >= 0
 * (rtcommon.glsl:181-202) */
static int triangle_hit(v3 o, v3 d, v3 pa, v3 pb, v3 pc, v3* hitp) {
    const v3 e1 = sub(pb, pa);
    const v3 e2 = sub(pc, pa);
    const v3 p = cross(d, e2);
    const float det = dot(e1, p);
    if (fabsf(det) < SH_EPS) return 0;
    const float inv = 1.0f / det;
    const v3 s = sub(o, pa);
    const float u = dot(s, p) * inv;
    if (u < 0.0f || u > 1.0f) return 0;
    const v3 q = cross(s, e1);
    const float v = dot(d, q) * inv;
    if (v < 0.0f || u + v > 1.0f) return 0;
    const float t = dot(e2, q) * inv;
    *hitp = add(o, scl(d, t));
    return t >= 0.0f;
}

/* solid-angle pdf of direction d from o under uniform area sampling of the
 * triangle; 0 when d misses it (rtcommon.glsl:204-214) */
static float triangle_pdf(v3 o, v3 d, v3 v0, v3 v1, v3 v2) {
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

/* tangent and bitangent of a unit normal (rtcommon.glsl:218-224) */
static void make_tanspace(v3 n, v3* t, v3* b) {
    if (fabsf(n.x) > fabsf(n.y))
        *t = divs(mk(n.z, 0.0f, -n.x), sqrtf(n.x * n.x + n.z * n.z));
    else
        *t = divs(mk(0.0f, -n.z, n.y), sqrtf(n.y * n.y + n.z * n.z));
    *b = cross(n, *t);
}

static inline float power_heuristic(float a, float b) { return a * a / (a * a + b * b); }
static inline float luma(v3 c) { return 0.299f * c.x + 0.587f * c.y + 0.114f * c.z; }

/* slab test of the ray against a box, t >= 0 (rtcommon.glsl:242-251); min
 * and max ignore a NaN operand (0 * inf when the origin lies on a face). */
static int hit_bbox(v3 o, v3 d, v3 bmin, v3 bmax) {
    const v3 inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    const v3 t0 = mulv(sub(bmin, o), inv);
    const v3 t1 = mulv(sub(bmax, o), inv);
    const v3 tn = mk(fminf(t0.x, t1.x), fminf(t0.y, t1.y), fminf(t0.z, t1.z));
    const v3 tf = mk(fmaxf(t0.x, t1.x), fmaxf(t0.y, t1.y), fmaxf(t0.z, t1.z));
    const float near_max = fmaxf(fmaxf(tn.x, tn.y), fmaxf(tn.z, 0.0f));
    const float far_min = fminf(fminf(tf.x, tf.y), tf.z);
    return near_max <= far_min;
}

/* ===================================================================== */
/* materials (rtcommon.glsl:253-369)                                      */
/* ===================================================================== */

typedef struct {
    v3 albedo, emissive;
    float roughness;
    int use_tanspace; /* the object has a normal texture */
    v3 tn;            /* its tangent-space normal at the hit */
} mat_info;

typedef struct {
    v3 wo, t, b, n;
} shade_info;

/* normalised Blinn-Phong lobe, exponent 1 / roughness, as a pdf over wi
 * (rtcommon.glsl:255-266) */
static float bp_pdf(const mat_info* m, const shade_info* sh, v3 wi) {
    const float o_dn = dot(neg(sh->wo), sh->n);
    const float i_dn = dot(wi, sh->n);
    if (o_dn <= 0.0f || i_dn <= 0.0f) return 0.0f;
    const float ex = 1.0f / m->roughness;
    const v3 h = normalize3(sub(wi, sh->wo));
    const float cosine = fmaxf(dot(h, sh->n), 0.0f);
    const float n_pdf = (ex + 1.0f) / (2.0f * SH_PI) * sh_pow(cosine, ex);
    return n_pdf / (4.0f * dot(neg(sh->wo), h));
}
static v3 bp_eval(const mat_info* m, const shade_info* sh, v3 wi) { return scl(m->albedo, bp_pdf(m, sh, wi)); }
static int bp_sample(uint32_t* seed, const mat_info* m, const shade_info* sh, v3* wi) {
    const float ex = 1.0f / m->roughness;
    const v3 h = cospow_hemisphere(ex, seed, sh->t, sh->b, sh->n);
    *wi = reflect3(sh->wo, h);
    return dot(*wi, sh->n) > 0.0f;
}

/* GGX (Trowbridge-Reitz) with Schlick Fresnel and the Smith joint
 * visibility of rtcommon.glsl:281-343; a2 = roughness^2 */
static v3 ggx_f(v3 r0, float i_dn) {
    const float c5 = sh_pow(1.0f - i_dn, 5.0f);
    return mk(r0.x + (1.0f - r0.x) * c5, r0.y + (1.0f - r0.y) * c5, r0.z + (1.0f - r0.z) * c5);
}
static float ggx_g(float o_dn, float i_dn, float a2) {
    const float sq0 = sqrtf(a2 + (1.0f - a2) * i_dn * i_dn);
    const float sq1 = sqrtf(a2 + (1.0f - a2) * o_dn * o_dn);
    return 2.0f * o_dn * i_dn / (o_dn * sq0 + i_dn * sq1);
}
static float ggx_d(float n_dh, float a2) {
    const float b = n_dh * n_dh * (a2 - 1.0f) + 1.0f;
    return a2 / (SH_PI * b * b);
}
static float ggx_pdf(const mat_info* m, const shade_info* sh, v3 wi) {
    const float o_dn = dot(neg(sh->wo), sh->n);
    const float i_dn = dot(wi, sh->n);
    if (o_dn <= 0.0f || i_dn <= 0.0f) return 0.0f;
    const v3 h = normalize3(sub(wi, sh->wo));
    const float n_dh = fmaxf(dot(h, sh->n), 0.0f);
    const float o_dh = fmaxf(dot(wi, h), 0.0f);
    const float a2 = m->roughness * m->roughness;
    return ggx_d(n_dh, a2) * n_dh / (4.0f * o_dh);
}
static v3 ggx_eval(const mat_info* m, const shade_info* sh, v3 wi) {
    const float o_dn = dot(neg(sh->wo), sh->n);
    const float i_dn = dot(wi, sh->n);
    if (o_dn <= 0.0f || i_dn <= 0.0f) return mk(0.0f, 0.0f, 0.0f);
    const v3 h = normalize3(sub(wi, sh->wo));
    const float n_dh = fmaxf(dot(h, sh->n), 0.0f);
    const float a2 = m->roughness * m->roughness;
    const v3 f = ggx_f(m->albedo, i_dn);
    const float d = ggx_d(n_dh, a2);
    const float g = ggx_g(o_dn, i_dn, a2);
    const float den = 4.0f * o_dn;
    return mk(f.x * d * g / den, f.y * d * g / den, f.z * d * g / den);
}
static int ggx_sample(uint32_t* seed, const mat_info* m, const shade_info* sh, v3* wi) {
    const float a2 = m->roughness * m->roughness;
    const float xi_x = sh_randf(seed);
    const float xi_y = sh_randf(seed);
    const float phi = 2.0f * SH_PI * xi_x;
    const float cos_t = sqrtf((1.0f - xi_y) / (1.0f + (a2 - 1.0f) * xi_y));
    const float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float sp, cp;
    sh_sincos(phi, &sp, &cp);
    const v3 h = comb(sh->t, cp * sin_t, sh->b, sp * sin_t, sh->n, cos_t);
    *wi = reflect3(sh->wo, h);
    return dot(*wi, sh->n) > 0.0f;
}

static float mat_pdf(int brdf, const mat_info* m, const shade_info* sh, v3 wi) {
    return brdf == 0 ? bp_pdf(m, sh, wi) : ggx_pdf(m, sh, wi);
}
static v3 mat_eval(int brdf, const mat_info* m, const shade_info* sh, v3 wi) {
    return brdf == 0 ? bp_eval(m, sh, wi) : ggx_eval(m, sh, wi);
}
static int mat_sample(int brdf, uint32_t* seed, const mat_info* m, const shade_info* sh, v3* wi) {
    return brdf == 0 ? bp_sample(seed, m, sh, wi) : ggx_sample(seed, m, sh, wi);
}

/* ===================================================================== */
/* scene access                                                           */
/* ===================================================================== */

/* ===================================================================== */
/* textures (rt.rgen:100-129; images RGBA8 sRGB, linear filter, repeat)    */
/* ===================================================================== */

/* sRGB to linear of one 8-bit value, with this file's pow */
float orc_sh_srgb_decode(uint32_t byte) {
    const float c = (float)(byte & 255u) / 255.0f;
    return c <= 0.04045f ? c / 12.92f : sh_pow((c + 0.055f) / 1.055f, 2.4f);
}

static float g_srgb[256];
static pthread_once_t g_srgb_once = PTHREAD_ONCE_INIT;
static void srgb_init(void) {
    for (uint32_t i = 0; i < 256; ++i) g_srgb[i] = orc_sh_srgb_decode(i);
}

/* x mod 1 in [0, 1); NaN, the infinities and a difference that rounds up to
 * 1 give 0 */
static float wrap01(float x) {
    float f = x - floorf(x);
    if (!(f >= 0.0f && f < 1.0f)) f = 0.0f;
    return f;
}

static void texel(const uint8_t* texels, int64_t i, float t[4]) {
    for (int k = 0; k < 3; ++k) t[k] = g_srgb[texels[4 * i + k]];
    t[3] = (float)texels[4 * i + 3] / 255.0f;
}

/* bilinear blend at level 0 of the four texels around (u mod 1) w - 1/2,
 * (v mod 1) h - 1/2, neighbours wrapping around the edges */
void orc_sh_texture(int32_t w, int32_t h, const uint8_t* texels, float u, float v, float out[4]) {
    pthread_once(&g_srgb_once, srgb_init);
    const float fx = wrap01(u) * (float)w - 0.5f, fy = wrap01(v) * (float)h - 0.5f;
    const float x0 = floorf(fx), y0 = floorf(fy);
    const float ax = fx - x0, ay = fy - y0;
    int i0 = (int)x0, j0 = (int)y0; /* in [-1, w - 1] and [-1, h - 1] */
    if (i0 < 0) i0 = w - 1;
    if (j0 < 0) j0 = h - 1;
    const int i1 = i0 + 1 == w ? 0 : i0 + 1, j1 = j0 + 1 == h ? 0 : j0 + 1;
    float t00[4], t10[4], t01[4], t11[4];
    texel(texels, (int64_t)j0 * w + i0, t00);
    texel(texels, (int64_t)j0 * w + i1, t10);
    texel(texels, (int64_t)j1 * w + i0, t01);
    texel(texels, (int64_t)j1 * w + i1, t11);
    for (int k = 0; k < 4; ++k)
        out[k] = (t00[k] * (1.0f - ax) + t10[k] * ax) * (1.0f - ay) + (t01[k] * (1.0f - ax) + t11[k] * ax) * ay;
}

/* texture `tex` of the scene at (u, v) */
static void scene_tex(const orc_shade_scene* s, int32_t tex, float u, float v, float out[4]) {
    orc_sh_texture(s->tex_size[2 * tex], s->tex_size[2 * tex + 1], s->texels + 4 * s->tex_off[tex], u, v, out);
}

/* the object's texture of kind k (0 albedo, 1 emissive, 2 metal_rough,
 * 3 normal), or -1 */
static inline int32_t obj_tex(const orc_shade_scene* s, int32_t o, int k) {
    return s->obj_tex ? s->obj_tex[4 * o + k] : -1;
}

typedef struct {
    int32_t obj;
    int64_t first, count; /* the light object's triangles */
    v3 bmin, bmax;        /* their world box */
} light_rec;

typedef struct {
    const orc_shade_scene* s;
    const orc_shade_params* p;
    const orc_shade_temporal* tmp;
    int32_t width, height;
    light_rec* lights;
    uint32_t n_lights;
} ctx_t;

static inline v3 vert(const orc_shade_scene* s, int64_t t, int j) { return ld(s->verts + 9 * t + 3 * j); }
static inline v3 nrm(const orc_shade_scene* s, int64_t t, int j) { return ld(s->normals + 9 * t + 3 * j); }

/* The lights: every object with an emission component above zero, in object
 * order, with its triangle range and world box (rt.cpp:47-58). */
static int collect_lights(const orc_shade_scene* s, light_rec** out, uint32_t* n_out) {
    light_rec* l = (light_rec*)calloc((size_t)(s->nobj > 0 ? s->nobj : 1), sizeof(light_rec));
    if (!l) return -1;
    uint32_t n = 0;
    for (int32_t o = 0; o < s->nobj; ++o) {
        const v3 e = ld(s->emissive + 3 * o);
        if (!any_pos(e)) continue;
        int64_t first = -1, count = 0;
        for (int64_t t = 0; t < s->nt; ++t) {
            if (s->obj[t] != o) continue;
            if (first < 0) first = t;
            if (t != first + count) { /* triangles of an object must be contiguous */
                free(l);
                return -1;
            }
            ++count;
        }
        if (count == 0) continue;
        light_rec r;
        r.obj = o;
        r.first = first;
        r.count = count;
        r.bmin = mk(INFINITY, INFINITY, INFINITY);
        r.bmax = mk(-INFINITY, -INFINITY, -INFINITY);
        for (int64_t t = first; t < first + count; ++t)
            for (int j = 0; j < 3; ++j) {
                const v3 v = vert(s, t, j);
                r.bmin = mk(fminf(r.bmin.x, v.x), fminf(r.bmin.y, v.y), fminf(r.bmin.z, v.z));
                r.bmax = mk(fmaxf(r.bmax.x, v.x), fmaxf(r.bmax.y, v.y), fmaxf(r.bmax.z, v.z));
            }
        l[n++] = r;
    }
    *out = l;
    *n_out = n;
    return 0;
}

/* Möller-Trumbore with the FP32 operation order of the oracle's ray
 * restatement (cpq_oracle.c mt_f32, det epsilon 0): the closest hit. */
static int mt_hit(v3 o, v3 d, v3 a, v3 b, v3 c, float* t, float* u, float* v) {
    const v3 e1 = sub(b, a), e2 = sub(c, a);
    const v3 p = cross(d, e2);
    const float det = dot(e1, p);
    if (!(fabsf(det) > 0.0f)) return 0;
    const float inv = 1.0f / det;
    const v3 s = sub(o, a);
    const float uu = dot(s, p) * inv;
    if (uu < 0.0f || uu > 1.0f) return 0;
    const v3 q = cross(s, e1);
    const float vv = dot(d, q) * inv;
    if (vv < 0.0f || uu + vv > 1.0f) return 0;
    *t = dot(e2, q) * inv;
    *u = uu;
    *v = vv;
    return 1;
}

typedef struct {
    int hit;
    int64_t tri;
    float u, v;
} hit_rec;

/* nearest hit with t in [tmin, tmax]; the least triangle index among equal t */
static hit_rec trace(const orc_shade_scene* s, v3 o, v3 d, float tmin, float tmax, int any) {
    hit_rec h;
    h.hit = 0;
    h.tri = -1;
    h.u = h.v = 0.0f;
    float best = INFINITY;
    for (int64_t t = 0; t < s->nt; ++t) {
        float tt, u, v;
        if (!mt_hit(o, d, vert(s, t, 0), vert(s, t, 1), vert(s, t, 2), &tt, &u, &v)) continue;
        if (!(tt >= tmin && tt <= tmax)) continue;
        if (tt < best) {
            best = tt;
            h.hit = 1;
            h.tri = t;
            h.u = u;
            h.v = v;
            if (any) return h;
        }
    }
    return h;
}

/* visibility(a, b): 1 when something lies between (rt.rgen:271-289) */
static int occluded(const orc_shade_scene* s, v3 a, v3 b) {
    const v3 dir = sub(b, a);
    const float d = length3(dir);
    return trace(s, a, divs(dir, d), SH_EPS, d - SH_EPS, 1).hit;
}

typedef struct {
    v3 pos, normal, tangent;
    float tc[2];
} hit_info;

static inline v3 tng(const orc_shade_scene* s, int64_t t, int j) {
    if (!s->tangents) return mk(0.0f, 0.0f, 0.0f);
    const float* q = s->tangents + 12 * t + 4 * j;
    return scl(ld(q), q[3]);
}
static inline float tcd(const orc_shade_scene* s, int64_t t, int j, int k) {
    return s->texcoords ? s->texcoords[6 * t + 2 * j + k] : 0.0f;
}

/* interpolated world position, unit normal, unit tangent and texture
 * coordinates at a hit (rt.rgen:62-95; the model matrices are the identity
 * for world-space triangles) */
static hit_info make_hit_info(const orc_shade_scene* s, const hit_rec* h) {
    const float bx = 1.0f - h->u - h->v, by = h->u, bz = h->v;
    hit_info r;
    r.normal = normalize3(comb(nrm(s, h->tri, 0), bx, nrm(s, h->tri, 1), by, nrm(s, h->tri, 2), bz));
    r.tangent = normalize3(comb(tng(s, h->tri, 0), bx, tng(s, h->tri, 1), by, tng(s, h->tri, 2), bz));
    r.pos = comb(vert(s, h->tri, 0), bx, vert(s, h->tri, 1), by, vert(s, h->tri, 2), bz);
    for (int k = 0; k < 2; ++k)
        r.tc[k] = tcd(s, h->tri, 0, k) * bx + tcd(s, h->tri, 1, k) * by + tcd(s, h->tri, 2, k) * bz;
    return r;
}

/* material of the hit object at texture coordinates tc: each factor, or its
 * texture where the object has one (rt.rgen:97-129) */
static mat_info make_mat_info(const ctx_t* c, int32_t o, const float tc[2]) {
    const orc_shade_scene* s = c->s;
    mat_info m;
    float t[4];
    m.albedo = ld(s->albedo + 3 * o);
    if (obj_tex(s, o, 0) >= 0) {
        scene_tex(s, obj_tex(s, o, 0), tc[0], tc[1], t);
        m.albedo = mk(t[0], t[1], t[2]);
    }
    m.emissive = ld(s->emissive + 3 * o);
    if (obj_tex(s, o, 1) >= 0) {
        scene_tex(s, obj_tex(s, o, 1), tc[0], tc[1], t);
        m.emissive = mk(t[0], t[1], t[2]);
    }
    float metal = s->metal_rough[2 * o], rough = s->metal_rough[2 * o + 1];
    if (obj_tex(s, o, 2) >= 0) {
        scene_tex(s, obj_tex(s, o, 2), tc[0], tc[1], t);
        metal = t[0];
        rough = t[1];
    }
    m.roughness = rough;
    if (c->p->use_metalness) { /* mix(vec3(0.04), albedo, metal) */
        m.albedo = mk(0.04f * (1.0f - metal) + m.albedo.x * metal, 0.04f * (1.0f - metal) + m.albedo.y * metal,
                      0.04f * (1.0f - metal) + m.albedo.z * metal);
    }
    m.use_tanspace = obj_tex(s, o, 3) >= 0;
    m.tn = mk(0.0f, 0.0f, 0.0f);
    if (m.use_tanspace) { /* texture(...).xyz * 2.0 - 1.0 */
        scene_tex(s, obj_tex(s, o, 3), tc[0], tc[1], t);
        m.tn = mk(t[0] * 2.0f - 1.0f, t[1] * 2.0f - 1.0f, t[2] * 2.0f - 1.0f);
    }
    return m;
}

/* shading frame facing the incoming ray, the normal bent by the normal
 * map when it is on (rt.rgen:131-148) */
static shade_info make_shade_info(const ctx_t* c, v3 wo, const hit_info* hit, const mat_info* m) {
    shade_info sh;
    sh.wo = wo;
    v3 normal = hit->normal;
    if (dot(sh.wo, normal) > 0.0f) normal = neg(normal);
    sh.t = hit->tangent;
    sh.n = normal;
    if (m->use_tanspace && c->p->use_normal_map == 1) { /* N = normalize(mat3(T, B, N) * tn) */
        sh.b = cross(sh.n, sh.t);
        sh.n = normalize3(add(add(scl(sh.t, m->tn.x), scl(sh.b, m->tn.y)), scl(sh.n, m->tn.z)));
    }
    make_tanspace(sh.n, &sh.t, &sh.b);
    return sh;
}

typedef struct {
    v3 pos, normal, emissive;
    float pdf;
} light_sample_t;

/* a point on a uniformly chosen triangle of a uniformly chosen light
 * (rt.rgen:150-194) */
static light_sample_t light_sample(const ctx_t* c, uint32_t* seed, v3 p) {
    const orc_shade_scene* s = c->s;
    const uint32_t li = sh_randu(seed, 0, c->n_lights);
    const light_rec* L = &c->lights[li];
    const uint32_t n_tris = (uint32_t)L->count;
    const uint32_t ti = sh_randu(seed, 0, n_tris);
    const int64_t t = L->first + ti;
    const v3 v0 = vert(s, t, 0), v1 = vert(s, t, 1), v2 = vert(s, t, 2);
    const v3 bary = triangle_sample(seed);
    light_sample_t r;
    r.pos = comb(v0, bary.x, v1, bary.y, v2, bary.z);
    r.emissive = ld(s->emissive + 3 * L->obj);
    if (obj_tex(s, L->obj, 1) >= 0) {
        /* the shader's coordinates: u interpolated, v vertex 1's at every
         * corner (rt.rgen:175) */
        const float tu = tcd(s, t, 0, 0) * bary.x + tcd(s, t, 1, 0) * bary.y + tcd(s, t, 2, 0) * bary.z;
        const float tv = tcd(s, t, 1, 1) * bary.x + tcd(s, t, 1, 1) * bary.y + tcd(s, t, 1, 1) * bary.z;
        float e[4];
        scene_tex(s, obj_tex(s, L->obj, 1), tu, tv, e);
        r.emissive = mk(e[0], e[1], e[2]);
    }
    const v3 narea = cross(sub(v1, v0), sub(v2, v0));
    const float a = 2.0f / length3(narea);
    const v3 dist = sub(r.pos, p);
    const v3 n = normalize3(narea);
    const v3 d = normalize3(dist);
    const float g = dot(dist, dist) / fabsf(dot(n, d));
    r.normal = n;
    r.pdf = a * g / (float)(n_tris * c->n_lights);
    return r;
}

/* direction to a uniform point on a uniformly chosen light triangle
 * (rt.rgen:196-220) */
static v3 light_sample_dir(const ctx_t* c, uint32_t* seed, v3 p) {
    const orc_shade_scene* s = c->s;
    const uint32_t li = sh_randu(seed, 0, c->n_lights);
    const light_rec* L = &c->lights[li];
    const uint32_t ti = sh_randu(seed, 0, (uint32_t)L->count);
    const int64_t t = L->first + ti;
    const v3 bary = triangle_sample(seed);
    const v3 pt = comb(vert(s, t, 0), bary.x, vert(s, t, 1), bary.y, vert(s, t, 2), bary.z);
    return normalize3(sub(pt, p));
}

/* brute-force solid-angle pdf of light sampling for direction d
 * (rt.rgen:222-255) */
static float light_pdf(const ctx_t* c, v3 p, v3 d) {
    const orc_shade_scene* s = c->s;
    float oacc = 0.0f;
    for (uint32_t l = 0; l < c->n_lights; ++l) {
        const light_rec* L = &c->lights[l];
        float tacc = 0.0f;
        if (!hit_bbox(p, d, L->bmin, L->bmax)) continue;
        for (int64_t t = L->first; t < L->first + L->count; ++t)
            tacc += triangle_pdf(p, d, vert(s, t, 0), vert(s, t, 1), vert(s, t, 2));
        oacc += tacc / (float)L->count;
    }
    return oacc / (float)c->n_lights;
}

typedef struct {
    v3 o, d, acc, throughput;
    int depth;
    float mis;
} trace_info;

/* emission of what the ray hits first, or the environment (rt.rgen:291-299) */
static v3 direct_light(const ctx_t* c, v3 o, v3 d) {
    const hit_rec h = trace(c->s, o, d, SH_EPS, SH_LARGE_DIST, 0);
    if (!h.hit) return ld(c->p->env);
    const hit_info hit = make_hit_info(c->s, &h);
    return make_mat_info(c, c->s->obj[h.tri], hit.tc).emissive;
}

/* rt.rgen:301-355 */
static void integrate_mis(const ctx_t* c, uint32_t* seed, trace_info* tr, const hit_info* hit, const mat_info* m,
                          const shade_info* sh) {
    const int brdf = c->p->brdf;
    if (any_pos(m->emissive)) {
        tr->acc = add(tr->acc, mulv(scl(tr->throughput, tr->mis), m->emissive));
        tr->depth = c->p->max_depth;
        return;
    }
    tr->o = hit->pos;
    if (m->roughness == 0.0f) {
        tr->d = reflect3(sh->wo, sh->n);
        tr->throughput = mulv(tr->throughput, m->albedo);
        tr->mis = 1.0f;
        return;
    }
    const v3 wi_light = light_sample_dir(c, seed, hit->pos);
    const float pdf_l = light_pdf(c, hit->pos, wi_light);
    if (pdf_l != 0.0f) {
        const float pdf_m = mat_pdf(brdf, m, sh, wi_light);
        const v3 atten = mat_eval(brdf, m, sh, wi_light);
        const v3 weight = scl(divs(atten, pdf_l), power_heuristic(pdf_l, pdf_m));
        tr->acc = add(tr->acc, mulv(mulv(tr->throughput, weight), direct_light(c, hit->pos, wi_light)));
    }
    v3 wi;
    if (!mat_sample(brdf, seed, m, sh, &wi)) {
        tr->depth = c->p->max_depth;
        return;
    }
    const float pdf_m = mat_pdf(brdf, m, sh, wi);
    if (pdf_m != 0.0f) {
        const float pdf_l2 = light_pdf(c, hit->pos, wi);
        const v3 atten = mat_eval(brdf, m, sh, wi);
        tr->throughput = mulv(tr->throughput, divs(atten, pdf_m));
        tr->mis = power_heuristic(pdf_m, pdf_l2);
    } else {
        tr->depth = c->p->max_depth;
        return;
    }
    tr->d = wi;
}

/* rt.rgen:357-390 */
static void integrate_mats(const ctx_t* c, uint32_t* seed, trace_info* tr, const hit_info* hit, const mat_info* m,
                           const shade_info* sh) {
    const int brdf = c->p->brdf;
    if (any_pos(m->emissive)) {
        tr->acc = add(tr->acc, mulv(m->emissive, tr->throughput));
        tr->depth = c->p->max_depth;
        return;
    }
    tr->o = hit->pos;
    if (m->roughness == 0.0f) {
        tr->d = reflect3(sh->wo, sh->n);
        tr->throughput = mulv(tr->throughput, m->albedo);
        return;
    }
    v3 wi;
    if (!mat_sample(brdf, seed, m, sh, &wi)) {
        tr->depth = c->p->max_depth;
        return;
    }
    const float pdf = mat_pdf(brdf, m, sh, wi);
    const v3 atten = mat_eval(brdf, m, sh, wi);
    if (pdf != 0.0f) {
        tr->throughput = mulv(tr->throughput, divs(atten, pdf));
    } else {
        tr->depth = c->p->max_depth;
        return;
    }
    tr->d = wi;
}

/* rt.rgen:392-412 */
static void integrate_direct(const ctx_t* c, uint32_t* seed, trace_info* tr, const hit_info* hit,
                             const mat_info* m, const shade_info* sh) {
    tr->depth = c->p->max_depth;
    if (any_pos(m->emissive)) {
        tr->acc = add(tr->acc, m->emissive);
        return;
    }
    if (m->roughness != 0.0f) {
        const light_sample_t L = light_sample(c, seed, hit->pos);
        const v3 wi = normalize3(sub(L.pos, hit->pos));
        const v3 atten = mat_eval(c->p->brdf, m, sh, wi);
        if (L.pdf != 0.0f) {
            const float shadow = occluded(c->s, hit->pos, L.pos) ? 0.0f : 1.0f;
            tr->acc = add(tr->acc, scl(mulv(divs(atten, L.pdf), L.emissive), shadow));
        }
    }
}

/* ---- ReSTIR (restir.glsl; rt.rgen:414-548) ---- */

typedef struct {
    v3 pos, normal, emissive;
    float w_sum, w;
    uint32_t n_seen;
} reservoir;

static reservoir res_new(void) {
    reservoir r;
    memset(&r, 0, sizeof r);
    return r;
}

static reservoir res_load(const orc_shade_reservoir* o) {
    reservoir r;
    r.pos = ld(o->pos);
    r.normal = ld(o->normal);
    r.emissive = ld(o->emissive);
    r.w_sum = o->w_sum;
    r.w = o->w;
    r.n_seen = o->n_seen;
    return r;
}

static void res_store(const reservoir* r, orc_shade_reservoir* o) {
    const float f[9] = {r->pos.x, r->pos.y, r->pos.z, r->normal.x, r->normal.y, r->normal.z,
                        r->emissive.x, r->emissive.y, r->emissive.z};
    memcpy(o->pos, f, 3 * sizeof(float));
    memcpy(o->normal, f + 3, 3 * sizeof(float));
    memcpy(o->emissive, f + 6, 3 * sizeof(float));
    o->w_sum = r->w_sum;
    o->w = r->w;
    o->n_seen = r->n_seen;
}

/* The previous frame's reservoir for a hit, when the reprojected first hit
 * agrees in position, albedo and normal (rt.rgen:457-479): returns 0 where
 * the shader leaves the reuse loop.  Buffers are read with the nearest texel
 * and repeat addressing of the G-buffer sampler (rt.cpp:449-450,
 * vulkan.cpp:522-531); a reservoir index at the image edge is clamped. */
/* A point projected into the previous frame (rt.rgen:459-461, 648-650):
 * returns 0 unless it lands inside the image; then uv holds its image
 * coordinates and g the previous first-hit buffer's nearest texel (zeros
 * where there is no buffer). */
static int prev_texel(const ctx_t* c, v3 pos, float uv[2], float g[9]) {
    const orc_shade_temporal* T = c->tmp;
    float pp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (T && T->prev_pv) {
        const float* M = T->prev_pv;
        for (int i = 0; i < 4; ++i) pp[i] = M[4 * i] * pos.x + M[4 * i + 1] * pos.y + M[4 * i + 2] * pos.z + M[4 * i + 3];
    }
    pp[0] = pp[0] / pp[3];
    pp[1] = pp[1] / pp[3];
    pp[0] = (pp[0] + 1.0f) * 0.5f;
    pp[1] = (pp[1] + 1.0f) * 0.5f;
    if (!(pp[0] > 0.0f && pp[1] > 0.0f && pp[0] < 1.0f && pp[1] < 1.0f)) return 0;
    const int W = c->width, H = c->height;
    const int tx = (int)floorf(pp[0] * (float)W) % W, ty = (int)floorf(pp[1] * (float)H) % H;
    memset(g, 0, 9 * sizeof(float));
    if (T && T->prev_gbuf) memcpy(g, T->prev_gbuf + 9 * ((int64_t)ty * W + tx), 9 * sizeof(float));
    uv[0] = pp[0];
    uv[1] = pp[1];
    return 1;
}

static int temporal_reservoir(const ctx_t* c, const hit_info* hit, const mat_info* m, const shade_info* sh,
                              reservoir* prev) {
    const orc_shade_temporal* T = c->tmp;
    float pp[2], g[9];
    if (!prev_texel(c, hit->pos, pp, g)) return 0;
    const int W = c->width, H = c->height;
    const v3 pd = sub(ld(g), hit->pos);
    if (dot(pd, pd) > 0.01f) return 0;
    const v3 ad = sub(ld(g + 6), m->albedo);
    if (dot(ad, ad) > 0.01f) return 0;
    if (dot(ld(g + 3), sh->n) < 0.5f) return 0;
    int fx = (int)(pp[0] * (float)W), fy = (int)(pp[1] * (float)H);
    fx = fx < W ? fx : W - 1;
    fy = fy < H ? fy : H - 1;
    if (T && T->prev_res)
        *prev = res_load(&T->prev_res[(int64_t)fy * W + fx]);
    else
        *prev = res_new();
    return 1;
}

static void res_update(uint32_t* seed, reservoir* r, float weight, v3 pos, v3 normal, v3 emissive) {
    r->n_seen++;
    r->w_sum += weight;
    if (sh_randf(seed) < weight / r->w_sum) {
        r->pos = pos;
        r->normal = normal;
        r->emissive = emissive;
    }
}

static float update_weight(const ctx_t* c, reservoir* r, const hit_info* hit, const mat_info* m,
                           const shade_info* sh) {
    if (r->n_seen == 0) {
        r->w = 0.0f;
        return 0.0f;
    }
    const v3 dir = sub(r->pos, hit->pos);
    const v3 wi = normalize3(dir);
    const v3 atten = mat_eval(c->p->brdf, m, sh, wi);
    const float g = fabsf(dot(r->normal, wi)) / dot(dir, dir);
    const v3 contrib = mulv(scl(atten, g), r->emissive);
    const float p_hat = luma(contrib);
    r->w = (1.0f / p_hat) * (r->w_sum / (float)r->n_seen);
    if (p_hat == 0.0f) r->w = 0.0f;
    return p_hat;
}

/* rt.rgen:425-507: candidates, then reuse of the previous frame's reservoir
 * (first sample, temporal reuse on) or of this pixel's previous sample */
static void reservoir_sample(const ctx_t* c, uint32_t* seed, trace_info* tr, const hit_info* hit,
                             const mat_info* m, const shade_info* sh, reservoir* prev, int first) {
    reservoir nr = res_new();
    for (int i = 0; i < c->p->new_samples; ++i) {
        const light_sample_t L = light_sample(c, seed, hit->pos);
        const v3 wi = normalize3(sub(L.pos, hit->pos));
        const v3 atten = mat_eval(c->p->brdf, m, sh, wi);
        const v3 contrib = divs(mulv(atten, L.emissive), L.pdf);
        res_update(seed, &nr, luma(contrib), L.pos, L.normal, L.emissive);
    }
    const float new_p = update_weight(c, &nr, hit, m, sh);
    if (new_p != 0.0f && occluded(c->s, hit->pos, nr.pos)) nr.w = 0.0f;

    if (first && c->p->use_temporal && !temporal_reservoir(c, hit, m, sh, prev)) goto done;
    reservoir tres = res_new();
    res_update(seed, &tres, new_p * nr.w * (float)nr.n_seen, nr.pos, nr.normal, nr.emissive);
    const float old_p = update_weight(c, prev, hit, m, sh);
    const uint32_t cap = (uint32_t)c->p->temporal_multiplier * nr.n_seen;
    prev->n_seen = cap < prev->n_seen ? cap : prev->n_seen;
    res_update(seed, &tres, old_p * prev->w * (float)prev->n_seen, prev->pos, prev->normal, prev->emissive);
    tres.n_seen = nr.n_seen + prev->n_seen;
    (void)update_weight(c, &tres, hit, m, sh);
    nr = tres;

done:
    if (nr.w != 0.0f) {
        const v3 dir = sub(nr.pos, hit->pos);
        const v3 wi = normalize3(dir);
        const v3 atten = mat_eval(c->p->brdf, m, sh, wi);
        const v3 contrib = mulv(atten, nr.emissive);
        const float g = fabsf(dot(nr.normal, wi)) / dot(dir, dir);
        tr->acc = add(tr->acc, scl(scl(contrib, nr.w), g));
    }
    *prev = nr;
}

/* rt.rgen:509-548 */
static void integrate_restir(const ctx_t* c, uint32_t* seed, trace_info* tr, const hit_info* hit,
                             const mat_info* m, const shade_info* sh, int d_only, reservoir* prev, int first) {
    const int brdf = c->p->brdf;
    if (any_pos(m->emissive)) {
        tr->acc = add(tr->acc, scl(mulv(m->emissive, tr->throughput), tr->mis));
        tr->depth = c->p->max_depth;
        return;
    }
    tr->o = hit->pos;
    if (m->roughness == 0.0f) {
        tr->d = reflect3(sh->wo, sh->n);
        tr->throughput = mulv(tr->throughput, m->albedo);
        tr->mis = 1.0f;
    } else {
        if (tr->depth == 0) reservoir_sample(c, seed, tr, hit, m, sh, prev, first);
        v3 wi;
        if (!mat_sample(brdf, seed, m, sh, &wi)) {
            tr->depth = c->p->max_depth;
            return;
        }
        const float pdf = mat_pdf(brdf, m, sh, wi);
        if (pdf != 0.0f) {
            const v3 atten = mat_eval(brdf, m, sh, wi);
            tr->throughput = mulv(tr->throughput, divs(atten, pdf));
            tr->mis = tr->depth == 0 ? 0.0f : 1.0f;
        } else {
            tr->depth = c->p->max_depth;
            return;
        }
        tr->d = wi;
    }
    if (d_only) tr->depth = c->p->max_depth;
}

/* camera ray of sample s through pixel (x, y) (rt.rgen:550-565); the frame
 * replaces the inverse view and projection matrices, row 0 at the top */
static v3 camera_ray(const orc_shade_camera* cam, const orc_shade_params* p, uint32_t* seed, int s, int x, int y) {
    float jx, jy;
    if (p->qmc == 0) {
        if (p->frame == 0) {
            jx = 0.5f;
            jy = 0.5f;
        } else {
            jx = sh_randf(seed);
            jy = sh_randf(seed);
        }
    } else {
        const uint32_t i = (uint32_t)(s + p->samples * p->frame), n = (uint32_t)(p->samples * p->max_frame);
        jx = (float)i / (float)n;
        jy = sh_radical_inverse(i);
    }
    const float ux = ((float)x + jx) / (float)cam->width;
    const float uy = ((float)y + jy) / (float)cam->height;
    const float nx = ux * 2.0f - 1.0f, ny = uy * 2.0f - 1.0f;
    const v3 r = ld(cam->right), u = ld(cam->up), f = ld(cam->fwd);
    /* as the inverse projection's product would: scale x by tan * aspect */
    const float sx = nx * (cam->tan_half_y * cam->aspect), sy = -(ny * cam->tan_half_y);
    return normalize3(comb(r, sx, u, sy, f, 1.0f));
}

/* rt.rgen:567-677 for one pixel */
static void render_pixel(const ctx_t* c, const orc_shade_camera* cam, int x, int y, float* out, float* gbuf) {
    const orc_shade_params* p = c->p;
    const orc_shade_scene* s = c->s;
    uint32_t seed = sh_tea((uint32_t)(y * cam->width + x), p->seed);
    v3 acc = mk(0.0f, 0.0f, 0.0f);
    const v3 eye = ld(cam->eye);
    v3 g_pos = mk(0, 0, 0), g_norm = mk(0, 0, 0), g_alb = mk(0, 0, 0);
    reservoir prev = res_new();
    for (int smp = 0; smp < p->samples; ++smp) {
        trace_info tr;
        tr.o = eye;
        tr.d = camera_ray(cam, p, &seed, smp, x, y);
        tr.acc = mk(0, 0, 0);
        tr.throughput = mk(1, 1, 1);
        tr.depth = 0;
        tr.mis = 1.0f;
        for (; tr.depth < p->max_depth; tr.depth++) {
            const hit_rec h = trace(s, tr.o, tr.d, SH_EPS, SH_LARGE_DIST, 0);
            if (!h.hit) {
                if (tr.depth == 0)
                    tr.acc = ld(p->clear);
                else
                    tr.acc = add(tr.acc, mulv(ld(p->env), tr.throughput));
                break;
            }
            const hit_info hit = make_hit_info(s, &h);
            const mat_info m = make_mat_info(c, s->obj[h.tri], hit.tc);
            const shade_info sh = make_shade_info(c, tr.d, &hit, &m);
            if (smp == 0 && tr.depth == 0) {
                g_pos = hit.pos;
                g_norm = sh.n;
                g_alb = m.albedo;
            }
            switch (p->integrator) {
                case 0: integrate_direct(c, &seed, &tr, &hit, &m, &sh); break;
                case 1: integrate_mats(c, &seed, &tr, &hit, &m, &sh); break;
                case 2: integrate_mis(c, &seed, &tr, &hit, &m, &sh); break;
                case 3: integrate_restir(c, &seed, &tr, &hit, &m, &sh, 1, &prev, smp == 0); break;
                default: integrate_restir(c, &seed, &tr, &hit, &m, &sh, 0, &prev, smp == 0); break;
            }
            if (p->use_rr) {
                const float pc = fminf(fmaxf(tr.throughput.x, fmaxf(tr.throughput.y, tr.throughput.z)) + 0.001f, 0.95f);
                if (sh_randf(&seed) >= pc) break;
                tr.throughput = divs(tr.throughput, pc);
            }
        }
        acc = add(acc, tr.acc);
    }
    if (p->integrator >= 3 && c->tmp && c->tmp->out_res)
        res_store(&prev, &c->tmp->out_res[(int64_t)y * cam->width + x]);
    const v3 avg = divs(acc, (float)p->samples);
    if (p->frame > 0) { /* mix(old, avg, 1 / (frame + 1)) */
        const float a = 1.0f / (float)(p->frame + 1);
        out[0] = out[0] * (1.0f - a) + avg.x * a;
        out[1] = out[1] * (1.0f - a) + avg.y * a;
        out[2] = out[2] * (1.0f - a) + avg.z * a;
    } else {
        out[0] = avg.x;
        out[1] = avg.y;
        out[2] = avg.z;
    }
    if (p->debug_view > 0) { /* the previous frame's buffers, reprojected (rt.rgen:647-671) */
        float uv[2], g[9];
        if (dot(g_norm, g_norm) > 0.5f && prev_texel(c, g_pos, uv, g)) {
            if (p->debug_view <= 3) memcpy(out, g + 3 * (p->debug_view - 1), 3 * sizeof(float));
        } else {
            out[0] = out[1] = out[2] = 0.0f;
        }
    }
    if (gbuf) {
        const float g[9] = {g_pos.x, g_pos.y, g_pos.z, g_norm.x, g_norm.y, g_norm.z, g_alb.x, g_alb.y, g_alb.z};
        memcpy(gbuf, g, sizeof g);
    }
}

/* ===================================================================== */
/* tone mapping (tonemap.frag)                                            */
/* ===================================================================== */

/* Hable's filmic curve with the shader's constants (tonemap.frag:16-25) */
static float filmic(float c) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((c * (A * c + C * B) + D * E) / (c * (A * c + B) + D * F)) - E / F;
}

/* type 0 filmic (tonemap.frag:27-31), 1 exponential (:33-37), 2 none */
static float tonemap1(int type, float c, float exposure, float gamma) {
    if (type == 0) {
        const float w = 1.0f / filmic(11.2f);
        return sh_pow(filmic(c * exposure) * w, 1.0f / gamma);
    }
    if (type == 1) return sh_pow(1.0f - sh_exp(-c * exposure), 1.0f / gamma);
    return c;
}

/* ===================================================================== */
/* exported batch entry points                                            */
/* ===================================================================== */

void orc_sh_tea(int64_t n, const uint32_t* v0, const uint32_t* v1, uint32_t* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = sh_tea(v0[i], v1[i]);
}

void orc_sh_lcg_stream(uint32_t seed, int64_t n, uint32_t* lcg_out, float* randf_out) {
    uint32_t a = seed, b = seed;
    for (int64_t i = 0; i < n; ++i) {
        if (lcg_out) lcg_out[i] = sh_lcg(&a);
        if (randf_out) randf_out[i] = sh_randf(&b);
    }
}

void orc_sh_radical_inverse(int64_t n, const uint32_t* bits, float* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = sh_radical_inverse(bits[i]);
}

void orc_sh_math(int32_t kind, int64_t n, const float* x, const float* y, float* out) {
    for (int64_t i = 0; i < n; ++i)
        out[i] = kind == 0 ? sh_sin(x[i]) : kind == 1 ? sh_cos(x[i]) : kind == 2 ? sh_pow(x[i], y[i]) : sh_exp(x[i]);
}

int orc_sh_tonemap(int32_t type, float exposure, float gamma, int64_t n, const float* in, float* out) {
    if (type < 0 || type > 2 || n < 0) return -1;
    for (int64_t i = 0; i < n; ++i) out[i] = tonemap1(type, in[i], exposure, gamma);
    return 0;
}

void orc_sh_sample(int32_t kind, int64_t n, uint32_t seed, const float* frame9, float param, const float* wo,
                   float* dirs, uint8_t* ok) {
    const v3 t = ld(frame9), b = ld(frame9 + 3), nn = ld(frame9 + 6);
    shade_info sh;
    sh.t = t;
    sh.b = b;
    sh.n = nn;
    sh.wo = wo ? ld(wo) : mk(0, 0, -1);
    mat_info m;
    m.albedo = mk(1, 1, 1);
    m.emissive = mk(0, 0, 0);
    m.roughness = param;
    for (int64_t i = 0; i < n; ++i) {
        v3 d = mk(0, 0, 0);
        int good = 1;
        switch (kind) {
            case 0: d = uniform_hemisphere(&seed, t, b, nn); break;
            case 1: d = cosine_hemisphere(&seed, t, b, nn); break;
            case 2: d = cospow_hemisphere(param, &seed, t, b, nn); break;
            case 3: good = ggx_sample(&seed, &m, &sh, &d); break;
            case 4: good = bp_sample(&seed, &m, &sh, &d); break;
            default: d = triangle_sample(&seed); break;
        }
        dirs[3 * i] = d.x;
        dirs[3 * i + 1] = d.y;
        dirs[3 * i + 2] = d.z;
        ok[i] = (uint8_t)good;
    }
}

void orc_sh_material(int32_t brdf, int64_t n, const float* albedo3, float roughness, const float* wo,
                     const float* frame9, const float* wi, float* pdf, float* eval3) {
    mat_info m;
    m.albedo = ld(albedo3);
    m.emissive = mk(0, 0, 0);
    m.roughness = roughness;
    shade_info sh;
    sh.wo = ld(wo);
    sh.t = ld(frame9);
    sh.b = ld(frame9 + 3);
    sh.n = ld(frame9 + 6);
    for (int64_t i = 0; i < n; ++i) {
        const v3 w = ld(wi + 3 * i);
        pdf[i] = mat_pdf(brdf, &m, &sh, w);
        const v3 e = mat_eval(brdf, &m, &sh, w);
        eval3[3 * i] = e.x;
        eval3[3 * i + 1] = e.y;
        eval3[3 * i + 2] = e.z;
    }
}

float orc_sh_sin(float x) { return sh_sin(x); }
float orc_sh_cos(float x) { return sh_cos(x); }
float orc_sh_pow(float x, float y) { return sh_pow(x, y); }
float orc_sh_exp(float x) { return sh_exp(x); }

int32_t orc_sh_trace(const orc_shade_scene* s, const float* o, const float* d, float tmin, float tmax, int32_t any,
                     float* u, float* v) {
    const hit_rec h = trace(s, ld(o), ld(d), tmin, tmax, any);
    *u = h.u;
    *v = h.v;
    return h.hit ? (int32_t)h.tri : -1;
}

void orc_sh_reservoir_stream(uint32_t seed, int64_t n, const float* weights, int32_t* chosen, float* w_sum) {
    reservoir r = res_new();
    for (int64_t i = 0; i < n; ++i) {
        res_update(&seed, &r, weights[i], mk((float)i, 0.0f, 0.0f), mk(0, 0, 0), mk(0, 0, 0));
        chosen[i] = (int32_t)r.pos.x;
        w_sum[i] = r.w_sum;
    }
}

void orc_sh_triangle_pdf(int64_t n, const float* o, const float* d, const float* tri9, float* out) {
    const v3 a = ld(tri9), b = ld(tri9 + 3), c = ld(tri9 + 6);
    for (int64_t i = 0; i < n; ++i) out[i] = triangle_pdf(ld(o + 3 * i), ld(d + 3 * i), a, b, c);
}

void orc_sh_hit_bbox(int64_t n, const float* o, const float* d, const float* bmin, const float* bmax, uint8_t* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = (uint8_t)hit_bbox(ld(o + 3 * i), ld(d + 3 * i), ld(bmin), ld(bmax));
}

void orc_sh_make_tanspace(int64_t n, const float* N, float* T, float* B) {
    for (int64_t i = 0; i < n; ++i) {
        v3 t, b;
        make_tanspace(ld(N + 3 * i), &t, &b);
        T[3 * i] = t.x;
        T[3 * i + 1] = t.y;
        T[3 * i + 2] = t.z;
        B[3 * i] = b.x;
        B[3 * i + 1] = b.y;
        B[3 * i + 2] = b.z;
    }
}

static int valid_scene(const orc_shade_scene* s) {
    if (!s || s->nt < 0 || s->nobj < 0) return 0;
    if (s->nt > 0 && (!s->verts || !s->normals || !s->obj)) return 0;
    if (s->nobj > 0 && (!s->albedo || !s->emissive || !s->metal_rough)) return 0;
    for (int64_t t = 0; t < s->nt; ++t)
        if (s->obj[t] < 0 || s->obj[t] >= s->nobj) return 0;
    return 1;
}

void orc_sh_light_pdf(const orc_shade_scene* s, int64_t n, const float* p, const float* d, float* out) {
    ctx_t c;
    memset(&c, 0, sizeof c);
    c.s = s;
    if (!valid_scene(s) || collect_lights(s, &c.lights, &c.n_lights) != 0) {
        for (int64_t i = 0; i < n; ++i) out[i] = NAN;
        return;
    }
    for (int64_t i = 0; i < n; ++i) out[i] = c.n_lights ? light_pdf(&c, ld(p + 3 * i), ld(d + 3 * i)) : 0.0f;
    free(c.lights);
}

typedef struct {
    const ctx_t* c;
    const orc_shade_camera* cam;
    float *image, *gbuf;
    atomic_int next_row;
} render_job;

/* rows handed out one at a time; every pixel seeds its own stream, so the
 * image does not depend on the number of threads */
static void* render_rows(void* arg) {
    render_job* j = (render_job*)arg;
    for (;;) {
        const int y = atomic_fetch_add(&j->next_row, 1);
        if (y >= j->cam->height) break;
        for (int x = 0; x < j->cam->width; ++x) {
            const int64_t px = (int64_t)y * j->cam->width + x;
            render_pixel(j->c, j->cam, x, y, j->image + 3 * px, j->gbuf ? j->gbuf + 9 * px : NULL);
        }
    }
    return NULL;
}

int orc_sh_render(const orc_shade_scene* s, const orc_shade_camera* cam, const orc_shade_params* p, float* image,
                  float* gbuf, const orc_shade_temporal* temporal) {
    if (!valid_scene(s) || !cam || !p || !image) return -1;
    if (cam->width <= 0 || cam->height <= 0 || p->samples <= 0 || p->max_depth < 0) return -1;
    if (p->integrator < 0 || p->integrator > 4 || p->brdf < 0 || p->brdf > 1) return -1;
    if (p->qmc && p->max_frame <= 0) return -1;
    ctx_t c;
    memset(&c, 0, sizeof c);
    c.s = s;
    c.p = p;
    c.tmp = temporal;
    c.width = cam->width;
    c.height = cam->height;
    if (collect_lights(s, &c.lights, &c.n_lights) != 0) return -1;
    /* every integrator but material sampling samples lights */
    if (c.n_lights == 0 && p->integrator != 1) {
        free(c.lights);
        return -1;
    }
    render_job job;
    job.c = &c;
    job.cam = cam;
    job.image = image;
    job.gbuf = gbuf;
    atomic_init(&job.next_row, 0);
    long hw = sysconf(_SC_NPROCESSORS_ONLN);
    int nth = hw > 1 ? (int)(hw < 64 ? hw : 64) : 1;
    if (nth > cam->height) nth = cam->height;
    pthread_t th[64];
    int started = 0;
    for (int i = 1; i < nth; ++i)
        if (pthread_create(&th[started], NULL, render_rows, &job) == 0) ++started;
    render_rows(&job);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    free(c.lights);
    return 0;
}
