/*
 * shade_oracle.h — ORACLE: test infrastructure only.
 *
 * A CPU restatement, in FP32, of the reference's path-tracer shading math
 * (src/shaders/rt/rtcommon.glsl, rt.rgen, restir.glsl): its random numbers,
 * hemisphere / lobe / triangle samplers, the Blinn-Phong and GGX materials,
 * the light sampling and brute-force light pdf, the five integrators
 * (direct, material sampling, MIS, ReSTIR direct-only, ReSTIR) with Russian
 * roulette, the per-pixel camera ray, and the tone mapping of tonemap.frag.
 * It is the checker for shading kernels; nothing in the product links it.
 *
 * Where the shader leaves a value to the GLSL implementation or the clock,
 * this restatement fixes it:
 *  - sin, cos, pow and exp are computed by this file's own routines (Cody-Waite
 *    reduction with Taylor polynomials; exp2 / log2 through the atanh
 *    series), so a device implementation spelling out the same operations
 *    can match it bit for bit; every other operation is one IEEE FP32
 *    operation (compiled with -ffp-contract=off);
 *  - the pixel seed is tea(pixel, caller seed) where the shader uses the
 *    clock (rt.rgen:569);
 *  - a new reservoir's sample (position, normal, emission) starts at zero
 *    (restir.glsl:29-35 leaves it undefined);
 *  - scenes are world-space triangles with per-vertex world normals,
 *    texture coordinates and tangents, and a material per object whose
 *    factors (albedo, emission, metalness / roughness) may be replaced by
 *    textures, with an optional normal map (rt.rgen:100-129, 131-148);
 *  - texture() on the reference's material textures (RGBA8 sRGB images, one
 *    level, linear filter, repeat addressing: rt.cpp:439-447) is this file's
 *    own: each texel's colour decoded from sRGB with this file's pow
 *    (alpha as stored / 255), then a bilinear blend at level 0 of the four
 *    texels around (u mod 1) w - 1/2, (v mod 1) h - 1/2, in a fixed order;
 *  - the closest hit is the nearest Möller-Trumbore hit over all triangles
 *    with t in [1e-5, 1e7] (the shader's EPS and LARGE_DIST, rt.rgen:257-269),
 *    a zero determinant counting as a miss; barycentrics (1-u-v, u, v) as
 *    rt.rchit:12.
 *
 * Checked bit for bit against the reference's own rtcommon.glsl, restir.glsl
 * and rt.rgen compiled as C++ (make_ref_shade.py), which take from this file
 * only what GLSL leaves to the implementation: sin / cos / pow / exp and the
 * scene tracer.
 */
#ifndef SHADE_ORACLE_H
#define SHADE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int64_t nt;             /* triangles */
    const float* verts;     /* nt x 3 vertices x xyz, world space */
    const float* normals;   /* nt x 3 vertices x xyz, world space (need not be unit) */
    const int32_t* obj;     /* object of each triangle; an object's triangles are contiguous */
    int32_t nobj;
    const float* albedo;    /* nobj x 3 */
    const float* emissive;  /* nobj x 3; an object with any component > 0 is a light */
    const float* metal_rough; /* nobj x 2: metalness, roughness */
    /* optional (NULL / 0: none) */
    const float* texcoords;   /* nt x 3 vertices x (u, v) */
    const float* tangents;    /* nt x 3 vertices x (xyz, w): the tangent is xyz * w */
    const int32_t* obj_tex;   /* nobj x 4: albedo, emissive, metal_rough, normal texture, or -1 */
    int32_t ntex;
    const int32_t* tex_size;  /* ntex x (width, height) */
    const int64_t* tex_off;   /* ntex + 1 texel offsets into texels */
    const uint8_t* texels;    /* RGBA8 texels, sRGB colour, row 0 first */
} orc_shade_scene;

typedef struct {
    float eye[3], right[3], up[3], fwd[3]; /* orthonormal camera frame; rays leave the eye */
    float tan_half_y, aspect;              /* tan of half the vertical field of view; width / height */
    int32_t width, height;                 /* row 0 at the top */
} orc_shade_camera;

typedef struct {
    float clear[3];        /* colour of a primary miss (consts.clear_col) */
    float env[3];          /* environment light of a secondary miss (env_scale * env) */
    int32_t samples;       /* samples per pixel per frame */
    int32_t max_depth;
    int32_t qmc;           /* 1: Hammersley jitter */
    int32_t integrator;    /* 0 direct, 1 material sampling, 2 MIS, 3 ReSTIR direct only, 4 ReSTIR */
    int32_t brdf;          /* 0 Blinn-Phong, 1 GGX */
    int32_t use_rr;
    int32_t use_metalness;
    int32_t frame;         /* 0: write the frame; > 0: blend into the image by 1 / (frame + 1) */
    int32_t max_frame;
    int32_t new_samples;   /* ReSTIR candidates per pixel */
    int32_t temporal_multiplier;
    int32_t use_temporal;  /* ReSTIR: reuse the previous frame's reservoirs (rt.rgen:456-479) */
    int32_t debug_view;    /* 1, 2, 3: write the previous frame's position, normal, albedo, reprojected */
    uint32_t seed;
    int32_t use_normal_map; /* 1: bend the shading normal by the object's normal texture (rt.rgen:141-144) */
} orc_shade_params;

/* A ReSTIR reservoir (restir.glsl:1-8). */
typedef struct {
    float pos[3], normal[3], emissive[3];
    float w_sum, w;
    uint32_t n_seen;
} orc_shade_reservoir;

/* State carried between frames for ReSTIR's temporal reuse.  Any pointer may
 * be NULL: a missing previous buffer reads as zeros, as an unwritten image. */
typedef struct {
    const float* prev_pv;                 /* 4 x 4 row-major: world to the previous frame's clip space */
    const float* prev_gbuf;               /* height x width x 9: the previous frame's first-hit buffer */
    const orc_shade_reservoir* prev_res;  /* height x width: the previous frame's final reservoirs */
    orc_shade_reservoir* out_res;         /* height x width: this frame's final reservoirs (written) */
} orc_shade_temporal;

/* random numbers (rtcommon.glsl:99-135) */
void orc_sh_tea(int64_t n, const uint32_t* v0, const uint32_t* v1, uint32_t* out);
void orc_sh_lcg_stream(uint32_t seed, int64_t n, uint32_t* lcg_out, float* randf_out);
void orc_sh_radical_inverse(int64_t n, const uint32_t* bits, float* out);

/* this file's own sin / cos / pow / exp: kind 0 sin(x), 1 cos(x), 2 pow(x, y), 3 exp(x) */
void orc_sh_math(int32_t kind, int64_t n, const float* x, const float* y, float* out);

/* the same routines one value at a time, and the renderer's scene tracer:
 * the nearest hit (or, with `any`, the first found) with t in [tmin, tmax],
 * its triangle (-1 on a miss) and the (u, v) of vertices 1 and 2 */
float orc_sh_sin(float x);
float orc_sh_cos(float x);
float orc_sh_pow(float x, float y);
float orc_sh_exp(float x);
int32_t orc_sh_trace(const orc_shade_scene* s, const float* o, const float* d, float tmin, float tmax, int32_t any,
                     float* u, float* v);

/* this file's texture(): the sample of a w x h RGBA8 sRGB image at (u, v),
 * and the sRGB decode of one 8-bit value */
void orc_sh_texture(int32_t w, int32_t h, const uint8_t* texels, float u, float v, float out[4]);
float orc_sh_srgb_decode(uint32_t byte);

/* tonemap.frag per colour component: type 0 Hable's filmic curve scaled to
 * white at 11.2, 1 exponential 1 - exp(-c exposure), both followed by
 * pow(., 1 / gamma); 2 unchanged.  Returns 0, or -1 for an unknown type. */
int orc_sh_tonemap(int32_t type, float exposure, float gamma, int64_t n, const float* in, float* out);

/* n samples drawn one after another from one lcg stream started at `seed`.
 * kind 0 uniform_hemisphere, 1 cosine_hemisphere, 2 cospow_hemisphere(param),
 * 3 GGX_sample(roughness = param), 4 bp_sample(roughness = param),
 * 5 triangle_sample (barycentrics into dirs).  frame9 = T, B, N; wo is the
 * incoming direction for kinds 3 and 4.  ok[i] is the sampler's return (1
 * for kinds without one). */
void orc_sh_sample(int32_t kind, int64_t n, uint32_t seed, const float* frame9, float param,
                   const float* wo, float* dirs, uint8_t* ok);

/* MAT_pdf and MAT_eval (brdf 0 Blinn-Phong, 1 GGX) for n directions wi at
 * one shading point: frame9 = T, B, N; wo incoming. */
void orc_sh_material(int32_t brdf, int64_t n, const float* albedo3, float roughness, const float* wo,
                     const float* frame9, const float* wi, float* pdf, float* eval3);

/* res_update (restir.glsl:17-27) over a stream of weights from one lcg
 * stream: after each update, the index of the selected candidate and w_sum */
void orc_sh_reservoir_stream(uint32_t seed, int64_t n, const float* weights, int32_t* chosen, float* w_sum);

/* triangle_pdf(o, d, v0, v1, v2) and hit_bbox(o, d, bmin, bmax) per ray */
void orc_sh_triangle_pdf(int64_t n, const float* o, const float* d, const float* tri9, float* out);
void orc_sh_hit_bbox(int64_t n, const float* o, const float* d, const float* bmin, const float* bmax,
                     uint8_t* out);
void orc_sh_make_tanspace(int64_t n, const float* N, float* T, float* B);

/* The light pdf of direction d at p (rt.rgen:222-255) over the scene's lights. */
void orc_sh_light_pdf(const orc_shade_scene* s, int64_t n, const float* p, const float* d, float* out);

/* One frame: image is height x width x 3 (read when frame > 0, written);
 * gbuf, when not NULL, receives per pixel the first hit's position, shading
 * normal and albedo of sample 0 (9 floats; zeros on a miss); temporal, when
 * not NULL, carries ReSTIR's state between frames.
 * Returns 0, or -1 on invalid arguments. */
int orc_sh_render(const orc_shade_scene* s, const orc_shade_camera* c, const orc_shade_params* p, float* image,
                  float* gbuf, const orc_shade_temporal* temporal);

#ifdef __cplusplus
}
#endif
#endif
