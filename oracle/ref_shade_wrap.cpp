// ref_shade_wrap.cpp — ORACLE: test infrastructure only.
//
// Batch entry points over the reference's own shading functions
// (rtcommon.glsl, restir.glsl compiled as C++ by make_ref_shade.py), shaped
// like the restatement's orc_sh_* so the tests can compare the two on the
// same inputs.
#include <cstdint>

#include "glsl_shim.h"
#include "rtcommon_ref.h"

namespace {
vec3 ld3(const float* p) { return vec3(p[0], p[1], p[2]); }
void st3(float* p, vec3 v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}
}  // namespace

extern "C" {

void ref_tea(int64_t n, const uint32_t* a, const uint32_t* b, uint32_t* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = tea(a[i], b[i]);
}

void ref_lcg_stream(uint32_t seed, int64_t n, uint32_t* u, float* f) {
    uint s1 = seed, s2 = seed;
    for (int64_t i = 0; i < n; ++i) {
        u[i] = lcg(s1);
        f[i] = randf(s2);
    }
}

void ref_radical_inverse(int64_t n, const uint32_t* bits, float* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = radical_inverse(bits[i]);
}

void ref_sample(int32_t kind, int64_t n, uint32_t seed, const float* frame9, float param, const float* wo,
                float* dirs, uint8_t* ok) {
    ShadeInfo sh;
    sh.T = ld3(frame9);
    sh.B = ld3(frame9 + 3);
    sh.N = ld3(frame9 + 6);
    sh.wo = wo ? ld3(wo) : vec3(0.0f, 0.0f, -1.0f);
    MatInfo m;
    m.albedo = vec3(1.0f);
    m.emissive = vec3(0.0f);
    m.roughness = param;
    m.use_tanspace = false;
    uint s = seed;
    for (int64_t i = 0; i < n; ++i) {
        vec3 d;
        bool good = true;
        switch (kind) {
            case 0: d = uniform_hemisphere(s, sh.T, sh.B, sh.N); break;
            case 1: d = cosine_hemisphere(s, sh.T, sh.B, sh.N); break;
            case 2: d = cospow_hemisphere(param, s, sh.T, sh.B, sh.N); break;
            case 3: good = GGX_sample(s, m, sh, d); break;
            case 4: good = bp_sample(s, m, sh, d); break;
            default: d = triangle_sample(s); break;
        }
        st3(dirs + 3 * i, d);
        ok[i] = good ? 1 : 0;
    }
}

void ref_material(int32_t brdf, int64_t n, const float* albedo3, float roughness, const float* wo,
                  const float* frame9, const float* wi, float* pdf, float* eval3) {
    consts.brdf = brdf;
    MatInfo m;
    m.albedo = ld3(albedo3);
    m.emissive = vec3(0.0f);
    m.roughness = roughness;
    m.use_tanspace = false;
    ShadeInfo sh;
    sh.wo = ld3(wo);
    sh.T = ld3(frame9);
    sh.B = ld3(frame9 + 3);
    sh.N = ld3(frame9 + 6);
    for (int64_t i = 0; i < n; ++i) {
        const vec3 w = ld3(wi + 3 * i);
        pdf[i] = MAT_pdf(m, sh, w);
        st3(eval3 + 3 * i, MAT_eval(m, sh, w));
    }
}

void ref_triangle_pdf(int64_t n, const float* o, const float* d, const float* tri9, float* out) {
    for (int64_t i = 0; i < n; ++i)
        out[i] = triangle_pdf(ld3(o + 3 * i), ld3(d + 3 * i), ld3(tri9), ld3(tri9 + 3), ld3(tri9 + 6));
}

void ref_hit_bbox(int64_t n, const float* o, const float* d, const float* bmin, const float* bmax, uint8_t* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = hit_bbox(ld3(o + 3 * i), ld3(d + 3 * i), ld3(bmin), ld3(bmax)) ? 1 : 0;
}

void ref_make_tanspace(int64_t n, const float* N, float* T, float* B) {
    for (int64_t i = 0; i < n; ++i) {
        vec3 t, b;
        make_tanspace(ld3(N + 3 * i), t, b);
        st3(T + 3 * i, t);
        st3(B + 3 * i, b);
    }
}

// res_update over a stream of weights: the index each update selects
void ref_reservoir_stream(uint32_t seed, int64_t n, const float* weights, int32_t* chosen, float* w_sum) {
    uint s = seed;
    Reservoir r = res_new();
    for (int64_t i = 0; i < n; ++i) {
        res_update(s, r, weights[i], vec3((float)i, 0.0f, 0.0f), vec3(0.0f), vec3(0.0f));
        chosen[i] = (int32_t)r.pos.x;
        w_sum[i] = r.w_sum;
    }
}

}  // extern "C"
