// ref_shade_wrap.cpp — ORACLE: test infrastructure only.
//
// Entry points over the reference's own shader code (rtcommon.glsl,
// restir.glsl and rt.rgen compiled as C++ by make_ref_shade.py), shaped like
// the restatement's orc_sh_* so the tests can run the two on the same
// inputs: batch calls of the shader functions, and ref_render, which runs
// rt.rgen's main over every pixel of a frame.
#include <cstdint>
#include <cstring>
#include <vector>

#include "glsl_shim.h"
#include "rtcommon_ref.h"

namespace tm {  // tonemap.frag has push constants of its own, also named Constants
#include "tonemap_ref.h"
}  // namespace tm

static_assert(sizeof(Reservoir) == sizeof(orc_shade_reservoir), "reservoir layouts differ");

namespace {
const orc_shade_scene* g_scene = nullptr;
std::vector<int64_t> g_first;  // first triangle of each object
}  // namespace

// The ray-tracing pipeline's effect on the payload: the closest-hit shader
// (rt.rchit:10-15) on a hit unless it is skipped, the miss shader
// (rt.rmiss:8-10) on a miss; the hit is the oracle's scene tracer's.
void traceRayEXT(accelerationStructureEXT, uint flags, uint, uint, uint, uint, vec3 o, float tmin, vec3 d, float tmax,
                 int) {
    const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
    float u = 0.0f, v = 0.0f;
    const int32_t t = orc_sh_trace(g_scene, of, df, tmin, tmax, (flags & gl_RayFlagsTerminateOnFirstHitEXT) ? 1 : 0, &u, &v);
    if (t < 0) {
        payload.hit = false;
        return;
    }
    if (flags & gl_RayFlagsSkipClosestHitShaderEXT) return;
    const int32_t ob = g_scene->obj[t];
    payload.hit = true;
    payload.barycentrics = vec3(1.0f - u - v, u, v);
    payload.obj_id = (uint)ob;
    payload.prim_id = (uint)(t - g_first[ob]);
}

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

// the shader's triangle_hit (rtcommon.glsl:181-202) per ray: hit flag and point
void ref_triangle_hit(int64_t n, const float* o, const float* d, const float* tri9, uint8_t* hit, float* hitp) {
    for (int64_t i = 0; i < n; ++i) {
        vec3 p;
        hit[i] = triangle_hit(ld3(o + 3 * i), ld3(d + 3 * i), ld3(tri9), ld3(tri9 + 3), ld3(tri9 + 6), p) ? 1 : 0;
        st3(hitp + 3 * i, p);
    }
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

// rt.rgen's main over every pixel.  Each object gets an identity model
// matrix (its vertices are already in world space, and the identity
// transform is exact) and its own vertex and index arrays; the camera's
// inverse view and projection are the matrices whose products give the
// restatement's camera ray operation for operation.
int ref_render(const orc_shade_scene* s, const orc_shade_camera* cam, const orc_shade_params* p, float* img,
               float* gbuf, const orc_shade_temporal* tmp) {
    if (!s || !cam || !p || !img || cam->width <= 0 || cam->height <= 0) return -1;
    const int W = cam->width, H = cam->height;
    const int32_t nobj = s->nobj;
    g_scene = s;
    g_first.assign((size_t)nobj, -1);
    std::vector<int64_t> count((size_t)nobj, 0);
    for (int64_t t = 0; t < s->nt; ++t) {
        const int32_t o = s->obj[t];
        if (g_first[o] < 0) g_first[o] = t;
        ++count[o];
    }
    mat4 I;
    std::memset(&I, 0, sizeof I);
    for (int k = 0; k < 4; ++k) I.m[k][k] = 1.0f;
    std::vector<Scene_Obj> objs((size_t)nobj);
    std::vector<std::vector<Vertex>> vtx((size_t)nobj);
    std::vector<std::vector<uint>> idx((size_t)nobj);
    std::vector<Vertices> vb((size_t)nobj);
    std::vector<Indices> ib((size_t)nobj);
    std::vector<Scene_Light> lts;
    for (int32_t o = 0; o < nobj; ++o) {
        Scene_Obj& so = objs[o];
        so.model = I;
        so.modelIT = I;
        so.albedo = vec4(ld3(s->albedo + 3 * o), 0.0f);
        so.emissive = vec4(ld3(s->emissive + 3 * o), 0.0f);
        so.metal_rough = vec4(s->metal_rough[2 * o], s->metal_rough[2 * o + 1], 0.0f, 0.0f);
        so.albedo_tex = so.emissive_tex = so.metal_rough_tex = so.normal_tex = -1;
        if (s->obj_tex) {
            so.albedo_tex = s->obj_tex[4 * o];
            so.emissive_tex = s->obj_tex[4 * o + 1];
            so.metal_rough_tex = s->obj_tex[4 * o + 2];
            so.normal_tex = s->obj_tex[4 * o + 3];
        }
        so.index = (uint)o;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t k = 0; k < count[o]; ++k)
            for (int j = 0; j < 3; ++j) {
                const float* pv = s->verts + 9 * (g_first[o] + k) + 3 * j;
                const int64_t t = g_first[o] + k;
                const float* tc = s->texcoords ? s->texcoords + 6 * t + 2 * j : nullptr;
                Vertex vx;
                vx.pos_tx = vec4(ld3(pv), tc ? tc[0] : 0.0f);
                vx.norm_ty = vec4(ld3(s->normals + 9 * t + 3 * j), tc ? tc[1] : 0.0f);
                vx.tangent = vec4();
                if (s->tangents) {
                    const float* tg = s->tangents + 12 * t + 4 * j;
                    vx.tangent = vec4(tg[0], tg[1], tg[2], tg[3]);
                }
                vtx[o].push_back(vx);
                idx[o].push_back((uint)(3 * k + j));
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::fmin(lo[a], pv[a]);
                    hi[a] = std::fmax(hi[a], pv[a]);
                }
            }
        vb[o].v = vtx[o].data();
        ib[o].i = idx[o].data();
        const float* e = s->emissive + 3 * o;
        if (count[o] > 0 && (e[0] > 0.0f || e[1] > 0.0f || e[2] > 0.0f)) {
            Scene_Light L;
            L.bb_min = vec4(ld3(lo), 0.0f);
            L.bb_max = vec4(ld3(hi), 0.0f);
            L.index = (uint)o;
            L.n_triangles = (uint)count[o];
            lts.push_back(L);
        }
    }
    objects = objs.data();
    lights = lts.data();
    vertices = vb.data();
    indices = ib.data();
    std::vector<sampler2D> texs((size_t)(s->ntex > 0 ? s->ntex : 0));
    for (int32_t k = 0; k < s->ntex; ++k)
        texs[k] = sampler2D{nullptr, s->tex_size[2 * k], s->tex_size[2 * k + 1], s->texels + 4 * s->tex_off[k]};
    Textures = texs.empty() ? nullptr : texs.data();

    consts.clear_col = vec4(ld3(p->clear), 1.0f);
    consts.env_light = vec4(ld3(p->env), 1.0f);
    consts.frame = p->frame;
    consts.samples = p->samples;
    consts.max_frame = p->max_frame;
    consts.qmc = p->qmc;
    consts.max_depth = p->max_depth;
    consts.use_normal_map = p->use_normal_map;
    consts.use_metalness = p->use_metalness;
    consts.use_temporal = p->use_temporal;
    consts.integrator = p->integrator;
    consts.brdf = p->brdf;
    consts.debug_view = p->debug_view;
    consts.use_rr = p->use_rr;
    consts.n_lights = (int)lts.size();
    consts.n_objs = nobj;

    std::memset(&uniforms, 0, sizeof uniforms);
    for (int r = 0; r < 3; ++r) {  // inverse view: columns right, up, -forward, eye
        uniforms.iV.m[0][r] = cam->right[r];
        uniforms.iV.m[1][r] = cam->up[r];
        uniforms.iV.m[2][r] = -cam->fwd[r];
        uniforms.iV.m[3][r] = cam->eye[r];
    }
    uniforms.iV.m[3][3] = 1.0f;
    uniforms.iP.m[0][0] = cam->tan_half_y * cam->aspect;  // inverse projection: (tan a x, -tan y, -1, 1)
    uniforms.iP.m[1][1] = -cam->tan_half_y;
    uniforms.iP.m[3][2] = -1.0f;
    uniforms.iP.m[3][3] = 1.0f;
    if (tmp && tmp->prev_pv)
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) uniforms.restir.prev_PV.m[j][i] = tmp->prev_pv[4 * i + j];
    uniforms.restir.new_samples = (uint)p->new_samples;
    uniforms.restir.temporal_multiplier = (uint)p->temporal_multiplier;

    const size_t np = (size_t)W * H;
    std::vector<float> im(4 * np, 0.0f), gp(4 * np, 0.0f), gn(4 * np, 0.0f), ga(4 * np, 0.0f);
    for (size_t k = 0; k < np; ++k)
        for (int a = 0; a < 3; ++a) im[4 * k + a] = img[3 * k + a];
    image = image2D{im.data(), W, H};
    pos_image = image2D{gp.data(), W, H};
    norm_image = image2D{gn.data(), W, H};
    alb_image = image2D{ga.data(), W, H};
    std::vector<float> pg, pn, pa;
    ppos_image = pnorm_image = palb_image = sampler2D{nullptr, W, H};
    if (tmp && tmp->prev_gbuf) {
        pg.assign(4 * np, 0.0f);
        pn.assign(4 * np, 0.0f);
        pa.assign(4 * np, 0.0f);
        for (size_t k = 0; k < np; ++k)
            for (int a = 0; a < 3; ++a) {
                pg[4 * k + a] = tmp->prev_gbuf[9 * k + a];
                pn[4 * k + a] = tmp->prev_gbuf[9 * k + 3 + a];
                pa[4 * k + a] = tmp->prev_gbuf[9 * k + 6 + a];
            }
        ppos_image = sampler2D{pg.data(), W, H};
        pnorm_image = sampler2D{pn.data(), W, H};
        palb_image = sampler2D{pa.data(), W, H};
    }
    std::vector<Reservoir> zero_prev(np), out(np);
    prevFrameReservoirs = (tmp && tmp->prev_res) ? reinterpret_cast<Reservoir*>(const_cast<orc_shade_reservoir*>(
                                                       tmp->prev_res))
                                                 : zero_prev.data();
    reservoirs = out.data();
    g_clock = p->seed;
    gl_LaunchSizeEXT = uvec3{(uint)W, (uint)H, 1u, uvec2{(uint)W, (uint)H}};
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            gl_LaunchIDEXT = uvec3{(uint)x, (uint)y, 0u, uvec2{(uint)x, (uint)y}};
            rt_main();
        }
    for (size_t k = 0; k < np; ++k)
        for (int a = 0; a < 3; ++a) {
            img[3 * k + a] = im[4 * k + a];
            if (gbuf) {
                gbuf[9 * k + a] = gp[4 * k + a];
                gbuf[9 * k + 3 + a] = gn[4 * k + a];
                gbuf[9 * k + 6 + a] = ga[4 * k + a];
            }
        }
    if (tmp && tmp->out_res && p->integrator >= 3) std::memcpy(tmp->out_res, out.data(), np * sizeof(Reservoir));
    return 0;
}

// tonemap.frag's curves per colour value: type 0 tonemapUT, 1 tonemapExp,
// 2 unchanged (its main)
int ref_tonemap(int32_t type, float exposure, float gamma, int64_t n, const float* in, float* out) {
    if (type < 0 || type > 2) return -1;
    tm::consts.exposure = exposure;
    tm::consts.gamma = gamma;
    tm::consts.type = type;
    for (int64_t i = 0; i < n; ++i) {
        const vec4 c(in[i], in[i], in[i], 1.0f);
        out[i] = type == 0 ? tm::tonemapUT(c).x : type == 1 ? tm::tonemapExp(c).x : c.x;
    }
    return 0;
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
