// ray.cu — ray queries through the closest-point BVH.
//
// The reference's own GPU query is a ray: `trace_ray` (closest hit over
// [EPS, LARGE_DIST], src/shaders/rt/rt.rgen:257-270) and `visibility`
// (terminate on the first hit of a segment, rt.rgen:272-291), answered by the
// driver's hardware traversal, with the payload {barycentrics, obj_id,
// prim_id, hit} (src/shaders/rt/rtcommon.glsl:55-60, rt.rchit:11-16).  Here
// the same wide BVH that serves closest-point queries is walked by one thread
// per ray: a slab test per child box (the reference's hit_bbox,
// rtcommon.glsl:242-251, made conservative), children visited nearest entry
// first, and at the leaves the Möller–Trumbore test of the reference's
// triangle_hit (rtcommon.glsl:181-202) in FP32.
//
// The triangle test is written with round-to-nearest intrinsics in
// triangle_hit's own evaluation order (dot = (x + y) + z, cross
// components as differences of products), so it is the same FP32 function
// as the CPU restatement; the closest hit is the least (t, triangle index)
// over every triangle the test accepts, and the slab test never rejects a box
// a ray enters, so the answer does not depend on the traversal order and
// equals the restatement's brute force bit for bit.
#include <cfloat>
#include <climits>

#include "bvh.cuh"
#include "ray.cuh"
#include "raywalk.cuh"

namespace cpq {

namespace {

using namespace raywalk;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int mesh_of(const int64_t* __restrict__ off, int nmeshes, int64_t i) {
    int lo = 0, hi = nmeshes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct RayArgs {
    const void* nodes;
    const TriRec* recs;
    const int32_t* wide_root;
    const int64_t* qoff;
    int nmeshes;
    const float* orig;
    const float* dir;
    const float* tmax_per_ray;  // optional
    int64_t n;
    float tmin, tmax, det_eps;
    int any_hit;
    const int32_t* perm;
    float* out_t;
    int32_t* out_tri;
    float* out_uv;
    unsigned long long* counter;
    uint32_t* status;
};

// One thread per ray, persistent over an atomic counter (32 rays per warp
// grab), each ray walked by ray_walk (raywalk.cuh: conservative slab tests,
// the reference's triangle_hit at the leaves).
template <int K>
__global__ void __launch_bounds__(256) k_ray(RayArgs a) {
    const int lane = threadIdx.x & 31;
    const WideNode<K>* __restrict__ nodes = static_cast<const WideNode<K>*>(a.nodes);
    int32_t stack[kRayStack];
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counter, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)a.n) break;
        const int64_t i = (int64_t)base + lane;
        if (i >= a.n) continue;
        const int64_t qi = a.perm ? (int64_t)a.perm[i] : i;
        const float ox = a.orig[3 * qi], oy = a.orig[3 * qi + 1], oz = a.orig[3 * qi + 2];
        const float dx = a.dir[3 * qi], dy = a.dir[3 * qi + 1], dz = a.dir[3 * qi + 2];
        float tmax = a.tmax;
        if (a.tmax_per_ray) tmax = fminf(tmax, a.tmax_per_ray[qi]);
        const int m = a.nmeshes > 1 ? mesh_of(a.qoff, a.nmeshes, qi) : 0;
        float bt = INFINITY, bu = 0.0f, bv = 0.0f;
        int bidx = INT_MAX;
        const bool found = ray_walk<K>(nodes, a.recs, a.wide_root[m], ox, oy, oz, dx, dy, dz, a.tmin, tmax,
                                       a.det_eps, a.any_hit != 0, stack, a.status, bt, bidx, bu, bv);
        if (a.out_t) a.out_t[qi] = found ? bt : INFINITY;
        if (a.out_tri) a.out_tri[qi] = found ? bidx : -1;
        if (a.out_uv) {
            a.out_uv[2 * qi] = found ? bu : 0.0f;
            a.out_uv[2 * qi + 1] = found ? bv : 0.0f;
        }
    }
}

template <int K>
cudaError_t launch_ray(const RayArgs& args, int block, cudaStream_t st) {
    auto kern = k_ray<K>;
    int sms = 0;
    cudaError_t e = sm_count(&sms);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = blocks_per_sm(reinterpret_cast<const void*>(kern), block, 0, &per_sm);
    if (e != cudaSuccess) return e;
    int64_t grid = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    const int64_t need = ((args.n + 31) / 32 * 32 + block - 1) / block;
    if (grid > need) grid = need;
    kern<<<(unsigned)grid, block, 0, st>>>(args); note_launch();
    return cudaGetLastError();
}

// ---- rays through instanced scenes ------------------------------------------
//
// The reference's trace_ray runs against a TLAS of transformed BLASes
// (src/vk/vulkan.cpp:777-856).  Here one thread per ray walks the scene's top
// level in world space with the same conservative slab test; at an instance
// the ray enters object space — o' = A (o - t), d' = A d, unnormalised, so the
// hit parameter t is the same in both spaces — and walks the mesh's BVH, or a
// general instance's world-space copy as it is.  The closest hit is the least
// (t, instance, triangle); t, the triangle's local index and its weights are
// those of the object-space Möller–Trumbore test.

struct SceneRayArgs {
    const void* tnodes;
    const TriRec* trecs;       // p2.y = instance
    const int32_t* troot;
    const void* bnodes;
    const TriRec* brecs;
    const int32_t* broot;      // per mesh
    const void* knodes;        // world-space copies (may be null)
    const TriRec* krecs;
    const int32_t* kroot;      // per copy
    const int32_t* inst_mesh;
    const int32_t* inst_baked;
    const float* inst_inv;     // 12 per instance (3 x 3 part used)
    const float* inst_fwd;     // 12 per instance (translation used)
    const float* orig;
    const float* dir;
    const float* tmax_per_ray;
    int64_t n;
    float tmin, tmax, det_eps;
    int any_hit;
    const int32_t* perm;
    float* out_t;
    int32_t* out_inst;
    int32_t* out_tri;
    float* out_uv;
    unsigned long long* counter;
    uint32_t* status;
};

__device__ __forceinline__ float safe_inv(float d) {
    return __fdiv_rn(1.0f, fabsf(d) < 1e-30f ? copysignf(1e-30f, d) : d);
}

// Entry parameter of each child box (+inf when the ray misses it or it starts
// beyond `limit`), the slab test of k_ray.
template <int K>
__device__ __forceinline__ void slab_children(const WideNode<K>* nd, float ox, float oy, float oz, float ix,
                                              float iy, float iz, float tmin, float limit, float (&tn)[K],
                                              int32_t (&ch)[K]) {
    float lox[K], hix[K], loy[K], hiy[K], loz[K], hiz[K];
    load_row<K>(nd->lox, lox);
    load_row<K>(nd->hix, hix);
    load_row<K>(nd->loy, loy);
    load_row<K>(nd->hiy, hiy);
    load_row<K>(nd->loz, loz);
    load_row<K>(nd->hiz, hiz);
    load_row_i<K>(nd->child, ch);
#pragma unroll
    for (int s = 0; s < K; ++s) {
        const float x0 = (lox[s] - ox) * ix, x1 = (hix[s] - ox) * ix;
        const float y0 = (loy[s] - oy) * iy, y1 = (hiy[s] - oy) * iy;
        const float z0 = (loz[s] - oz) * iz, z1 = (hiz[s] - oz) * iz;
        const float tnear = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
        float tfar = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), limit));
        tfar += fabsf(tfar) * 9.5367432e-7f;
        tn[s] = (tnear <= tfar && lox[s] <= hix[s]) ? tnear : INFINITY;
    }
}

// Entered children pushed farthest first.
template <int K>
__device__ __forceinline__ void push_children(float (&tn)[K], const int32_t (&ch)[K], int32_t* stack, int& sp,
                                              uint32_t* status) {
#pragma unroll
    for (int pass = 0; pass < K; ++pass) {
        int pick = -1;
        float far = -1.0f;
#pragma unroll
        for (int s = 0; s < K; ++s)
            if (tn[s] < INFINITY && tn[s] > far) {
                far = tn[s];
                pick = s;
            }
        if (pick < 0) break;
        if (sp < kRayStack) stack[sp++] = ch[pick];
        else atomicOr(status, 1u);
#pragma unroll
        for (int s = 0; s < K; ++s)
            if (s == pick) tn[s] = INFINITY;
    }
}

template <int K>
__global__ void __launch_bounds__(256) k_scene_ray(SceneRayArgs a) {
    const int lane = threadIdx.x & 31;
    const WideNode<K>* __restrict__ tnodes = static_cast<const WideNode<K>*>(a.tnodes);
    const int32_t troot = __ldg(a.troot);
    int32_t tstack[kRayStack];
    int32_t bstack[kRayStack];
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counter, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)a.n) break;
        const int64_t i = (int64_t)base + lane;
        if (i >= a.n) continue;
        const int64_t qi = a.perm ? (int64_t)a.perm[i] : i;
        const float ox = a.orig[3 * qi], oy = a.orig[3 * qi + 1], oz = a.orig[3 * qi + 2];
        const float dx = a.dir[3 * qi], dy = a.dir[3 * qi + 1], dz = a.dir[3 * qi + 2];
        const float ix = safe_inv(dx), iy = safe_inv(dy), iz = safe_inv(dz);
        float tmax = a.tmax;
        if (a.tmax_per_ray) tmax = fminf(tmax, a.tmax_per_ray[qi]);
        const float tmin = a.tmin;
        float bt = INFINITY, bu = 0.0f, bv = 0.0f;
        int binst = INT_MAX, bidx = INT_MAX;
        bool found = false;
        int tsp = 0;
        tstack[tsp++] = troot;
        while (tsp > 0 && !(found && a.any_hit)) {
            const int cur = tstack[--tsp];
            if (cur >= 0) {
                float tn[K];
                int32_t ch[K];
                slab_children<K>(tnodes + cur, ox, oy, oz, ix, iy, iz, tmin, fminf(bt, tmax), tn, ch);
                push_children<K>(tn, ch, tstack, tsp, a.status);
                continue;
            }
            const int first = leaf_first(cur), cnt = leaf_count(cur);
            for (int k = 0; k < cnt && !(found && a.any_hit); ++k) {
                const int inst = __float_as_int(__ldg(&a.trecs[first + k].p2.y));
                const int baked = a.inst_baked[inst];
                float rox = ox, roy = oy, roz = oz, rdx = dx, rdy = dy, rdz = dz;
                const WideNode<K>* bn;
                const TriRec* recs;
                int32_t root;
                if (baked >= 0) {
                    bn = static_cast<const WideNode<K>*>(a.knodes);
                    recs = a.krecs;
                    root = a.kroot[baked];
                } else {
                    const float* m = a.inst_inv + 12 * inst;
                    const float* f = a.inst_fwd + 12 * inst;
                    const float px = ox - f[3], py = oy - f[7], pz = oz - f[11];
                    rox = fmaf(m[0], px, fmaf(m[1], py, m[2] * pz));
                    roy = fmaf(m[4], px, fmaf(m[5], py, m[6] * pz));
                    roz = fmaf(m[8], px, fmaf(m[9], py, m[10] * pz));
                    rdx = fmaf(m[0], dx, fmaf(m[1], dy, m[2] * dz));
                    rdy = fmaf(m[4], dx, fmaf(m[5], dy, m[6] * dz));
                    rdz = fmaf(m[8], dx, fmaf(m[9], dy, m[10] * dz));
                    bn = static_cast<const WideNode<K>*>(a.bnodes);
                    recs = a.brecs;
                    root = a.broot[a.inst_mesh[inst]];
                }
                const float jx = safe_inv(rdx), jy = safe_inv(rdy), jz = safe_inv(rdz);
                int bsp = 0;
                bstack[bsp++] = root;
                while (bsp > 0) {
                    const int bc = bstack[--bsp];
                    if (bc >= 0) {
                        float tn[K];
                        int32_t ch[K];
                        slab_children<K>(bn + bc, rox, roy, roz, jx, jy, jz, tmin, fminf(bt, tmax), tn, ch);
                        push_children<K>(tn, ch, bstack, bsp, a.status);
                        continue;
                    }
                    const int f0 = leaf_first(bc), fc = leaf_count(bc);
                    for (int j = 0; j < fc; ++j) {
                        const float4* rp = reinterpret_cast<const float4*>(recs + f0 + j);
                        TriRec r;
                        r.p0 = __ldg(rp);
                        r.p1 = __ldg(rp + 1);
                        r.p2 = __ldg(rp + 2);
                        float t, u, v;
                        if (!mt_hit(rox, roy, roz, rdx, rdy, rdz, r, a.det_eps, t, u, v)) continue;
                        if (!(t >= tmin && t <= tmax)) continue;
                        const int idx = __float_as_int(r.p2.y);
                        if (t < bt || (t == bt && (inst < binst || (inst == binst && idx < bidx)))) {
                            bt = t;
                            bu = u;
                            bv = v;
                            binst = inst;
                            bidx = idx;
                            found = true;
                        }
                    }
                    if (found && a.any_hit) break;
                }
            }
        }
        if (a.out_t) a.out_t[qi] = found ? bt : INFINITY;
        if (a.out_inst) a.out_inst[qi] = found ? binst : -1;
        if (a.out_tri) a.out_tri[qi] = found ? bidx : -1;
        if (a.out_uv) {
            a.out_uv[2 * qi] = found ? bu : 0.0f;
            a.out_uv[2 * qi + 1] = found ? bv : 0.0f;
        }
    }
}

template <int K>
cudaError_t launch_scene_ray(const SceneRayArgs& args, int block, cudaStream_t st) {
    auto kern = k_scene_ray<K>;
    int sms = 0;
    cudaError_t e = sm_count(&sms);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = blocks_per_sm(reinterpret_cast<const void*>(kern), block, 0, &per_sm);
    if (e != cudaSuccess) return e;
    int64_t grid = (int64_t)sms * (per_sm > 0 ? per_sm : 1);
    const int64_t need = ((args.n + 31) / 32 * 32 + block - 1) / block;
    if (grid > need) grid = need;
    kern<<<(unsigned)grid, block, 0, st>>>(args); note_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t bvh_ray_query(const Bvh& b, const float* orig, const float* dir, const float* tmax_per_ray,
                          int64_t n, const int64_t* d_off, const RayParams& rp, float* out_t,
                          int32_t* out_tri, float* out_uv, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    RayArgs args;
    cudaError_t e = order_points(b, orig, n, d_off, rp.sort != 0, ws, ws_bytes, st, &args.perm, &args.counter,
                                 /*coarse=*/true);
    if (e != cudaSuccess) return e;
    args.nodes = b.nodes;
    args.recs = b.recs;
    args.wide_root = b.wide_root;
    args.qoff = d_off;
    args.nmeshes = b.nmeshes;
    args.orig = orig;
    args.dir = dir;
    args.tmax_per_ray = tmax_per_ray;
    args.n = n;
    args.tmin = rp.tmin;
    args.tmax = rp.tmax;
    args.det_eps = rp.det_eps;
    args.any_hit = rp.any_hit;
    args.out_t = out_t;
    args.out_tri = out_tri;
    args.out_uv = out_uv;
    args.status = b.status;
    switch (b.p.K) {
        case 2: return launch_ray<2>(args, rp.block, st);
        case 4: return launch_ray<4>(args, rp.block, st);
        default: return launch_ray<8>(args, rp.block, st);
    }
}

cudaError_t scene_ray_query(const Bvh& top, const Bvh& bottom, const InstanceSet& is, const float* orig,
                            const float* dir, const float* tmax_per_ray, int64_t n, const RayParams& rp,
                            float* out_t, int32_t* out_inst, int32_t* out_tri, float* out_uv, void* ws,
                            size_t ws_bytes, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (top.p.K != bottom.p.K || (is.baked_bvh && is.baked_bvh->p.K != bottom.p.K)) return cudaErrorInvalidValue;
    SceneRayArgs a;
    cudaError_t e = order_points(top, orig, n, nullptr, rp.sort != 0, ws, ws_bytes, st, &a.perm, &a.counter,
                                 /*coarse=*/true);
    if (e != cudaSuccess) return e;
    a.tnodes = top.nodes;
    a.trecs = top.recs;
    a.troot = top.wide_root;
    a.bnodes = bottom.nodes;
    a.brecs = bottom.recs;
    a.broot = bottom.wide_root;
    a.knodes = is.baked_bvh ? is.baked_bvh->nodes : nullptr;
    a.krecs = is.baked_bvh ? is.baked_bvh->recs : nullptr;
    a.kroot = is.baked_bvh ? is.baked_bvh->wide_root : nullptr;
    a.inst_mesh = is.mesh;
    a.inst_baked = is.baked;
    a.inst_inv = is.inv;
    a.inst_fwd = is.fwd;
    a.orig = orig;
    a.dir = dir;
    a.tmax_per_ray = tmax_per_ray;
    a.n = n;
    a.tmin = rp.tmin;
    a.tmax = rp.tmax;
    a.det_eps = rp.det_eps;
    a.any_hit = rp.any_hit;
    a.out_t = out_t;
    a.out_inst = out_inst;
    a.out_tri = out_tri;
    a.out_uv = out_uv;
    a.status = bottom.status;
    switch (top.p.K) {
        case 2: return launch_scene_ray<2>(a, rp.block, st);
        case 4: return launch_scene_ray<4>(a, rp.block, st);
        default: return launch_scene_ray<8>(a, rp.block, st);
    }
}

}  // namespace cpq
