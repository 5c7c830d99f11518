// raywalk.cuh — one thread's walk of a wide BVH for one ray: the closest
// hit (least t, then least triangle index) or any hit with t in [tmin, tmax].
//
// Shared by the ray-query kernels (ray.cu) and the path tracer's scene tracer
// (shade.cu).  Per node: the slab entry/exit of every child box against the
// current hit distance; entered children are pushed farthest first.  The exit
// distance is widened by 2^-20 of its magnitude (four times the rounding of a
// subtraction and a product on each side), so a box the ray enters is never
// rejected.  The slab test divides by the direction with zero components
// replaced by a signed 1e-30, so an origin lying on a slab plane gives 0
// rather than the NaN of 0 * inf; the triangle test uses the ray as given.
// At the leaves: the reference's triangle_hit (src/shaders/rt/rtcommon.glsl:
// 181-202) in FP32 with round-to-nearest intrinsics in its own evaluation
// order (dot = (x + y) + z, cross components as differences of products).
// Since the slab test never rejects an entered box and the answer is the
// least (t, index) over every accepted hit, it does not depend on the
// traversal order: it equals a brute force over all triangles bit for bit.
#pragma once

#include <climits>

#include "bvh.cuh"

namespace cpq {
namespace raywalk {

constexpr int kRayStack = 264;  // > (K-1)(depth+1) + 1: cp_mesh_create refuses (K-1)(depth+1) > 256

__device__ __forceinline__ float dot_rn(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// triangle_hit of the reference: t, and the weights u (of b) and v (of c).
// |det| <= det_eps (and det = 0 always) is a miss.
__device__ __forceinline__ bool mt_hit(float ox, float oy, float oz, float dx, float dy, float dz,
                                       const TriRec& r, float det_eps, float& t, float& u, float& v) {
    const float ax = r.p0.x, ay = r.p0.y, az = r.p0.z;
    const float v1x = __fsub_rn(r.p0.w, ax), v1y = __fsub_rn(r.p1.x, ay), v1z = __fsub_rn(r.p1.y, az);
    const float v2x = __fsub_rn(r.p1.z, ax), v2y = __fsub_rn(r.p1.w, ay), v2z = __fsub_rn(r.p2.x, az);
    // p = cross(d, v2)
    const float px = __fsub_rn(__fmul_rn(dy, v2z), __fmul_rn(dz, v2y));
    const float py = __fsub_rn(__fmul_rn(dz, v2x), __fmul_rn(dx, v2z));
    const float pz = __fsub_rn(__fmul_rn(dx, v2y), __fmul_rn(dy, v2x));
    const float det = dot_rn(v1x, v1y, v1z, px, py, pz);
    if (!(fabsf(det) > det_eps)) return false;
    const float inv = __fdiv_rn(1.0f, det);
    const float sx = __fsub_rn(ox, ax), sy = __fsub_rn(oy, ay), sz = __fsub_rn(oz, az);
    u = __fmul_rn(dot_rn(sx, sy, sz, px, py, pz), inv);
    if (u < 0.0f || u > 1.0f) return false;
    // q = cross(s, v1)
    const float qx = __fsub_rn(__fmul_rn(sy, v1z), __fmul_rn(sz, v1y));
    const float qy = __fsub_rn(__fmul_rn(sz, v1x), __fmul_rn(sx, v1z));
    const float qz = __fsub_rn(__fmul_rn(sx, v1y), __fmul_rn(sy, v1x));
    v = __fmul_rn(dot_rn(dx, dy, dz, qx, qy, qz), inv);
    if (v < 0.0f || __fadd_rn(u, v) > 1.0f) return false;
    t = __fmul_rn(dot_rn(v2x, v2y, v2z, qx, qy, qz), inv);
    return true;
}

template <int K>
__device__ __forceinline__ void load_row(const float* __restrict__ p, float (&r)[K]) {
    if constexpr (K == 2) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(p));
        r[0] = v.x; r[1] = v.y;
    } else {
#pragma unroll
        for (int j = 0; j < K; j += 4) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(p) + j / 4);
            r[j] = v.x; r[j + 1] = v.y; r[j + 2] = v.z; r[j + 3] = v.w;
        }
    }
}
template <int K>
__device__ __forceinline__ void load_row_i(const int32_t* __restrict__ p, int32_t (&r)[K]) {
    if constexpr (K == 2) {
        const int2 v = __ldg(reinterpret_cast<const int2*>(p));
        r[0] = v.x; r[1] = v.y;
    } else {
#pragma unroll
        for (int j = 0; j < K; j += 4) {
            const int4 v = __ldg(reinterpret_cast<const int4*>(p) + j / 4);
            r[j] = v.x; r[j + 1] = v.y; r[j + 2] = v.z; r[j + 3] = v.w;
        }
    }
}

// Walk from `root`; returns whether a hit was accepted, with its t, triangle
// index and weights (u of b, v of c).  `stack` holds kRayStack entries; an
// overflow (cannot happen for a tree cp_mesh_create accepts) sets bit 1 of
// *status and drops the child.
template <int K>
__device__ __forceinline__ bool ray_walk(const WideNode<K>* __restrict__ nodes, const TriRec* __restrict__ recs,
                                         int32_t root, float ox, float oy, float oz, float dx, float dy, float dz,
                                         float tmin, float tmax, float det_eps, bool any_hit, int32_t* stack,
                                         uint32_t* status, float& bt, int& bidx, float& bu, float& bv) {
    const float ix = __fdiv_rn(1.0f, fabsf(dx) < 1e-30f ? copysignf(1e-30f, dx) : dx);
    const float iy = __fdiv_rn(1.0f, fabsf(dy) < 1e-30f ? copysignf(1e-30f, dy) : dy);
    const float iz = __fdiv_rn(1.0f, fabsf(dz) < 1e-30f ? copysignf(1e-30f, dz) : dz);
    bool found = false;
    int sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const int cur = stack[--sp];
        if (cur >= 0) {
            const WideNode<K>* nd = nodes + cur;
            float lox[K], hix[K], loy[K], hiy[K], loz[K], hiz[K];
            int32_t ch[K];
            load_row<K>(nd->lox, lox);
            load_row<K>(nd->hix, hix);
            load_row<K>(nd->loy, loy);
            load_row<K>(nd->hiy, hiy);
            load_row<K>(nd->loz, loz);
            load_row<K>(nd->hiz, hiz);
            load_row_i<K>(nd->child, ch);
            const float limit = fminf(bt, tmax);
            float tn[K];
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const float x0 = (lox[s] - ox) * ix, x1 = (hix[s] - ox) * ix;
                const float y0 = (loy[s] - oy) * iy, y1 = (hiy[s] - oy) * iy;
                const float z0 = (loz[s] - oz) * iz, z1 = (hiz[s] - oz) * iz;
                const float tnear = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
                float tfar = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), limit));
                tfar += fabsf(tfar) * 9.5367432e-7f;
                // empty slots (lo = +inf) give tnear = +inf or NaN: never entered
                tn[s] = (tnear <= tfar && lox[s] <= hix[s]) ? tnear : INFINITY;
            }
            // push entered children, farthest first (insertion order by tn)
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
        } else {
            const int first = leaf_first(cur), cnt = leaf_count(cur);
            for (int k = 0; k < cnt; ++k) {
                const float4* rp = reinterpret_cast<const float4*>(recs + first + k);
                TriRec r;
                r.p0 = __ldg(rp);
                r.p1 = __ldg(rp + 1);
                r.p2 = __ldg(rp + 2);
                float t, u, v;
                if (!mt_hit(ox, oy, oz, dx, dy, dz, r, det_eps, t, u, v)) continue;
                if (!(t >= tmin && t <= tmax)) continue;
                const int idx = __float_as_int(r.p2.y);
                if (t < bt || (t == bt && idx < bidx)) {
                    bt = t;
                    bu = u;
                    bv = v;
                    bidx = idx;
                    found = true;
                }
            }
            if (found && any_hit) break;
        }
    }
    return found;
}

}  // namespace raywalk
}  // namespace cpq
