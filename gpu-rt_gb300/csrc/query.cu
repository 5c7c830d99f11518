// query.cu — closest-point traversal, query ordering, instanced scenes and the
// adjoint kernel.
//
// Replaces the reference's per-pixel traceRayEXT over its TLAS
// (src/shaders/rt/rt.rgen:257-270) and the slab test hit_bbox
// (src/shaders/rt/rtcommon.glsl:242-251) with a closest-first descent: a
// child box is visited only while its squared distance lower bound is below
// the best squared distance found so far.  Candidates are ranked with an FP32
// point-triangle distance in each triangle's own frame; the winner is
// re-evaluated in float-float by the Voronoi-region method (Ericson 2005,
// section 5.1.5).
//
// Kernels (GB300, 152 SMs; each a persistent grid of SMs x resident blocks
// taking 32 consecutive Hilbert-ordered queries per warp from a global
// counter, with a warp-uniform exit):
//   k_traverse_packet  the default: the 32 lanes walk one shared stack in
//                      shared memory, one entry per wide level;
//   k_traverse         one query per thread, the top `S` stack entries in
//                      shared memory ([slot][thread], 32 distinct banks),
//                      older ones spilled to local memory;
//   k_instances_packet, k_instances
//                      the same two shapes over an instanced scene: a top
//                      level of instance boxes, each instance's mesh walked
//                      with the query in its object space (or on a world-space
//                      copy), the winner finished in world space;
//   k_backward         the adjoint of the distance.
// Node rows and triangle records are read with 128-bit read-only loads.
#include <cfloat>
#include <climits>
#include <mutex>
#include <utility>
#include <vector>
#include <algorithm>

#include "bvh.cuh"
#include "sort.cuh"

namespace cpq {

namespace {

constexpr int kStackTotal = 256;   // >= (K-1)(depth+1) for any 64+32-bit-key LBVH

// Packet traversal work claims: `seed_chunk` (a query option) consecutive
// packets per claim, each packet after a chunk's first seeding its limits from
// kSeedPoints closest points of the packet before it, then kTailPackets single
// packets per warp at the end.  The tail trades seeds for balance: on the
// large heightfield (16M queries, chunks of 4) 16 tail packets per warp
// took 10.05 ms against 10.25 with 4 and 10.40 with 32; claiming the tail two
// at a time (half of it seeded) took 10.11.
#ifndef CPQ_SEED_POINTS
#define CPQ_SEED_POINTS 16
#endif
constexpr int kSeedPoints = CPQ_SEED_POINTS;
#ifndef CPQ_TAIL_PACKETS
#define CPQ_TAIL_PACKETS 16
#endif
constexpr unsigned long long kTailPackets = CPQ_TAIL_PACKETS;
static_assert(kSeedPoints == 1 || kSeedPoints == 2 || kSeedPoints == 4 || kSeedPoints == 8 ||
                  kSeedPoints == 16 || kSeedPoints == 32, "seed points: a power of two up to 32");
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int mesh_of(const int64_t* __restrict__ off, int nmeshes, int64_t i) {
    int lo = 0, hi = nmeshes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int K>
__device__ __forceinline__ void load_row(const float* __restrict__ p, float (&r)[K]) {
    if constexpr (K == 2) {
        float2 v = __ldg(reinterpret_cast<const float2*>(p));
        r[0] = v.x; r[1] = v.y;
    } else if constexpr (K == 4) {
        float4 v = __ldg(reinterpret_cast<const float4*>(p));
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
    } else {
        float4 v = __ldg(reinterpret_cast<const float4*>(p));
        float4 u = __ldg(reinterpret_cast<const float4*>(p) + 1);
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
        r[4] = u.x; r[5] = u.y; r[6] = u.z; r[7] = u.w;
    }
}
template <int K>
__device__ __forceinline__ void load_row_i(const int32_t* __restrict__ p, int32_t (&r)[K]) {
    if constexpr (K == 2) {
        int2 v = __ldg(reinterpret_cast<const int2*>(p));
        r[0] = v.x; r[1] = v.y;
    } else if constexpr (K == 4) {
        int4 v = __ldg(reinterpret_cast<const int4*>(p));
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
    } else {
        int4 v = __ldg(reinterpret_cast<const int4*>(p));
        int4 u = __ldg(reinterpret_cast<const int4*>(p) + 1);
        r[0] = v.x; r[1] = v.y; r[2] = v.z; r[3] = v.w;
        r[4] = u.x; r[5] = u.y; r[6] = u.z; r[7] = u.w;
    }
}

__device__ __forceinline__ void cswap(float& a, float& b, int& x, int& y) {
    if (b < a) {
        float t = a; a = b; b = t;
        int u = x; x = y; y = u;
    }
}

// Ascending sorting networks (2: 1 exchange, 4: 5, 8: 19).
template <int K>
__device__ __forceinline__ void sort_children(float (&d)[K], int (&c)[K]) {
    if constexpr (K == 2) {
        cswap(d[0], d[1], c[0], c[1]);
    } else if constexpr (K == 4) {
        cswap(d[0], d[1], c[0], c[1]); cswap(d[2], d[3], c[2], c[3]);
        cswap(d[0], d[2], c[0], c[2]); cswap(d[1], d[3], c[1], c[3]);
        cswap(d[1], d[2], c[1], c[2]);
    } else {
        cswap(d[0], d[1], c[0], c[1]); cswap(d[2], d[3], c[2], c[3]);
        cswap(d[4], d[5], c[4], c[5]); cswap(d[6], d[7], c[6], c[7]);
        cswap(d[0], d[2], c[0], c[2]); cswap(d[1], d[3], c[1], c[3]);
        cswap(d[4], d[6], c[4], c[6]); cswap(d[5], d[7], c[5], c[7]);
        cswap(d[1], d[2], c[1], c[2]); cswap(d[5], d[6], c[5], c[6]);
        cswap(d[0], d[4], c[0], c[4]); cswap(d[3], d[7], c[3], c[7]);
        cswap(d[1], d[5], c[1], c[5]); cswap(d[2], d[6], c[2], c[6]);
        cswap(d[1], d[4], c[1], c[4]); cswap(d[3], d[6], c[3], c[6]);
        cswap(d[2], d[4], c[2], c[4]); cswap(d[3], d[5], c[3], c[5]);
        cswap(d[3], d[4], c[3], c[4]);
    }
}

// max(a, b, c) in one instruction (three-input max.f32, sm_100 and later).
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// min(a, b, c) in one instruction (three-input min.f32, sm_100 and later).
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ float box_lb2(float qx, float qy, float qz, float lox, float hix,
                                         float loy, float hiy, float loz, float hiz) {
    const float dx = max3f(lox - qx, qx - hix, 0.0f);
    const float dy = max3f(loy - qy, qy - hiy, 0.0f);
    const float dz = max3f(loz - qz, qz - hiz, 0.0f);
    return dx * dx + dy * dy + dz * dz;
}

// Packed f32x2 arithmetic (sm_100 and later): one instruction applies the
// same IEEE single-precision operation, rounded to nearest even, to both
// halves of a 64-bit register pair, so two children's box tests issue as
// one.  Half .x is the low word.  (Triangle tests stay scalar: paired, their
// unpacking and per-half selects cost as many ALU instructions as the packing
// saved on the FMA pipe.)
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float x, float y) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ void f2_unpack(f32x2 v, float& x, float& y) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(v));
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Box distance along one axis for two children: max(lo - q, q - hi, 0).
__device__ __forceinline__ f32x2 box_axis2(f32x2 q, f32x2 lo, f32x2 hi) {
    float a0, a1, b0, b1;
    f2_unpack(f2_sub(lo, q), a0, a1);
    f2_unpack(f2_sub(q, hi), b0, b1);
    return f2_pack(max3f(a0, b0, 0.0f), max3f(a1, b1, 0.0f));
}

// A node row of K floats as K/2 pairs (children 2j, 2j+1), 16-byte loads.
template <int K>
__device__ __forceinline__ void load_row2(const float* __restrict__ p, f32x2 (&r)[K / 2]) {
    if constexpr (K == 2) {
        r[0] = __ldg(reinterpret_cast<const unsigned long long*>(p));
    } else {
#pragma unroll
        for (int j = 0; j < K / 2; j += 2) {
            const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p) + j / 2);
            r[j] = v.x;
            r[j + 1] = v.y;
        }
    }
}

// Branch-free squared distance for the traversal, on a FastTri record: the
// query's offset from a in the triangle's frame, (u, v) in the plane and h
// off it, then h^2 plus the squared 2D distance to the triangle (a, b, c) =
// ((0, 0), (L1, 0), (x2, y2)) — zero inside, else the nearest of the three
// edge segments, each clamped with a saturating multiply.  The ALU pipe is
// the kernel's busiest, so clamps and the inside test are written for the
// FMA pipe: the distance along ab beyond [0, L1] is (|u| + |u - L1| - L1) / 2
// (abs is an operand modifier), and "inside" becomes a factor
// sat(max of the three edge functions * 2^126), 0 when none is positive.
// Lanes that test the same triangle from different Voronoi regions do not
// diverge.  The frame is rounded from FP64, so the value is the distance to
// the triangle to a few ulps of |q - a|; the winner is re-evaluated exactly.
__device__ __forceinline__ float tri_d2_fast(float qx, float qy, float qz, const FastTri& f) {
    const float apx = qx - f.p0.x, apy = qy - f.p0.y, apz = qz - f.p0.z;
    const float u = fmaf(f.p1.x, apx, fmaf(f.p1.y, apy, f.p1.z * apz));
    const float v = fmaf(f.p2.x, apx, fmaf(f.p2.y, apy, f.p2.z * apz));
    const float h = fmaf(f.p3.x, apx, fmaf(f.p3.y, apy, f.p3.z * apz));
    const float L1 = f.p0.w, x2 = f.p1.w, y2 = f.p2.w, bx = f.p3.w;
    const float bu = u - L1;
    // edge ab: twice the distance along the u axis outside [0, L1]
    const float xa = (fabsf(u) + fabsf(bu)) - L1;
    const float d_ab = fmaf(0.25f * xa, xa, v * v);
    // edge ac: from the origin to (x2, y2)
    const float s2 = __saturatef(fmaf(u, x2, v * y2) * f.p4.x);
    const float cx = fmaf(-s2, x2, u), cy = fmaf(-s2, y2, v);
    const float d_ac = fmaf(cx, cx, cy * cy);
    // edge bc: from (L1, 0) to (x2, y2)
    const float s3 = __saturatef(fmaf(bu, bx, v * y2) * f.p4.y);
    const float ex = fmaf(-s3, bx, bu), ey = fmaf(-s3, y2, v);
    const float d_bc = fmaf(ex, ex, ey * ey);
    // outside ab, ca or bc (counter-clockwise, y2 >= 0); vmin = +inf marks a
    // zero-area triangle, never inside
    const float out = max3f(f.p4.z - v, fmaf(v, x2, -u * y2), fmaf(bu, y2, -v * bx));
    return fmaf(h, h, min3f(d_ab, d_ac, d_bc) * __saturatef(out * 0x1p126f));
}

// Degenerate triangle in FP32 with barycentrics (weights of b and c).
__device__ void degenerate_bary(float qx, float qy, float qz, const TriRec& r, float& ov, float& ow) {
    const float ax = r.p0.x, ay = r.p0.y, az = r.p0.z;
    const float bx = r.p0.w, by = r.p1.x, bz = r.p1.y;
    const float cx = r.p1.z, cy = r.p1.w, cz = r.p2.x;
    const float px[3] = {ax, bx, ax}, py[3] = {ay, by, ay}, pz[3] = {az, bz, az};
    const float ex[3] = {bx - ax, cx - bx, cx - ax}, ey[3] = {by - ay, cy - by, cy - ay},
                ez[3] = {bz - az, cz - bz, cz - az};
    float best = FLT_MAX;
    ov = 0.0f;
    ow = 0.0f;
    for (int e = 0; e < 3; ++e) {
        float wx = qx - px[e], wy = qy - py[e], wz = qz - pz[e];
        float l = ex[e] * ex[e] + ey[e] * ey[e] + ez[e] * ez[e];
        float t = l > 0.0f ? __saturatef((wx * ex[e] + wy * ey[e] + wz * ez[e]) / l) : 0.0f;
        wx -= t * ex[e]; wy -= t * ey[e]; wz -= t * ez[e];
        float d2 = wx * wx + wy * wy + wz * wz;
        if (d2 < best) {
            best = d2;
            if (e == 0) { ov = t; ow = 0.0f; }
            else if (e == 1) { ov = 1.0f - t; ow = t; }
            else { ov = 0.0f; ow = t; }
        }
    }
}

// Exact float-float differences of FP32 values (one two-sum each).
__device__ __forceinline__ ff ff_diff(float a, float b) { return ff_two_sum(a, -b); }
__device__ __forceinline__ ff3 ff3_diff(float ax, float ay, float az, float bx, float by, float bz) {
    return {ff_diff(ax, bx), ff_diff(ay, by), ff_diff(az, bz)};
}
// Float-float sum whose error is ~2^-48 of the larger operand (the low parts
// added once): enough for the region tests, which only need signs and ratios.
__device__ __forceinline__ ff ff_add_fast(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return ff_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff3_dot_fast(const ff3& a, const ff3& b) {
    return ff_add_fast(ff_add_fast(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}
// 1 / b to float-float precision: an FP32 quotient and one correction step.
__device__ __forceinline__ ff ff_recip(ff b) {
    const float q1 = __fdiv_rn(1.0f, b.hi);
    const ff r = ff_sub(ff_from(1.0f), ff_mul(b, ff_from(q1)));
    return ff_fast_two_sum(q1, __fmul_rn(r.hi, q1));
}
__device__ __forceinline__ ff ff_select(bool c, ff a, ff b) { return c ? a : b; }

// The triangle's exact edge vectors and the query's offset from a.
struct TriDiff {
    ff3 ab, ac, ap;
};
__device__ __forceinline__ TriDiff tri_diff(float qx, float qy, float qz, const TriRec& r) {
    return {ff3_diff(r.p0.w, r.p1.x, r.p1.y, r.p0.x, r.p0.y, r.p0.z),
            ff3_diff(r.p1.z, r.p1.w, r.p2.x, r.p0.x, r.p0.y, r.p0.z),
            ff3_diff(qx, qy, qz, r.p0.x, r.p0.y, r.p0.z)};
}

// Barycentric weights (of b and c) of the closest point on the triangle:
// the Voronoi-region logic (Ericson 2005, 5.1.5) in float-float on exact
// differences, evaluated branch-free — every region's weights are a
// (numerator v, numerator w, denominator) triple, the one of the region
// found is kept, and one reciprocal finishes it — so lanes of a warp in
// different regions do not serialise.
// The region logic on float-float edge vectors ab, ac and offsets ap, bp, cp
// of the query from a, b and c.
__device__ void precise_bary_core(const TriDiff& t, const ff3& bp, const ff3& cp, ff& v, ff& w) {
    const ff d1 = ff3_dot_fast(t.ab, t.ap), d2 = ff3_dot_fast(t.ac, t.ap);
    const ff d3 = ff3_dot_fast(t.ab, bp), d4 = ff3_dot_fast(t.ac, bp);
    const ff d5 = ff3_dot_fast(t.ab, cp), d6 = ff3_dot_fast(t.ac, cp);
    const ff vc = ff_sub(ff_mul(d1, d4), ff_mul(d3, d2));
    const ff vb = ff_sub(ff_mul(d5, d2), ff_mul(d1, d6));
    const ff va = ff_sub(ff_mul(d3, d6), ff_mul(d5, d4));
    const ff d43 = ff_sub(d4, d3), d56 = ff_sub(d5, d6);
    const ff zero = ff_from(0.0f), one = ff_from(1.0f);
    // face, then the regions that take precedence over it, last one wins
    ff nv = vb, nw = vc, dn = ff_add(ff_add(va, vb), vc);
    bool c = ff_le0(va) && ff_ge0(d43) && ff_ge0(d56);  // edge bc
    nv = ff_select(c, d56, nv);
    nw = ff_select(c, d43, nw);
    dn = ff_select(c, ff_add(d43, d56), dn);
    c = ff_le0(vb) && ff_ge0(d2) && ff_le0(d6);  // edge ac
    nv = ff_select(c, zero, nv);
    nw = ff_select(c, d2, nw);
    dn = ff_select(c, ff_sub(d2, d6), dn);
    c = ff_ge0(d6) && ff_le(d5, d6);  // vertex c
    nv = ff_select(c, zero, nv);
    nw = ff_select(c, one, nw);
    dn = ff_select(c, one, dn);
    c = ff_le0(vc) && ff_ge0(d1) && ff_le0(d3);  // edge ab
    nv = ff_select(c, d1, nv);
    nw = ff_select(c, zero, nw);
    dn = ff_select(c, ff_sub(d1, d3), dn);
    c = ff_ge0(d3) && ff_le(d4, d3);  // vertex b
    nv = ff_select(c, one, nv);
    nw = ff_select(c, zero, nw);
    dn = ff_select(c, one, dn);
    c = ff_le0(d1) && ff_le0(d2);  // vertex a
    nv = ff_select(c, zero, nv);
    nw = ff_select(c, zero, nw);
    dn = ff_select(c, one, dn);
    const ff rd = ff_recip(dn);
    v = ff_mul(nv, rd);
    w = ff_mul(nw, rd);
}

__device__ void precise_bary_d(float qx, float qy, float qz, const TriRec& r, const TriDiff& t, ff& v,
                               ff& w) {
    if (__float_as_uint(r.p2.z) & kTriDegenerate) {
        float fv, fw;
        degenerate_bary(qx, qy, qz, r, fv, fw);
        v = ff_from(fv);
        w = ff_from(fw);
        return;
    }
    precise_bary_core(t, ff3_diff(qx, qy, qz, r.p0.w, r.p1.x, r.p1.y),
                      ff3_diff(qx, qy, qz, r.p1.z, r.p1.w, r.p2.x), v, w);
}

__device__ void precise_bary(float qx, float qy, float qz, const TriRec& r, ff& v, ff& w) {
    precise_bary_d(qx, qy, qz, r, tri_diff(qx, qy, qz, r), v, w);
}

// Residual q - p and offset p - a for p = a + v (b - a) + w (c - a), in
// float-float: the differences of FP32 inputs are exact, so the residual of a
// query very close to the surface keeps its relative accuracy.
__device__ __forceinline__ void precise_residual_d(const TriDiff& t, ff v, ff w, ff3& res, ff3& off) {
    off = {ff_add(ff_mul(v, t.ab.x), ff_mul(w, t.ac.x)), ff_add(ff_mul(v, t.ab.y), ff_mul(w, t.ac.y)),
           ff_add(ff_mul(v, t.ab.z), ff_mul(w, t.ac.z))};
    res = ff3_sub(t.ap, off);
}
__device__ __forceinline__ void precise_residual(float qx, float qy, float qz, const TriRec& r,
                                                 ff v, ff w, ff3& res, ff3& off) {
    precise_residual_d(tri_diff(qx, qy, qz, r), v, w, res, off);
}

// Final answer for the winning triangle: distance to ~2^-44 relative, the
// closest point and its barycentric weights rounded once to FP32.
__device__ void precise_closest(float qx, float qy, float qz, const TriRec& r, float& dist,
                                float& px, float& py, float& pz, float& ov, float& ow) {
    const TriDiff t = tri_diff(qx, qy, qz, r);
    ff v, w;
    precise_bary_d(qx, qy, qz, r, t, v, w);
    ff3 res, off;
    precise_residual_d(t, v, w, res, off);
    dist = ff_to_float(ff_sqrt(ff3_dot(res, res)));
    px = ff_to_float(ff_add(ff_from(r.p0.x), off.x));
    py = ff_to_float(ff_add(ff_from(r.p0.y), off.y));
    pz = ff_to_float(ff_add(ff_from(r.p0.z), off.z));
    ov = ff_to_float(v);
    ow = ff_to_float(w);
}

// q_i - s_i - t1 - t2 for exact float-float products t1, t2: one rounding of
// the three-term sum's error parts.
__device__ __forceinline__ ff ff_sub3(ff d, ff t1, ff t2) {
    const ff s1 = ff_two_sum(d.hi, -t1.hi);
    const ff s2 = ff_two_sum(s1.hi, -t2.hi);
    const float lo = __fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(d.lo, t1.lo), t2.lo), s1.lo), s2.lo);
    return ff_fast_two_sum(s2.hi, lo);
}
// alpha * e for FP32 alpha and float-float e, to float-float precision.
__device__ __forceinline__ ff ff_scale_f(float alpha, ff e) {
    ff t = ff_two_prod(alpha, e.hi);
    t.lo = __fmaf_rn(alpha, e.lo, t.lo);
    return t;
}
// e . r for float-float vectors, rounded once to FP32.
__device__ __forceinline__ float ff3_dot_f(ff ex, ff ey, ff ez, ff rx, ff ry, ff rz) {
    ff px = ff_two_prod(ex.hi, rx.hi), py = ff_two_prod(ey.hi, ry.hi), pz = ff_two_prod(ez.hi, rz.hi);
    px.lo = __fmaf_rn(ex.hi, rx.lo, __fmaf_rn(ex.lo, rx.hi, px.lo));
    py.lo = __fmaf_rn(ey.hi, ry.lo, __fmaf_rn(ey.lo, ry.hi, py.lo));
    pz.lo = __fmaf_rn(ez.hi, rz.lo, __fmaf_rn(ez.lo, rz.hi, pz.lo));
    const ff t = ff_add(ff_add(px, py), pz);
    return __fadd_rn(t.hi, t.lo);
}

// The winner's closest point from its FP32 frame record and exact vertices,
// at a fraction of precise_closest's float-float work; false when the lane
// must take precise_closest instead.
//   1. Feature: the query's in-plane coordinates (u, w) in the frame give
//      the margins of the seven Voronoi regions (face, edges ab / ac / bc,
//      vertices a / b / c); the largest margin picks the feature.  FP32
//      puts (u, w) within delta = 1e-6 (|q - a|_1 + perimeter) of the exact
//      values, so a feature picked with a smaller margin may be a neighbour
//      of the true one, whose point lies within ~delta of the true closest
//      point: a distance error of at most delta^2 / (2 d^2), negligible unless
//      the query is close to the plane (then precise_closest).
//   2. Residual: r = q - (s + alpha (P - s) + beta (R - s)) for the
//      feature's start vertex s and FP32 parameters, in float-float on exact
//      vertex differences, so the point lies exactly on the feature's line
//      or plane whatever alpha and beta are.
//   3. Two refinements, each restricted to the feature (both in-plane
//      directions on the face, the edge's direction on an edge, none at a
//      vertex) and applied to r as parameter changes times the exact edge
//      vectors (exact two-products), so the point never leaves the
//      feature's plane or line.  The first takes the move from r's FP32
//      projection on the frame axes: well conditioned on slivers, it leaves
//      ~2e-7 of the first step's error, so a query farther than 1e-9 of the
//      scale from the plane gets its distance to ~1e-9 relative (closer ones
//      take precise_closest); but the FP32 axes are ~6e-8 off the plane,
//      which leaks ~6e-8 of r's normal part into the move.  The second
//      removes that: r's components along the exact edge vectors
//      (float-float dot products, no leak), solved for the parameters in
//      FP32, which is accurate enough for a correction that small.
//   4. |r| in FP32 from r's leading parts (a sum of squares, no cancellation):
//      a few ulps.  The point is q - r; barycentrics follow the feature and
//      are clamped to it.
// Zero-area triangles take precise_closest.
__device__ __forceinline__ bool closest_by_frame(float qx, float qy, float qz, const TriRec& r, const FastTri& f,
                                                 float& dist, float& px, float& py, float& pz, float& ov,
                                                 float& ow) {
    if (__float_as_uint(r.p2.z) & kTriDegenerate) return false;
    const float ax = r.p0.x, ay = r.p0.y, az = r.p0.z;
    const float bxv = r.p0.w, byv = r.p1.x, bzv = r.p1.y;
    const float cxv = r.p1.z, cyv = r.p1.w, czv = r.p2.x;
    const float apx = qx - ax, apy = qy - ay, apz = qz - az;
    const float u = fmaf(f.p1.x, apx, fmaf(f.p1.y, apy, f.p1.z * apz));
    const float w = fmaf(f.p2.x, apx, fmaf(f.p2.y, apy, f.p2.z * apz));
    const float h = fmaf(f.p3.x, apx, fmaf(f.p3.y, apy, f.p3.z * apz));
    const float L1 = f.p0.w, x2 = f.p1.w, y2 = f.p2.w, bx = f.p3.w;
    const float L2 = sqrtf(fmaf(x2, x2, y2 * y2)), L3 = sqrtf(fmaf(bx, bx, y2 * y2));
    const float il2 = f.p4.x * L2, il3 = f.p4.y * L3;  // 1 / |ac|, 1 / |bc|
    const float bu = u - L1;
    // outside distances of the three edge lines, positions along the edges
    const float A1 = -w, A2 = fmaf(w, x2, -u * y2) * il2, A3 = fmaf(bu, y2, -w * bx) * il3;
    const float P1 = u, P2 = fmaf(u, x2, w * y2) * il2, P3 = fmaf(bu, bx, w * y2) * il3;
    // margins: face, ab, ac, bc, a, b, c; the largest wins
    float mbest = min3f(-A1, -A2, -A3);
    int feat = 0;
    const float m1 = min3f(A1, P1, L1 - P1), m2 = min3f(A2, P2, L2 - P2), m3 = min3f(A3, P3, L3 - P3);
    const float m4 = fminf(-P1, -P2), m5 = fminf(P1 - L1, -P3), m6 = fminf(P2 - L2, P3 - L3);
    if (m1 > mbest) { mbest = m1; feat = 1; }
    if (m2 > mbest) { mbest = m2; feat = 2; }
    if (m3 > mbest) { mbest = m3; feat = 3; }
    if (m4 > mbest) { mbest = m4; feat = 4; }
    if (m5 > mbest) { mbest = m5; feat = 5; }
    if (m6 > mbest) { mbest = m6; feat = 6; }
    const float scale = fabsf(apx) + fabsf(apy) + fabsf(apz) + L1 + L2 + L3;
    const float delta = 1e-6f * scale, ah = fabsf(h);
    // (a frame whose edge lengths or inverses are zero or not finite, from
    // extreme scales, also goes to precise_closest)
    if (!(ah >= 1e-9f * scale) || (mbest < delta && ah < 2.3e3f * delta) || !(L1 > 0.0f && y2 > 0.0f) ||
        !(il2 < INFINITY && il3 < INFINITY && scale < INFINITY))
        return false;
    const float iL1 = __frcp_rn(L1), iy2 = __frcp_rn(y2);

    // start vertex s and the two others (cyclic), the parameters, the
    // refinement direction (dx, dy) in frame coordinates (face: both axes)
    const bool from_b = feat == 3 || feat == 5, from_c = feat == 6;
    const float sx = from_b ? bxv : (from_c ? cxv : ax), sy = from_b ? byv : (from_c ? cyv : ay),
                sz = from_b ? bzv : (from_c ? czv : az);
    const float Px = from_b ? cxv : (from_c ? ax : bxv), Py = from_b ? cyv : (from_c ? ay : byv),
                Pz = from_b ? czv : (from_c ? az : bzv);
    const float Rx = from_b ? ax : (from_c ? bxv : cxv), Ry = from_b ? ay : (from_c ? byv : cyv),
                Rz = from_b ? az : (from_c ? bzv : czv);
    const float wf = w * iy2, vf = (u - wf * x2) * iL1;  // face barycentrics
    float alpha = 0.0f, beta = 0.0f, dx = 0.0f, dy = 0.0f;
    if (feat == 0) { alpha = vf; beta = wf; }
    else if (feat == 1) { alpha = P1 * iL1; dx = 1.0f; }
    else if (feat == 2) { beta = P2 * il2; dx = x2 * il2; dy = y2 * il2; }
    else if (feat == 3) { alpha = P3 * il3; dx = bx * il3; dy = y2 * il3; }
    // exact edge vectors from s, the residual
    const ff EPx = ff_two_sum(Px, -sx), EPy = ff_two_sum(Py, -sy), EPz = ff_two_sum(Pz, -sz);
    const ff ERx = ff_two_sum(Rx, -sx), ERy = ff_two_sum(Ry, -sy), ERz = ff_two_sum(Rz, -sz);
    ff rx = ff_sub3(ff_two_sum(qx, -sx), ff_scale_f(alpha, EPx), ff_scale_f(beta, ERx));
    ff ry = ff_sub3(ff_two_sum(qy, -sy), ff_scale_f(alpha, EPy), ff_scale_f(beta, ERy));
    ff rz = ff_sub3(ff_two_sum(qz, -sz), ff_scale_f(alpha, EPz), ff_scale_f(beta, ERz));
    // first refinement: r's projection on the frame axes, within the feature
    const float e1x = f.p1.x, e1y = f.p1.y, e1z = f.p1.z, e2x = f.p2.x, e2y = f.p2.y, e2z = f.p2.z;
    const float rho1 = fmaf(e1x, rx.hi, fmaf(e1y, ry.hi, e1z * rz.hi));
    const float rho2 = fmaf(e2x, rx.hi, fmaf(e2y, ry.hi, e2z * rz.hi));
    const float along = fmaf(dx, rho1, dy * rho2);
    // as parameter changes, applied along the exact edge vectors, so the
    // point stays on the feature's plane or line
    float da1 = 0.0f, db1 = 0.0f;
    if (feat == 0) {
        db1 = rho2 * iy2;
        da1 = (rho1 - db1 * x2) * iL1;
    } else if (feat == 1) {
        da1 = along * iL1;
    } else if (feat == 2) {
        db1 = along * il2;
    } else if (feat == 3) {
        da1 = along * il3;
    }
    rx = ff_sub3(rx, ff_scale_f(da1, EPx), ff_scale_f(db1, ERx));
    ry = ff_sub3(ry, ff_scale_f(da1, EPy), ff_scale_f(db1, ERy));
    rz = ff_sub3(rz, ff_scale_f(da1, EPz), ff_scale_f(db1, ERz));
    alpha += da1;
    beta += db1;
    // second refinement: r along the exact edge vectors, solved in FP32
    if (feat <= 3) {
        const float rP = ff3_dot_f(EPx, EPy, EPz, rx, ry, rz), rR = ff3_dot_f(ERx, ERy, ERz, rx, ry, rz);
        const float gPP = fmaf(EPx.hi, EPx.hi, fmaf(EPy.hi, EPy.hi, EPz.hi * EPz.hi));
        const float gRR = fmaf(ERx.hi, ERx.hi, fmaf(ERy.hi, ERy.hi, ERz.hi * ERz.hi));
        const float gPR = fmaf(EPx.hi, ERx.hi, fmaf(EPy.hi, ERy.hi, EPz.hi * ERz.hi));
        float da = 0.0f, db = 0.0f;
        if (feat == 0) {
            const float det = fmaf(gPP, gRR, -gPR * gPR);
            if (det > 0.0f) {
                const float id = __frcp_rn(det);
                da = fmaf(gRR, rP, -gPR * rR) * id;
                db = fmaf(gPP, rR, -gPR * rP) * id;
            }
        } else if (feat == 2) {
            db = rR * __frcp_rn(gRR);
        } else {
            da = rP * __frcp_rn(gPP);
        }
        rx = ff_sub3(rx, ff_scale_f(da, EPx), ff_scale_f(db, ERx));
        ry = ff_sub3(ry, ff_scale_f(da, EPy), ff_scale_f(db, ERy));
        rz = ff_sub3(rz, ff_scale_f(da, EPz), ff_scale_f(db, ERz));
        alpha += da;
        beta += db;
    }
    dist = sqrtf(fmaf(rx.hi, rx.hi, fmaf(ry.hi, ry.hi, rz.hi * rz.hi)));
    px = __fsub_rn(__fsub_rn(qx, rx.hi), rx.lo);
    py = __fsub_rn(__fsub_rn(qy, ry.hi), ry.lo);
    pz = __fsub_rn(__fsub_rn(qz, rz.hi), rz.lo);
    // barycentrics (weights of b and c), clamped to the feature
    float v = 0.0f, wb = 0.0f;
    if (feat == 0) {
        wb = __saturatef(beta);
        v = fminf(__saturatef(alpha), 1.0f - wb);
    } else if (feat == 1) {
        v = __saturatef(alpha);
    } else if (feat == 2) {
        wb = __saturatef(beta);
    } else if (feat == 3) {
        wb = __saturatef(alpha);
        v = 1.0f - wb;
    } else if (feat == 5) {
        v = 1.0f;
    } else if (feat == 6) {
        wb = 1.0f;
    }
    ov = v;
    ow = wb;
    return true;
}

struct TraverseArgs {
    const void* nodes;
    const TriRec* recs;   // exact vertices: the winner's re-evaluation
    const FastTri* fast;  // distance-test records, same order
    const int32_t* inv_order;  // triangle (mesh offset + local index) -> record
    const int64_t* toff;       // per-mesh triangle offsets
    const int32_t* wide_root;
    const int64_t* qoff;
    int nmeshes;
    const float* queries;
    const int32_t* perm;
    int64_t nq;
    float* out_point;
    float* out_dist;
    int32_t* out_tri;
    float* out_bary;
    unsigned long long* counter;  // [0] chunk claims, [1] single-packet claims (packet kernel)
    uint32_t* status;
    unsigned long long* stats;  // optional: node visits, leaf triangle tests, pops, skipped pops
    const float* box;           // binary node boxes (lo xyz, hi xyz); a mesh's box at its root
    const int32_t* mesh_root;   // per mesh: its binary root
    int seed_chunk;             // packet kernel: packets per claim (1: no seeding)
};

template <int K, int S>
__global__ void __launch_bounds__(256) k_traverse(TraverseArgs a) {
    extern __shared__ float2 s_stack[];
    const int lane = threadIdx.x & 31;
    const int nth = blockDim.x;
    float2* my = s_stack + threadIdx.x;
    float2 spill[kStackTotal - S];
    const WideNode<K>* __restrict__ nodes = static_cast<const WideNode<K>*>(a.nodes);

    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counter, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)a.nq) break;  // warp-uniform exit
        const int64_t i = (int64_t)base + lane;
        if (i >= a.nq) continue;
        const int64_t qi = a.perm ? (int64_t)a.perm[i] : i;
        const float qx = a.queries[3 * qi], qy = a.queries[3 * qi + 1], qz = a.queries[3 * qi + 2];
        const int m = a.nmeshes > 1 ? mesh_of(a.qoff, a.nmeshes, qi) : 0;

        float best = INFINITY;
        int best_rec = -1;
        int best_idx = INT_MAX;
        int sp = 0;
        int cur = a.wide_root[m];
        bool have = true;
        while (have) {
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
                float lb[K];
#pragma unroll
                for (int s = 0; s < K; ++s) {
                    float d = box_lb2(qx, qy, qz, lox[s], hix[s], loy[s], hiy[s], loz[s], hiz[s]);
                    lb[s] = d < best ? d : INFINITY;
                }
                sort_children<K>(lb, ch);
#pragma unroll
                for (int s = K - 1; s >= 1; --s) {
                    if (lb[s] < INFINITY) {
                        // push (far children first so the nearest is on top)
                        const int slot = (sp & (S - 1)) * nth;
                        if (sp >= S) {
                            const int ov = sp - S;
                            if (ov < kStackTotal - S) spill[ov] = my[slot];
                            else atomicOr(a.status, 1u);
                        }
                        my[slot] = make_float2(lb[s], __int_as_float(ch[s]));
                        ++sp;
                    }
                }
                if (lb[0] < INFINITY) {
                    cur = ch[0];
                    continue;
                }
            } else {
                const int first = leaf_first(cur), cnt = leaf_count(cur);
                for (int k = 0; k < cnt; ++k) {
                    const FastTri f = load_fast(a.fast + first + k);
                    const float d2 = tri_d2_fast(qx, qy, qz, f);
                    const int idx = fast_index(f);
                    if (d2 < best || (d2 == best && idx < best_idx)) {
                        best = d2;
                        best_rec = first + k;
                        best_idx = idx;
                    }
                }
            }
            // pop the nearest entry that can still hold a closer triangle
            have = false;
            while (sp > 0) {
                --sp;
                const int slot = (sp & (S - 1)) * nth;
                const float2 e = my[slot];
                if (sp >= S) my[slot] = spill[sp - S];
                if (e.x < best) {
                    cur = __float_as_int(e.y);
                    have = true;
                    break;
                }
            }
        }

        float dist = __int_as_float(0x7fc00000), px = dist, py = dist, pz = dist, bv = dist, bw = dist;
        if (best_rec >= 0) {
            const float4* rp = reinterpret_cast<const float4*>(a.recs + best_rec);
            TriRec r;
            r.p0 = __ldg(rp);
            r.p1 = __ldg(rp + 1);
            r.p2 = __ldg(rp + 2);
            if (!closest_by_frame(qx, qy, qz, r, load_fast(a.fast + best_rec), dist, px, py, pz, bv, bw))
                precise_closest(qx, qy, qz, r, dist, px, py, pz, bv, bw);
        } else {
            atomicOr(a.status, 4u);
        }
        if (a.out_dist) a.out_dist[qi] = dist;
        if (a.out_tri) a.out_tri[qi] = best_rec >= 0 ? best_idx : -1;
        if (a.out_point) {
            a.out_point[3 * qi] = px;
            a.out_point[3 * qi + 1] = py;
            a.out_point[3 * qi + 2] = pz;
        }
        if (a.out_bary) {
            a.out_bary[2 * qi] = bv;
            a.out_bary[2 * qi + 1] = bw;
        }
    }
}

// Streaming (evict-first) access for data a traversal touches once: the
// queries gathered through the ordering and the results scattered back.  The
// hint keeps them from displacing the tree's nodes and triangle records,
// which neighbouring packets re-read, from L2.
#ifndef CPQ_STREAM_IO
#define CPQ_STREAM_IO 1
#endif
template <typename T>
__device__ __forceinline__ T ld_stream(const T* p) {
    if constexpr (CPQ_STREAM_IO) return __ldcs(p);
    else return *p;
}
template <typename T>
__device__ __forceinline__ void st_stream(T* p, T v) {
    if constexpr (CPQ_STREAM_IO) __stcs(p, v);
    else *p = v;
}

// The winner's float-float re-evaluation and the outputs; the closest point
// (NaN when nothing was found) is also returned in (px, py, pz).
__device__ __forceinline__ void write_result(const TraverseArgs& a, int64_t qi, float qx, float qy,
                                             float qz, int best_rec, int best_idx, float& px, float& py,
                                             float& pz) {
    float dist = __int_as_float(0x7fc00000), bv = dist, bw = dist;
    px = dist;
    py = dist;
    pz = dist;
    if (best_rec >= 0) {
        const float4* rp = reinterpret_cast<const float4*>(a.recs + best_rec);
        TriRec r;
        r.p0 = __ldg(rp);
        r.p1 = __ldg(rp + 1);
        r.p2 = __ldg(rp + 2);
        if (!closest_by_frame(qx, qy, qz, r, load_fast(a.fast + best_rec), dist, px, py, pz, bv, bw))
            precise_closest(qx, qy, qz, r, dist, px, py, pz, bv, bw);
    } else {
        atomicOr(a.status, 4u);
    }
    // results land in the caller's (random) query order and are written once:
    // evict-first stores, so they do not push the tree out of L2
    if (a.out_dist) st_stream(a.out_dist + qi, dist);
    if (a.out_tri) st_stream(a.out_tri + qi, best_rec >= 0 ? best_idx : -1);
    if (a.out_point) {
        st_stream(a.out_point + 3 * qi, px);
        st_stream(a.out_point + 3 * qi + 1, py);
        st_stream(a.out_point + 3 * qi + 2, pz);
    }
    if (a.out_bary) {
        st_stream(a.out_bary + 2 * qi, bv);
        st_stream(a.out_bary + 2 * qi + 1, bw);
    }
}

// Slot lists of the packet stack: entry m lists the set bits of m, lowest
// first, one per nibble (m < 256 covers nodes up to 8 wide).
struct SlotLists {
    uint32_t v[256];
};
constexpr SlotLists make_slot_lists() {
    SlotLists t{};
    for (int m = 0; m < 256; ++m) {
        uint32_t l = 0;
        int p = 0;
        for (int s = 0; s < 8; ++s)
            if ((m >> s) & 1) l |= (uint32_t)s << (4 * p++);
        t.v[m] = l;
    }
    return t;
}
__constant__ SlotLists c_slot_lists = make_slot_lists();

// Store K consecutive 4-byte values with vector stores (dst 8- or 16-byte
// aligned as K is 2 or more).
template <int K, typename T>
__device__ __forceinline__ void store_row(T* dst, const T (&v)[K]) {
    static_assert(sizeof(T) == 4, "4-byte elements");
    if constexpr (K == 2) {
        *reinterpret_cast<uint2*>(dst) = make_uint2(__builtin_bit_cast(uint32_t, v[0]),
                                                    __builtin_bit_cast(uint32_t, v[1]));
    } else {
#pragma unroll
        for (int j = 0; j < K; j += 4)
            *reinterpret_cast<uint4*>(dst + j) =
                make_uint4(__builtin_bit_cast(uint32_t, v[j]), __builtin_bit_cast(uint32_t, v[j + 1]),
                           __builtin_bit_cast(uint32_t, v[j + 2]), __builtin_bit_cast(uint32_t, v[j + 3]));
    }
}

// Shared memory of one warp: the packet stack of `cap` entries (every lane's
// K bounds [entry][lane][slot], the K child refs [entry][slot], the (slot
// list, count) of entries below the top [entry]; rounded to 16 bytes), then
// the leaf-compaction slots (32 query points) when the kernel compacts, then
// the previous packet's kSeedPoints closest points (x, y, z, mesh), then the
// warp's chunk cursor (next packet, chunk end).
__host__ __device__ constexpr size_t packet_stack_bytes(int K, int cap) {
    return ((size_t)cap * (128 * K + 4 * K + 8) + 15) & ~size_t(15);
}
__host__ __device__ constexpr size_t packet_warp_bytes(int K, int cap, bool compact) {
    return packet_stack_bytes(K, cap) + (compact ? 32 * sizeof(float4) : 0) + (kSeedPoints + 1) * sizeof(float4);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// A lane's best candidate as one unsigned key: the squared distance's bits
// (non-negative floats order as their bit patterns) over the triangle index,
// so the unsigned minimum is the nearest triangle, ties to the smallest index.
__device__ __forceinline__ unsigned long long best_key(float d2, int idx) {
    return ((unsigned long long)__float_as_uint(d2) << 32) | (uint32_t)idx;
}
__device__ __forceinline__ float key_d2(unsigned long long k) {
    return __uint_as_float((uint32_t)(k >> 32));
}
constexpr unsigned long long kNoKey = 0x7f8000007fffffffull;  // (+inf, INT_MAX): nothing found
constexpr unsigned long long kSeedKeyLow = 0x7fffffffull;     // a seed's index: INT_MAX, no triangle's

// Leaf compaction with na active lanes (1..16): kpr = 32 / na triangles per
// round and 1 / na.
struct LeafSplit {
    int kpr;
    float inv;
};
struct LeafSplits {
    LeafSplit v[17];
};
constexpr LeafSplits make_leaf_splits() {
    LeafSplits t{};
    for (int na = 1; na <= 16; ++na) t.v[na] = {32 / na, 1.0f / (float)na};
    return t;
}
__constant__ LeafSplits c_leaf_splits = make_leaf_splits();

// Warp-packet traversal.  The 32 lanes of a warp hold 32 consecutive queries
// of the Hilbert order (neighbours in space) and walk ONE shared stack: a
// child is visited when any lane's box lower bound beats that lane's best, so
// every node row is a single broadcast load and node tests run with all
// lanes converged; child bounds are computed two children per packed f32x2
// operation.  A visit goes on at once to the needed child nearest to any
// lane (one warp min); if other children are needed the node becomes ONE
// stack entry holding every lane's K bounds, the K child refs and the list of
// the needed slots still to visit (in slot order).  On a pop the
// top entry's next slot is re-checked against every lane's current best and
// skipped when no lane still needs it.  Only the top entry can be used up,
// and a push reuses it, so the stack holds one entry per wide level at most;
// `cap` (max wide depth + 1) is that bound, so it cannot overflow.  Lanes of
// different meshes in one packet (batches) are served one mesh at a time.
// With seed_chunk > 1 a warp claims that many consecutive packets at once;
// each packet after the first starts every lane's limit at a padded upper
// bound from the previous packet's closest points (its neighbours along the
// curve), so the first leaves a packet reaches are not tested against an
// infinite limit.  Chunks spread the packets in flight over more of the
// curve, which costs cache locality; on coherent queries (points near a
// surface) the seeds save more than that, on scattered ones less.
// kCompact (trees whose leaves hold 3 or more triangles) spreads a leaf's
// (query, triangle) pairs over the warp when few lanes need the leaf; it
// costs 512 bytes of shared memory per warp, which with 2-triangle leaves
// is better spent on resident warps.  kStats adds per-warp visit counters (a
// diagnostic build of the kernel).
template <int K, bool kCompact, bool kStats>
__global__ void __launch_bounds__(256, K == 8 ? 2 : 4) k_traverse_packet(TraverseArgs a, int cap) {
    extern __shared__ __align__(16) unsigned char s_pk[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool lane0 = lane == 0;
    unsigned char* wbase = s_pk + (size_t)warp * packet_warp_bytes(K, cap, kCompact);
    float* st_bnd = reinterpret_cast<float*>(wbase) + lane * K;  // entry e, slot s at [e * 32 * K + s]
    int32_t* st_ch = reinterpret_cast<int32_t*>(wbase + (size_t)cap * 128 * K);
    uint2* st_state = reinterpret_cast<uint2*>(wbase + (size_t)cap * 132 * K);
    float4* st_q = reinterpret_cast<float4*>(wbase + packet_stack_bytes(K, cap));
    float4* st_seed = st_q + (kCompact ? 32 : 0);
    const uint32_t lt_mask = lanemask_lt();
    const WideNode<K>* __restrict__ nodes = static_cast<const WideNode<K>*>(a.nodes);
    unsigned long long n_nodes = 0, n_tris = 0, n_pops = 0, n_skips = 0, n_lane_tris = 0, n_rounds = 0,
                       n_lane_nodes = 0;

    // Work: packets of 32 consecutive ordered queries.  Up to `split` they are
    // claimed `seed_chunk` at a time from counter[0]; the last kTailPackets per
    // warp one at a time from counter[1], so that the warps finish together.
    // The warp's position in its chunk lives in shared memory (lane 0 reads
    // and advances it between packets), so no register holds it across the
    // traversal.
    const uint32_t npk = (uint32_t)(((unsigned long long)a.nq + 31) / 32);
    const uint32_t tail = gridDim.x * (blockDim.x >> 5) * kTailPackets;
    const uint32_t chunk = (uint32_t)a.seed_chunk;
    const uint32_t split = npk > tail ? (npk - tail) / chunk * chunk : 0u;
    uint32_t* st_work = reinterpret_cast<uint32_t*>(st_seed + kSeedPoints);  // next packet, chunk end
    if (lane0) {
        st_work[0] = 0;
        st_work[1] = 0;
    }
    for (;;) {
        uint32_t pk = 0, seeded = 0;
        if (lane0) {
            pk = st_work[0];
            if (pk < st_work[1]) {
                seeded = 1;  // the next packet of this warp's chunk
            } else {
                pk = (uint32_t)(atomicAdd(a.counter, (unsigned long long)chunk));
                if (pk < split) {
                    st_work[1] = min(pk + chunk, split);
                } else {
                    pk = split + (uint32_t)atomicAdd(a.counter + 1, 1ull);
                    st_work[1] = 0;
                }
            }
            st_work[0] = pk + 1;
        }
        pk = __shfl_sync(kFull, pk, 0);
        seeded = __shfl_sync(kFull, seeded, 0);
        if (pk >= npk) break;  // warp-uniform exit
        const int64_t i = (int64_t)pk * 32 + lane;
        const bool valid = i < a.nq;
        int64_t qi = 0;
        float qx = 0.f, qy = 0.f, qz = 0.f;
        int m = 0;
        if (valid) {
            qi = a.perm ? (int64_t)ld_stream(a.perm + i) : i;
            qx = ld_stream(a.queries + 3 * qi);
            qy = ld_stream(a.queries + 3 * qi + 1);
            qz = ld_stream(a.queries + 3 * qi + 2);
            m = a.nmeshes > 1 ? mesh_of(a.qoff, a.nmeshes, qi) : 0;
        }
        // Seed: after a chunk's first packet each lane starts from its least
        // distance to the previous packet's kSeedPoints closest points (same
        // mesh), padded.  Those points lie on the mesh up to FP32 rounding,
        // so the padded distance (1 + 1e-4 relative, plus 4e-6 of the mesh's
        // extent, the query's magnitude and the distance) exceeds the query's
        // true distance by far more than the box and triangle tests err: no
        // box or triangle that can hold the nearest triangle is pruned, and
        // the answer is the unseeded one.  The seed enters as the lane's best
        // key (its squared distance over the index INT_MAX, which no triangle
        // has), so traversal prunes against it like any candidate.
        unsigned long long best = kNoKey;
        if (seeded) {
            __syncwarp();  // the previous packet's slot writes come first
            float m2 = INFINITY;
#pragma unroll
            for (int j = 0; j < kSeedPoints; ++j) {
                const float4 sp4 = st_seed[j];
                const float dx = qx - sp4.x, dy = qy - sp4.y, dz = qz - sp4.z;
                const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                if (__float_as_int(sp4.w) == m && d2 < m2) m2 = d2;  // a NaN point fails the compare
            }
            if (valid && m2 < INFINITY) {
                const float* bx = a.box + 6 * (int64_t)__ldg(a.mesh_root + m);
                const float ext = max3f(__ldg(bx + 3) - __ldg(bx), __ldg(bx + 4) - __ldg(bx + 1),
                                        __ldg(bx + 5) - __ldg(bx + 2));
                const float qa = max3f(fabsf(qx), fabsf(qy), fabsf(qz));
                const float d = sqrtf(m2);
                const float sd = fmaf(d, 1.0001f, 4e-6f * (ext + qa + d));
                best = kSeedKeyLow | ((unsigned long long)__float_as_uint(sd * sd) << 32);
            }
        }
        unsigned pending = __ballot_sync(kFull, valid);
        bool retried = false;
        while (pending) {
            const int leader = __ffs(pending) - 1;
            const int mesh = __shfl_sync(kFull, m, leader);
            const bool mine = ((pending >> lane) & 1u) && m == mesh;
            pending &= ~__ballot_sync(kFull, mine);
            // lanes outside this round never need anything: bound -inf
            float lim = mine ? key_d2(best) : -INFINITY;
            int sp = 0;            // stack entries; only the top one can be used up
            uint32_t t_order = 0;  // the top entry's slots still to visit, next in the low nibble
            int t_cnt = 0;         // and their number
            int cur = a.wide_root[mesh];
            // this lane's bound admitted the node being visited (the root, a
            // wide node, admits the round's lanes); used at leaves
            bool leaf_active = mine;
            for (;;) {
                if (cur >= 0) {
                    if (kStats) {
                        ++n_nodes;
                        n_lane_nodes += __popc(__ballot_sync(kFull, leaf_active));
                    }
                    const WideNode<K>* nd = nodes + cur;
                    f32x2 lox[K / 2], hix[K / 2], loy[K / 2], hiy[K / 2], loz[K / 2], hiz[K / 2];
                    int32_t ch[K];
                    load_row2<K>(nd->lox, lox);
                    load_row2<K>(nd->hix, hix);
                    load_row2<K>(nd->loy, loy);
                    load_row2<K>(nd->hiy, hiy);
                    load_row2<K>(nd->loz, loz);
                    load_row2<K>(nd->hiz, hiz);
                    load_row_i<K>(nd->child, ch);
                    // box lower bounds, two children per packed operation
                    // (the query's packed copies made here, not held across
                    // the traversal: three register pairs fewer in the loop,
                    // 0.5% faster on the large workload)
                    const f32x2 qx2 = f2_pack(qx, qx), qy2 = f2_pack(qy, qy), qz2 = f2_pack(qz, qz);
                    float lb[K];
#pragma unroll
                    for (int j = 0; j < K / 2; ++j) {
                        const f32x2 dx = box_axis2(qx2, lox[j], hix[j]);
                        const f32x2 dy = box_axis2(qy2, loy[j], hiy[j]);
                        const f32x2 dz = box_axis2(qz2, loz[j], hiz[j]);
                        f2_unpack(f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx))), lb[2 * j], lb[2 * j + 1]);
                    }
                    // each lane's needed children, and its nearest as the least
                    // (bound bits | slot) unsigned key: non-negative floats
                    // order as their bit patterns, and the cleared sign bit
                    // keeps every needed key below the sentinel
                    uint32_t mine_need = 0, kmine = 0xFFFFFFFFu;
#pragma unroll
                    for (int s = 0; s < K; ++s) {
                        const bool want = lb[s] < lim;
                        mine_need |= (want ? 1u : 0u) << s;
                        kmine = min(kmine, want ? ((__float_as_uint(lb[s]) & 0x7FFFFFF8u) | (uint32_t)s)
                                                : 0xFFFFFFFFu);
                    }
                    const uint32_t need = __reduce_or_sync(kFull, mine_need);
                    if (need != 0) {
                        // go first to the child nearest to any lane
                        const int f = (int)(__reduce_min_sync(kFull, kmine) & 7u);
                        const uint32_t rest = need & ~(1u << f);
                        int32_t cf = ch[0];
#pragma unroll
                        for (int s = 1; s < K; ++s) cf = f == s ? ch[s] : cf;
                        if (rest != 0) {
                            // the node becomes the top entry; a used-up top
                            // entry is overwritten, a live one keeps its list
                            if (sp > 0) {
                                if (t_cnt == 0) --sp;
                                else if (lane0) st_state[sp - 1] = make_uint2(t_order, (uint32_t)t_cnt);
                            }
                            if (sp >= cap) {  // cannot happen: cap bounds the depth
                                atomicOr(a.status, 1u);
                                sp = cap - 1;
                            }
                            store_row<K>(st_bnd + sp * 32 * K, lb);
                            if (lane0) store_row<K>(st_ch + sp * K, ch);
                            t_order = c_slot_lists.v[rest];
                            t_cnt = __popc(rest);
                            ++sp;
                            __syncwarp();
                        }
                        cur = cf;
                        leaf_active = (mine_need >> f) & 1u;
                        continue;
                    }
                } else {
                    const int first = leaf_first(cur), cnt = leaf_count(cur);
                    if (kStats) n_tris += cnt;
                    const uint32_t act = __ballot_sync(kFull, leaf_active);
                    const int na = __popc(act);
                    if (kStats) n_lane_tris += (unsigned long long)na * cnt;
                    if (kCompact && cnt >= 2 && na >= 1 && na <= 16) {
                        // Few lanes need this leaf: spread its (query, triangle)
                        // pairs over the warp.  A round covers kpr = 32 / na
                        // triangles: lane w tests triangle k0 + w / na against
                        // the (w % na)-th active lane's query, and each active
                        // lane takes the minimum of its keys (order-free, so
                        // the result is the same).
                        const LeafSplit sp2 = c_leaf_splits.v[na];
                        const int r = __popc(act & lt_mask);
                        if (leaf_active) st_q[r] = make_float4(qx, qy, qz, 0.0f);
                        __syncwarp();
                        // w / na, exact: (w + 1/2) / na is at least 1/32 from an integer
                        const int kk = (int)(((float)lane + 0.5f) * sp2.inv);
                        const bool worker = lane < sp2.kpr * na;
                        const float4 qq = st_q[worker ? lane - kk * na : 0];
                        // a worker serves the same query in every round: keep
                        // its minimum and gather once
                        unsigned long long key = kNoKey;
                        for (int k0 = 0; k0 < cnt; k0 += sp2.kpr) {
                            if (kStats) ++n_rounds;
                            const int k = k0 + kk;
                            if (worker && k < cnt) {
                                const FastTri f = load_fast(a.fast + first + k);
                                key = min(key, best_key(tri_d2_fast(qq.x, qq.y, qq.z, f), fast_index(f)));
                            }
                        }
                        const int nk = min(sp2.kpr, cnt);
                        for (int j = 0; j < nk; ++j) {
                            const unsigned long long got = __shfl_sync(kFull, key, (r + j * na) & 31);
                            if (leaf_active) best = min(best, got);
                        }
                    } else {
                        if (kStats) n_rounds += cnt;
                        for (int k = 0; k < cnt; ++k) {
                            const FastTri f = load_fast(a.fast + first + k);
                            if (leaf_active)
                                best = min(best, best_key(tri_d2_fast(qx, qy, qz, f), fast_index(f)));
                        }
                    }
                    if (mine) lim = key_d2(best);
                }
                // pop: the top entry's next slot that some lane still needs
                bool found = false;
                for (;;) {
                    if (t_cnt == 0) {
                        if (sp <= 1) break;
                        --sp;
                        const uint2 s2 = st_state[sp - 1];
                        t_order = s2.x;
                        t_cnt = (int)s2.y;
                        continue;
                    }
                    const int s = (int)(t_order & 15u);
                    t_order >>= 4;
                    --t_cnt;
                    const int e = sp - 1;
                    const bool want = st_bnd[e * 32 * K + s] < lim;
                    if (kStats) ++n_pops;
                    if (__any_sync(kFull, want)) {
                        cur = st_ch[e * K + s];
                        leaf_active = want;
                        found = true;
                        break;
                    }
                    if (kStats) ++n_skips;
                }
                __syncwarp();  // the reads above come before a push's writes
                if (!found) break;
            }
            // after the last mesh group: a lane whose seed left it no
            // triangle (not expected: the seed is an upper bound with a
            // margin) runs again unseeded
            if (!pending && !retried) {
                retried = true;
                const bool empty = valid && (uint32_t)best == (uint32_t)kSeedKeyLow && best != kNoKey;
                pending = __ballot_sync(kFull, empty);
                if (empty) best = kNoKey;
            }
        }
        float px = __int_as_float(0x7fc00000), py = px, pz = px;
        if (valid) {
            // the winner's record: its triangle through the build's inverse order
            const int idx = (int)(uint32_t)best;
            const int rec = best == kNoKey ? -1 : a.inv_order[a.toff[m] + idx];
            write_result(a, qi, qx, qy, qz, rec, idx, px, py, pz);
        }
        // this packet's closest points seed the next one
        constexpr int kStride = 32 / kSeedPoints;
        if (lane % kStride == 0) st_seed[lane / kStride] = make_float4(px, py, pz, __int_as_float(valid ? m : -1));
    }
    if (kStats && a.stats && lane == 0) {
        atomicAdd(&a.stats[0], n_nodes);
        atomicAdd(&a.stats[1], n_tris);
        atomicAdd(&a.stats[2], n_pops);
        atomicAdd(&a.stats[3], n_skips);
        atomicAdd(&a.stats[4], n_lane_tris);
        atomicAdd(&a.stats[5], n_rounds);
        atomicAdd(&a.stats[6], n_lane_nodes);
    }
}

// Index of cell (x, y, z) along the 3D Hilbert curve of 2^bits cells per axis
// (Skilling 2004, "Programming the Hilbert curve": undo the excess rotations
// and reflections level by level, Gray-encode, then read the transposed
// coordinates out bit-interleaved).  Consecutive indices are face-adjacent
// cells, unlike Morton order, which jumps at every octant boundary; a warp
// of 32 consecutive queries is therefore a tighter cluster, and the next
// warp's cluster lies next to it.
__device__ __forceinline__ uint64_t hilbert3(uint32_t x, uint32_t y, uint32_t z, int bits) {
    uint32_t X[3] = {x, y, z};
    const uint32_t top = 1u << (bits - 1);
    for (uint32_t Q = top; Q > 1; Q >>= 1) {
        const uint32_t P = Q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                const uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];
    X[2] ^= X[1];
    uint32_t t = 0;
    for (uint32_t Q = top; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    return (spread3(X[0]) << 2) | (spread3(X[1]) << 1) | spread3(X[2]);
}

// bit k of a 10-bit x to bit 3k, in 32-bit arithmetic
__device__ __forceinline__ uint32_t spread3_10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// hilbert3 for 10 bits per axis (every single-mesh ordering), unrolled, with
// selects in place of branches and 32-bit bit spreading: the same index.
__device__ __forceinline__ uint32_t hilbert3_10(uint32_t x, uint32_t y, uint32_t z) {
    uint32_t X0 = x, X1 = y, X2 = z;
#pragma unroll
    for (int b = 9; b >= 1; --b) {
        const uint32_t Q = 1u << b, P = Q - 1;
        X0 ^= (X0 & Q) ? P : 0u;
        const uint32_t t1 = (X0 ^ X1) & P;
        const bool h1 = (X1 & Q) != 0u;
        X0 ^= h1 ? P : t1;
        X1 ^= h1 ? 0u : t1;
        const uint32_t t2 = (X0 ^ X2) & P;
        const bool h2 = (X2 & Q) != 0u;
        X0 ^= h2 ? P : t2;
        X2 ^= h2 ? 0u : t2;
    }
    X1 ^= X0;
    X2 ^= X1;
    uint32_t t = 0;
#pragma unroll
    for (int b = 9; b >= 1; --b) t ^= (X2 & (1u << b)) ? ((1u << b) - 1u) : 0u;
    X0 ^= t;
    X1 ^= t;
    X2 ^= t;
    return (spread3_10(X0) << 2) | (spread3_10(X1) << 1) | spread3_10(X2);
}

// Ordering key of each query: its mesh in the high bits, then the Hilbert
// index of its cell in the mesh's isotropic query frame.
template <typename KeyT>
__global__ void k_query_keys(const float* __restrict__ q, int64_t nq, const int64_t* __restrict__ qoff,
                             int nmeshes, const float* __restrict__ frame, int qbits,
                             KeyT* __restrict__ keys) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const int m = nmeshes > 1 ? mesh_of(qoff, nmeshes, i) : 0;
    const float* f = frame + 6 * m;
    const float maxcell = (float)((1u << qbits) - 1u);
    uint32_t c[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float t = (q[3 * i + k] - f[k]) * f[3 + k];
        t = fminf(fmaxf(t, 0.0f), maxcell);  // NaN -> 0
        c[k] = (uint32_t)t;
    }
    const uint64_t h = qbits == 10 ? hilbert3_10(c[0], c[1], c[2]) : hilbert3(c[0], c[1], c[2], qbits);
    keys[i] = (KeyT)(((uint64_t)m << (3 * qbits)) | h);
}

__device__ __forceinline__ void atomic_min_pos(float* addr, float v) {
    if (v >= 0.0f) atomicMin(reinterpret_cast<int*>(addr), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned*>(addr), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_pos(float* addr, float v) {
    if (v >= 0.0f) atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned*>(addr), __float_as_uint(v));
}

__global__ void k_init_qbounds(float* __restrict__ qb, int nmeshes) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * nmeshes) qb[i] = (i % 6) < 3 ? INFINITY : -INFINITY;
}

// Per-mesh bounding box of the finite query points.  Each block reduces one
// contiguous chunk; a thread keeps a running box and flushes it with atomics
// only when the mesh changes and at the end (warp-reduced when the warp's
// lanes agree on the mesh), so a 16M-query call issues a few thousand atomics
// rather than one set per warp of queries.
__device__ __forceinline__ void flush_box(float* __restrict__ qb, int m, const float* lo,
                                          const float* hi) {
    for (int k = 0; k < 3; ++k) {
        atomic_min_pos(&qb[6 * m + k], lo[k]);
        atomic_max_pos(&qb[6 * m + 3 + k], hi[k]);
    }
}

__global__ void __launch_bounds__(256) k_query_bounds(const float* __restrict__ q, int64_t nq,
                                                      const int64_t* __restrict__ qoff, int nmeshes,
                                                      float* __restrict__ qb) {
    const int64_t per_block = (nq + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = (int64_t)blockIdx.x * per_block;
    const int64_t b1 = min(nq, b0 + per_block);
    int cur = -1;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const float x = q[3 * i], y = q[3 * i + 1], z = q[3 * i + 2];
        if (!(isfinite(x) && isfinite(y) && isfinite(z))) continue;
        const int m = nmeshes > 1 ? mesh_of(qoff, nmeshes, i) : 0;
        if (m != cur) {
            if (cur >= 0) flush_box(qb, cur, lo, hi);
            cur = m;
            lo[0] = lo[1] = lo[2] = INFINITY;
            hi[0] = hi[1] = hi[2] = -INFINITY;
        }
        lo[0] = fminf(lo[0], x); lo[1] = fminf(lo[1], y); lo[2] = fminf(lo[2], z);
        hi[0] = fmaxf(hi[0], x); hi[1] = fmaxf(hi[1], y); hi[2] = fmaxf(hi[2], z);
    }
    const int c0 = __shfl_sync(kFull, cur, 0);
    if (__all_sync(kFull, cur == c0)) {
        if (c0 < 0) return;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(kFull, lo[k], o));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(kFull, hi[k], o));
            }
        if ((threadIdx.x & 31) == 0) flush_box(qb, c0, lo, hi);
    } else if (cur >= 0) {
        flush_box(qb, cur, lo, hi);
    }
}

// Isotropic Morton frame over each mesh's query box: the same cell size on
// every axis, so 32 consecutive codes are a compact cluster of queries (with
// the mesh's box instead, queries above or below a flat mesh collapse into
// one clamped layer of cells and a warp's queries spread far apart).
__global__ void k_query_frame(float* __restrict__ qb, int nmeshes, float cells) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmeshes) return;
    float ext = 0.0f;
    for (int k = 0; k < 3; ++k) {
        const float e = qb[6 * m + 3 + k] - qb[6 * m + k];
        if (e > ext) ext = e;  // NaN / empty boxes leave ext at 0
    }
    const float scale = ext > 0.0f && ext < INFINITY ? cells / ext : 0.0f;
    for (int k = 0; k < 3; ++k) {
        if (!(qb[6 * m + k] > -INFINITY && qb[6 * m + k] < INFINITY)) qb[6 * m + k] = 0.0f;
        qb[6 * m + 3 + k] = scale;
    }
}

// Adjoint: recompute p from (tri, bary), scatter -b_k g (q - p)/d to the
// triangle's vertices.  Lanes that hit the same vertex are summed inside the
// warp first (match_any + an ordered shuffle loop) and one lane adds.
__device__ __forceinline__ void warp_add3(float* __restrict__ base, int vid, float x, float y, float z) {
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(kFull, vid);
    const bool shared = __any_sync(kFull, vid >= 0 && __popc(peers) > 1);
    if (!shared) {
        if (vid >= 0) {
            atomicAdd(base + 3 * (int64_t)vid, x);
            atomicAdd(base + 3 * (int64_t)vid + 1, y);
            atomicAdd(base + 3 * (int64_t)vid + 2, z);
        }
        return;
    }
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
#pragma unroll 1
    for (int src = 0; src < 32; ++src) {
        const float vx = __shfl_sync(kFull, x, src);
        const float vy = __shfl_sync(kFull, y, src);
        const float vz = __shfl_sync(kFull, z, src);
        if ((peers >> src) & 1u) {
            sx += vx;
            sy += vy;
            sz += vz;
        }
    }
    if (vid >= 0 && (__ffs(peers) - 1) == lane) {
        atomicAdd(base + 3 * (int64_t)vid, sx);
        atomicAdd(base + 3 * (int64_t)vid + 1, sy);
        atomicAdd(base + 3 * (int64_t)vid + 2, sz);
    }
}

__global__ void __launch_bounds__(256) k_backward(const TriRec* __restrict__ recs,
                                                   const int32_t* __restrict__ inv_order,
                                                   const int32_t* __restrict__ tris, int64_t nt,
                                                   const float* __restrict__ q,
                                                   const int32_t* __restrict__ tri,
                                                   const float* __restrict__ bary,
                                                   const float* __restrict__ grad, int64_t nq,
                                                   float* __restrict__ grad_q,
                                                   float* __restrict__ grad_v,
                                                   uint32_t* __restrict__ status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int32_t t = -1;
    float gx = 0.f, gy = 0.f, gz = 0.f, u = 0.f, v = 0.f, w = 0.f;
    if (i < nq) {
        t = tri[i];
        if (t >= nt) {
            atomicOr(status, 2u);
            t = -1;
        }
        if (t >= 0) {
            const float4* rp = reinterpret_cast<const float4*>(recs + inv_order[t]);
            TriRec r;
            r.p0 = __ldg(rp);
            r.p1 = __ldg(rp + 1);
            r.p2 = __ldg(rp + 2);
            const float qx = q[3 * i], qy = q[3 * i + 1], qz = q[3 * i + 2];
            ff fv, fw;
            if (bary) {
                fv = ff_from(bary[2 * i]);
                fw = ff_from(bary[2 * i + 1]);
            } else {
                precise_bary(qx, qy, qz, r, fv, fw);
            }
            ff3 res, off;
            precise_residual(qx, qy, qz, r, fv, fw, res, off);
            const float d = ff_to_float(ff_sqrt(ff3_dot(res, res)));
            v = ff_to_float(fv);
            w = ff_to_float(fw);
            u = ff_to_float(ff_sub(ff_sub(ff_from(1.0f), fv), fw));
            const float s = d > 0.0f ? grad[i] / d : 0.0f;
            gx = s * ff_to_float(res.x);
            gy = s * ff_to_float(res.y);
            gz = s * ff_to_float(res.z);
        }
        if (grad_q) {
            grad_q[3 * i] = gx;
            grad_q[3 * i + 1] = gy;
            grad_q[3 * i + 2] = gz;
        }
    }
    if (grad_v == nullptr) return;  // uniform across the grid
    int v0 = -1, v1 = -1, v2 = -1;
    if (t >= 0) {
        v0 = tris[3 * (int64_t)t];
        v1 = tris[3 * (int64_t)t + 1];
        v2 = tris[3 * (int64_t)t + 2];
    }
    warp_add3(grad_v, v0, -u * gx, -u * gy, -u * gz);
    warp_add3(grad_v, v1, -v * gx, -v * gy, -v * gz);
    warp_add3(grad_v, v2, -w * gx, -w * gy, -w * gz);
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct QueryLayout {
    size_t keys = 0, vals = 0, keys_alt = 0, vals_alt = 0, sort_ws = 0, counter = 0, total = 0;
    size_t sort_ws_bytes = 0, frame = 0;
};

QueryLayout layout(int64_t nq, int nmeshes, bool sort) {
    QueryLayout L;
    size_t off = 0;
    L.counter = off;
    off += 256;
    if (sort && nq > 1) {
        L.frame = off; off += align256(sizeof(float) * 6 * nmeshes);
        L.keys = off; off += align256(sizeof(uint64_t) * nq);
        L.vals = off; off += align256(sizeof(int32_t) * nq);
        L.keys_alt = off; off += align256(sizeof(uint64_t) * nq);
        L.vals_alt = off; off += align256(sizeof(int32_t) * nq);
        L.sort_ws = off;
        L.sort_ws_bytes = radix_sort_workspace_bytes(nq);
        off += align256(L.sort_ws_bytes);
    }
    L.total = off;
    return L;
}

// Opt-in CUDA-event timing of every traversal launch (cp_timing_*).
struct TraverseTiming {
    std::mutex mu;
    bool on = false;        // events around each traversal launch
    bool counters = false;  // packet traversals run their counting build
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    double ms = 0.0;
    int64_t launches = 0;
    unsigned long long* stats = nullptr;  // device: packet visit counters
};
TraverseTiming g_timing;

template <int K, int S>
cudaError_t launch_traverse(const TraverseArgs& args, int block, int blocks_per_sm, cudaStream_t st,
                            bool allow_timing) {
    const size_t smem = (size_t)S * block * sizeof(float2);
    auto kern = k_traverse<K, S>;
    int sms = 0;
    cudaError_t e = sm_count(&sms);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm <= 0) {
        e = cpq::blocks_per_sm(reinterpret_cast<const void*>(kern), block, smem, &blocks_per_sm);
        if (e != cudaSuccess) return e;
    }
    int64_t grid = (int64_t)sms * blocks_per_sm;
    const int64_t need = (args.nq + 31) / 32 * 32 / block + 1;
    if (grid > need) grid = need;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool timed = false;
    {
        std::lock_guard<std::mutex> lock(g_timing.mu);
        timed = g_timing.on && allow_timing;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cap);
    if (timed && cap == cudaStreamCaptureStatusNone) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, st);
    } else {
        timed = false;
    }
    kern<<<(unsigned)grid, block, smem, st>>>(args); note_launch();
    e = cudaGetLastError();
    if (timed) {
        cudaEventRecord(e1, st);
        std::lock_guard<std::mutex> lock(g_timing.mu);
        g_timing.pending.emplace_back(e0, e1);
    }
    return e;
}

template <int K>
cudaError_t launch_packet(const TraverseArgs& args, int cap, bool compact, int block,
                          int blocks_per_sm, cudaStream_t st, bool allow_timing) {
    if (cap < 1) cap = 1;
    size_t smem = (size_t)(block / 32) * packet_warp_bytes(K, cap, compact);
    cudaError_t e;
    if (smem > 48 * 1024) {
        // very deep trees: fewer warps per block until the stacks fit
        int dev = 0, optin = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        while (block > 32 && smem > (size_t)optin) {
            block /= 2;
            smem = (size_t)(block / 32) * packet_warp_bytes(K, cap, compact);
        }
    }
    auto kern = compact ? (args.stats ? k_traverse_packet<K, true, true> : k_traverse_packet<K, true, false>)
                        : (args.stats ? k_traverse_packet<K, false, true> : k_traverse_packet<K, false, false>);
    e = ensure_smem_limit(reinterpret_cast<const void*>(kern), smem);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = sm_count(&sms);
    if (e != cudaSuccess) return e;
    if (blocks_per_sm <= 0) {
        e = cpq::blocks_per_sm(reinterpret_cast<const void*>(kern), block, smem, &blocks_per_sm);
        if (e != cudaSuccess) return e;
    }
    int64_t grid = (int64_t)sms * blocks_per_sm;
    const int64_t need = ((args.nq + 31) / 32 * 32 + block - 1) / block;
    if (grid > need) grid = need;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool timed = false;
    {
        std::lock_guard<std::mutex> lock(g_timing.mu);
        timed = g_timing.on && allow_timing;
    }
    cudaStreamCaptureStatus capst = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &capst);
    if (timed && capst == cudaStreamCaptureStatusNone) {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, st);
    } else {
        timed = false;
    }
    kern<<<(unsigned)grid, block, smem, st>>>(args, cap); note_launch();
    e = cudaGetLastError();
    if (timed) {
        cudaEventRecord(e1, st);
        std::lock_guard<std::mutex> lock(g_timing.mu);
        g_timing.pending.emplace_back(e0, e1);
    }
    return e;
}

template <int K>
cudaError_t launch_k(const TraverseArgs& args, const QueryParams& qp, int cap, bool compact,
                     cudaStream_t st) {
    // packet traversal needs spatially coherent warps: the default whenever
    // the queries are walked in Hilbert order
    const bool packet = qp.traversal == 2 || (qp.traversal == 0 && qp.sort);
    const bool allow_timing = !qp.no_timing;
    if (packet) return launch_packet<K>(args, cap, compact, qp.block, qp.blocks_per_sm, st, allow_timing);
    switch (qp.short_stack) {
        case 4: return launch_traverse<K, 4>(args, qp.block, qp.blocks_per_sm, st, allow_timing);
        case 16: return launch_traverse<K, 16>(args, qp.block, qp.blocks_per_sm, st, allow_timing);
        default: return launch_traverse<K, 8>(args, qp.block, qp.blocks_per_sm, st, allow_timing);
    }
}

// ---- instances: two-level traversal ------------------------------------------
//
// The reference places meshes with a TLAS of transformed BLAS instances
// (Accel::recreate(blas, T), src/vk/vulkan.cpp:777-856; per-object model
// matrices, src/rt/rt.cpp:31-45).  Here a top-level wide BVH over the
// instances' world boxes is walked closest first in world space; at an
// instance the query is taken to the mesh's object space and the mesh's own
// BVH (a batch's) is walked with the world bound divided by the instance's
// squared scale — instances are similarity transforms, under which distances
// scale by s.  The winner is re-evaluated in float-float in WORLD space: its
// object-space barycentrics give the point, the instance's 3x4 matrix takes
// it to world space in float-float, and the residual to the query is formed
// there, so the distance keeps the accuracy of the plain path.

struct InstArgs {
    const void* tnodes;        // top level: wide BVH over the instances' world boxes
    const TriRec* trecs;       // its leaf records; p2.y = instance index
    const int32_t* troot;      // device: its root reference
    const void* bnodes;        // bottom level: the batch's meshes
    const FastTri* bfast;
    const TriRec* brecs;
    const int32_t* broot;      // per mesh
    const int32_t* binv_order; // the batch's global triangle -> record position
    const int64_t* btoff;      // the batch's per-mesh triangle offsets
    const void* knodes;        // baked level: world-space copies of the general-affine instances
    const FastTri* kfast;
    const int32_t* kroot;      // per baked instance
    const int32_t* inst_mesh;  // per instance
    const int32_t* inst_baked; // per instance: its baked copy, or -1 (a similarity)
    const float* inst_inv;     // 12 per instance: object <- world, row-major 3 x 4 (3 x 3 part used)
    const float* inst_fwd;     // 12 per instance: world <- object
    const float* inst_s2;      // 2 per instance: squared scale (ranking), its lower bound (pruning)
    const float* queries;
    const int32_t* perm;
    int64_t nq;
    float* out_point;
    float* out_dist;
    int32_t* out_inst;
    int32_t* out_tri;
    float* out_bary;
    unsigned long long* counter;
    uint32_t* status;
};

__device__ __forceinline__ void affine(const float* m, float x, float y, float z, float& ox, float& oy,
                                       float& oz) {
    ox = fmaf(m[0], x, fmaf(m[1], y, fmaf(m[2], z, m[3])));
    oy = fmaf(m[4], x, fmaf(m[5], y, fmaf(m[6], z, m[7])));
    oz = fmaf(m[8], x, fmaf(m[9], y, fmaf(m[10], z, m[11])));
}

// World to object coordinates: the translation off first, then the inverse's
// 3 x 3 part, so the rounding is relative to the point's distance from the
// instance's origin and not to its world coordinates.
__device__ __forceinline__ void to_object(const float* inv, const float* fwd, float x, float y, float z,
                                          float& ox, float& oy, float& oz) {
    const float dx = x - fwd[3], dy = y - fwd[7], dz = z - fwd[11];
    ox = fmaf(inv[0], dx, fmaf(inv[1], dy, inv[2] * dz));
    oy = fmaf(inv[4], dx, fmaf(inv[5], dy, inv[6] * dz));
    oz = fmaf(inv[8], dx, fmaf(inv[9], dy, inv[10] * dz));
}

// Closest-first walk of one mesh's BVH from `root` for one point: nodes whose
// box bound is below `lim` are visited nearest first; on return `lim` is the
// best squared distance found (unchanged if none), with its record and index.
// The stack holds at most (K-1)(depth+1) <= kStackTotal entries.
template <int K>
__device__ void walk_mesh(const WideNode<K>* __restrict__ nodes, const FastTri* __restrict__ fast,
                     const TriRec* __restrict__ recs, int32_t root, float qx, float qy, float qz,
                     float& lim, int& rec, int& idx, float2* stack, uint32_t* status) {
    int sp = 0;
    stack[sp++] = make_float2(0.0f, __int_as_float(root));
    while (sp > 0) {
        const float2 e = stack[--sp];
        if (!(e.x < lim)) continue;
        const int cur = __float_as_int(e.y);
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
            float lb[K];
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const float d = box_lb2(qx, qy, qz, lox[s], hix[s], loy[s], hiy[s], loz[s], hiz[s]);
                lb[s] = d < lim ? d : INFINITY;
            }
            sort_children<K>(lb, ch);
#pragma unroll
            for (int s = K - 1; s >= 0; --s) {
                if (lb[s] < INFINITY) {
                    if (sp < kStackTotal) stack[sp++] = make_float2(lb[s], __int_as_float(ch[s]));
                    else atomicOr(status, 1u);
                }
            }
        } else {
            const int first = leaf_first(cur), cnt = leaf_count(cur);
            for (int k = 0; k < cnt; ++k) {
                const FastTri f = load_fast(fast + first + k);
                const float d2 = tri_d2_fast(qx, qy, qz, f);
                const int i = fast_index(f);
                if (d2 < lim || (d2 == lim && rec >= 0 && i < idx)) {
                    lim = d2;
                    rec = first + k;
                    idx = i;
                }
            }
        }
    }
}

// The winner of an instanced query, finished in world space from its exact
// object-space record (any walk: per thread or packet), and the outputs.
__device__ void instance_finish(const InstArgs& a, int64_t qi, float qx, float qy, float qz, int binst,
                                int bidx) {
    float dist = __int_as_float(0x7fc00000), px = dist, py = dist, pz = dist, bv = dist, bw = dist;
    // the winner's exact object-space record, whichever level found it
    const int brec = binst >= 0 ? a.binv_order[a.btoff[a.inst_mesh[binst]] + bidx] : -1;
    if (brec >= 0) {
        const float4* rp = reinterpret_cast<const float4*>(a.brecs + brec);
        TriRec r;
        r.p0 = __ldg(rp);
        r.p1 = __ldg(rp + 1);
        r.p2 = __ldg(rp + 2);
        // the world triangle: the instance matrix applied to the FP32
        // vertices in float-float (products exact, sums to ~2^-44)
        const float* f = a.inst_fwd + 12 * binst;
        const float ov[3][3] = {{r.p0.x, r.p0.y, r.p0.z}, {r.p0.w, r.p1.x, r.p1.y}, {r.p1.z, r.p1.w, r.p2.x}};
        ff3 wv[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            ff c[3];
#pragma unroll
            for (int j = 0; j < 3; ++j)
                c[j] = ff_add(ff_add(ff_two_prod(f[4 * j], ov[k][0]), ff_two_prod(f[4 * j + 1], ov[k][1])),
                              ff_add(ff_two_prod(f[4 * j + 2], ov[k][2]), ff_from(f[4 * j + 3])));
            wv[k] = {c[0], c[1], c[2]};
        }
        const ff3 q3 = ff3_from(qx, qy, qz);
        TriDiff t;
        t.ab = ff3_sub(wv[1], wv[0]);
        t.ac = ff3_sub(wv[2], wv[0]);
        t.ap = ff3_sub(q3, wv[0]);
        ff v, w;
        // degenerate in world space: the object triangle's flag, or the same
        // area test on the rounded world edges (a singular matrix flattens
        // triangles)
        const float e1x = ff_to_float(t.ab.x), e1y = ff_to_float(t.ab.y), e1z = ff_to_float(t.ab.z);
        const float e2x = ff_to_float(t.ac.x), e2y = ff_to_float(t.ac.y), e2z = ff_to_float(t.ac.z);
        const float cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
        const float l1 = e1x * e1x + e1y * e1y + e1z * e1z, l2 = e2x * e2x + e2y * e2y + e2z * e2z;
        const bool flat = !(cx * cx + cy * cy + cz * cz > 1e-10f * (l1 * l2));
        if ((__float_as_uint(r.p2.z) & kTriDegenerate) || flat) {
            TriRec rw = r;  // degenerate: the FP32 edge search on the rounded world vertices
            rw.p0 = make_float4(ff_to_float(wv[0].x), ff_to_float(wv[0].y), ff_to_float(wv[0].z),
                                ff_to_float(wv[1].x));
            rw.p1 = make_float4(ff_to_float(wv[1].y), ff_to_float(wv[1].z), ff_to_float(wv[2].x),
                                ff_to_float(wv[2].y));
            rw.p2.x = ff_to_float(wv[2].z);
            float fv, fw;
            degenerate_bary(qx, qy, qz, rw, fv, fw);
            v = ff_from(fv);
            w = ff_from(fw);
        } else {
            precise_bary_core(t, ff3_sub(q3, wv[1]), ff3_sub(q3, wv[2]), v, w);
        }
        ff3 res, off;
        precise_residual_d(t, v, w, res, off);
        dist = ff_to_float(ff_sqrt(ff3_dot(res, res)));
        px = ff_to_float(ff_add(wv[0].x, off.x));
        py = ff_to_float(ff_add(wv[0].y, off.y));
        pz = ff_to_float(ff_add(wv[0].z, off.z));
        bv = ff_to_float(v);
        bw = ff_to_float(w);
    } else {
        atomicOr(a.status, 4u);
    }
    if (a.out_dist) a.out_dist[qi] = dist;
    if (a.out_inst) a.out_inst[qi] = binst;
    if (a.out_tri) a.out_tri[qi] = brec >= 0 ? bidx : -1;
    if (a.out_point) {
        a.out_point[3 * qi] = px;
        a.out_point[3 * qi + 1] = py;
        a.out_point[3 * qi + 2] = pz;
    }
    if (a.out_bary) {
        a.out_bary[2 * qi] = bv;
        a.out_bary[2 * qi + 1] = bw;
    }
}

// One query of the two-level walk (index i in the work order).
template <int K>
__device__ void instance_point(const InstArgs& a, const WideNode<K>* __restrict__ tnodes,
                               const WideNode<K>* __restrict__ bnodes, int32_t troot, int64_t i,
                               float2* tstack, float2* bstack) {
    const int64_t qi = a.perm ? (int64_t)a.perm[i] : i;
    const float qx = a.queries[3 * qi], qy = a.queries[3 * qi + 1], qz = a.queries[3 * qi + 2];
    float best = INFINITY;
    int binst = -1, bidx = INT_MAX;
    // top level: closest first over instance boxes, instances walked as found
    int tsp = 0;
    tstack[tsp++] = make_float2(0.0f, __int_as_float(troot));
    while (tsp > 0) {
        const float2 e = tstack[--tsp];
        if (!(e.x < best)) continue;
        const int cur = __float_as_int(e.y);
        if (cur >= 0) {
            const WideNode<K>* nd = tnodes + cur;
            float lox[K], hix[K], loy[K], hiy[K], loz[K], hiz[K];
            int32_t ch[K];
            load_row<K>(nd->lox, lox);
            load_row<K>(nd->hix, hix);
            load_row<K>(nd->loy, loy);
            load_row<K>(nd->hiy, hiy);
            load_row<K>(nd->loz, loz);
            load_row<K>(nd->hiz, hiz);
            load_row_i<K>(nd->child, ch);
            float lb[K];
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const float d = box_lb2(qx, qy, qz, lox[s], hix[s], loy[s], hiy[s], loz[s], hiz[s]);
                lb[s] = d < best ? d : INFINITY;
            }
            sort_children<K>(lb, ch);
#pragma unroll
            for (int s = K - 1; s >= 0; --s) {
                if (lb[s] < INFINITY) {
                    if (tsp < kStackTotal) tstack[tsp++] = make_float2(lb[s], __int_as_float(ch[s]));
                    else atomicOr(a.status, 1u);
                }
            }
            continue;
        }
        const int first = leaf_first(cur), cnt = leaf_count(cur);
        for (int k = 0; k < cnt; ++k) {
            const int inst = __float_as_int(__ldg(&a.trecs[first + k].p2.y));
            const int baked = a.inst_baked[inst];
            int rec = -1, idx = INT_MAX;
            float d2w;
            if (baked >= 0) {
                // a general affine instance: its world-space copy, no transform
                float lim = best;
                walk_mesh<K>(static_cast<const WideNode<K>*>(a.knodes), a.kfast, nullptr, a.kroot[baked], qx, qy,
                             qz, lim, rec, idx, bstack, a.status);
                d2w = lim;
            } else {
                float ox, oy, oz;
                to_object(a.inst_inv + 12 * inst, a.inst_fwd + 12 * inst, qx, qy, qz, ox, oy, oz);
                const float s2 = a.inst_s2[2 * inst], s2lo = a.inst_s2[2 * inst + 1];
                // object-space bound: below it lies every triangle whose world
                // distance can beat `best` (s2lo bounds the transform's
                // smallest squared stretch), widened for the FP32 rounding
                float lim = best < INFINITY ? best / s2lo * (1.0f + 1e-5f) : INFINITY;
                walk_mesh<K>(bnodes, a.bfast, a.brecs, a.broot[a.inst_mesh[inst]], ox, oy, oz, lim, rec, idx,
                             bstack, a.status);
                d2w = lim * s2;
            }
            if (rec < 0) continue;
            if (d2w < best || (d2w == best && (inst < binst || (inst == binst && idx < bidx)))) {
                best = d2w;
                binst = inst;
                bidx = idx;
            }
        }
    }
    instance_finish(a, qi, qx, qy, qz, binst, bidx);
}

template <int K>
__global__ void __launch_bounds__(128) k_instances(InstArgs a) {
    const int lane = threadIdx.x & 31;
    const WideNode<K>* __restrict__ tnodes = static_cast<const WideNode<K>*>(a.tnodes);
    const WideNode<K>* __restrict__ bnodes = static_cast<const WideNode<K>*>(a.bnodes);
    float2 tstack[kStackTotal];
    float2 bstack[kStackTotal];
    const int32_t troot = __ldg(a.troot);
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counter, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)a.nq) break;
        const int64_t i = (int64_t)base + lane;
        if (i < a.nq) instance_point<K>(a, tnodes, bnodes, troot, i, tstack, bstack);
    }
}

// ---- instances: packet walk ---------------------------------------------------
//
// The warp-packet traversal of k_traverse_packet as a device function over
// any wide BVH: per-lane query and bound, one shared stack entry per level in
// `stk` (packet_stack_bytes(K, cap)), the packet descending first into the
// child nearest to any lane.  Leaves go to `leaf(first, count, admitted,
// lim)`, which tests them for the lanes its bound admitted and lowers `lim`.
// Lanes that take no part enter with lim = -inf.  The scene kernel nests it:
// at the top level a leaf is an instance, whose handler runs the same walk
// over that instance's mesh with the lanes' object-space queries.
template <int K, class Leaf>
__device__ __forceinline__ void packet_walk(const WideNode<K>* __restrict__ nodes, int32_t root, float qx, float qy,
                                            float qz, bool active, float& lim, unsigned char* stk, int cap,
                                            uint32_t* status, Leaf& leaf) {
    const int lane = threadIdx.x & 31;
    const bool lane0 = lane == 0;
    float* st_bnd = reinterpret_cast<float*>(stk) + lane * K;  // entry e, slot s at [e * 32 * K + s]
    int32_t* st_ch = reinterpret_cast<int32_t*>(stk + (size_t)cap * 128 * K);
    uint2* st_state = reinterpret_cast<uint2*>(stk + (size_t)cap * 132 * K);
    const f32x2 qx2 = f2_pack(qx, qx), qy2 = f2_pack(qy, qy), qz2 = f2_pack(qz, qz);
    int sp = 0;
    uint32_t t_order = 0;
    int t_cnt = 0;
    int cur = root;
    bool leaf_active = active;
    for (;;) {
        if (cur >= 0) {
            const WideNode<K>* nd = nodes + cur;
            f32x2 lox[K / 2], hix[K / 2], loy[K / 2], hiy[K / 2], loz[K / 2], hiz[K / 2];
            int32_t ch[K];
            load_row2<K>(nd->lox, lox);
            load_row2<K>(nd->hix, hix);
            load_row2<K>(nd->loy, loy);
            load_row2<K>(nd->hiy, hiy);
            load_row2<K>(nd->loz, loz);
            load_row2<K>(nd->hiz, hiz);
            load_row_i<K>(nd->child, ch);
            float lb[K];
#pragma unroll
            for (int j = 0; j < K / 2; ++j) {
                const f32x2 dx = box_axis2(qx2, lox[j], hix[j]);
                const f32x2 dy = box_axis2(qy2, loy[j], hiy[j]);
                const f32x2 dz = box_axis2(qz2, loz[j], hiz[j]);
                f2_unpack(f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx))), lb[2 * j], lb[2 * j + 1]);
            }
            uint32_t mine_need = 0, kmine = 0xFFFFFFFFu;
#pragma unroll
            for (int s = 0; s < K; ++s) {
                const bool want = lb[s] < lim;
                mine_need |= (want ? 1u : 0u) << s;
                kmine = min(kmine, want ? ((__float_as_uint(lb[s]) & 0x7FFFFFF8u) | (uint32_t)s) : 0xFFFFFFFFu);
            }
            const uint32_t need = __reduce_or_sync(kFull, mine_need);
            if (need != 0) {
                const int f = (int)(__reduce_min_sync(kFull, kmine) & 7u);
                const uint32_t rest = need & ~(1u << f);
                if (rest != 0) {
                    if (sp > 0) {
                        if (t_cnt == 0) --sp;
                        else if (lane0) st_state[sp - 1] = make_uint2(t_order, (uint32_t)t_cnt);
                    }
                    if (sp >= cap) {  // cannot happen: cap bounds the depth
                        atomicOr(status, 1u);
                        sp = cap - 1;
                    }
                    store_row<K>(st_bnd + sp * 32 * K, lb);
                    if (lane0) store_row<K>(st_ch + sp * K, ch);
                    t_order = c_slot_lists.v[rest];
                    t_cnt = __popc(rest);
                    ++sp;
                    __syncwarp();
                }
                int32_t cf = ch[0];
#pragma unroll
                for (int s = 1; s < K; ++s) cf = f == s ? ch[s] : cf;
                cur = cf;
                leaf_active = (mine_need >> f) & 1u;
                continue;
            }
        } else {
            leaf(leaf_first(cur), leaf_count(cur), leaf_active, lim);
        }
        bool found = false;
        for (;;) {
            if (t_cnt == 0) {
                if (sp <= 1) break;
                --sp;
                const uint2 s2 = st_state[sp - 1];
                t_order = s2.x;
                t_cnt = (int)s2.y;
                continue;
            }
            const int s = (int)(t_order & 15u);
            t_order >>= 4;
            --t_cnt;
            const int e = sp - 1;
            const bool want = st_bnd[e * 32 * K + s] < lim;
            if (__any_sync(kFull, want)) {
                cur = st_ch[e * K + s];
                leaf_active = want;
                found = true;
                break;
            }
        }
        __syncwarp();
        if (!found) break;
    }
}

__host__ __device__ constexpr size_t scene_warp_bytes(int K, int cap_t, int cap_b) {
    return packet_stack_bytes(K, cap_t) + packet_stack_bytes(K, cap_b) + 32 * sizeof(float4);
}

// 7 blocks of 128 per SM: what two 4-wide stacks per warp leave of shared
// memory on the scenes measured; the register cap it implies (73) spills 32
// bytes, and 28 warps instead of 24 gave 1% more queries per second.
template <int K>
__global__ void __launch_bounds__(128, 7) k_instances_packet(InstArgs a, int cap_t, int cap_b) {
    extern __shared__ __align__(16) unsigned char s_sc[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned char* stk_t = s_sc + (size_t)warp * scene_warp_bytes(K, cap_t, cap_b);
    unsigned char* stk_b = stk_t + packet_stack_bytes(K, cap_t);
    float4* st_q = reinterpret_cast<float4*>(stk_b + packet_stack_bytes(K, cap_b));
    const uint32_t lt_mask = lanemask_lt();
    const WideNode<K>* __restrict__ tnodes = static_cast<const WideNode<K>*>(a.tnodes);
    const int32_t troot = __ldg(a.troot);
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counter, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)a.nq) break;
        const int64_t i = (int64_t)base + lane;
        const bool valid = i < a.nq;
        int64_t qi = 0;
        float qx = 0.f, qy = 0.f, qz = 0.f;
        if (valid) {
            qi = a.perm ? (int64_t)a.perm[i] : i;
            qx = a.queries[3 * qi];
            qy = a.queries[3 * qi + 1];
            qz = a.queries[3 * qi + 2];
        }
        // world best: squared distance, then (instance, triangle) for ties
        float best = INFINITY;
        int binst = -1, bidx = INT_MAX;
        // the instance being walked: this lane's object-space query and key
        float ox = 0.f, oy = 0.f, oz = 0.f;
        unsigned long long okey = kNoKey;
        const FastTri* mfast = nullptr;
        auto mesh_leaf = [&](int first, int cnt, bool admitted, float& lim) {
            const uint32_t act = __ballot_sync(kFull, admitted);
            const int na = __popc(act);
            if (cnt >= 2 && na >= 1 && na <= 16) {
                // (query, triangle) pairs spread over the warp, as in k_traverse_packet
                const LeafSplit sp2 = c_leaf_splits.v[na];
                const int r = __popc(act & lt_mask);
                if (admitted) st_q[r] = make_float4(ox, oy, oz, 0.0f);
                __syncwarp();
                const int kk = (int)(((float)lane + 0.5f) * sp2.inv);
                const bool worker = lane < sp2.kpr * na;
                const float4 qq = st_q[worker ? lane - kk * na : 0];
                unsigned long long key = kNoKey;
                for (int k0 = 0; k0 < cnt; k0 += sp2.kpr) {
                    const int k = k0 + kk;
                    if (worker && k < cnt) {
                        const FastTri f = load_fast(mfast + first + k);
                        key = min(key, best_key(tri_d2_fast(qq.x, qq.y, qq.z, f), fast_index(f)));
                    }
                }
                const int nk = min(sp2.kpr, cnt);
                for (int j = 0; j < nk; ++j) {
                    const unsigned long long got = __shfl_sync(kFull, key, (r + j * na) & 31);
                    if (admitted) okey = min(okey, got);
                }
                __syncwarp();  // st_q is read before the next leaf writes it
            } else {
                for (int k = 0; k < cnt; ++k) {
                    const FastTri f = load_fast(mfast + first + k);
                    if (admitted) okey = min(okey, best_key(tri_d2_fast(ox, oy, oz, f), fast_index(f)));
                }
            }
            lim = fminf(lim, key_d2(okey));
        };
        auto instance_leaf = [&](int first, int cnt, bool admitted, float& lim) {
            for (int k = 0; k < cnt; ++k) {
                const int inst = __float_as_int(__ldg(&a.trecs[first + k].p2.y));
                const int baked = a.inst_baked[inst];
                const bool act = admitted;
                float lim0, s2 = 1.0f;
                const WideNode<K>* bn;
                int32_t root;
                if (baked >= 0) {
                    ox = qx;
                    oy = qy;
                    oz = qz;
                    lim0 = best;
                    bn = static_cast<const WideNode<K>*>(a.knodes);
                    mfast = a.kfast;
                    root = a.kroot[baked];
                } else {
                    to_object(a.inst_inv + 12 * inst, a.inst_fwd + 12 * inst, qx, qy, qz, ox, oy, oz);
                    s2 = a.inst_s2[2 * inst];
                    const float s2lo = a.inst_s2[2 * inst + 1];
                    lim0 = best < INFINITY ? best / s2lo * (1.0f + 1e-5f) : INFINITY;
                    bn = static_cast<const WideNode<K>*>(a.bnodes);
                    mfast = a.bfast;
                    root = a.broot[a.inst_mesh[inst]];
                }
                okey = kNoKey;
                float limb = act ? lim0 : -INFINITY;
                if (__any_sync(kFull, act)) packet_walk<K>(bn, root, ox, oy, oz, act, limb, stk_b, cap_b, a.status, mesh_leaf);
                const float d2o = key_d2(okey);
                if (act && d2o < lim0) {
                    const float d2w = d2o * s2;
                    const int idx = (int)(uint32_t)okey;
                    if (d2w < best || (d2w == best && (inst < binst || (inst == binst && idx < bidx)))) {
                        best = d2w;
                        binst = inst;
                        bidx = idx;
                    }
                }
            }
            if (admitted) lim = best;
        };
        float limw = valid ? INFINITY : -INFINITY;
        packet_walk<K>(tnodes, troot, qx, qy, qz, valid, limw, stk_t, cap_t, a.status, instance_leaf);
        if (valid) instance_finish(a, qi, qx, qy, qz, binst, bidx);
    }
}

// Returns cudaErrorNotSupported (nothing launched) when even one warp's two
// stacks exceed a block's shared memory: the caller takes the per-thread walk.
template <int K>
cudaError_t launch_instances_packet(const InstArgs& args, int cap_t, int cap_b, cudaStream_t st) {
    auto kern = k_instances_packet<K>;
    int block = 128;
    size_t smem = (size_t)(block / 32) * scene_warp_bytes(K, cap_t, cap_b);
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    while (block > 32 && smem > (size_t)optin) {  // very deep trees: fewer warps per block
        block /= 2;
        smem = (size_t)(block / 32) * scene_warp_bytes(K, cap_t, cap_b);
    }
    if (smem > (size_t)optin) return cudaErrorNotSupported;
    e = ensure_smem_limit(reinterpret_cast<const void*>(kern), smem);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = sm_count(&sms);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cpq::blocks_per_sm(reinterpret_cast<const void*>(kern), block, smem, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorNotSupported;
    int64_t grid = (int64_t)sms * per_sm;
    const int64_t need = ((args.nq + 31) / 32 * 32 + block - 1) / block;
    if (grid > need) grid = need;
    kern<<<(unsigned)grid, block, smem, st>>>(args, cap_t, cap_b);
    note_launch();
    return cudaGetLastError();
}

// One proxy triangle (lo, hi, hi) per instance: the world box of its mesh's
// root box (the 8 corners through the instance matrix), padded by 2^-20 of
// the terms' magnitude so that FP32 rounding cannot shrink it.
__global__ void k_instance_proxies(const float* __restrict__ box, const int32_t* __restrict__ mesh_root,
                                   const int32_t* __restrict__ inst_mesh, const float* __restrict__ fwd,
                                   int32_t n, float* __restrict__ verts, int32_t* __restrict__ tris) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* bx = box + 6 * (int64_t)mesh_root[inst_mesh[i]];
    const float* m = fwd + 12 * i;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
        float w[3];
        affine(m, bx[(c & 1) ? 3 : 0], bx[(c & 2) ? 4 : 1], bx[(c & 4) ? 5 : 2], w[0], w[1], w[2]);
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], w[k]);
            hi[k] = fmaxf(hi[k], w[k]);
        }
    }
    const float ax = fmaxf(fabsf(bx[0]), fabsf(bx[3])), ay = fmaxf(fabsf(bx[1]), fabsf(bx[4])),
                az = fmaxf(fabsf(bx[2]), fabsf(bx[5]));
    for (int k = 0; k < 3; ++k) {
        const float mag = fabsf(m[4 * k]) * ax + fabsf(m[4 * k + 1]) * ay + fabsf(m[4 * k + 2]) * az +
                          fabsf(m[4 * k + 3]);
        const float pad = mag * 0x1p-20f + 1e-30f;
        verts[6 * (int64_t)i + k] = lo[k] - pad;
        verts[6 * (int64_t)i + 3 + k] = hi[k] + pad;
    }
    tris[3 * (int64_t)i] = 2 * i;
    tris[3 * (int64_t)i + 1] = 2 * i + 1;
    tris[3 * (int64_t)i + 2] = 2 * i + 1;
}

// World-space copies of general-affine instances, one triangle per thread:
// triangle g of the output is local triangle i of baked instance j (g =
// out_off[j] + i), its exact record through the batch's inverse order, its
// vertices through the instance matrix in FP64 and rounded once; the copy
// keeps the mesh's local triangle order, so its indices are the mesh's.
__global__ void k_bake_instances(const TriRec* __restrict__ recs, const int32_t* __restrict__ inv_order,
                                 const int64_t* __restrict__ toff, const int32_t* __restrict__ baked_inst,
                                 const int32_t* __restrict__ inst_mesh, const float* __restrict__ fwd,
                                 const int64_t* __restrict__ out_off, int32_t nb, int64_t total,
                                 float* __restrict__ verts, int32_t* __restrict__ tris) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = nb - 1;  // the last j with out_off[j] <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (out_off[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    const int64_t i = g - out_off[lo];
    const int inst = baked_inst[lo];
    const TriRec r = recs[inv_order[toff[inst_mesh[inst]] + i]];
    const float* m = fwd + 12 * (int64_t)inst;
    const float v[3][3] = {{r.p0.x, r.p0.y, r.p0.z}, {r.p0.w, r.p1.x, r.p1.y}, {r.p1.z, r.p1.w, r.p2.x}};
    for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c)
            verts[9 * g + 3 * k + c] = (float)((double)m[4 * c] * v[k][0] + (double)m[4 * c + 1] * v[k][1] +
                                               (double)m[4 * c + 2] * v[k][2] + (double)m[4 * c + 3]);
    tris[3 * g] = (int32_t)(3 * i);
    tris[3 * g + 1] = (int32_t)(3 * i + 1);
    tris[3 * g + 2] = (int32_t)(3 * i + 2);
}

template <int K>
cudaError_t launch_instances(const InstArgs& args, cudaStream_t st) {
    auto kern = k_instances<K>;
    int sms = 0;
    cudaError_t e = sm_count(&sms);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cpq::blocks_per_sm(reinterpret_cast<const void*>(kern), 128, 0, &per_sm);
    if (e != cudaSuccess) return e;
    int64_t grid = (int64_t)sms * per_sm;
    const int64_t need = ((args.nq + 31) / 32 * 32 + 127) / 128;
    if (grid > need) grid = need;
    kern<<<(unsigned)grid, 128, 0, st>>>(args); note_launch();
    return cudaGetLastError();
}

}  // namespace

void timing_enable(bool events, bool counters) {
    std::lock_guard<std::mutex> lock(g_timing.mu);
    g_timing.on = events;
    g_timing.counters = counters;
    if (counters && !g_timing.stats) {
        if (cudaMalloc(&g_timing.stats, kStatCount * sizeof(unsigned long long)) == cudaSuccess)
            cudaMemset(g_timing.stats, 0, kStatCount * sizeof(unsigned long long));
        else
            g_timing.stats = nullptr;
    }
}

cudaError_t traversal_stats(unsigned long long* out, bool reset) {
    std::lock_guard<std::mutex> lock(g_timing.mu);
    for (int k = 0; k < kStatCount; ++k) out[k] = 0;
    if (!g_timing.stats) return cudaSuccess;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(out, g_timing.stats, kStatCount * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(g_timing.stats, 0, kStatCount * sizeof(unsigned long long));
    return e;
}

cudaError_t timing_read(double* ms, int64_t* launches, bool reset) {
    std::lock_guard<std::mutex> lock(g_timing.mu);
    cudaError_t err = cudaSuccess;
    for (auto& pr : g_timing.pending) {
        float t = 0.0f;
        cudaError_t e = cudaEventSynchronize(pr.second);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, pr.first, pr.second);
        if (e != cudaSuccess) err = e;
        g_timing.ms += t;
        g_timing.launches += 1;
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    g_timing.pending.clear();
    if (ms) *ms = g_timing.ms;
    if (launches) *launches = g_timing.launches;
    if (reset) {
        g_timing.ms = 0.0;
        g_timing.launches = 0;
    }
    return err;
}

size_t query_workspace_bytes(const Bvh& b, int64_t nq, const QueryParams& qp) {
    return layout(nq, b.nmeshes, qp.sort != 0).total;
}

cudaError_t order_points(const Bvh& b, const float* queries, int64_t nq, const int64_t* d_qoff,
                         bool sort, void* ws, size_t ws_bytes, cudaStream_t st, const int32_t** perm_out,
                         unsigned long long** counter_out, bool coarse, uint32_t* keys_out) {
    const QueryLayout L = layout(nq, b.nmeshes, sort);
    if (ws_bytes < L.total) return cudaErrorInvalidValue;
    unsigned char* w = static_cast<unsigned char*>(ws);
    unsigned long long* counter = reinterpret_cast<unsigned long long*>(w + L.counter);
    *counter_out = counter;
    *perm_out = nullptr;
    cudaError_t e = cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const int32_t* perm = nullptr;
    if (sort && nq > 1) {
        uint64_t* keys = reinterpret_cast<uint64_t*>(w + L.keys);
        int32_t* vals = reinterpret_cast<int32_t*>(w + L.vals);
        uint64_t* keys_alt = reinterpret_cast<uint64_t*>(w + L.keys_alt);
        int32_t* vals_alt = reinterpret_cast<int32_t*>(w + L.vals_alt);
        const int qbits = (64 - b.mesh_bits) / 3 < 10 ? (64 - b.mesh_bits) / 3 : 10;
        float* frame = reinterpret_cast<float*>(w + L.frame);
        k_init_qbounds<<<(unsigned)((6 * b.nmeshes + 255) / 256), 256, 0, st>>>(frame, b.nmeshes); note_launch();
        // ~8 blocks per SM of 152, each over a contiguous chunk of >= 4096 queries
        const unsigned bgrid = (unsigned)std::min<int64_t>((nq + 4095) / 4096, 1216);
        k_query_bounds<<<bgrid, 256, 0, st>>>(queries, nq, d_qoff, b.nmeshes,
                                                                     frame); note_launch();
        k_query_frame<<<(unsigned)((b.nmeshes + 255) / 256), 256, 0, st>>>(frame, b.nmeshes,
                                                                           (float)(1u << qbits)); note_launch();
        const int key_bits = 3 * qbits + b.mesh_bits;
        // Coarse: only the Hilbert index's top bits are sorted, about 16
        // points per curve segment on average, a radix pass less per 10 bits
        // dropped.  Per-thread ray walks gain (4% on 16M rays); packets of
        // closest-point queries lose far more (near-surface queries crowd
        // into few segments, 35% more node visits), so they sort every bit.
        int begin_bit = 0;
        if (coarse) {
            int floor_log2 = 0;
            while ((int64_t(1) << (floor_log2 + 1)) <= nq) ++floor_log2;
            const int keep = std::min(3 * qbits, std::max(floor_log2 - 4, std::min(3 * qbits, 12)));
            begin_bit = 3 * qbits - keep;
        }
        const unsigned kgrid = (unsigned)((nq + 255) / 256);
        bool in_alt = false;
        if (key_bits <= 32) {
            // 32-bit keys (a single mesh: 30 bits) move a third less data per sort pass
            uint32_t* k32 = reinterpret_cast<uint32_t*>(keys);
            uint32_t* k32_alt = reinterpret_cast<uint32_t*>(keys_alt);
            k_query_keys<uint32_t><<<kgrid, 256, 0, st>>>(queries, nq, d_qoff, b.nmeshes, frame, qbits,
                                                          k32); note_launch();
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            if (keys_out) {
                e = cudaMemcpyAsync(keys_out, k32, sizeof(uint32_t) * nq, cudaMemcpyDeviceToDevice, st);
                if (e != cudaSuccess) return e;
            }
            e = radix_sort_pairs<uint32_t>(k32, vals, k32_alt, vals_alt, nq, begin_bit, key_bits,
                                           w + L.sort_ws, L.sort_ws_bytes, st, &in_alt, true);
        } else {
            k_query_keys<uint64_t><<<kgrid, 256, 0, st>>>(queries, nq, d_qoff, b.nmeshes, frame, qbits,
                                                          keys); note_launch();
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
            e = radix_sort_pairs<uint64_t>(keys, vals, keys_alt, vals_alt, nq, begin_bit, key_bits,
                                           w + L.sort_ws, L.sort_ws_bytes, st, &in_alt, true);
        }
        if (e != cudaSuccess) return e;
        perm = in_alt ? vals_alt : vals;
    }
    *perm_out = perm;
    return cudaSuccess;
}

cudaError_t bvh_query(const Bvh& b, const float* queries, int64_t nq, const int64_t* d_qoff,
                      const QueryParams& qp, float* out_point, float* out_dist, int32_t* out_tri,
                      float* out_bary, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    const int32_t* perm = nullptr;
    unsigned long long* counter = nullptr;
    cudaError_t e = order_points(b, queries, nq, d_qoff, qp.sort != 0, ws, ws_bytes, st, &perm, &counter);
    if (e != cudaSuccess) return e;
    TraverseArgs args;
    args.nodes = b.nodes;
    args.recs = b.recs;
    args.fast = b.fast;
    args.inv_order = b.inv_order;
    args.toff = b.d_toff;
    args.wide_root = b.wide_root;
    args.qoff = d_qoff;
    args.nmeshes = b.nmeshes;
    args.queries = queries;
    args.perm = perm;
    args.nq = nq;
    args.out_point = out_point;
    args.out_dist = out_dist;
    args.out_tri = out_tri;
    args.out_bary = out_bary;
    args.counter = counter;
    args.status = b.status;
    args.stats = nullptr;
    args.box = b.box;
    args.mesh_root = b.mesh_root;
    args.seed_chunk = qp.seed_chunk;
    {
        cudaStreamCaptureStatus capst = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &capst);
        std::lock_guard<std::mutex> lock(g_timing.mu);
        if (g_timing.counters && !qp.no_timing && capst == cudaStreamCaptureStatusNone)
            args.stats = g_timing.stats;
    }
    // the packet stack holds one entry per wide level at most
    const int packet_cap = b.max_wide_depth + 1;
    // leaf compaction pays once leaves can hold 3 or more triangles
    const bool compact = b.p.leaf_size >= 3;
    switch (b.p.K) {
        case 2: return launch_k<2>(args, qp, packet_cap, compact, st);
        case 4: return launch_k<4>(args, qp, packet_cap, compact, st);
        default: return launch_k<8>(args, qp, packet_cap, compact, st);
    }
}

cudaError_t bvh_backward(const Bvh& b, const float* queries, const int32_t* tri, const float* bary,
                         const float* grad_dist, int64_t nq, float* grad_q, float* grad_verts,
                         cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    k_backward<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(b.recs, b.inv_order, b.tris, b.nt,
                                                             queries, tri, bary, grad_dist, nq,
                                                             grad_q, grad_verts, b.status); note_launch();
    return cudaGetLastError();
}

cudaError_t instance_proxies(const Bvh& bottom, const int32_t* inst_mesh, const float* inst_fwd,
                             int32_t n, float* verts, int32_t* tris, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_instance_proxies<<<(n + 127) / 128, 128, 0, st>>>(bottom.box, bottom.mesh_root, inst_mesh, inst_fwd, n,
                                                        verts, tris);
    note_launch();
    return cudaGetLastError();
}

cudaError_t instance_bake(const Bvh& bottom, const int32_t* baked_inst, const int32_t* inst_mesh,
                          const float* inst_fwd, const int64_t* out_off, int32_t nb, int64_t total, float* verts,
                          int32_t* tris, cudaStream_t st) {
    if (total <= 0) return cudaSuccess;
    k_bake_instances<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(bottom.recs, bottom.inv_order, bottom.d_toff,
                                                                      baked_inst, inst_mesh, inst_fwd, out_off, nb,
                                                                      total, verts, tris);
    note_launch();
    return cudaGetLastError();
}

cudaError_t bvh_instance_query(const Bvh& top, const Bvh& bottom, const InstanceSet& is, const float* queries,
                               int64_t nq, bool sort, float* out_point, float* out_dist, int32_t* out_inst,
                               int32_t* out_tri, float* out_bary, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    if (top.p.K != bottom.p.K || (is.baked_bvh && is.baked_bvh->p.K != bottom.p.K)) return cudaErrorInvalidValue;
    InstArgs a;
    cudaError_t e = order_points(top, queries, nq, nullptr, sort, ws, ws_bytes, st, &a.perm, &a.counter);
    if (e != cudaSuccess) return e;
    a.tnodes = top.nodes;
    a.trecs = top.recs;
    a.troot = top.wide_root;
    a.bnodes = bottom.nodes;
    a.bfast = bottom.fast;
    a.brecs = bottom.recs;
    a.broot = bottom.wide_root;
    a.binv_order = bottom.inv_order;
    a.btoff = bottom.d_toff;
    a.knodes = is.baked_bvh ? is.baked_bvh->nodes : nullptr;
    a.kfast = is.baked_bvh ? is.baked_bvh->fast : nullptr;
    a.kroot = is.baked_bvh ? is.baked_bvh->wide_root : nullptr;
    a.inst_mesh = is.mesh;
    a.inst_baked = is.baked;
    a.inst_inv = is.inv;
    a.inst_fwd = is.fwd;
    a.inst_s2 = is.s2;
    a.queries = queries;
    a.nq = nq;
    a.out_point = out_point;
    a.out_dist = out_dist;
    a.out_inst = out_inst;
    a.out_tri = out_tri;
    a.out_bary = out_bary;
    a.status = bottom.status;
    if (sort) {
        // Hilbert-ordered queries: warp packets at both levels
        const int cap_t = top.max_wide_depth + 1;
        const int cap_b = std::max(bottom.max_wide_depth, is.baked_bvh ? is.baked_bvh->max_wide_depth : 0) + 1;
        switch (top.p.K) {
            case 2: e = launch_instances_packet<2>(a, cap_t, cap_b, st); break;
            case 4: e = launch_instances_packet<4>(a, cap_t, cap_b, st); break;
            default: e = launch_instances_packet<8>(a, cap_t, cap_b, st); break;
        }
        if (e != cudaErrorNotSupported) return e;
        // the stacks do not fit in shared memory: the per-thread walk below
    }
    switch (top.p.K) {
        case 2: return launch_instances<2>(a, st);
        case 4: return launch_instances<4>(a, st);
        default: return launch_instances<8>(a, st);
    }
}

}  // namespace cpq
