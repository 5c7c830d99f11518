// common.cuh — shared device types and helpers of the GB300 closest-point engine.
//
// Data layout in HBM (all arrays 256-byte aligned, owned by a Bvh):
//   WideNode<K>  K-wide BVH node, 32*K bytes, one 128-byte line for K = 4:
//                six K-float SoA rows of child bounds (lo x, hi x, lo y, hi y,
//                lo z, hi z) and one K-int row of packed child references,
//                padded to 8 rows so every row is a 16-byte vector load.
//   TriRec       48-byte triangle record in leaf (Morton) order: three float4
//                {a.x a.y a.z b.x} {b.y b.z c.x c.y} {c.z idx flags 0}.
// A child reference >= 0 is an inner node; a leaf of `count` triangles
// starting at record `first` is stored as ~((first << 4) | (count - 1)).
// Empty slots have lo = +inf, hi = -inf, so their box distance is +inf.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>

namespace cpq {

constexpr int kLeafShift = 4;             // bits for (count - 1) in a packed leaf
constexpr int kMaxLeafSize = 15;
constexpr int64_t kMaxTriangles = (int64_t(1) << 27) - 1;  // first must fit in 27 bits

constexpr uint32_t kTriDegenerate = 1u;   // TriRec flags: zero-area triangle

// Host side: count one kernel launch of this library (cp_kernel_launches).
void note_launch();

// Host side, cached per device and kernel: raise the kernel's dynamic
// shared-memory limit to at least `smem` (the runtime call is made only when
// the cached limit is lower), and the kernel's resident blocks per SM for a
// block size and shared-memory size.  Keeps per-query host work free of
// runtime calls that could wait for the device.
cudaError_t ensure_smem_limit(const void* kernel, size_t smem);
cudaError_t blocks_per_sm(const void* kernel, int block, size_t smem, int* out);
cudaError_t sm_count(int* out);

template <int K>
struct alignas(16) WideNode {
    float lox[K], hix[K], loy[K], hiy[K], loz[K], hiz[K];
    int32_t child[K];
    int32_t pad[K];
};
static_assert(sizeof(WideNode<4>) == 128, "BVH4 node must be one 128-byte line");
static_assert(sizeof(WideNode<8>) == 256, "BVH8 node must be two lines");
static_assert(sizeof(WideNode<2>) == 64, "BVH2 node must be 64 bytes");

struct alignas(16) TriRec {
    float4 p0, p1, p2;
};

// 80-byte record for the traversal's distance test, in the same (leaf) order
// as TriRec.  The triangle in its own orthonormal frame (e1 along ab, e2 in
// the plane towards c, n = e1 x e2): a at the origin, b at (L1, 0), c at
// (x2, y2) with y2 >= 0, so a query's offset from a gives in-plane (u, v) and
// height h by three dot products, and the rest is a 2D point-triangle test:
//   {a.xyz L1} {e1.xyz x2} {e2.xyz y2} {n.xyz x2 - L1}
//   {1/|ac|^2 1/|bc|^2 vmin idx}
// vmin is 0, or +inf for a zero-area triangle (never "inside"); zero-length
// edges store 0 for their inverse.
struct alignas(16) FastTri {
    float4 p0, p1, p2, p3, p4;
};
static_assert(sizeof(FastTri) == 80, "FastTri is five 16-byte loads");

__device__ __forceinline__ FastTri load_fast(const FastTri* p) {
    const float4* fp = reinterpret_cast<const float4*>(p);
    FastTri f;
    f.p0 = __ldg(fp);
    f.p1 = __ldg(fp + 1);
    f.p2 = __ldg(fp + 2);
    f.p3 = __ldg(fp + 3);
    f.p4 = __ldg(fp + 4);
    return f;
}
__device__ __forceinline__ int fast_index(const FastTri& f) { return __float_as_int(f.p4.w); }

__host__ __device__ inline int32_t pack_leaf(int32_t first, int32_t count) {
    return ~((first << kLeafShift) | (count - 1));
}
__host__ __device__ inline bool ref_is_leaf(int32_t ref) { return ref < 0; }
__host__ __device__ inline int32_t leaf_first(int32_t ref) { return (~ref) >> kLeafShift; }
__host__ __device__ inline int32_t leaf_count(int32_t ref) {
    return ((~ref) & ((1 << kLeafShift) - 1)) + 1;
}

// ---------------------------------------------------------------------------
// Morton codes: bit k of x moves to bit 3k (x < 2^21).
__host__ __device__ inline uint64_t spread3(uint64_t x) {
    x &= 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Quantise one centroid-sum coordinate: t = (s - lo) * scale, rounded to
// nearest in FP32 with no contraction, truncated and clamped to maxcell.
__device__ __forceinline__ uint32_t quantise(float s, float lo, float scale, uint32_t maxcell) {
    float t = __fmul_rn(__fsub_rn(s, lo), scale);
    if (!(t < (float)maxcell)) return maxcell;
    return (uint32_t)t;
}

// Half surface area of a box, (ex*ez + ex*ey) + ey*ez in that rounding order:
// the order of the reference's BBox::surface_area (src/lib/bbox.h:55-59),
// whose factor 2 is exact, so twice this is its value bit for bit (the SAH
// building block; the factor cancels in every cost comparison).
__device__ __forceinline__ float half_area(float lx, float ly, float lz, float hx, float hy, float hz) {
    float ex = __fsub_rn(hx, lx), ey = __fsub_rn(hy, ly), ez = __fsub_rn(hz, lz);
    return __fadd_rn(__fadd_rn(__fmul_rn(ex, ez), __fmul_rn(ex, ey)), __fmul_rn(ey, ez));
}

__device__ __forceinline__ float fmin_t(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float fmax_t(float a, float b) { return a > b ? a : b; }

// ---------------------------------------------------------------------------
// Float-float ("double-float") arithmetic for the final re-evaluation of the
// winning triangle, so the reported distance is within a few FP32 ulps of the
// exact distance without FP64 on the device.  Error-free transforms:
// Knuth's two-sum, the FMA-based two-product (Dekker 1971 with a fused
// multiply-add), and pair arithmetic as in the double-double literature
// (Hida, Li and Bailey 2001), restated for float pairs.
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, err};
}
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float err = __fsub_rn(b, __fsub_rn(s, a));
    return {s, err};
}
__device__ __forceinline__ ff ff_two_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float err = __fmaf_rn(a, b, -p);
    return {p, err};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = ff_two_sum(a.hi, b.hi);
    ff t = ff_two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = ff_fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return ff_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    ff p = ff_two_prod(a.hi, b.hi);
    float t = __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
    p.lo = __fadd_rn(p.lo, t);
    return ff_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ ff ff_div(ff a, ff b) {
    float q1 = __fdiv_rn(a.hi, b.hi);
    ff r = ff_sub(a, ff_mul(b, {q1, 0.0f}));
    float q2 = __fdiv_rn(r.hi, b.hi);
    r = ff_sub(r, ff_mul(b, {q2, 0.0f}));
    float q3 = __fdiv_rn(r.hi, b.hi);
    ff q = ff_fast_two_sum(q1, q2);
    return ff_add(q, {q3, 0.0f});
}
__device__ __forceinline__ ff ff_from(float a) { return {a, 0.0f}; }
__device__ __forceinline__ ff ff_sqrt(ff a) {
    if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
    float x = __fsqrt_rn(a.hi);
    // one Newton step: x + (a - x^2) / (2x)
    ff xx = ff_two_prod(x, x);
    ff r = ff_sub(a, xx);
    float corr = __fdiv_rn(r.hi, __fmul_rn(2.0f, x));
    return ff_fast_two_sum(x, corr);
}
__device__ __forceinline__ float ff_to_float(ff a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ bool ff_le0(ff a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo <= 0.0f); }
__device__ __forceinline__ bool ff_ge0(ff a) { return a.hi > 0.0f || (a.hi == 0.0f && a.lo >= 0.0f); }
__device__ __forceinline__ bool ff_le(ff a, ff b) { return ff_le0(ff_sub(a, b)); }

struct ff3 {
    ff x, y, z;
};
__device__ __forceinline__ ff3 ff3_sub(ff3 a, ff3 b) {
    return {ff_sub(a.x, b.x), ff_sub(a.y, b.y), ff_sub(a.z, b.z)};
}
__device__ __forceinline__ ff ff3_dot(ff3 a, ff3 b) {
    return ff_add(ff_add(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_mul(a.z, b.z));
}
__device__ __forceinline__ ff3 ff3_scale(ff3 a, ff s) {
    return {ff_mul(a.x, s), ff_mul(a.y, s), ff_mul(a.z, s)};
}
__device__ __forceinline__ ff3 ff3_from(float x, float y, float z) {
    return {ff_from(x), ff_from(y), ff_from(z)};
}

}  // namespace cpq
