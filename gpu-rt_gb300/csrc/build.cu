// build.cu — GPU LBVH build: Morton keys -> radix sort -> Karras hierarchy ->
// bottom-up refit with SAH leaf decisions -> leaf clusters -> K-wide collapse.
//
// Every FP32 expression that decides a key, a box or a leaf is written with
// round-to-nearest intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn) and the same
// operation order as the CPU restatement, so Morton codes, topology, boxes and
// collapse decisions match it bit for bit.  Published methods: Morton order
// (Lauterbach et al. 2009), the binary radix tree of Karras 2012, SAH
// (MacDonald and Booth 1990).  The reference's counterpart is the closed
// driver build behind VK::Accel::recreate (src/vk/vulkan.cpp:881-936); its
// only box vocabulary is BBox::enclose / surface_area (src/lib/bbox.h:35-59).
#include <algorithm>
#include <cfloat>
#include <cstring>

#include "bvh.cuh"
#include "sort.cuh"

namespace cpq {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int threads = kThreads) {
    return (unsigned)((n + threads - 1) / threads);
}

__device__ __forceinline__ int mesh_of(const int64_t* __restrict__ off, int nmeshes, int64_t i) {
    // last m with off[m] <= i
    int lo = 0, hi = nmeshes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void atomic_min_f(float* addr, float v) {
    if (v >= 0.0f) atomicMin(reinterpret_cast<int*>(addr), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned*>(addr), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_f(float* addr, float v) {
    if (v >= 0.0f) atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned*>(addr), __float_as_uint(v));
}

__device__ __forceinline__ float3 load_vert(const float* __restrict__ verts, int64_t stride,
                                            int64_t v) {
    const float* p = verts + v * stride;
    return make_float3(p[0], p[1], p[2]);
}

__global__ void k_validate(const float* __restrict__ verts, int64_t stride,
                           const int32_t* __restrict__ tris, int64_t nt,
                           const int64_t* __restrict__ voff, const int64_t* __restrict__ toff,
                           int nmeshes, uint32_t* __restrict__ bad) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int m = mesh_of(toff, nmeshes, t);
    int64_t nvm = voff[m + 1] - voff[m];
    uint32_t flags = 0;
    for (int k = 0; k < 3; ++k) {
        int32_t ix = tris[3 * t + k];
        if (ix < 0 || ix >= nvm) {
            flags |= 2u;
            continue;
        }
        float3 v = load_vert(verts, stride, voff[m] + ix);
        if (!isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z)) flags |= 4u;
    }
    if (flags) atomicOr(bad, flags);
}

__global__ void k_centroid_bounds(const float* __restrict__ verts, int64_t stride,
                                  const int32_t* __restrict__ tris, int64_t nt,
                                  const int64_t* __restrict__ voff,
                                  const int64_t* __restrict__ toff, int nmeshes,
                                  float* __restrict__ csum, float* __restrict__ mbox) {
    // Each block owns a contiguous chunk; a thread keeps a running box and
    // flushes it with atomics only when the mesh changes and at the end (min
    // and max are exact, so any reduction order gives the same bounds).
    const int64_t per_block = (nt + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = (int64_t)blockIdx.x * per_block;
    const int64_t b1 = min(nt, b0 + per_block);
    int cur = -1;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t t = b0 + threadIdx.x; t < b1; t += blockDim.x) {
        const int m = nmeshes > 1 ? mesh_of(toff, nmeshes, t) : 0;
        const int64_t vb = voff[m];
        const float3 a = load_vert(verts, stride, vb + tris[3 * t + 0]);
        const float3 b = load_vert(verts, stride, vb + tris[3 * t + 1]);
        const float3 c = load_vert(verts, stride, vb + tris[3 * t + 2]);
        const float s[3] = {__fadd_rn(__fadd_rn(a.x, b.x), c.x), __fadd_rn(__fadd_rn(a.y, b.y), c.y),
                            __fadd_rn(__fadd_rn(a.z, b.z), c.z)};
        csum[3 * t + 0] = s[0];
        csum[3 * t + 1] = s[1];
        csum[3 * t + 2] = s[2];
        if (m != cur) {
            if (cur >= 0)
                for (int k = 0; k < 3; ++k) {
                    atomic_min_f(&mbox[6 * cur + k], lo[k]);
                    atomic_max_f(&mbox[6 * cur + 3 + k], hi[k]);
                }
            cur = m;
            lo[0] = lo[1] = lo[2] = INFINITY;
            hi[0] = hi[1] = hi[2] = -INFINITY;
        }
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], s[k]);
            hi[k] = fmaxf(hi[k], s[k]);
        }
    }
    const unsigned full = 0xffffffffu;
    const int c0 = __shfl_sync(full, cur, 0);
    if (__all_sync(full, cur == c0)) {
        if (c0 < 0) return;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                lo[k] = fminf(lo[k], __shfl_xor_sync(full, lo[k], o));
                hi[k] = fmaxf(hi[k], __shfl_xor_sync(full, hi[k], o));
            }
        if ((threadIdx.x & 31) == 0)
            for (int k = 0; k < 3; ++k) {
                atomic_min_f(&mbox[6 * c0 + k], lo[k]);
                atomic_max_f(&mbox[6 * c0 + 3 + k], hi[k]);
            }
    } else if (cur >= 0) {
        for (int k = 0; k < 3; ++k) {
            atomic_min_f(&mbox[6 * cur + k], lo[k]);
            atomic_max_f(&mbox[6 * cur + 3 + k], hi[k]);
        }
    }
}

__global__ void k_init_boxes(float* __restrict__ mbox, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        int k = i % 6;
        mbox[i] = k < 3 ? INFINITY : -INFINITY;
    }
}

// Per mesh: (lo, scale) of the build's quantisation frame.  The frame is
// isotropic (one cell size on every axis, from the largest extent): on a
// flat or 2.5D mesh, per-axis scaling would give the thin axis as many bits
// as the wide ones and the hierarchy would split it far too often, leaving
// wide, flat boxes whose distance bounds prune poorly (about 25% more node
// visits and triangle tests on the heightfield workload).
__global__ void k_build_frames(const float* __restrict__ mbox, int nmeshes, float cells,
                               float* __restrict__ lo_scale) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmeshes) return;
    float emax = 0.0f;
    for (int k = 0; k < 3; ++k) {
        const float e = __fsub_rn(mbox[6 * m + 3 + k], mbox[6 * m + k]);
        if (e > emax) emax = e;
    }
    float scale = emax > 0.0f ? __fdiv_rn(cells, emax) : 0.0f;
    if (!(scale <= FLT_MAX)) scale = 0.0f;
    for (int k = 0; k < 3; ++k) {
        lo_scale[6 * m + k] = mbox[6 * m + k];
        lo_scale[6 * m + 3 + k] = scale;
    }
}

__global__ void k_morton(const float* __restrict__ csum, int64_t nt,
                         const int64_t* __restrict__ toff, int nmeshes,
                         const float* __restrict__ lo_scale, int bits, uint64_t* __restrict__ keys,
                         int32_t* __restrict__ vals) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int m = nmeshes > 1 ? mesh_of(toff, nmeshes, t) : 0;
    const uint32_t maxcell = (1u << bits) - 1u;
    uint64_t code = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        uint32_t cell = quantise(csum[3 * t + k], lo_scale[6 * m + k], lo_scale[6 * m + 3 + k], maxcell);
        code |= spread3(cell) << (2 - k);
    }
    keys[t] = ((uint64_t)m << (3 * bits)) | code;
    vals[t] = (int32_t)t;
}

__global__ void k_key_and_or(const uint64_t* __restrict__ keys, int64_t n,
                             unsigned long long* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long a = ~0ull, o = 0ull;
    for (; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        a &= keys[i];
        o |= keys[i];
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        a &= __shfl_xor_sync(0xffffffffu, a, s);
        o |= __shfl_xor_sync(0xffffffffu, o, s);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAnd(&out[0], a);
        atomicOr(&out[1], o);
    }
}

__device__ __forceinline__ int delta(const uint64_t* __restrict__ keys, int64_t n, int64_t i,
                                     int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t x = keys[i] ^ keys[j];
    if (x) return __clzll((long long)x);
    return 64 + __clz((int)((uint32_t)i ^ (uint32_t)j));
}

// Karras 2012: each internal node i finds its range from the direction of
// the longer common prefix, then the split by binary search.
__global__ void k_karras(const uint64_t* __restrict__ keys, int64_t n, int bits, int nmeshes,
                         const int64_t* __restrict__ toff, int32_t* __restrict__ left,
                         int32_t* __restrict__ right, int32_t* __restrict__ parent,
                         int32_t* __restrict__ first, int32_t* __restrict__ last,
                         int32_t* __restrict__ mesh_root) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) > 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int64_t lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int64_t j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int64_t s = 0;
    for (int64_t div = 2;; div *= 2) {
        int64_t t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t <= 1) break;
    }
    int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
    int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    int32_t lc = (lo == gamma) ? (int32_t)(n - 1 + gamma) : (int32_t)gamma;
    int32_t rc = (hi == gamma + 1) ? (int32_t)(n - 1 + gamma + 1) : (int32_t)(gamma + 1);
    left[i] = lc;
    right[i] = rc;
    parent[lc] = (int32_t)i;
    parent[rc] = (int32_t)i;
    first[i] = (int32_t)lo;
    last[i] = (int32_t)hi;
    int m = nmeshes > 1 ? (int)(keys[lo] >> (3 * bits)) : 0;
    if ((int64_t)lo == toff[m] && (int64_t)hi == toff[m + 1] - 1) mesh_root[m] = (int32_t)i;
}

__global__ void k_leaf_init(int64_t n, int32_t* __restrict__ first, int32_t* __restrict__ last,
                            int32_t* __restrict__ parent_root) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    first[n - 1 + k] = (int32_t)k;
    last[n - 1 + k] = (int32_t)k;
    if (k == 0) parent_root[0] = -1;  // the root (node 0) has no parent
}

__global__ void k_single_tri_roots(const int64_t* __restrict__ toff, int nmeshes, int64_t n,
                                   int32_t* __restrict__ mesh_root) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmeshes) return;
    if (toff[m + 1] - toff[m] == 1) mesh_root[m] = (int32_t)(n - 1 + toff[m]);
}

__device__ __forceinline__ uint32_t degenerate_flag(float3 a, float3 b, float3 c) {
    float abx = __fsub_rn(b.x, a.x), aby = __fsub_rn(b.y, a.y), abz = __fsub_rn(b.z, a.z);
    float acx = __fsub_rn(c.x, a.x), acy = __fsub_rn(c.y, a.y), acz = __fsub_rn(c.z, a.z);
    float nx = __fsub_rn(__fmul_rn(aby, acz), __fmul_rn(abz, acy));
    float ny = __fsub_rn(__fmul_rn(abz, acx), __fmul_rn(abx, acz));
    float nz = __fsub_rn(__fmul_rn(abx, acy), __fmul_rn(aby, acx));
    float nn = __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
    float lab = __fadd_rn(__fadd_rn(__fmul_rn(abx, abx), __fmul_rn(aby, aby)), __fmul_rn(abz, abz));
    float lac = __fadd_rn(__fadd_rn(__fmul_rn(acx, acx), __fmul_rn(acy, acy)), __fmul_rn(acz, acz));
    return (nn > __fmul_rn(1e-10f, __fmul_rn(lab, lac))) ? 0u : kTriDegenerate;
}

// The frame is computed in FP64 from the FP32 vertices and each stored value
// rounded once, so its directions are within half an ulp of the exact ones:
// the test's error is then the FP32 arithmetic of the query alone.
__device__ __forceinline__ FastTri make_fast_tri(float3 a, float3 b, float3 c, int32_t local,
                                                 bool degenerate) {
    const double abx = (double)b.x - a.x, aby = (double)b.y - a.y, abz = (double)b.z - a.z;
    const double acx = (double)c.x - a.x, acy = (double)c.y - a.y, acz = (double)c.z - a.z;
    const double aa = abx * abx + aby * aby + abz * abz;
    const double cc = acx * acx + acy * acy + acz * acz;
    // e1: along ab, else along ac, else any axis (a point)
    double e1x = 1.0, e1y = 0.0, e1z = 0.0;
    if (aa > 0.0) {
        const double r = 1.0 / sqrt(aa);
        e1x = abx * r; e1y = aby * r; e1z = abz * r;
    } else if (cc > 0.0) {
        const double r = 1.0 / sqrt(cc);
        e1x = acx * r; e1y = acy * r; e1z = acz * r;
    }
    // e2: ac's part across e1; for a zero-area triangle any unit vector
    // across e1 (from the axis e1 leans on least)
    const double ce = acx * e1x + acy * e1y + acz * e1z;
    double wx = acx - ce * e1x, wy = acy - ce * e1y, wz = acz - ce * e1z;
    double ww = wx * wx + wy * wy + wz * wz;
    if (degenerate || !(ww > 0.0)) {
        const double ax = fabs(e1x), ay = fabs(e1y), az = fabs(e1z);
        const double tx = (ax <= ay && ax <= az) ? 1.0 : 0.0;
        const double ty = (tx == 0.0 && ay <= az) ? 1.0 : 0.0;
        const double tz = (tx == 0.0 && ty == 0.0) ? 1.0 : 0.0;
        const double te = tx * e1x + ty * e1y + tz * e1z;
        wx = tx - te * e1x; wy = ty - te * e1y; wz = tz - te * e1z;
        ww = wx * wx + wy * wy + wz * wz;
    }
    const double rw = 1.0 / sqrt(ww);
    const double e2x = wx * rw, e2y = wy * rw, e2z = wz * rw;
    const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    const double L1 = abx * e1x + aby * e1y + abz * e1z;
    const double x2 = ce;
    const double y2 = fmax(acx * e2x + acy * e2y + acz * e2z, 0.0);
    const double bx = x2 - L1;
    const double l2 = x2 * x2 + y2 * y2, l3 = bx * bx + y2 * y2;
    FastTri f;
    f.p0 = make_float4(a.x, a.y, a.z, (float)L1);
    f.p1 = make_float4((float)e1x, (float)e1y, (float)e1z, (float)x2);
    f.p2 = make_float4((float)e2x, (float)e2y, (float)e2z, (float)y2);
    f.p3 = make_float4((float)nx, (float)ny, (float)nz, (float)bx);
    f.p4 = make_float4(l2 > 0.0 ? (float)(1.0 / l2) : 0.0f, l3 > 0.0 ? (float)(1.0 / l3) : 0.0f,
                       degenerate ? INFINITY : 0.0f, __int_as_float(local));
    return f;
}

// Leaf boxes + triangle records, then the bottom-up walk: the second thread
// to reach a node merges its children (min/max are order-free; SAH costs use
// only the children's values), so the result does not depend on scheduling.
template <bool kBuild>
__global__ void k_refit(const float* __restrict__ verts, int64_t stride,
                        const int32_t* __restrict__ tris, const int32_t* __restrict__ order,
                        const uint64_t* __restrict__ keys, int64_t n,
                        const int64_t* __restrict__ voff, const int64_t* __restrict__ toff,
                        int nmeshes, int key_mesh_shift, const int32_t* __restrict__ left,
                        const int32_t* __restrict__ right, const int32_t* __restrict__ parent,
                        const int32_t* __restrict__ first, const int32_t* __restrict__ last,
                        float* box, float* cost, uint8_t* __restrict__ leaf_flag,
                        uint32_t* __restrict__ arrive, TriRec* __restrict__ recs,
                        FastTri* __restrict__ fast, int32_t* __restrict__ inv_order,
                        int leaf_size, const int32_t* __restrict__ mesh_leaf, int collapse, float c_node,
                        float c_tri) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int32_t t = order[k];
    const int m = nmeshes > 1 ? (int)(keys[k] >> key_mesh_shift) : 0;
    const int64_t vb = voff[m];
    const int32_t* ix = tris + 3 * (int64_t)t;
    float3 a = load_vert(verts, stride, vb + ix[0]);
    float3 b = load_vert(verts, stride, vb + ix[1]);
    float3 c = load_vert(verts, stride, vb + ix[2]);
    const int32_t local = (int32_t)(t - toff[m]);
    TriRec r;
    r.p0 = make_float4(a.x, a.y, a.z, b.x);
    r.p1 = make_float4(b.y, b.z, c.x, c.y);
    const uint32_t degenerate = degenerate_flag(a, b, c);
    r.p2 = make_float4(c.z, __int_as_float(local), __uint_as_float(degenerate), 0.0f);
    recs[k] = r;
    fast[k] = make_fast_tri(a, b, c, local, degenerate != 0);
    if (kBuild) inv_order[t] = (int32_t)k;

    const int64_t node = n - 1 + k;
    float lo[3], hi[3];
    {
        float av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z}, cv[3] = {c.x, c.y, c.z};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            float l = av[q] < bv[q] ? av[q] : bv[q];
            l = l < cv[q] ? l : cv[q];
            float h = av[q] > bv[q] ? av[q] : bv[q];
            h = h > cv[q] ? h : cv[q];
            lo[q] = l;
            hi[q] = h;
        }
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        box[6 * node + q] = lo[q];
        box[6 * node + 3 + q] = hi[q];
    }
    if (kBuild) {
        float A = half_area(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]);
        cost[node] = collapse == 1 ? __fmul_rn(__fmul_rn(c_tri, 1.0f), A) : 0.0f;
        leaf_flag[node] = 1;
    }
    int32_t p = parent[node];
    while (p >= 0) {
        __threadfence();
        uint32_t old = atomicAdd(&arrive[p], 1u);
        if (old == 0) break;
        __threadfence();
        const int32_t l = left[p], rr = right[p];
        float pl[3], ph[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            float ll = __ldcg(&box[6 * (int64_t)l + q]), rl = __ldcg(&box[6 * (int64_t)rr + q]);
            float lh = __ldcg(&box[6 * (int64_t)l + 3 + q]), rh = __ldcg(&box[6 * (int64_t)rr + 3 + q]);
            pl[q] = ll < rl ? ll : rl;
            ph[q] = lh > rh ? lh : rh;
            box[6 * (int64_t)p + q] = pl[q];
            box[6 * (int64_t)p + 3 + q] = ph[q];
        }
        if (kBuild) {
            const int32_t f = first[p], e = last[p];
            const int32_t size = e - f + 1;
            bool same_mesh = nmeshes <= 1 || ((keys[f] >> key_mesh_shift) == (keys[e] >> key_mesh_shift));
            const int limit = mesh_leaf ? mesh_leaf[nmeshes > 1 ? (int)(keys[f] >> key_mesh_shift) : 0] : leaf_size;
            bool leafable = size <= limit && same_mesh;
            if (collapse == 1) {
                float Ap = half_area(pl[0], pl[1], pl[2], ph[0], ph[1], ph[2]);
                float split = __fmul_rn(c_node, Ap);
                split = __fadd_rn(split, __ldcg(&cost[l]));
                split = __fadd_rn(split, __ldcg(&cost[rr]));
                float leafc = __fmul_rn(__fmul_rn(c_tri, (float)size), Ap);
                bool lf = leafable && leafc <= split;
                leaf_flag[p] = lf ? 1 : 0;
                cost[p] = lf ? leafc : split;
            } else {
                leaf_flag[p] = leafable ? 1 : 0;
                cost[p] = 0.0f;
            }
        }
        p = parent[p];
    }
}

// Cluster flags, depth below the mesh root and "starts a wide node" flags.
__global__ void k_wide_flags(int64_t n, const uint64_t* __restrict__ keys, int nmeshes,
                             int key_mesh_shift, const int32_t* __restrict__ parent,
                             const int32_t* __restrict__ first, const int32_t* __restrict__ last,
                             const uint8_t* __restrict__ leaf_flag,
                             const int32_t* __restrict__ mesh_root, int k_levels,
                             uint8_t* __restrict__ cluster, uint32_t* __restrict__ wide_flag,
                             int32_t* __restrict__ max_depth) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nn = 2 * n - 1;
    if (v >= nn) return;
    int m = 0;
    if (nmeshes > 1) {
        m = (int)(keys[first[v]] >> key_mesh_shift);
        if ((int)(keys[last[v]] >> key_mesh_shift) != m) {
            cluster[v] = 0;
            wide_flag[v] = 0;
            return;
        }
    }
    const int32_t root = mesh_root[m];
    int32_t d = 0;
    bool anc_leaf = false;
    int64_t u = v;
    while (u != root) {
        u = parent[u];
        if (u < 0) {  // no mesh root above v: not part of any mesh's tree
            cluster[v] = 0;
            wide_flag[v] = 0;
            return;
        }
        ++d;
        anc_leaf |= leaf_flag[u] != 0;
    }
    const bool lf = leaf_flag[v] != 0;
    cluster[v] = (lf && !anc_leaf) ? 1 : 0;
    bool is_wide = (v == root) || (!anc_leaf && !lf && v < n - 1 && (d % k_levels) == 0);
    wide_flag[v] = is_wide ? 1u : 0u;
    if (is_wide) atomicMax(max_depth, d / k_levels);
}

template <int K>
__global__ void k_wide_emit(int64_t n, int k_levels, const uint32_t* __restrict__ wide_flag,
                            const uint32_t* __restrict__ wide_id, const uint64_t* __restrict__ keys,
                            int nmeshes, int key_mesh_shift, const int32_t* __restrict__ left,
                            const int32_t* __restrict__ right, const int32_t* __restrict__ first,
                            const int32_t* __restrict__ last, const float* __restrict__ box,
                            const uint8_t* __restrict__ cluster,
                            const int32_t* __restrict__ mesh_root, WideNode<K>* __restrict__ nodes,
                            int32_t* __restrict__ wide_src, int32_t* __restrict__ slot_src,
                            int32_t* __restrict__ wide_root, uint32_t* __restrict__ leaf_count) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nn = 2 * n - 1;
    if (v >= nn || !wide_flag[v]) return;
    const uint32_t w = wide_id[v];
    // Expand k_levels times: every inner, non-cluster slot is replaced in
    // place by its two children, in order (the CPU restatement's list walk).
    int32_t cur[K];
    int nc = 1;
    cur[0] = (int32_t)v;
    if (!cluster[v]) {
        for (int lev = 0; lev < k_levels; ++lev) {
            int32_t nxt[K];
            int nx = 0;
            for (int s = 0; s < nc; ++s) {
                int32_t x = cur[s];
                if (x < n - 1 && !cluster[x]) {
                    nxt[nx++] = left[x];
                    nxt[nx++] = right[x];
                } else {
                    nxt[nx++] = x;
                }
            }
            for (int s = 0; s < nx; ++s) cur[s] = nxt[s];
            nc = nx;
        }
    }
    WideNode<K> nd;
    uint32_t leaves = 0;
    for (int s = 0; s < K; ++s) {
        if (s < nc) {
            const int32_t x = cur[s];
            const float* b = box + 6 * (int64_t)x;
            nd.lox[s] = b[0]; nd.hix[s] = b[3];
            nd.loy[s] = b[1]; nd.hiy[s] = b[4];
            nd.loz[s] = b[2]; nd.hiz[s] = b[5];
            if (cluster[x]) {
                nd.child[s] = pack_leaf(first[x], last[x] - first[x] + 1);
                ++leaves;
            } else {
                nd.child[s] = (int32_t)wide_id[x];
            }
            slot_src[(int64_t)w * K + s] = x;
        } else {
            nd.lox[s] = INFINITY; nd.hix[s] = -INFINITY;
            nd.loy[s] = INFINITY; nd.hiy[s] = -INFINITY;
            nd.loz[s] = INFINITY; nd.hiz[s] = -INFINITY;
            nd.child[s] = 0;
            slot_src[(int64_t)w * K + s] = -1;
        }
        nd.pad[s] = 0;
    }
    nodes[w] = nd;
    wide_src[w] = (int32_t)v;
    if (leaves) atomicAdd(leaf_count, leaves);
    int m = nmeshes > 1 ? (int)(keys[first[v]] >> key_mesh_shift) : 0;
    if (mesh_root[m] == (int32_t)v) wide_root[m] = (int32_t)w;
}

// Refit path: copy each slot's refitted binary box into the wide node.
template <int K>
__global__ void k_wide_boxes(int64_t num_wide, const int32_t* __restrict__ slot_src,
                             const float* __restrict__ box, WideNode<K>* __restrict__ nodes) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_wide * K) return;
    int64_t w = i / K;
    int s = (int)(i % K);
    int32_t x = slot_src[i];
    if (x < 0) return;
    const float* b = box + 6 * (int64_t)x;
    WideNode<K>& nd = nodes[w];
    nd.lox[s] = b[0]; nd.hix[s] = b[3];
    nd.loy[s] = b[1]; nd.hiy[s] = b[4];
    nd.loz[s] = b[2]; nd.hiz[s] = b[5];
}

// Query Morton frame per mesh from the refitted root box.
__global__ void k_query_frames(const float* __restrict__ box, const int32_t* __restrict__ mesh_root,
                               int nmeshes, float cells, float* __restrict__ frame) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmeshes) return;
    const float* b = box + 6 * (int64_t)mesh_root[m];
    for (int k = 0; k < 3; ++k) {
        float ext = b[3 + k] - b[k];
        float scale = ext > 0.0f ? cells / ext : 0.0f;
        if (!(scale <= FLT_MAX)) scale = 0.0f;
        frame[6 * m + k] = b[k];
        frame[6 * m + 3 + k] = scale;
    }
}

template <typename T>
cudaError_t dalloc(Bvh& b, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    size_t bytes = count * sizeof(T);
    if (alloc_fault()) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), bytes);
    if (e != cudaSuccess) return e;
    b.allocations.push_back(*p);
    b.device_bytes += bytes;
    return cudaSuccess;
}

struct TmpAlloc {
    std::vector<void*> ptrs;
    cudaStream_t st;
    explicit TmpAlloc(cudaStream_t s) : st(s) {}
    template <typename T>
    cudaError_t get(T** p, size_t count) {
        if (count == 0) count = 1;
        if (alloc_fault()) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(p), count * sizeof(T), st);
        if (e == cudaSuccess) ptrs.push_back(*p);
        return e;
    }
    ~TmpAlloc() {
        for (void* p : ptrs) cudaFreeAsync(p, st);
    }
};

int ceil_log2(int64_t v) {
    int b = 0;
    while ((int64_t(1) << b) < v) ++b;
    return b;
}

#define CK(x)                                \
    do {                                     \
        cudaError_t e_ = (x);                \
        if (e_ != cudaSuccess) return e_;    \
    } while (0)

}  // namespace

void bvh_free(Bvh& b) {
    for (void* p : b.allocations) cudaFree(p);
    b.allocations.clear();
    b.device_bytes = 0;
    b.nodes = nullptr;
    b.recs = nullptr;
    b.mesh_leaf = nullptr;
}

cudaError_t bvh_build(Bvh& b, const float* verts, int64_t vstride, const int32_t* tris,
                      const std::vector<int64_t>& h_voff, const std::vector<int64_t>& h_toff,
                      const BuildParams& p, cudaStream_t st, bool* bad_input, std::string* why) {
    *bad_input = false;
    // the two timing events are destroyed on every return path
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events() {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    CK(cudaEventCreate(&ev.a));
    CK(cudaEventCreate(&ev.b));
    cudaEvent_t ev0 = ev.a, ev1 = ev.b;
    CK(cudaEventRecord(ev0, st));
    CK(cudaGetDevice(&b.device));
    b.p = p;
    b.nmeshes = (int32_t)(h_toff.size() - 1);
    b.nt = h_toff.back();
    b.nv = h_voff.back();
    b.h_voff = h_voff;
    b.h_toff = h_toff;
    const int64_t n = b.nt, nn = 2 * n - 1;
    const int nm = b.nmeshes;
    b.mesh_bits = nm > 1 ? ceil_log2(nm) : 0;
    b.morton_bits = (64 - b.mesh_bits) / 3;
    if (b.morton_bits > 21) b.morton_bits = 21;
    const int bits = b.morton_bits;
    const int key_shift = 3 * bits;
    const int k_levels = p.K == 2 ? 1 : (p.K == 4 ? 2 : 3);

    CK(dalloc(b, &b.tris, (size_t)3 * n));
    CK(dalloc(b, &b.d_voff, (size_t)nm + 1));
    CK(dalloc(b, &b.d_toff, (size_t)nm + 1));
    CK(dalloc(b, &b.keys, (size_t)n));
    CK(dalloc(b, &b.order, (size_t)n));
    CK(dalloc(b, &b.inv_order, (size_t)n));
    CK(dalloc(b, &b.left, (size_t)(n > 1 ? n - 1 : 1)));
    CK(dalloc(b, &b.right, (size_t)(n > 1 ? n - 1 : 1)));
    CK(dalloc(b, &b.parent, (size_t)nn));
    CK(dalloc(b, &b.first, (size_t)nn));
    CK(dalloc(b, &b.last, (size_t)nn));
    CK(dalloc(b, &b.box, (size_t)6 * nn));
    CK(dalloc(b, &b.cost, (size_t)nn));
    CK(dalloc(b, &b.leaf_flag, (size_t)nn));
    CK(dalloc(b, &b.cluster, (size_t)nn));
    CK(dalloc(b, &b.arrive, (size_t)nn));
    CK(dalloc(b, &b.mesh_root, (size_t)nm));
    CK(dalloc(b, &b.wide_root, (size_t)nm));
    CK(dalloc(b, &b.frame, (size_t)6 * nm));
    CK(dalloc(b, &b.recs, (size_t)n));
    CK(dalloc(b, &b.fast, (size_t)n));
    CK(dalloc(b, &b.status, (size_t)64));
    if (!p.mesh_leaf.empty()) {
        if ((int)p.mesh_leaf.size() != nm) return cudaErrorInvalidValue;
        CK(dalloc(b, &b.mesh_leaf, (size_t)nm));
        CK(cudaMemcpyAsync(b.mesh_leaf, b.p.mesh_leaf.data(), sizeof(int32_t) * nm, cudaMemcpyHostToDevice, st));
    }

    CK(cudaMemcpyAsync(b.tris, tris, sizeof(int32_t) * 3 * n, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(b.d_voff, h_voff.data(), sizeof(int64_t) * (nm + 1), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(b.d_toff, h_toff.data(), sizeof(int64_t) * (nm + 1), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(b.status, 0, 64 * sizeof(uint32_t), st));
    CK(cudaMemsetAsync(b.mesh_root, 0xff, sizeof(int32_t) * nm, st));
    CK(cudaMemsetAsync(b.wide_root, 0, sizeof(int32_t) * nm, st));

    TmpAlloc tmp(st);
    float* csum;
    float* mbox;
    float* lo_scale;
    int32_t* vals;
    uint64_t* keys_alt;
    int32_t* vals_alt;
    uint32_t* wide_id;
    uint32_t* scratch;  // [0] bad-input flags, [1] max depth, [2] num wide, [4..7] key and/or
    CK(tmp.get(&csum, (size_t)3 * n));
    CK(tmp.get(&mbox, (size_t)6 * nm));
    CK(tmp.get(&lo_scale, (size_t)6 * nm));
    CK(tmp.get(&vals, (size_t)n));
    CK(tmp.get(&keys_alt, (size_t)n));
    CK(tmp.get(&vals_alt, (size_t)n));
    CK(tmp.get(&wide_id, (size_t)nn));
    CK(tmp.get(&scratch, (size_t)16));
    const size_t sort_ws = radix_sort_workspace_bytes(n);
    const size_t scan_ws = scan_workspace_bytes(nn);
    unsigned char* ws;
    CK(tmp.get(&ws, sort_ws > scan_ws ? sort_ws : scan_ws));
    CK(cudaMemsetAsync(scratch, 0, 16 * sizeof(uint32_t), st));
    CK(cudaMemsetAsync(scratch + 4, 0xff, 2 * sizeof(uint32_t), st));  // AND identity

    // validate indices and coordinates before any kernel reads a vertex by index
    k_validate<<<grid_for(n), kThreads, 0, st>>>(verts, vstride, b.tris, n, b.d_voff, b.d_toff, nm,
                                                scratch); note_launch();
    CK(cudaGetLastError());
    uint32_t h_scr[16];
    CK(cudaMemcpyAsync(h_scr, scratch, sizeof(h_scr), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h_scr[0] != 0) {
        *bad_input = true;
        if (why) *why = (h_scr[0] & 2u) ? "triangle index out of range" : "non-finite vertex coordinate";
        return cudaSuccess;
    }
    k_init_boxes<<<grid_for(6 * nm), kThreads, 0, st>>>(mbox, 6 * nm); note_launch();
    k_centroid_bounds<<<(unsigned)std::min<int64_t>((n + 2047) / 2048, 1216), kThreads, 0, st>>>(
        verts, vstride, b.tris, n, b.d_voff,
                                                       b.d_toff, nm, csum, mbox); note_launch();
    CK(cudaGetLastError());
    k_build_frames<<<grid_for(nm), kThreads, 0, st>>>(mbox, nm, (float)(1u << bits), lo_scale); note_launch();
    k_morton<<<grid_for(n), kThreads, 0, st>>>(csum, n, b.d_toff, nm, lo_scale, bits, b.keys, vals); note_launch();
    CK(cudaGetLastError());
    // sort only the digits whose bits vary
    k_key_and_or<<<256, kThreads, 0, st>>>(b.keys, n, reinterpret_cast<unsigned long long*>(scratch + 4)); note_launch();
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h_scr, scratch, sizeof(h_scr), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    uint64_t kand, kor;
    std::memcpy(&kand, &h_scr[4], 8);
    std::memcpy(&kor, &h_scr[6], 8);
    uint64_t vary = kand ^ kor;
    int begin_bit = 0, end_bit = 0;
    if (vary) {
        int lo_bit = __builtin_ctzll(vary), hi_bit = 63 - __builtin_clzll(vary);
        begin_bit = (lo_bit / 8) * 8;
        end_bit = (hi_bit / 8 + 1) * 8;
    }
    bool in_alt = false;
    CK(radix_sort_pairs<uint64_t>(b.keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, ws,
                                  sort_ws, st, &in_alt));
    if (in_alt) {
        CK(cudaMemcpyAsync(b.keys, keys_alt, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(b.order, vals_alt, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
    } else {
        CK(cudaMemcpyAsync(b.order, vals, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st));
    }

    k_leaf_init<<<grid_for(n), kThreads, 0, st>>>(n, b.first, b.last, b.parent); note_launch();
    CK(cudaGetLastError());
    if (n > 1) {
        k_karras<<<grid_for(n - 1), kThreads, 0, st>>>(b.keys, n, bits, nm, b.d_toff, b.left,
                                                       b.right, b.parent, b.first, b.last,
                                                       b.mesh_root); note_launch();
        CK(cudaGetLastError());
    }
    k_single_tri_roots<<<grid_for(nm), kThreads, 0, st>>>(b.d_toff, nm, n, b.mesh_root); note_launch();
    CK(cudaMemsetAsync(b.arrive, 0, sizeof(uint32_t) * nn, st));
    k_refit<true><<<grid_for(n), kThreads, 0, st>>>(
        verts, vstride, b.tris, b.order, b.keys, n, b.d_voff, b.d_toff, nm, key_shift, b.left,
        b.right, b.parent, b.first, b.last, b.box, b.cost, b.leaf_flag, b.arrive, b.recs,
        b.fast, b.inv_order, p.leaf_size, b.mesh_leaf, p.collapse, p.c_node, p.c_tri); note_launch();
    CK(cudaGetLastError());
    int32_t* max_depth = reinterpret_cast<int32_t*>(scratch + 1);
    k_wide_flags<<<grid_for(nn), kThreads, 0, st>>>(n, b.keys, nm, key_shift, b.parent, b.first,
                                                   b.last, b.leaf_flag, b.mesh_root, k_levels,
                                                   b.cluster, wide_id, max_depth); note_launch();
    CK(cudaGetLastError());
    uint32_t* wide_flag;
    CK(tmp.get(&wide_flag, (size_t)nn));
    CK(cudaMemcpyAsync(wide_flag, wide_id, sizeof(uint32_t) * nn, cudaMemcpyDeviceToDevice, st));
    CK(exclusive_scan_u32(wide_id, nn, scratch + 2, ws, scan_ws, st));
    CK(cudaMemcpyAsync(h_scr, scratch, sizeof(h_scr), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    b.max_wide_depth = (int32_t)h_scr[1];
    b.num_wide = h_scr[2];
    b.stack_bound = (p.K - 1) * (b.max_wide_depth + 1);

    const size_t node_bytes = (size_t)32 * p.K;
    {
        void* nodes = nullptr;
        CK(cudaMalloc(&nodes, node_bytes * (size_t)b.num_wide));
        b.allocations.push_back(nodes);
        b.device_bytes += node_bytes * (size_t)b.num_wide;
        b.nodes = nodes;
    }
    CK(dalloc(b, &b.wide_src, (size_t)b.num_wide));
    CK(dalloc(b, &b.slot_src, (size_t)b.num_wide * p.K));
    switch (p.K) {
        case 2:
            k_wide_emit<2><<<grid_for(nn), kThreads, 0, st>>>(
                n, k_levels, wide_flag, wide_id, b.keys, nm, key_shift, b.left, b.right, b.first,
                b.last, b.box, b.cluster, b.mesh_root, static_cast<WideNode<2>*>(b.nodes),
                b.wide_src, b.slot_src, b.wide_root, scratch + 3); note_launch();
            break;
        case 4:
            k_wide_emit<4><<<grid_for(nn), kThreads, 0, st>>>(
                n, k_levels, wide_flag, wide_id, b.keys, nm, key_shift, b.left, b.right, b.first,
                b.last, b.box, b.cluster, b.mesh_root, static_cast<WideNode<4>*>(b.nodes),
                b.wide_src, b.slot_src, b.wide_root, scratch + 3); note_launch();
            break;
        default:
            k_wide_emit<8><<<grid_for(nn), kThreads, 0, st>>>(
                n, k_levels, wide_flag, wide_id, b.keys, nm, key_shift, b.left, b.right, b.first,
                b.last, b.box, b.cluster, b.mesh_root, static_cast<WideNode<8>*>(b.nodes),
                b.wide_src, b.slot_src, b.wide_root, scratch + 3); note_launch();
            break;
    }
    CK(cudaGetLastError());
    const int qbits = (64 - b.mesh_bits) / 3 < 10 ? (64 - b.mesh_bits) / 3 : 10;
    k_query_frames<<<grid_for(nm), kThreads, 0, st>>>(b.box, b.mesh_root, nm, (float)(1u << qbits),
                                                     b.frame); note_launch();
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h_scr, scratch, sizeof(h_scr), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ev1, st));
    CK(cudaEventSynchronize(ev1));
    cudaEventElapsedTime(&b.build_ms, ev0, ev1);
    b.num_leaves = h_scr[3];
    return cudaSuccess;
}

cudaError_t bvh_refit(Bvh& b, const float* verts, int64_t vstride, cudaStream_t st) {
    const int64_t n = b.nt, nn = 2 * n - 1;
    const int key_shift = 3 * b.morton_bits;
    CK(cudaMemsetAsync(b.arrive, 0, sizeof(uint32_t) * nn, st));
    k_refit<false><<<grid_for(n), kThreads, 0, st>>>(
        verts, vstride, b.tris, b.order, b.keys, n, b.d_voff, b.d_toff, b.nmeshes, key_shift,
        b.left, b.right, b.parent, b.first, b.last, b.box, b.cost, b.leaf_flag, b.arrive, b.recs,
        b.fast, b.inv_order, b.p.leaf_size, nullptr, b.p.collapse, b.p.c_node, b.p.c_tri); note_launch();
    CK(cudaGetLastError());
    const int64_t slots = b.num_wide * b.p.K;
    switch (b.p.K) {
        case 2:
            k_wide_boxes<2><<<grid_for(slots), kThreads, 0, st>>>(b.num_wide, b.slot_src, b.box,
                                                                 static_cast<WideNode<2>*>(b.nodes)); note_launch();
            break;
        case 4:
            k_wide_boxes<4><<<grid_for(slots), kThreads, 0, st>>>(b.num_wide, b.slot_src, b.box,
                                                                 static_cast<WideNode<4>*>(b.nodes)); note_launch();
            break;
        default:
            k_wide_boxes<8><<<grid_for(slots), kThreads, 0, st>>>(b.num_wide, b.slot_src, b.box,
                                                                 static_cast<WideNode<8>*>(b.nodes)); note_launch();
            break;
    }
    CK(cudaGetLastError());
    const int qbits = (64 - b.mesh_bits) / 3 < 10 ? (64 - b.mesh_bits) / 3 : 10;
    k_query_frames<<<grid_for(b.nmeshes), kThreads, 0, st>>>(b.box, b.mesh_root, b.nmeshes,
                                                            (float)(1u << qbits), b.frame); note_launch();
    return cudaGetLastError();
}

}  // namespace cpq
