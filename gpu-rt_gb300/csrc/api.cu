// api.cu — the extern "C" boundary declared in include/cpq.h.
//
// Handles own device memory; arrays passed in are caller-owned.  Every entry
// point catches its own failures and returns a cp_status with a message in a
// thread-local string; nothing here exits the process (the reference's die()
// does, src/lib/log.h:46-49).  Workspaces that the caller does not provide
// come from a per-device stream-ordered memory pool, so a query allocates
// nothing synchronously and stays on its stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <new>
#include <string>
#include <vector>

#include "../../include/cpq.h"
#include "bvh.cuh"
#include "handles.cuh"
#include "sort.cuh"
#include "ray.cuh"

using namespace cpq;

namespace cpq {
static std::atomic<uint64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// Allocations still to succeed before one fails; -1: off.  Firing disarms it.
static std::atomic<int64_t> g_fail_after{-1};
bool alloc_fault() {
    int64_t v = g_fail_after.load(std::memory_order_relaxed);
    while (v >= 0) {
        if (g_fail_after.compare_exchange_weak(v, v - 1, std::memory_order_relaxed)) return v == 0;
    }
    return false;
}

namespace {
struct KernelCache {
    std::mutex mu;
    std::map<std::pair<const void*, int>, size_t> smem_limit;                   // (kernel, device)
    std::map<std::tuple<const void*, int, int, size_t>, int> occupancy;  // + block, smem
    std::map<int, int> sms;
};
KernelCache& kernel_cache() {
    static KernelCache c;
    return c;
}
}  // namespace

cudaError_t sm_count(int* out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    KernelCache& c = kernel_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    auto it = c.sms.find(dev);
    if (it == c.sms.end()) {
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        it = c.sms.emplace(dev, n).first;
    }
    *out = it->second;
    return cudaSuccess;
}

cudaError_t ensure_smem_limit(const void* kernel, size_t smem) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    KernelCache& c = kernel_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    size_t& have = c.smem_limit[{kernel, dev}];
    if (have >= smem) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) have = smem;
    return e;
}

cudaError_t blocks_per_sm(const void* kernel, int block, size_t smem, int* out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    KernelCache& c = kernel_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    auto key = std::make_tuple(kernel, dev, block, smem);
    auto it = c.occupancy.find(key);
    if (it == c.occupancy.end()) {
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, smem);
        if (e != cudaSuccess) return e;
        it = c.occupancy.emplace(key, n < 1 ? 1 : n).first;
    }
    *out = it->second;
    return cudaSuccess;
}
}  // namespace cpq

struct cp_batch {
    Bvh bvh;
    int64_t* d_qoff = nullptr;
    std::vector<int64_t> h_qoff;
    // CUDA-graph cache of the last captured query launch sequence
    cudaGraphExec_t exec = nullptr;
    std::vector<uintptr_t> graph_key;
    cudaStream_t capture_stream = nullptr;
};

namespace {

thread_local std::string g_last_error;

cp_status fail(cp_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

cp_status cuda_fail(cudaError_t e, const char* where) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(CP_ERROR_OUT_OF_MEMORY, std::string(where) + ": " + cudaGetErrorString(e));
    }
    return fail(CP_ERROR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CP_CUDA(call, where)                          \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, where); \
    } while (0)

cp_status require_gpu() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(CP_ERROR_NOT_SUPPORTED, "no CUDA device is available");
    }
    return CP_SUCCESS;
}

// Per-device pool for stream-ordered workspaces that stays warm between calls.
std::mutex g_pool_mu;
std::vector<cudaMemPool_t> g_pools;

cudaError_t get_pool(cudaMemPool_t* out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if ((int)g_pools.size() <= dev) g_pools.resize(dev + 1, nullptr);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        e = cudaMemPoolCreate(&pool, &props);
        if (e != cudaSuccess) return e;
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        // An allocation never waits on another stream's pending free: the pool
        // grows instead, so calls on two streams (a double-buffered stream of
        // host batches) keep overlapping rather than queueing behind each other.
        int no_internal_waits = 0;
        cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no_internal_waits);
        g_pools[dev] = pool;
    }
    *out = g_pools[dev];
    return cudaSuccess;
}

cudaError_t ws_alloc(void** p, size_t bytes, cudaStream_t st) {
    if (alloc_fault()) return cudaErrorMemoryAllocation;
    cudaMemPool_t pool;
    cudaError_t e = get_pool(&pool);
    if (e != cudaSuccess) return e;
    return cudaMallocFromPoolAsync(p, bytes ? bytes : 256, pool, st);
}

cp_status to_build_params(const cp_build_opts* o, BuildParams* p) {
    cp_build_opts d;
    cp_build_opts_default(&d);
    if (!o) o = &d;
    if (o->branching != 2 && o->branching != 4 && o->branching != 8)
        return fail(CP_ERROR_INVALID_VALUE, "branching must be 2, 4 or 8");
    if (o->leaf_size < 1 || o->leaf_size > kMaxLeafSize)
        return fail(CP_ERROR_INVALID_VALUE, "leaf_size must be in 1..15");
    if (o->collapse != CP_COLLAPSE_COUNT && o->collapse != CP_COLLAPSE_SAH)
        return fail(CP_ERROR_INVALID_VALUE, "collapse must be CP_COLLAPSE_COUNT or CP_COLLAPSE_SAH");
    if (o->collapse == CP_COLLAPSE_SAH &&
        !(o->sah_node_cost >= 0.0f && o->sah_tri_cost > 0.0f && std::isfinite(o->sah_node_cost) &&
          std::isfinite(o->sah_tri_cost)))
        return fail(CP_ERROR_INVALID_VALUE, "SAH costs must be finite, node >= 0, triangle > 0");
    p->K = o->branching;
    p->leaf_size = o->leaf_size;
    p->collapse = o->collapse;
    p->c_node = o->sah_node_cost;
    p->c_tri = o->sah_tri_cost;
    return CP_SUCCESS;
}

cp_status to_query_params(const cp_query_opts* o, QueryParams* q) {
    cp_query_opts d;
    cp_query_opts_default(&d);
    if (!o) o = &d;
    int block = o->block_size ? o->block_size : d.block_size;
    if (block < 32 || block > 256 || block % 32)
        return fail(CP_ERROR_INVALID_VALUE, "block_size must be a multiple of 32 in 32..256");
    int ss = o->short_stack ? o->short_stack : d.short_stack;
    if (ss != 4 && ss != 8 && ss != 16)
        return fail(CP_ERROR_INVALID_VALUE, "short_stack must be 4, 8 or 16");
    if (o->blocks_per_sm < 0 || o->blocks_per_sm > 64)
        return fail(CP_ERROR_INVALID_VALUE, "blocks_per_sm must be in 0..64");
    if (o->traversal < CP_TRAVERSAL_AUTO || o->traversal > CP_TRAVERSAL_PACKET)
        return fail(CP_ERROR_INVALID_VALUE, "traversal must be CP_TRAVERSAL_AUTO, _THREAD or _PACKET");
    if (o->seed_chunk < 0 || o->seed_chunk > 16)
        return fail(CP_ERROR_INVALID_VALUE, "seed_chunk must be in 0..16");
    q->block = block;
    q->sort = o->sort_queries ? 1 : 0;
    q->blocks_per_sm = o->blocks_per_sm;
    q->short_stack = ss;
    q->traversal = o->traversal;
    q->seed_chunk = o->seed_chunk ? o->seed_chunk : 1;
    return CP_SUCCESS;
}

cp_status build_common(Bvh& b, const float* verts, int64_t vstride_bytes, const int32_t* tris,
                       const std::vector<int64_t>& voff, const std::vector<int64_t>& toff,
                       const cp_build_opts* opts, cp_stream_t stream, const int32_t* mesh_leaf = nullptr) {
    BuildParams p;
    cp_status s = to_build_params(opts, &p);
    if (s != CP_SUCCESS) return s;
    if (mesh_leaf) {
        const int32_t nm = (int32_t)toff.size() - 1;
        p.mesh_leaf.assign(mesh_leaf, mesh_leaf + nm);
        int32_t mx = 1;
        for (int32_t i = 0; i < nm; ++i) {
            if (p.mesh_leaf[i] < 1 || p.mesh_leaf[i] > kMaxLeafSize)
                return fail(CP_ERROR_INVALID_VALUE, "leaf size of mesh " + std::to_string(i) + " must be in 1..15");
            mx = std::max(mx, p.mesh_leaf[i]);
        }
        p.leaf_size = mx;
    }
    if (vstride_bytes < 12 || vstride_bytes % 4)
        return fail(CP_ERROR_INVALID_VALUE, "vertex stride must be a multiple of 4 bytes and >= 12");
    bool bad = false;
    std::string why;
    cudaError_t e = bvh_build(b, verts, vstride_bytes / 4, tris, voff, toff, p,
                              reinterpret_cast<cudaStream_t>(stream), &bad, &why);
    if (e != cudaSuccess) {
        bvh_free(b);
        return cuda_fail(e, "BVH build");
    }
    if (bad) {
        bvh_free(b);
        return fail(CP_ERROR_INVALID_VALUE, "BVH build: " + why);
    }
    if (b.stack_bound > 256) {
        bvh_free(b);
        return fail(CP_ERROR_NOT_SUPPORTED, "BVH deeper than the traversal stack supports");
    }
    return CP_SUCCESS;
}

}  // namespace

namespace cpq {
cp_status parse_query_opts(const cp_query_opts* opts, QueryParams* out) {
    return to_query_params(opts, out);
}
cp_status set_error(cp_status s, const std::string& msg) { return fail(s, msg); }
}  // namespace cpq

extern "C" {

CP_API void cp_build_opts_default(cp_build_opts* o) {
    if (!o) return;
    o->branching = 2;
    o->leaf_size = 4;
    o->collapse = CP_COLLAPSE_COUNT;
    o->sah_node_cost = 1.0f;
    o->sah_tri_cost = 1.0f;
}

CP_API void cp_query_opts_default(cp_query_opts* o) {
    if (!o) return;
    o->block_size = 256;
    o->sort_queries = 1;
    o->blocks_per_sm = 0;
    o->short_stack = 8;
    o->traversal = CP_TRAVERSAL_AUTO;
    o->seed_chunk = 1;
}

CP_API const char* cp_last_error_string(void) { return g_last_error.c_str(); }

CP_API const char* cp_status_string(cp_status s) {
    switch (s) {
        case CP_SUCCESS: return "success";
        case CP_ERROR_INVALID_VALUE: return "invalid value";
        case CP_ERROR_OUT_OF_MEMORY: return "out of memory";
        case CP_ERROR_CUDA: return "CUDA error";
        case CP_ERROR_DEVICE_FAULT: return "device fault";
        case CP_ERROR_NOT_SUPPORTED: return "not supported";
        case CP_ERROR_SCRATCH_TOO_SMALL: return "scratch too small";
    }
    return "unknown status";
}

CP_API int32_t cp_version(void) { return 100; }

CP_API uint64_t cp_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

CP_API void cp_debug_fail_allocation(int64_t after) {
    g_fail_after.store(after < 0 ? -1 : after, std::memory_order_relaxed);
}

// Values 0..n-1: the identity permutation the sort starts from.
__global__ void k_iota(int32_t* __restrict__ v, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = (int32_t)i;
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

CP_API cp_status cp_timing_enable(int32_t flags) {
    if (flags & ~(CP_TIMING_EVENTS | CP_TIMING_COUNTERS))
        return fail(CP_ERROR_INVALID_VALUE, "cp_timing_enable: unknown flag bits");
    timing_enable((flags & CP_TIMING_EVENTS) != 0, (flags & CP_TIMING_COUNTERS) != 0);
    return CP_SUCCESS;
}

CP_API cp_status cp_timing_read(double* traverse_ms, int64_t* launches, int32_t reset) {
    CP_CUDA(timing_read(traverse_ms, launches, reset != 0), "timing read");
    return CP_SUCCESS;
}

CP_API cp_status cp_traversal_stats(uint64_t* counts7, int32_t reset) {
    if (!counts7) return fail(CP_ERROR_INVALID_VALUE, "counts7 is NULL");
    unsigned long long c[kStatCount];
    CP_CUDA(traversal_stats(c, reset != 0), "traversal stats");
    for (int k = 0; k < kStatCount; ++k) counts7[k] = c[k];
    return CP_SUCCESS;
}

CP_API int32_t cp_size_class(int64_t nt) {
    int32_t c = 0;
    while (nt > 1) {
        nt >>= 1;
        ++c;
    }
    return c;
}

CP_API cp_status cp_mesh_create(const float* verts, int64_t nv, int64_t vstride, const int32_t* tris,
                                int64_t nt, const cp_build_opts* opts, cp_stream_t stream,
                                cp_mesh** out) {
    if (!out) return fail(CP_ERROR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (!verts || !tris) return fail(CP_ERROR_INVALID_VALUE, "verts or tris is NULL");
    if (nv <= 0 || nt <= 0) return fail(CP_ERROR_INVALID_VALUE, "mesh needs at least one vertex and one triangle");
    if (nt > kMaxTriangles) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^27 - 1 triangles");
    if (nv > INT32_MAX) return fail(CP_ERROR_INVALID_VALUE, "more than 2^31 - 1 vertices");
    cp_status s = require_gpu();
    if (s != CP_SUCCESS) return s;
    cp_mesh* m = new (std::nothrow) cp_mesh();
    if (!m) return fail(CP_ERROR_OUT_OF_MEMORY, "host allocation of the handle failed");
    s = build_common(m->bvh, verts, vstride, tris, {0, nv}, {0, nt}, opts, stream);
    if (s != CP_SUCCESS) {
        delete m;
        return s;
    }
    *out = m;
    return CP_SUCCESS;
}

CP_API cp_status cp_mesh_refit(cp_mesh* m, const float* verts, int64_t vstride, cp_stream_t stream) {
    if (!m || !verts) return fail(CP_ERROR_INVALID_VALUE, "mesh or verts is NULL");
    if (vstride < 12 || vstride % 4)
        return fail(CP_ERROR_INVALID_VALUE, "vertex stride must be a multiple of 4 bytes and >= 12");
    CP_CUDA(bvh_refit(m->bvh, verts, vstride / 4, reinterpret_cast<cudaStream_t>(stream)), "refit");
    return CP_SUCCESS;
}

CP_API cp_status cp_mesh_save(const cp_mesh* m, const char* path) {
    if (!m || !path) return fail(CP_ERROR_INVALID_VALUE, "mesh or path is NULL");
    std::string why;
    cudaError_t e = bvh_save(const_cast<cp_mesh*>(m)->bvh, path, &why);
    if (!why.empty()) return fail(CP_ERROR_INVALID_VALUE, "cp_mesh_save: " + why);
    if (e != cudaSuccess) return cuda_fail(e, "cp_mesh_save");
    return CP_SUCCESS;
}

CP_API cp_status cp_mesh_load(const char* path, cp_stream_t stream, cp_mesh** out) {
    if (!out || !path) return fail(CP_ERROR_INVALID_VALUE, "path or out is NULL");
    *out = nullptr;
    cp_mesh* m = new (std::nothrow) cp_mesh();
    if (!m) return fail(CP_ERROR_OUT_OF_MEMORY, "host allocation of the handle failed");
    std::string why;
    bool bad = false;
    cudaError_t e = bvh_load(m->bvh, path, reinterpret_cast<cudaStream_t>(stream), &why, &bad);
    if (e == cudaSuccess && m->bvh.nmeshes != 1) {
        bad = true;
        why = "the file holds a batch of " + std::to_string(m->bvh.nmeshes) + " meshes, not one mesh";
    }
    if (bad || e != cudaSuccess) {
        bvh_free(m->bvh);
        delete m;
        if (bad) return fail(CP_ERROR_INVALID_VALUE, std::string("cp_mesh_load: ") + path + ": " + why);
        return cuda_fail(e, "cp_mesh_load");
    }
    *out = m;
    return CP_SUCCESS;
}

CP_API cp_status cp_mesh_destroy(cp_mesh* m) {
    if (!m) return CP_SUCCESS;
    bvh_free(m->bvh);
    delete m;
    return CP_SUCCESS;
}

CP_API cp_status cp_mesh_info(const cp_mesh* m, cp_mesh_info_t* o) {
    if (!m || !o) return fail(CP_ERROR_INVALID_VALUE, "mesh or out is NULL");
    const Bvh& b = m->bvh;
    o->num_vertices = b.nv;
    o->num_triangles = b.nt;
    o->num_binary_nodes = 2 * b.nt - 1;
    o->num_wide_nodes = b.num_wide;
    o->num_leaves = b.num_leaves;
    o->branching = b.p.K;
    o->leaf_size = b.p.leaf_size;
    o->max_wide_depth = b.max_wide_depth;
    o->stack_bound = b.stack_bound;
    o->device_bytes = (int64_t)b.device_bytes;
    o->build_ms = b.build_ms;
    return CP_SUCCESS;
}

CP_API cp_status cp_mesh_device_status(cp_mesh* m, cp_stream_t stream, uint32_t* bits) {
    if (!m || !bits) return fail(CP_ERROR_INVALID_VALUE, "mesh or bits is NULL");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint32_t h = 0;
    CP_CUDA(cudaMemcpyAsync(&h, m->bvh.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "status read");
    CP_CUDA(cudaStreamSynchronize(st), "status read");
    CP_CUDA(cudaMemsetAsync(m->bvh.status, 0, sizeof(uint32_t), st), "status clear");
    *bits = h;
    return CP_SUCCESS;
}

CP_API cp_status cp_query_workspace_size(const cp_mesh* m, int64_t nq, const cp_query_opts* opts,
                                         size_t* bytes) {
    if (!m || !bytes) return fail(CP_ERROR_INVALID_VALUE, "mesh or bytes is NULL");
    if (nq < 0) return fail(CP_ERROR_INVALID_VALUE, "negative query count");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    *bytes = query_workspace_bytes(m->bvh, nq, qp);
    return CP_SUCCESS;
}

static cp_status query_impl(const Bvh& b, const float* q, int64_t nq, const int64_t* d_qoff,
                            const QueryParams& qp, float* op, float* od, int32_t* ot, float* ob,
                            void* ws, size_t ws_bytes, cudaStream_t st) {
    const size_t need = query_workspace_bytes(b, nq, qp);
    void* own = nullptr;
    if (!ws) {
        CP_CUDA(ws_alloc(&own, need, st), "workspace allocation");
        ws = own;
        ws_bytes = need;
    } else if (ws_bytes < need) {
        return fail(CP_ERROR_SCRATCH_TOO_SMALL, "workspace smaller than cp_query_workspace_size()");
    }
    cudaError_t e = bvh_query(b, q, nq, d_qoff, qp, op, od, ot, ob, ws, ws_bytes, st);
    if (own) cudaFreeAsync(own, st);
    if (e != cudaSuccess) return cuda_fail(e, "query");
    return CP_SUCCESS;
}

CP_API cp_status cp_query(const cp_mesh* m, const float* queries, int64_t nq,
                          const cp_query_opts* opts, float* out_point, float* out_dist,
                          int32_t* out_tri, float* out_bary, void* workspace, size_t ws_bytes,
                          cp_stream_t stream) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (nq < 0) return fail(CP_ERROR_INVALID_VALUE, "negative query count");
    if (nq > INT32_MAX) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^31 - 1 queries in one call");
    if (nq == 0) return CP_SUCCESS;
    if (!queries) return fail(CP_ERROR_INVALID_VALUE, "queries is NULL");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    return query_impl(m->bvh, queries, nq, nullptr, qp, out_point, out_dist, out_tri, out_bary,
                      workspace, ws_bytes, reinterpret_cast<cudaStream_t>(stream));
}

CP_API cp_status cp_query_order(cp_mesh* m, const float* queries, int64_t nq, int32_t* perm, uint32_t* keys,
                                cp_stream_t stream) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (nq < 2 || nq > INT32_MAX) return fail(CP_ERROR_INVALID_VALUE, "cp_query_order: nq must be in 2..2^31 - 1");
    if (!queries || !perm) return fail(CP_ERROR_INVALID_VALUE, "queries and perm are required");
    if (m->bvh.nmeshes != 1) return fail(CP_ERROR_NOT_SUPPORTED, "cp_query_order: single meshes only");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    QueryParams qp;
    cp_status s = to_query_params(nullptr, &qp);
    if (s != CP_SUCCESS) return s;
    qp.sort = 1;
    const size_t need = query_workspace_bytes(m->bvh, nq, qp);
    void* ws = nullptr;
    CP_CUDA(ws_alloc(&ws, need, st), "workspace allocation");
    const int32_t* order = nullptr;
    unsigned long long* counter = nullptr;
    cudaError_t e = order_points(m->bvh, queries, nq, nullptr, true, ws, need, st, &order, &counter, false, keys);
    if (e == cudaSuccess && order)
        e = cudaMemcpyAsync(perm, order, sizeof(int32_t) * nq, cudaMemcpyDeviceToDevice, st);
    cudaFreeAsync(ws, st);
    if (e != cudaSuccess) return cuda_fail(e, "cp_query_order");
    return CP_SUCCESS;
}

CP_API cp_status cp_debug_order_sort(const void* keys, int32_t key_bytes, int64_t n, int32_t begin_bit,
                                     int32_t end_bit, int32_t* perm, cp_stream_t stream) {
    if (!keys || !perm) return fail(CP_ERROR_INVALID_VALUE, "keys and perm are required");
    if (key_bytes != 4 && key_bytes != 8) return fail(CP_ERROR_INVALID_VALUE, "key_bytes must be 4 or 8");
    if (n < 2 || n > INT32_MAX) return fail(CP_ERROR_INVALID_VALUE, "n must be in 2..2^31 - 1");
    if (begin_bit < 0 || end_bit <= begin_bit || end_bit > 8 * key_bytes)
        return fail(CP_ERROR_INVALID_VALUE, "need 0 <= begin_bit < end_bit <= key width");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t kb = align256((size_t)key_bytes * n), vb = align256(sizeof(int32_t) * n);
    const size_t sb = radix_sort_workspace_bytes(n);
    unsigned char* ws = nullptr;
    CP_CUDA(ws_alloc(reinterpret_cast<void**>(&ws), 2 * kb + 2 * vb + sb, st), "workspace allocation");
    int32_t* vals = reinterpret_cast<int32_t*>(ws + 2 * kb);
    int32_t* vals_alt = reinterpret_cast<int32_t*>(ws + 2 * kb + vb);
    cudaError_t e = cudaMemcpyAsync(ws, keys, (size_t)key_bytes * n, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) {
        k_iota<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(vals, n); note_launch();
        e = cudaGetLastError();
    }
    bool in_alt = false;
    if (e == cudaSuccess)
        e = key_bytes == 4 ? radix_sort_pairs<uint32_t>(reinterpret_cast<uint32_t*>(ws), vals,
                                                         reinterpret_cast<uint32_t*>(ws + kb), vals_alt, n,
                                                         begin_bit, end_bit, ws + 2 * kb + 2 * vb, sb, st, &in_alt)
                           : radix_sort_pairs<uint64_t>(reinterpret_cast<uint64_t*>(ws), vals,
                                                         reinterpret_cast<uint64_t*>(ws + kb), vals_alt, n,
                                                         begin_bit, end_bit, ws + 2 * kb + 2 * vb, sb, st, &in_alt);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(perm, in_alt ? vals_alt : vals, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, st);
    cudaFreeAsync(ws, st);
    if (e != cudaSuccess) return cuda_fail(e, "cp_debug_order_sort");
    return CP_SUCCESS;
}

CP_API cp_status cp_query_host(const cp_mesh* m, const float* queries, int64_t nq,
                               const cp_query_opts* opts, float* out_point, float* out_dist,
                               int32_t* out_tri, float* out_bary, cp_stream_t stream) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (nq < 0) return fail(CP_ERROR_INVALID_VALUE, "negative query count");
    if (nq == 0) return CP_SUCCESS;
    if (!queries) return fail(CP_ERROR_INVALID_VALUE, "queries is NULL");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    const Bvh& b = m->bvh;
    cudaStream_t user = reinterpret_cast<cudaStream_t>(stream);
    // One ordering over as many queries as possible: a 32-query packet's
    // extent shrinks with the density of the ordered set, so splitting a batch
    // into chunks costs more traversal time (16M queries in 4M chunks: +4 ms)
    // than overlapping their copies with it saves (H2D + D2H: 2.7 ms).  Only
    // batches beyond 64M queries (about 4 GB of scratch) are pipelined.
    const int64_t chunk = nq < (int64_t(1) << 26) ? nq : (int64_t(1) << 26);
    const int64_t nchunks = (nq + chunk - 1) / chunk;
    const int nslots = nchunks > 1 ? 2 : 1;
    cudaStream_t st[2] = {nullptr, nullptr};
    cudaEvent_t start = nullptr, done[2] = {nullptr, nullptr};
    struct Slot {
        float *q, *p, *d, *b;
        int32_t* t;
        void* ws;
    } slot[2] = {};
    const size_t wsb = query_workspace_bytes(b, chunk, qp);
    cp_status result = CP_SUCCESS;
    auto check = [&](cudaError_t e, const char* where) {
        if (e != cudaSuccess && result == CP_SUCCESS) result = cuda_fail(e, where);
        return e == cudaSuccess;
    };
    check(cudaEventCreateWithFlags(&start, cudaEventDisableTiming), "event");
    check(cudaEventRecord(start, user), "event");
    for (int k = 0; k < nslots && result == CP_SUCCESS; ++k) {
        check(cudaStreamCreateWithFlags(&st[k], cudaStreamNonBlocking), "stream");
        check(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming), "event");
        check(cudaStreamWaitEvent(st[k], start, 0), "stream wait");
        check(ws_alloc(reinterpret_cast<void**>(&slot[k].q), sizeof(float) * 3 * chunk, st[k]), "alloc");
        if (out_point) check(ws_alloc(reinterpret_cast<void**>(&slot[k].p), sizeof(float) * 3 * chunk, st[k]), "alloc");
        if (out_dist) check(ws_alloc(reinterpret_cast<void**>(&slot[k].d), sizeof(float) * chunk, st[k]), "alloc");
        if (out_tri) check(ws_alloc(reinterpret_cast<void**>(&slot[k].t), sizeof(int32_t) * chunk, st[k]), "alloc");
        if (out_bary) check(ws_alloc(reinterpret_cast<void**>(&slot[k].b), sizeof(float) * 2 * chunk, st[k]), "alloc");
        check(ws_alloc(&slot[k].ws, wsb, st[k]), "alloc");
    }
    for (int64_t c = 0; c < nchunks && result == CP_SUCCESS; ++c) {
        const int k = (int)(c % nslots);
        const int64_t off = c * chunk;
        const int64_t cnt = (nq - off) < chunk ? (nq - off) : chunk;
        Slot& sl = slot[k];
        check(cudaMemcpyAsync(sl.q, queries + 3 * off, sizeof(float) * 3 * cnt, cudaMemcpyHostToDevice, st[k]), "H2D");
        if (result != CP_SUCCESS) break;
        cudaError_t e = bvh_query(b, sl.q, cnt, nullptr, qp, sl.p, sl.d, sl.t, sl.b, sl.ws, wsb, st[k]);
        if (!check(e, "query")) break;
        if (out_point) check(cudaMemcpyAsync(out_point + 3 * off, sl.p, sizeof(float) * 3 * cnt, cudaMemcpyDeviceToHost, st[k]), "D2H");
        if (out_dist) check(cudaMemcpyAsync(out_dist + off, sl.d, sizeof(float) * cnt, cudaMemcpyDeviceToHost, st[k]), "D2H");
        if (out_tri) check(cudaMemcpyAsync(out_tri + off, sl.t, sizeof(int32_t) * cnt, cudaMemcpyDeviceToHost, st[k]), "D2H");
        if (out_bary) check(cudaMemcpyAsync(out_bary + 2 * off, sl.b, sizeof(float) * 2 * cnt, cudaMemcpyDeviceToHost, st[k]), "D2H");
    }
    for (int k = 0; k < nslots; ++k) {
        if (!st[k]) continue;
        void* ptrs[6] = {slot[k].q, slot[k].p, slot[k].d, slot[k].t, slot[k].b, slot[k].ws};
        for (void* p : ptrs)
            if (p) cudaFreeAsync(p, st[k]);
        if (done[k]) {
            cudaEventRecord(done[k], st[k]);
            cudaStreamWaitEvent(user, done[k], 0);
        }
    }
    check(cudaStreamSynchronize(user), "synchronise");
    for (int k = 0; k < nslots; ++k) {
        if (st[k]) cudaStreamDestroy(st[k]);
        if (done[k]) cudaEventDestroy(done[k]);
    }
    if (start) cudaEventDestroy(start);
    return result;
}

// Pinned (page-locked) host memory, or memory the device maps directly.
static bool is_pinned_host(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

CP_API cp_status cp_query_host_async(const cp_mesh* m, const float* queries, int64_t nq,
                                     const cp_query_opts* opts, float* out_point, float* out_dist,
                                     int32_t* out_tri, float* out_bary, cp_stream_t stream) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (nq < 0) return fail(CP_ERROR_INVALID_VALUE, "negative query count");
    if (nq > INT32_MAX) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^31 - 1 queries in one call");
    if (nq == 0) return CP_SUCCESS;
    if (!queries) return fail(CP_ERROR_INVALID_VALUE, "queries is NULL");
    const void* host[5] = {queries, out_point, out_dist, out_tri, out_bary};
    for (const void* p : host)
        if (p && !is_pinned_host(p))
            return fail(CP_ERROR_INVALID_VALUE,
                        "cp_query_host_async: every host array must be pinned (cudaHostAlloc / cudaHostRegister)");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    const Bvh& b = m->bvh;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t wsb = query_workspace_bytes(b, nq, qp);
    void* buf[6] = {};  // queries, point, dist, tri, bary, workspace
    const size_t bytes[6] = {sizeof(float) * 3 * nq, out_point ? sizeof(float) * 3 * nq : 0,
                             out_dist ? sizeof(float) * nq : 0, out_tri ? sizeof(int32_t) * nq : 0,
                             out_bary ? sizeof(float) * 2 * nq : 0, wsb};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 6 && e == cudaSuccess; ++k)
        if (bytes[k]) e = ws_alloc(&buf[k], bytes[k], st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf[0], queries, bytes[0], cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = bvh_query(b, static_cast<float*>(buf[0]), nq, nullptr, qp, static_cast<float*>(buf[1]),
                      static_cast<float*>(buf[2]), static_cast<int32_t*>(buf[3]), static_cast<float*>(buf[4]), buf[5],
                      wsb, st);
    void* outs[4] = {out_point, out_dist, out_tri, out_bary};
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
        if (outs[k]) e = cudaMemcpyAsync(outs[k], buf[k + 1], bytes[k + 1], cudaMemcpyDeviceToHost, st);
    for (void* p : buf)
        if (p) cudaFreeAsync(p, st);
    if (e != cudaSuccess) return cuda_fail(e, "cp_query_host_async");
    return CP_SUCCESS;
}

CP_API cp_status cp_backward(const cp_mesh* m, const float* queries, const int32_t* tri,
                             const float* bary, const float* grad_dist, int64_t nq,
                             float* grad_queries, float* grad_verts, cp_stream_t stream) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (nq < 0) return fail(CP_ERROR_INVALID_VALUE, "negative query count");
    if (nq == 0) return CP_SUCCESS;
    if (!queries || !tri || !grad_dist)
        return fail(CP_ERROR_INVALID_VALUE, "queries, tri and grad_dist are required");
    CP_CUDA(bvh_backward(m->bvh, queries, tri, bary, grad_dist, nq, grad_queries, grad_verts,
                         reinterpret_cast<cudaStream_t>(stream)),
            "backward");
    return CP_SUCCESS;
}

// ---- rays ------------------------------------------------------------------

CP_API void cp_ray_opts_default(cp_ray_opts* o) {
    if (!o) return;
    o->tmin = 0.0f;
    o->tmax = INFINITY;
    o->det_epsilon = 0.0f;
    o->any_hit = 0;
    o->sort_rays = 1;
    o->block_size = 256;
}

static cp_status to_ray_params(const cp_ray_opts* o, RayParams* r) {
    cp_ray_opts d;
    cp_ray_opts_default(&d);
    if (!o) o = &d;
    const int block = o->block_size ? o->block_size : d.block_size;
    if (block < 32 || block > 256 || block % 32)
        return fail(CP_ERROR_INVALID_VALUE, "block_size must be a multiple of 32 in 32..256");
    if (std::isnan(o->tmin) || std::isnan(o->tmax) || !(o->tmin <= o->tmax))
        return fail(CP_ERROR_INVALID_VALUE, "tmin and tmax must satisfy tmin <= tmax");
    if (!(o->det_epsilon >= 0.0f) || std::isinf(o->det_epsilon))
        return fail(CP_ERROR_INVALID_VALUE, "det_epsilon must be finite and >= 0");
    r->tmin = o->tmin;
    r->tmax = o->tmax;
    r->det_eps = o->det_epsilon;
    r->any_hit = o->any_hit ? 1 : 0;
    r->sort = o->sort_rays ? 1 : 0;
    r->block = block;
    return CP_SUCCESS;
}

CP_API cp_status cp_ray_workspace_size(const cp_mesh* m, int64_t n, const cp_ray_opts* opts,
                                       size_t* bytes) {
    if (!m || !bytes) return fail(CP_ERROR_INVALID_VALUE, "mesh or bytes is NULL");
    if (n < 0) return fail(CP_ERROR_INVALID_VALUE, "negative ray count");
    RayParams rp;
    cp_status s = to_ray_params(opts, &rp);
    if (s != CP_SUCCESS) return s;
    QueryParams qp;
    qp.sort = rp.sort;
    *bytes = query_workspace_bytes(m->bvh, n, qp);
    return CP_SUCCESS;
}

CP_API cp_status cp_ray_query(const cp_mesh* m, const float* origins, const float* directions,
                              const float* tmax_per_ray, int64_t n, const cp_ray_opts* opts,
                              float* out_t, int32_t* out_tri, float* out_uv, void* workspace,
                              size_t ws_bytes, cp_stream_t stream) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    if (n < 0) return fail(CP_ERROR_INVALID_VALUE, "negative ray count");
    if (n > INT32_MAX) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^31 - 1 rays in one call");
    if (n == 0) return CP_SUCCESS;
    if (!origins || !directions) return fail(CP_ERROR_INVALID_VALUE, "origins and directions are required");
    RayParams rp;
    cp_status s = to_ray_params(opts, &rp);
    if (s != CP_SUCCESS) return s;
    QueryParams qp;
    qp.sort = rp.sort;
    const size_t need = query_workspace_bytes(m->bvh, n, qp);
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    void* own = nullptr;
    if (!workspace) {
        CP_CUDA(ws_alloc(&own, need, st), "workspace allocation");
        workspace = own;
        ws_bytes = need;
    } else if (ws_bytes < need) {
        return fail(CP_ERROR_SCRATCH_TOO_SMALL, "workspace smaller than cp_ray_workspace_size()");
    }
    cudaError_t e = bvh_ray_query(m->bvh, origins, directions, tmax_per_ray, n, nullptr, rp, out_t,
                                  out_tri, out_uv, workspace, ws_bytes, st);
    if (own) cudaFreeAsync(own, st);
    if (e != cudaSuccess) return cuda_fail(e, "ray query");
    return CP_SUCCESS;
}

// ---- batches ---------------------------------------------------------------

CP_API cp_status cp_batch_create(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                                 const int64_t* tri_offsets, int32_t nmeshes,
                                 const cp_build_opts* opts, cp_stream_t stream, cp_batch** out) {
    return cp_batch_create_leaves(verts, vert_offsets, tris, tri_offsets, nmeshes, nullptr, opts, stream, out);
}

CP_API cp_status cp_batch_create_leaves(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                                        const int64_t* tri_offsets, int32_t nmeshes, const int32_t* leaf_sizes,
                                        const cp_build_opts* opts, cp_stream_t stream, cp_batch** out) {
    if (!out) return fail(CP_ERROR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (!verts || !tris || !vert_offsets || !tri_offsets)
        return fail(CP_ERROR_INVALID_VALUE, "NULL array");
    if (nmeshes <= 0) return fail(CP_ERROR_INVALID_VALUE, "nmeshes must be positive");
    if (nmeshes > (1 << 20)) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^20 meshes");
    std::vector<int64_t> voff(vert_offsets, vert_offsets + nmeshes + 1);
    std::vector<int64_t> toff(tri_offsets, tri_offsets + nmeshes + 1);
    if (voff[0] != 0 || toff[0] != 0) return fail(CP_ERROR_INVALID_VALUE, "offsets must start at 0");
    for (int32_t i = 0; i < nmeshes; ++i) {
        if (toff[i + 1] <= toff[i]) return fail(CP_ERROR_INVALID_VALUE, "every mesh needs at least one triangle");
        if (voff[i + 1] <= voff[i]) return fail(CP_ERROR_INVALID_VALUE, "every mesh needs at least one vertex");
    }
    if (toff.back() > kMaxTriangles) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^27 - 1 triangles");
    cp_status s = require_gpu();
    if (s != CP_SUCCESS) return s;
    cp_batch* bt = new (std::nothrow) cp_batch();
    if (!bt) return fail(CP_ERROR_OUT_OF_MEMORY, "host allocation of the handle failed");
    s = build_common(bt->bvh, verts, 12, tris, voff, toff, opts, stream, leaf_sizes);
    if (s != CP_SUCCESS) {
        delete bt;
        return s;
    }
    if (cudaMalloc(&bt->d_qoff, sizeof(int64_t) * (nmeshes + 1)) != cudaSuccess) {
        bvh_free(bt->bvh);
        delete bt;
        return fail(CP_ERROR_OUT_OF_MEMORY, "query offsets");
    }
    *out = bt;
    return CP_SUCCESS;
}

CP_API cp_status cp_batch_destroy(cp_batch* bt) {
    if (!bt) return CP_SUCCESS;
    if (bt->exec) cudaGraphExecDestroy(bt->exec);
    if (bt->capture_stream) cudaStreamDestroy(bt->capture_stream);
    if (bt->d_qoff) cudaFree(bt->d_qoff);
    bvh_free(bt->bvh);
    delete bt;
    return CP_SUCCESS;
}

CP_API cp_status cp_batch_save(const cp_batch* bt, const char* path) {
    if (!bt || !path) return fail(CP_ERROR_INVALID_VALUE, "batch or path is NULL");
    std::string why;
    cudaError_t e = bvh_save(const_cast<cp_batch*>(bt)->bvh, path, &why);
    if (!why.empty()) return fail(CP_ERROR_INVALID_VALUE, "cp_batch_save: " + why);
    if (e != cudaSuccess) return cuda_fail(e, "cp_batch_save");
    return CP_SUCCESS;
}

CP_API cp_status cp_batch_load(const char* path, cp_stream_t stream, cp_batch** out) {
    if (!out || !path) return fail(CP_ERROR_INVALID_VALUE, "path or out is NULL");
    *out = nullptr;
    cp_batch* bt = new (std::nothrow) cp_batch();
    if (!bt) return fail(CP_ERROR_OUT_OF_MEMORY, "host allocation of the handle failed");
    std::string why;
    bool bad = false;
    cudaError_t e = bvh_load(bt->bvh, path, reinterpret_cast<cudaStream_t>(stream), &why, &bad);
    if (e == cudaSuccess && !bad) {
        if (alloc_fault()) e = cudaErrorMemoryAllocation;
        else e = cudaMalloc(&bt->d_qoff, sizeof(int64_t) * (bt->bvh.nmeshes + 1));
    }
    if (bad || e != cudaSuccess) {
        if (bt->d_qoff) cudaFree(bt->d_qoff);
        bt->d_qoff = nullptr;
        bvh_free(bt->bvh);
        delete bt;
        if (bad) return fail(CP_ERROR_INVALID_VALUE, std::string("cp_batch_load: ") + path + ": " + why);
        return cuda_fail(e, "cp_batch_load");
    }
    *out = bt;
    return CP_SUCCESS;
}

CP_API cp_status cp_batch_info(const cp_batch* bt, int32_t* nmeshes, int64_t* num_wide,
                               int64_t* num_tris, int32_t* stack_bound) {
    if (!bt) return fail(CP_ERROR_INVALID_VALUE, "batch is NULL");
    if (nmeshes) *nmeshes = bt->bvh.nmeshes;
    if (num_wide) *num_wide = bt->bvh.num_wide;
    if (num_tris) *num_tris = bt->bvh.nt;
    if (stack_bound) *stack_bound = bt->bvh.stack_bound;
    return CP_SUCCESS;
}

CP_API cp_status cp_batch_query_workspace_size(const cp_batch* bt, int64_t nq,
                                               const cp_query_opts* opts, size_t* bytes) {
    if (!bt || !bytes) return fail(CP_ERROR_INVALID_VALUE, "batch or bytes is NULL");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    *bytes = query_workspace_bytes(bt->bvh, nq, qp);
    return CP_SUCCESS;
}

CP_API cp_status cp_batch_query(cp_batch* bt, const float* queries, const int64_t* q_offsets,
                                const cp_query_opts* opts, float* out_point, float* out_dist,
                                int32_t* out_tri, float* out_bary, void* workspace,
                                size_t ws_bytes, int32_t use_graph, cp_stream_t stream) {
    if (!bt || !q_offsets) return fail(CP_ERROR_INVALID_VALUE, "batch or q_offsets is NULL");
    const int nm = bt->bvh.nmeshes;
    if (q_offsets[0] != 0) return fail(CP_ERROR_INVALID_VALUE, "q_offsets must start at 0");
    for (int i = 0; i < nm; ++i)
        if (q_offsets[i + 1] < q_offsets[i]) return fail(CP_ERROR_INVALID_VALUE, "q_offsets must not decrease");
    const int64_t nq = q_offsets[nm];
    if (nq > INT32_MAX) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^31 - 1 queries in one call");
    if (nq == 0) return CP_SUCCESS;
    if (!queries) return fail(CP_ERROR_INVALID_VALUE, "queries is NULL");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const bool changed = bt->h_qoff.size() != (size_t)(nm + 1) ||
                         std::memcmp(bt->h_qoff.data(), q_offsets, sizeof(int64_t) * (nm + 1)) != 0;
    if (changed) {
        bt->h_qoff.assign(q_offsets, q_offsets + nm + 1);
        CP_CUDA(cudaMemcpyAsync(bt->d_qoff, bt->h_qoff.data(), sizeof(int64_t) * (nm + 1),
                                cudaMemcpyHostToDevice, st),
                "query offsets upload");
        CP_CUDA(cudaStreamSynchronize(st), "query offsets upload");
    }
    if (!use_graph)
        return query_impl(bt->bvh, queries, nq, bt->d_qoff, qp, out_point, out_dist, out_tri,
                          out_bary, workspace, ws_bytes, st);
    if (!workspace) return fail(CP_ERROR_INVALID_VALUE, "graph mode needs a caller workspace");
    const size_t need = query_workspace_bytes(bt->bvh, nq, qp);
    if (ws_bytes < need) return fail(CP_ERROR_SCRATCH_TOO_SMALL, "workspace smaller than cp_batch_query_workspace_size()");
    std::vector<uintptr_t> key = {(uintptr_t)queries, (uintptr_t)out_point, (uintptr_t)out_dist,
                                  (uintptr_t)out_tri, (uintptr_t)out_bary, (uintptr_t)workspace,
                                  (uintptr_t)qp.block, (uintptr_t)qp.sort, (uintptr_t)qp.blocks_per_sm,
                                  (uintptr_t)qp.short_stack, (uintptr_t)qp.traversal, (uintptr_t)qp.seed_chunk,
                                  (uintptr_t)nq};
    for (int i = 0; i <= nm; ++i) key.push_back((uintptr_t)q_offsets[i]);
    if (!bt->exec || key != bt->graph_key) {
        if (bt->exec) {
            cudaGraphExecDestroy(bt->exec);
            bt->exec = nullptr;
        }
        // Capture on a private stream: the caller's stream may be the legacy
        // default stream, which cannot be captured.  Captured work does not
        // run, so the private stream needs no ordering with the caller's.
        if (!bt->capture_stream)
            CP_CUDA(cudaStreamCreateWithFlags(&bt->capture_stream, cudaStreamNonBlocking), "graph capture");
        cudaStream_t cs = bt->capture_stream;
        CP_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "graph capture");
        cudaError_t e = bvh_query(bt->bvh, queries, nq, bt->d_qoff, qp, out_point, out_dist, out_tri,
                                  out_bary, workspace, ws_bytes, cs);
        cudaGraph_t graph = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
        if (e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return cuda_fail(e, "graph capture");
        }
        if (e2 != cudaSuccess) return cuda_fail(e2, "graph capture");
        e = cudaGraphInstantiate(&bt->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            bt->exec = nullptr;
            return cuda_fail(e, "graph instantiate");
        }
        bt->graph_key = key;
    }
    CP_CUDA(cudaGraphLaunch(bt->exec, st), "graph launch");
    return CP_SUCCESS;
}

}  // extern "C"

// ---- instanced scenes ------------------------------------------------------

struct cp_scene {
    Bvh top;                    // over the instances' proxies, one per instance
    Bvh baked;                  // world-space copies of the general-affine instances
    bool has_baked = false;
    bool valid = false;         // false while a build is under way or after one failed
    const cp_batch* batch = nullptr;
    int32_t n = 0;
    int32_t n_baked = 0;
    int32_t* d_inst_mesh = nullptr;
    int32_t* d_baked = nullptr; // n: baked copy of each instance, or -1
    float* d_fwd = nullptr;     // n x 12 world <- object
    float* d_inv = nullptr;     // n x 12 object <- world
    float* d_s2 = nullptr;      // n x 2: squared scale, lower bound of the squared stretch
    std::vector<int32_t> h_baked;  // host copy of d_baked (which instances have world-space copies)
    std::vector<int64_t> bake_off; // triangle offsets of the baked copies (n_baked + 1)
};

namespace {

// Per instance: the matrix as given and whether it is a similarity (M^T M =
// s^2 I within 1e-5 s^2, invertible) — such instances are walked in object
// space with the inverse (FP64, rounded once), s^2 for ranking and a
// Gershgorin lower bound of M^T M's eigenvalues for pruning; every other
// affine matrix (non-uniform scale, shear, singular) is baked.  Refuses
// non-finite matrices.
cp_status instance_frames(const float* T, int32_t n, std::vector<float>& fwd, std::vector<float>& inv,
                          std::vector<float>& s2, std::vector<int32_t>& baked) {
    fwd.assign(T, T + (size_t)12 * n);
    inv.assign((size_t)12 * n, 0.0f);
    s2.assign((size_t)2 * n, 1.0f);
    baked.assign((size_t)n, -1);
    int32_t nb = 0;
    for (int32_t i = 0; i < n; ++i) {
        const float* t = T + (size_t)12 * i;
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(t[k]))
                return fail(CP_ERROR_INVALID_VALUE, "instance " + std::to_string(i) + ": non-finite transform");
        double M[3][3], tr[3];
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) M[r][c] = t[4 * r + c];
            tr[r] = t[4 * r + 3];
        }
        double G[3][3];
        for (int j = 0; j < 3; ++j)
            for (int k = 0; k < 3; ++k) G[j][k] = M[0][j] * M[0][k] + M[1][j] * M[1][k] + M[2][j] * M[2][k];
        const double s = (G[0][0] + G[1][1] + G[2][2]) / 3.0;
        double dev = 0.0, lo = INFINITY;
        for (int j = 0; j < 3; ++j) {
            double off = 0.0;
            for (int k = 0; k < 3; ++k) {
                dev = std::max(dev, std::fabs(G[j][k] - (j == k ? s : 0.0)));
                if (k != j) off += std::fabs(G[j][k]);
            }
            lo = std::min(lo, G[j][j] - off);
        }
        const double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                           M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                           M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
        const bool similarity = s > 1e-30 && std::isfinite(s) && dev <= 1e-5 * s && det != 0.0 && lo > 0.0;
        if (!similarity) {
            baked[i] = nb++;
            continue;
        }
        double A[3][3];  // inverse by the adjugate
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                const int r1 = (c + 1) % 3, r2 = (c + 2) % 3, c1 = (r + 1) % 3, c2 = (r + 2) % 3;
                A[r][c] = (M[r1][c1] * M[r2][c2] - M[r1][c2] * M[r2][c1]) / det;
            }
        float* o = inv.data() + (size_t)12 * i;
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) o[4 * r + c] = (float)A[r][c];
            o[4 * r + 3] = (float)-(A[r][0] * tr[0] + A[r][1] * tr[1] + A[r][2] * tr[2]);
        }
        s2[2 * i] = (float)s;
        s2[2 * i + 1] = (float)(lo * (1.0 - 1e-6));
    }
    return CP_SUCCESS;
}

// Frames to the device, world-space copies of the general-affine instances,
// proxies, top-level build.  Every level has the batch's branching factor;
// the top level holds one instance per leaf, the baked copies the batch's
// leaf size.
cp_status scene_build(cp_scene* sc, const float* T, cudaStream_t st) {
    std::vector<float> fwd, inv, s2;
    std::vector<int32_t> baked;
    cp_status s = instance_frames(T, sc->n, fwd, inv, s2, baked);
    if (s != CP_SUCCESS) return s;  // nothing changed: the scene stays as it was
    sc->valid = false;              // from here on a failure leaves it unusable
    const size_t n = (size_t)sc->n;
    const Bvh& bottom = sc->batch->bvh;
    CP_CUDA(cudaMemcpyAsync(sc->d_fwd, fwd.data(), sizeof(float) * 12 * n, cudaMemcpyHostToDevice, st), "scene upload");
    CP_CUDA(cudaMemcpyAsync(sc->d_inv, inv.data(), sizeof(float) * 12 * n, cudaMemcpyHostToDevice, st), "scene upload");
    CP_CUDA(cudaMemcpyAsync(sc->d_s2, s2.data(), sizeof(float) * 2 * n, cudaMemcpyHostToDevice, st), "scene upload");
    CP_CUDA(cudaMemcpyAsync(sc->d_baked, baked.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st),
            "scene upload");
    // world-space copies, one mesh each, in the mesh's local triangle order
    std::vector<int32_t> list;
    std::vector<int64_t> out_off(1, 0), voff(1, 0);
    std::vector<int32_t> h_mesh(n);
    CP_CUDA(cudaMemcpyAsync(h_mesh.data(), sc->d_inst_mesh, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st),
            "scene upload");
    CP_CUDA(cudaStreamSynchronize(st), "scene upload");
    for (size_t i = 0; i < n; ++i) {
        if (baked[i] < 0) continue;
        const int m = h_mesh[i];
        const int64_t nt = bottom.h_toff[m + 1] - bottom.h_toff[m];
        list.push_back((int32_t)i);
        out_off.push_back(out_off.back() + nt);
        voff.push_back(3 * out_off.back());
    }
    const int64_t total = out_off.back();
    if (total > kMaxTriangles) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^27 - 1 baked triangles");
    sc->h_baked = baked;
    sc->bake_off = out_off;
    bvh_free(sc->baked);
    sc->baked = Bvh();
    sc->has_baked = false;
    sc->n_baked = (int32_t)list.size();
    if (total > 0) {
        float* verts = nullptr;
        int32_t *tris = nullptr, *d_list = nullptr;
        int64_t* d_off = nullptr;
        cudaError_t e = cudaMalloc(&verts, sizeof(float) * 9 * total);
        if (e == cudaSuccess) e = cudaMalloc(&tris, sizeof(int32_t) * 3 * total);
        if (e == cudaSuccess) e = cudaMalloc(&d_list, sizeof(int32_t) * list.size());
        if (e == cudaSuccess) e = cudaMalloc(&d_off, sizeof(int64_t) * out_off.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_list, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_off, out_off.data(), sizeof(int64_t) * out_off.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = instance_bake(bottom, d_list, sc->d_inst_mesh, sc->d_fwd, d_off, (int32_t)list.size(), total, verts,
                              tris, st);
        cp_status bs = CP_SUCCESS;
        if (e == cudaSuccess) {
            cp_build_opts bo;
            cp_build_opts_default(&bo);
            bo.branching = bottom.p.K;
            bo.leaf_size = bottom.p.leaf_size;
            std::vector<int64_t> toff(out_off.begin(), out_off.end());
            bs = build_common(sc->baked, verts, 12, tris, voff, toff, &bo, st);
        }
        cudaError_t e2 = cudaStreamSynchronize(st);
        cudaFree(verts);
        cudaFree(tris);
        cudaFree(d_list);
        cudaFree(d_off);
        if (e != cudaSuccess) return cuda_fail(e, "scene bake");
        if (bs != CP_SUCCESS) return bs;
        if (e2 != cudaSuccess) return cuda_fail(e2, "scene bake");
        sc->has_baked = true;
    }
    float* verts = nullptr;
    int32_t* tris = nullptr;
    if (cudaMalloc(&verts, sizeof(float) * 6 * n) != cudaSuccess ||
        cudaMalloc(&tris, sizeof(int32_t) * 3 * n) != cudaSuccess) {
        cudaFree(verts);
        return fail(CP_ERROR_OUT_OF_MEMORY, "scene proxies");
    }
    cudaError_t e = instance_proxies(bottom, sc->d_inst_mesh, sc->d_fwd, sc->n, verts, tris, st);
    if (e == cudaSuccess) {
        bvh_free(sc->top);
        sc->top = Bvh();
        cp_build_opts bo;
        cp_build_opts_default(&bo);
        bo.branching = bottom.p.K;
        bo.leaf_size = 1;
        s = build_common(sc->top, verts, 12, tris, {0, (int64_t)(2 * n)}, {0, (int64_t)n}, &bo, st);
    }
    cudaError_t e2 = cudaStreamSynchronize(st);
    cudaFree(verts);
    cudaFree(tris);
    if (e != cudaSuccess) return cuda_fail(e, "scene proxies");
    if (s != CP_SUCCESS) return s;
    if (e2 != cudaSuccess) return cuda_fail(e2, "scene build");
    sc->valid = true;
    return CP_SUCCESS;
}

// New transforms with the scene's instance kinds unchanged: the top level and
// the world-space copies keep their topology; the copies are re-baked, the
// proxies recomputed, and both trees refit bottom-up (boxes and triangle
// records), as a TLAS update does instead of a rebuild.
cp_status scene_refit(cp_scene* sc, const float* T, cudaStream_t st) {
    std::vector<float> fwd, inv, s2;
    std::vector<int32_t> baked;
    cp_status s = instance_frames(T, sc->n, fwd, inv, s2, baked);
    if (s != CP_SUCCESS) return s;  // nothing changed: the scene stays as it was
    if (!sc->valid || baked != sc->h_baked) return scene_build(sc, T, st);  // kinds changed: rebuild
    sc->valid = false;
    const size_t n = (size_t)sc->n;
    const Bvh& bottom = sc->batch->bvh;
    CP_CUDA(cudaMemcpyAsync(sc->d_fwd, fwd.data(), sizeof(float) * 12 * n, cudaMemcpyHostToDevice, st), "scene upload");
    CP_CUDA(cudaMemcpyAsync(sc->d_inv, inv.data(), sizeof(float) * 12 * n, cudaMemcpyHostToDevice, st), "scene upload");
    CP_CUDA(cudaMemcpyAsync(sc->d_s2, s2.data(), sizeof(float) * 2 * n, cudaMemcpyHostToDevice, st), "scene upload");
    cudaError_t e = cudaSuccess;
    if (sc->has_baked) {
        std::vector<int32_t> list;
        for (size_t i = 0; i < n; ++i)
            if (baked[i] >= 0) list.push_back((int32_t)i);
        const int64_t total = sc->bake_off.back();
        float* verts = nullptr;
        int32_t *tris = nullptr, *d_list = nullptr;
        int64_t* d_off = nullptr;
        e = cudaMalloc(&verts, sizeof(float) * 9 * total);
        if (e == cudaSuccess) e = cudaMalloc(&tris, sizeof(int32_t) * 3 * total);
        if (e == cudaSuccess) e = cudaMalloc(&d_list, sizeof(int32_t) * list.size());
        if (e == cudaSuccess) e = cudaMalloc(&d_off, sizeof(int64_t) * sc->bake_off.size());
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_list, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_off, sc->bake_off.data(), sizeof(int64_t) * sc->bake_off.size(),
                                cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = instance_bake(bottom, d_list, sc->d_inst_mesh, sc->d_fwd, d_off, (int32_t)list.size(), total, verts,
                              tris, st);
        if (e == cudaSuccess) e = bvh_refit(sc->baked, verts, 3, st);
        cudaError_t e2 = cudaStreamSynchronize(st);
        cudaFree(verts);
        cudaFree(tris);
        cudaFree(d_list);
        cudaFree(d_off);
        if (e == cudaSuccess) e = e2;
        if (e != cudaSuccess) return cuda_fail(e, "scene refit (copies)");
    }
    float* verts = nullptr;
    int32_t* tris = nullptr;
    if (cudaMalloc(&verts, sizeof(float) * 6 * n) != cudaSuccess ||
        cudaMalloc(&tris, sizeof(int32_t) * 3 * n) != cudaSuccess) {
        cudaFree(verts);
        return fail(CP_ERROR_OUT_OF_MEMORY, "scene proxies");
    }
    e = instance_proxies(bottom, sc->d_inst_mesh, sc->d_fwd, sc->n, verts, tris, st);
    if (e == cudaSuccess) e = bvh_refit(sc->top, verts, 3, st);
    cudaError_t e2 = cudaStreamSynchronize(st);
    cudaFree(verts);
    cudaFree(tris);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_fail(e, "scene refit");
    sc->valid = true;
    return CP_SUCCESS;
}

void scene_free(cp_scene* sc) {
    cudaFree(sc->d_inst_mesh);
    cudaFree(sc->d_baked);
    cudaFree(sc->d_fwd);
    cudaFree(sc->d_inv);
    cudaFree(sc->d_s2);
    bvh_free(sc->top);
    bvh_free(sc->baked);
    delete sc;
}

}  // namespace

extern "C" {

CP_API cp_status cp_scene_create(const cp_batch* batch, const int32_t* instance_mesh,
                                 const float* instance_transform, int32_t n_instances,
                                 cp_stream_t stream, cp_scene** out) {
    if (!out) return fail(CP_ERROR_INVALID_VALUE, "out is NULL");
    *out = nullptr;
    if (!batch || !instance_mesh || !instance_transform) return fail(CP_ERROR_INVALID_VALUE, "NULL argument");
    if (n_instances <= 0) return fail(CP_ERROR_INVALID_VALUE, "a scene needs at least one instance");
    if (n_instances > kMaxTriangles) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^27 - 1 instances");
    for (int32_t i = 0; i < n_instances; ++i)
        if (instance_mesh[i] < 0 || instance_mesh[i] >= batch->bvh.nmeshes)
            return fail(CP_ERROR_INVALID_VALUE, "instance " + std::to_string(i) + ": mesh id out of range");
    cp_status s = require_gpu();
    if (s != CP_SUCCESS) return s;
    cp_scene* sc = new (std::nothrow) cp_scene();
    if (!sc) return fail(CP_ERROR_OUT_OF_MEMORY, "host allocation of the handle failed");
    sc->batch = batch;
    sc->n = n_instances;
    const size_t n = (size_t)n_instances;
    if (cudaMalloc(&sc->d_inst_mesh, sizeof(int32_t) * n) != cudaSuccess ||
        cudaMalloc(&sc->d_baked, sizeof(int32_t) * n) != cudaSuccess ||
        cudaMalloc(&sc->d_fwd, sizeof(float) * 12 * n) != cudaSuccess ||
        cudaMalloc(&sc->d_inv, sizeof(float) * 12 * n) != cudaSuccess ||
        cudaMalloc(&sc->d_s2, sizeof(float) * 2 * n) != cudaSuccess) {
        scene_free(sc);
        return fail(CP_ERROR_OUT_OF_MEMORY, "scene instance arrays");
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(sc->d_inst_mesh, instance_mesh, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        scene_free(sc);
        return cuda_fail(e, "scene upload");
    }
    s = scene_build(sc, instance_transform, st);
    if (s != CP_SUCCESS) {
        scene_free(sc);
        return s;
    }
    *out = sc;
    return CP_SUCCESS;
}

CP_API cp_status cp_scene_update(cp_scene* scene, const float* instance_transform, cp_stream_t stream) {
    if (!scene || !instance_transform) return fail(CP_ERROR_INVALID_VALUE, "scene or transforms is NULL");
    return scene_build(scene, instance_transform, reinterpret_cast<cudaStream_t>(stream));
}

CP_API cp_status cp_scene_refit(cp_scene* scene, const float* instance_transform, cp_stream_t stream) {
    if (!scene || !instance_transform) return fail(CP_ERROR_INVALID_VALUE, "scene or transforms is NULL");
    return scene_refit(scene, instance_transform, reinterpret_cast<cudaStream_t>(stream));
}

CP_API cp_status cp_scene_destroy(cp_scene* scene) {
    if (scene) scene_free(scene);
    return CP_SUCCESS;
}

CP_API cp_status cp_scene_query_workspace_size(const cp_scene* scene, int64_t nq,
                                               const cp_query_opts* opts, size_t* bytes) {
    if (!scene || !bytes) return fail(CP_ERROR_INVALID_VALUE, "scene or bytes is NULL");
    if (nq < 0) return fail(CP_ERROR_INVALID_VALUE, "negative query count");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    *bytes = query_workspace_bytes(scene->top, nq, qp);
    return CP_SUCCESS;
}

CP_API cp_status cp_scene_query(const cp_scene* scene, const float* queries, int64_t nq,
                                const cp_query_opts* opts, float* out_point, float* out_dist,
                                int32_t* out_instance, int32_t* out_tri, float* out_bary,
                                void* workspace, size_t ws_bytes, cp_stream_t stream) {
    if (!scene) return fail(CP_ERROR_INVALID_VALUE, "scene is NULL");
    if (!scene->valid) return fail(CP_ERROR_INVALID_VALUE, "scene unusable: its last update failed");
    if (nq < 0) return fail(CP_ERROR_INVALID_VALUE, "negative query count");
    if (nq > INT32_MAX) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^31 - 1 queries in one call");
    if (nq == 0) return CP_SUCCESS;
    if (!queries) return fail(CP_ERROR_INVALID_VALUE, "queries is NULL");
    QueryParams qp;
    cp_status s = to_query_params(opts, &qp);
    if (s != CP_SUCCESS) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t need = query_workspace_bytes(scene->top, nq, qp);
    void* own = nullptr;
    if (!workspace) {
        CP_CUDA(ws_alloc(&own, need, st), "workspace allocation");
        workspace = own;
        ws_bytes = need;
    } else if (ws_bytes < need) {
        return fail(CP_ERROR_SCRATCH_TOO_SMALL, "workspace smaller than cp_scene_query_workspace_size()");
    }
    InstanceSet is;
    is.mesh = scene->d_inst_mesh;
    is.baked = scene->d_baked;
    is.inv = scene->d_inv;
    is.fwd = scene->d_fwd;
    is.s2 = scene->d_s2;
    is.baked_bvh = scene->has_baked ? &scene->baked : nullptr;
    cudaError_t e = bvh_instance_query(scene->top, scene->batch->bvh, is, queries, nq, qp.sort != 0, out_point,
                                       out_dist, out_instance, out_tri, out_bary, workspace, ws_bytes, st);
    if (own) cudaFreeAsync(own, st);
    if (e != cudaSuccess) return cuda_fail(e, "scene query");
    return CP_SUCCESS;
}

CP_API cp_status cp_scene_ray_workspace_size(const cp_scene* scene, int64_t n, const cp_ray_opts* opts,
                                             size_t* bytes) {
    if (!scene || !bytes) return fail(CP_ERROR_INVALID_VALUE, "scene or bytes is NULL");
    if (n < 0) return fail(CP_ERROR_INVALID_VALUE, "negative ray count");
    RayParams rp;
    cp_status s = to_ray_params(opts, &rp);
    if (s != CP_SUCCESS) return s;
    QueryParams qp;
    qp.sort = rp.sort;
    *bytes = query_workspace_bytes(scene->top, n, qp);
    return CP_SUCCESS;
}

CP_API cp_status cp_scene_ray_query(const cp_scene* scene, const float* origins, const float* directions,
                                    const float* tmax_per_ray, int64_t n, const cp_ray_opts* opts,
                                    float* out_t, int32_t* out_instance, int32_t* out_tri, float* out_uv,
                                    void* workspace, size_t ws_bytes, cp_stream_t stream) {
    if (!scene) return fail(CP_ERROR_INVALID_VALUE, "scene is NULL");
    if (!scene->valid) return fail(CP_ERROR_INVALID_VALUE, "scene unusable: its last update failed");
    if (n < 0) return fail(CP_ERROR_INVALID_VALUE, "negative ray count");
    if (n > INT32_MAX) return fail(CP_ERROR_NOT_SUPPORTED, "more than 2^31 - 1 rays in one call");
    if (n == 0) return CP_SUCCESS;
    if (!origins || !directions) return fail(CP_ERROR_INVALID_VALUE, "origins or directions is NULL");
    RayParams rp;
    cp_status s = to_ray_params(opts, &rp);
    if (s != CP_SUCCESS) return s;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    QueryParams qp;
    qp.sort = rp.sort;
    const size_t need = query_workspace_bytes(scene->top, n, qp);
    void* own = nullptr;
    if (!workspace) {
        CP_CUDA(ws_alloc(&own, need, st), "workspace allocation");
        workspace = own;
        ws_bytes = need;
    } else if (ws_bytes < need) {
        return fail(CP_ERROR_SCRATCH_TOO_SMALL, "workspace smaller than cp_scene_ray_workspace_size()");
    }
    InstanceSet is;
    is.mesh = scene->d_inst_mesh;
    is.baked = scene->d_baked;
    is.inv = scene->d_inv;
    is.fwd = scene->d_fwd;
    is.s2 = scene->d_s2;
    is.baked_bvh = scene->has_baked ? &scene->baked : nullptr;
    cudaError_t e = scene_ray_query(scene->top, scene->batch->bvh, is, origins, directions, tmax_per_ray, n, rp,
                                    out_t, out_instance, out_tri, out_uv, workspace, ws_bytes, st);
    if (own) cudaFreeAsync(own, st);
    if (e != cudaSuccess) return cuda_fail(e, "scene ray query");
    return CP_SUCCESS;
}

// ---- inspection ------------------------------------------------------------

}  // extern "C"

namespace {

cp_status export_build(const Bvh& b, uint64_t* keys, int32_t* order, int32_t* left, int32_t* right,
                       int32_t* parent, uint8_t* cluster, int32_t* wide_src) {
    const int64_t n = b.nt, nn = 2 * n - 1;
    CP_CUDA(cudaDeviceSynchronize(), "export");
    if (keys) CP_CUDA(cudaMemcpy(keys, b.keys, 8 * n, cudaMemcpyDeviceToHost), "export");
    if (order) CP_CUDA(cudaMemcpy(order, b.order, 4 * n, cudaMemcpyDeviceToHost), "export");
    if (n > 1 && left) CP_CUDA(cudaMemcpy(left, b.left, 4 * (n - 1), cudaMemcpyDeviceToHost), "export");
    if (n > 1 && right) CP_CUDA(cudaMemcpy(right, b.right, 4 * (n - 1), cudaMemcpyDeviceToHost), "export");
    if (parent) CP_CUDA(cudaMemcpy(parent, b.parent, 4 * nn, cudaMemcpyDeviceToHost), "export");
    if (cluster) CP_CUDA(cudaMemcpy(cluster, b.cluster, nn, cudaMemcpyDeviceToHost), "export");
    if (wide_src) CP_CUDA(cudaMemcpy(wide_src, b.wide_src, 4 * b.num_wide, cudaMemcpyDeviceToHost), "export");
    return CP_SUCCESS;
}

cp_status export_wide(const Bvh& b, float* boxes, int32_t* refs, int32_t* counts) {
    const int K = b.p.K;
    const size_t node_bytes = (size_t)32 * K;
    std::vector<unsigned char> h(node_bytes * (size_t)b.num_wide);
    CP_CUDA(cudaDeviceSynchronize(), "export");
    CP_CUDA(cudaMemcpy(h.data(), b.nodes, h.size(), cudaMemcpyDeviceToHost), "export");
    for (int64_t w = 0; w < b.num_wide; ++w) {
        const float* rows = reinterpret_cast<const float*>(h.data() + node_bytes * w);
        const int32_t* child = reinterpret_cast<const int32_t*>(rows + 6 * K);
        for (int s = 0; s < K; ++s) {
            if (boxes)
                for (int r = 0; r < 6; ++r) boxes[(w * 6 + r) * K + s] = rows[r * K + s];
            const bool empty = std::isinf(rows[s]) && rows[s] > 0 && std::isinf(rows[K + s]) && rows[K + s] < 0;
            int32_t ref, cnt;
            if (empty) {
                ref = 0;
                cnt = -1;
            } else if (ref_is_leaf(child[s])) {
                ref = leaf_first(child[s]);
                cnt = leaf_count(child[s]);
            } else {
                ref = child[s];
                cnt = 0;
            }
            if (refs) refs[w * K + s] = ref;
            if (counts) counts[w * K + s] = cnt;
        }
    }
    return CP_SUCCESS;
}

}  // namespace

extern "C" {

CP_API cp_status cp_mesh_export_build(const cp_mesh* m, uint64_t* keys, int32_t* order, int32_t* left,
                                      int32_t* right, int32_t* parent, uint8_t* cluster,
                                      int32_t* wide_src) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    return export_build(m->bvh, keys, order, left, right, parent, cluster, wide_src);
}

CP_API cp_status cp_mesh_export_wide(const cp_mesh* m, float* boxes, int32_t* refs, int32_t* counts) {
    if (!m) return fail(CP_ERROR_INVALID_VALUE, "mesh is NULL");
    return export_wide(m->bvh, boxes, refs, counts);
}

CP_API cp_status cp_batch_export_build(const cp_batch* bt, uint64_t* keys, int32_t* order, int32_t* left,
                                       int32_t* right, int32_t* parent, uint8_t* cluster,
                                       int32_t* wide_src) {
    if (!bt) return fail(CP_ERROR_INVALID_VALUE, "batch is NULL");
    return export_build(bt->bvh, keys, order, left, right, parent, cluster, wide_src);
}

CP_API cp_status cp_batch_export_wide(const cp_batch* bt, float* boxes, int32_t* refs, int32_t* counts) {
    if (!bt) return fail(CP_ERROR_INVALID_VALUE, "batch is NULL");
    return export_wide(bt->bvh, boxes, refs, counts);
}

}  // extern "C"
