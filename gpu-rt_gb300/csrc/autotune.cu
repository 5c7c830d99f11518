// autotune.cu — per-size-class choice of branching, leaf size, block size and
// short-stack depth by timing real builds and queries on the caller's data.
// The reference has no tuner; its only knobs are UI sliders that feed push
// constants (src/gpurt.cpp:283-322, src/vk/rt.h:85-102).  Results are cached
// in a plain text file, one line per (triangle class, query class, branching):
//   <tri_class> <query_class> <branching> <leaf_size> <block_size> <short_stack> <ms> <seed_chunk>
// where a class is floor(log2(count)), short_stack 0 stands for the
// warp-packet traversal and seed_chunk is its packets per claim (1: unseeded;
// a line without the column reads as 1); batches (cp_batch_autotune) add lines of their own,
// marked B, with a leaf size per triangle class.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <algorithm>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cpq.h"

namespace {

struct Entry {
    int cls, qcls, K, leaf, block, stack;
    float ms;
    int seed = 1;  // packet traversal's seed chunk (lines without the column: 1)
};

std::vector<Entry> read_cache(const char* path) {
    std::vector<Entry> out;
    if (!path) return out;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        Entry e;
        if (is >> e.cls >> e.qcls >> e.K >> e.leaf >> e.block >> e.stack >> e.ms) {
            int seed = 1;
            if (is >> seed && seed >= 1 && seed <= 16) e.seed = seed;
            out.push_back(e);
        }
    }
    return out;
}

void write_cache(const char* path, const std::vector<Entry>& es) {
    if (!path) return;
    std::vector<std::string> batch_lines;  // a batch's lines (cp_batch_autotune) stay
    {
        std::ifstream in(path);
        std::string line;
        while (std::getline(in, line))
            if (!line.empty() && line[0] == 'B') batch_lines.push_back(line);
    }
    std::ofstream f(path, std::ios::trunc);
    for (const std::string& l : batch_lines) f << l << '\n';
    for (const Entry& e : es)
        f << e.cls << ' ' << e.qcls << ' ' << e.K << ' ' << e.leaf << ' ' << e.block << ' ' << e.stack
          << ' ' << e.ms << ' ' << e.seed << '\n';
}

}  // namespace

extern "C" CP_API cp_status cp_autotune(const float* verts, int64_t nv, const int32_t* tris,
                                        int64_t nt, const float* queries, int64_t nq,
                                        const char* cache_path, cp_build_opts* best_build,
                                        cp_query_opts* best_query) {
    if (!verts || !tris || !queries || !best_build || !best_query || nv <= 0 || nt <= 0 || nq <= 0)
        return CP_ERROR_INVALID_VALUE;
    const int cls = cp_size_class(nt);
    // query density decides how coherent a warp's queries are, so the query
    // count is part of the size class
    const int qcls = cp_size_class(nq);
    // a branching already set on entry (2, 4 or 8) restricts the search to it
    const int fixed_K = (best_build->branching == 2 || best_build->branching == 4 ||
                         best_build->branching == 8) ? best_build->branching : 0;
    std::vector<Entry> cache = read_cache(cache_path);
    cp_build_opts_default(best_build);
    cp_query_opts_default(best_query);
    for (const Entry& e : cache)
        if (e.cls == cls && e.qcls == qcls && (fixed_K == 0 || e.K == fixed_K)) {
            best_build->branching = e.K;
            best_build->leaf_size = e.leaf;
            best_query->block_size = e.block;
            best_query->short_stack = e.stack ? e.stack : 8;
            best_query->traversal = e.stack ? CP_TRAVERSAL_THREAD : CP_TRAVERSAL_PACKET;
            best_query->seed_chunk = e.stack ? 1 : e.seed;
            return CP_SUCCESS;
        }

    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return CP_ERROR_CUDA;
    float* dist = nullptr;
    int32_t* tri = nullptr;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cp_status result = CP_SUCCESS;
    if (cudaMalloc(&dist, sizeof(float) * nq) != cudaSuccess ||
        cudaMalloc(&tri, sizeof(int32_t) * nq) != cudaSuccess)
        result = CP_ERROR_OUT_OF_MEMORY;
    Entry best = {cls, qcls, fixed_K ? fixed_K : 2, 4, 256, 0, 1e30f};
    const int Ks[3] = {2, 4, 8};
    const int leaves[4] = {1, 2, 4, 8};
    const int blocks[2] = {128, 256};
    const int stacks[3] = {4, 8, 16};
    for (int ki = 0; ki < 3 && result == CP_SUCCESS; ++ki)
        for (int li = 0; li < 4 && result == CP_SUCCESS; ++li) {
            if (fixed_K && Ks[ki] != fixed_K) continue;
            cp_build_opts bo;
            cp_build_opts_default(&bo);
            bo.branching = Ks[ki];
            bo.leaf_size = leaves[li];
            cp_mesh* mesh = nullptr;
            cp_status s = cp_mesh_create(verts, nv, 12, tris, nt, &bo, st, &mesh);
            if (s != CP_SUCCESS) {
                result = s;
                break;
            }
            for (int bi = 0; bi < 2; ++bi)
                for (int si = 0; si < 5; ++si) {
                    // stacks[0..2]: per-thread traversal with that short stack;
                    // si == 3: warp-packet traversal; si == 4: packets seeded
                    // from the packet before (chunks of 4)
                    cp_query_opts qo;
                    cp_query_opts_default(&qo);
                    qo.block_size = blocks[bi];
                    qo.short_stack = si < 3 ? stacks[si] : 8;
                    qo.traversal = si < 3 ? CP_TRAVERSAL_THREAD : CP_TRAVERSAL_PACKET;
                    qo.seed_chunk = si == 4 ? 4 : 1;
                    size_t wsb = 0;
                    cp_query_workspace_size(mesh, nq, &qo, &wsb);
                    void* ws = nullptr;
                    if (cudaMalloc(&ws, wsb) != cudaSuccess) {
                        result = CP_ERROR_OUT_OF_MEMORY;
                        break;
                    }
                    float ms = 1e30f;
                    for (int rep = 0; rep < 3; ++rep) {
                        cudaEventRecord(e0, st);
                        s = cp_query(mesh, queries, nq, &qo, nullptr, dist, tri, nullptr, ws, wsb, st);
                        cudaEventRecord(e1, st);
                        cudaEventSynchronize(e1);
                        float t = 0.0f;
                        cudaEventElapsedTime(&t, e0, e1);
                        if (rep > 0 && t < ms) ms = t;  // first run warms caches and pools
                    }
                    cudaFree(ws);
                    if (s != CP_SUCCESS) {
                        result = s;
                        break;
                    }
                    if (ms < best.ms)
                        best = {cls, qcls, Ks[ki], leaves[li], blocks[bi], si < 3 ? stacks[si] : 0, ms,
                                si == 4 ? 4 : 1};
                }
            cp_mesh_destroy(mesh);
        }
    cudaFree(dist);
    cudaFree(tri);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (result != CP_SUCCESS) return result;
    best_build->branching = best.K;
    best_build->leaf_size = best.leaf;
    best_query->block_size = best.block;
    best_query->short_stack = best.stack ? best.stack : 8;
    best_query->traversal = best.stack ? CP_TRAVERSAL_THREAD : CP_TRAVERSAL_PACKET;
    best_query->seed_chunk = best.stack ? 1 : best.seed;
    if (cache_path) {
        std::vector<Entry> out;
        for (const Entry& e : cache)
            if (e.cls != cls || e.qcls != qcls || e.K != best.K) out.push_back(e);
        out.push_back(best);
        write_cache(cache_path, out);
    }
    return CP_SUCCESS;
}

// ---- batches: a leaf size per size class -----------------------------------
//
// Cache lines for batches: B <tri_class> <query_class> <branching> <leaf_size> <ms>
// (tri_class of the mesh, query_class of its mean queries per mesh).

namespace {

struct BatchEntry {
    int cls, qcls, K, leaf;
    float ms;
};

std::vector<BatchEntry> read_batch_cache(const char* path) {
    std::vector<BatchEntry> out;
    if (!path) return out;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string tag;
        BatchEntry e;
        if (is >> tag && tag == "B" && is >> e.cls >> e.qcls >> e.K >> e.leaf >> e.ms) out.push_back(e);
    }
    return out;
}

// Rewrite the cache file: its single-mesh lines as they were, then `batch`.
void write_batch_cache(const char* path, const std::vector<BatchEntry>& batch) {
    if (!path) return;
    std::vector<std::string> keep;
    {
        std::ifstream f(path);
        std::string line;
        while (std::getline(f, line))
            if (!line.empty() && line[0] != 'B') keep.push_back(line);
    }
    std::ofstream f(path, std::ios::trunc);
    for (const std::string& l : keep) f << l << '\n';
    for (const BatchEntry& e : batch)
        f << "B " << e.cls << ' ' << e.qcls << ' ' << e.K << ' ' << e.leaf << ' ' << e.ms << '\n';
}

}  // namespace

namespace {

// Query time (ms, best of 3 after a warm-up) of the whole batch built with
// the given per-mesh leaf sizes.
cp_status time_batch(const float* verts, const int64_t* voff, const int32_t* tris, const int64_t* toff,
                     int32_t nmeshes, const float* queries, const int64_t* qoff, int32_t branching,
                     const std::vector<int32_t>& leaves, float* dist, cudaStream_t st, cudaEvent_t e0,
                     cudaEvent_t e1, float* ms_out) {
    cp_build_opts bo;
    cp_build_opts_default(&bo);
    bo.branching = branching;
    cp_batch* b = nullptr;
    cp_status s = cp_batch_create_leaves(verts, voff, tris, toff, nmeshes, leaves.data(), &bo, st, &b);
    if (s != CP_SUCCESS) return s;
    cp_query_opts qo;
    cp_query_opts_default(&qo);
    const int64_t nq = qoff[nmeshes];
    size_t wsb = 0;
    cp_batch_query_workspace_size(b, nq, &qo, &wsb);
    void* ws = nullptr;
    if (cudaMalloc(&ws, wsb) != cudaSuccess) {
        cp_batch_destroy(b);
        return CP_ERROR_OUT_OF_MEMORY;
    }
    float ms = 1e30f;
    for (int rep = 0; rep < 4 && s == CP_SUCCESS; ++rep) {
        cudaEventRecord(e0, st);
        s = cp_batch_query(b, queries, qoff, &qo, nullptr, dist, nullptr, nullptr, ws, wsb, 0, st);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        if (rep > 0 && t < ms) ms = t;  // the first run warms caches
    }
    cudaFree(ws);
    cp_batch_destroy(b);
    *ms_out = ms;
    return s;
}

}  // namespace

extern "C" CP_API cp_status cp_batch_autotune(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                                              const int64_t* tri_offsets, int32_t nmeshes, const float* queries,
                                              const int64_t* q_offsets, int32_t branching, const char* cache_path,
                                              int32_t* leaf_sizes, cp_query_opts* best_query) {
    if (!verts || !vert_offsets || !tris || !tri_offsets || !queries || !q_offsets || !leaf_sizes || !best_query ||
        nmeshes <= 0)
        return CP_ERROR_INVALID_VALUE;
    if (branching != 2 && branching != 4 && branching != 8) return CP_ERROR_INVALID_VALUE;
    cp_query_opts_default(best_query);
    // size classes of the meshes, and each class's mean queries per mesh
    std::vector<int> cls(nmeshes);
    std::vector<int64_t> cls_meshes(64, 0), cls_queries(64, 0);
    for (int32_t m = 0; m < nmeshes; ++m) {
        const int64_t nt = tri_offsets[m + 1] - tri_offsets[m];
        if (nt <= 0 || vert_offsets[m + 1] <= vert_offsets[m] || q_offsets[m + 1] < q_offsets[m])
            return CP_ERROR_INVALID_VALUE;
        cls[m] = cp_size_class(nt);
        ++cls_meshes[cls[m]];
        cls_queries[cls[m]] += q_offsets[m + 1] - q_offsets[m];
    }
    std::vector<int> classes, qcls(64, 0);
    for (int c = 0; c < 64; ++c)
        if (cls_meshes[c]) {
            classes.push_back(c);
            const int64_t mean = cls_queries[c] / cls_meshes[c];
            qcls[c] = cp_size_class(mean > 0 ? mean : 1);
        }
    // all classes in the cache: no timing
    std::vector<BatchEntry> cache = read_batch_cache(cache_path);
    int leaf_of[64] = {0};
    bool all_cached = true;
    for (int c : classes) {
        bool hit = false;
        for (const BatchEntry& e : cache)
            if (e.cls == c && e.qcls == qcls[c] && e.K == branching) {
                leaf_of[c] = e.leaf;
                hit = true;
                break;
            }
        all_cached = all_cached && hit;
    }
    if (!all_cached) {
        // One build and one launch serve every class, so each choice is timed
        // on the whole batch: first the best uniform leaf size, then one class
        // at a time (most queries first) tries the other sizes, a change kept
        // when the whole batch gets at least 2% faster.
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return CP_ERROR_CUDA;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float* dist = nullptr;
        cp_status result = cudaMalloc(&dist, sizeof(float) * (q_offsets[nmeshes] + 1)) == cudaSuccess
                               ? CP_SUCCESS
                               : CP_ERROR_OUT_OF_MEMORY;
        const int sizes[4] = {1, 2, 4, 8};
        std::vector<int32_t> leaves(nmeshes, 2);
        float best_ms = 1e30f;
        int uniform = 2;
        for (int li = 0; li < 4 && result == CP_SUCCESS; ++li) {
            std::fill(leaves.begin(), leaves.end(), sizes[li]);
            float ms = 0.0f;
            result = time_batch(verts, vert_offsets, tris, tri_offsets, nmeshes, queries, q_offsets, branching, leaves,
                                dist, st, e0, e1, &ms);
            if (result == CP_SUCCESS && ms < best_ms) {
                best_ms = ms;
                uniform = sizes[li];
            }
        }
        for (int c : classes) leaf_of[c] = uniform;
        std::vector<int> order = classes;
        std::sort(order.begin(), order.end(), [&](int a, int b) { return cls_queries[a] > cls_queries[b]; });
        for (int c : order) {
            for (int li = 0; li < 4 && result == CP_SUCCESS; ++li) {
                if (sizes[li] == leaf_of[c]) continue;
                for (int32_t m = 0; m < nmeshes; ++m) leaves[m] = cls[m] == c ? sizes[li] : leaf_of[cls[m]];
                float ms = 0.0f;
                result = time_batch(verts, vert_offsets, tris, tri_offsets, nmeshes, queries, q_offsets, branching,
                                    leaves, dist, st, e0, e1, &ms);
                if (result == CP_SUCCESS && ms < 0.98f * best_ms) {
                    best_ms = ms;
                    leaf_of[c] = sizes[li];
                }
            }
        }
        cudaFree(dist);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaStreamDestroy(st);
        if (result != CP_SUCCESS) return result;
        if (cache_path) {
            std::vector<BatchEntry> out;
            for (const BatchEntry& e : cache) {
                bool replaced = false;
                for (int c : classes)
                    if (e.cls == c && e.qcls == qcls[c] && e.K == branching) replaced = true;
                if (!replaced) out.push_back(e);
            }
            for (int c : classes) out.push_back({c, qcls[c], branching, leaf_of[c], best_ms});
            write_batch_cache(cache_path, out);
        }
    }
    for (int32_t m = 0; m < nmeshes; ++m) leaf_sizes[m] = leaf_of[cls[m]];
    return CP_SUCCESS;
}
