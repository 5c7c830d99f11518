// autotune.cu — per-size-class choice of branching, leaf size, block size and
// short-stack depth by timing real builds and queries on the caller's data.
// The reference has no tuner; its only knobs are UI sliders that feed push
// constants (src/gpurt.cpp:283-322, src/vk/rt.h:85-102).  Results are cached
// in a plain text file, one line per (triangle class, query class, branching):
//   <tri_class> <query_class> <branching> <leaf_size> <block_size> <short_stack> <ms>
// where a class is floor(log2(count)) and short_stack 0 stands for the
// warp-packet traversal; batches (cp_batch_autotune) add lines of their own,
// marked B, with a leaf size per triangle class.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cpq.h"

namespace {

struct Entry {
    int cls, qcls, K, leaf, block, stack;
    float ms;
};

std::vector<Entry> read_cache(const char* path) {
    std::vector<Entry> out;
    if (!path) return out;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        Entry e;
        if (is >> e.cls >> e.qcls >> e.K >> e.leaf >> e.block >> e.stack >> e.ms) out.push_back(e);
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
          << ' ' << e.ms << '\n';
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
                for (int si = 0; si < 4; ++si) {
                    // stacks[0..2]: per-thread traversal with that short stack;
                    // si == 3: warp-packet traversal
                    cp_query_opts qo;
                    cp_query_opts_default(&qo);
                    qo.block_size = blocks[bi];
                    qo.short_stack = si < 3 ? stacks[si] : 8;
                    qo.traversal = si < 3 ? CP_TRAVERSAL_THREAD : CP_TRAVERSAL_PACKET;
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
                        best = {cls, qcls, Ks[ki], leaves[li], blocks[bi], si < 3 ? stacks[si] : 0, ms};
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

extern "C" CP_API cp_status cp_batch_autotune(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                                              const int64_t* tri_offsets, int32_t nmeshes, const float* queries,
                                              const int64_t* q_offsets, int32_t branching, const char* cache_path,
                                              int32_t* leaf_sizes, cp_query_opts* best_query) {
    if (!verts || !vert_offsets || !tris || !tri_offsets || !queries || !q_offsets || !leaf_sizes || !best_query ||
        nmeshes <= 0)
        return CP_ERROR_INVALID_VALUE;
    if (branching != 2 && branching != 4 && branching != 8) return CP_ERROR_INVALID_VALUE;
    cp_query_opts_default(best_query);
    // size classes of the meshes
    std::vector<int> cls(nmeshes);
    std::vector<std::vector<int32_t>> members(64);
    for (int32_t m = 0; m < nmeshes; ++m) {
        const int64_t nt = tri_offsets[m + 1] - tri_offsets[m];
        if (nt <= 0 || vert_offsets[m + 1] <= vert_offsets[m] || q_offsets[m + 1] < q_offsets[m])
            return CP_ERROR_INVALID_VALUE;
        cls[m] = cp_size_class(nt);
        members[cls[m]].push_back(m);
    }
    std::vector<BatchEntry> cache = read_batch_cache(cache_path);
    int best_leaf[64];
    for (int c = 0; c < 64; ++c) best_leaf[c] = 0;
    std::vector<BatchEntry> found;

    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return CP_ERROR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cp_status result = CP_SUCCESS;
    const int leaves[4] = {1, 2, 4, 8};
    for (int c = 0; c < 64 && result == CP_SUCCESS; ++c) {
        const std::vector<int32_t>& mem = members[c];
        if (mem.empty()) continue;
        // the class's meshes and queries, back to back
        std::vector<int64_t> voff{0}, toff{0}, qoff{0};
        for (int32_t m : mem) {
            voff.push_back(voff.back() + vert_offsets[m + 1] - vert_offsets[m]);
            toff.push_back(toff.back() + tri_offsets[m + 1] - tri_offsets[m]);
            qoff.push_back(qoff.back() + q_offsets[m + 1] - q_offsets[m]);
        }
        const int64_t nq = qoff.back();
        const int qcls = cp_size_class(nq / (int64_t)mem.size() > 0 ? nq / (int64_t)mem.size() : 1);
        bool cached = false;
        for (const BatchEntry& e : cache)
            if (e.cls == c && e.qcls == qcls && e.K == branching) {
                best_leaf[c] = e.leaf;
                found.push_back(e);
                cached = true;
                break;
            }
        if (cached) continue;
        if (nq == 0) {  // nothing to time: the single-mesh default
            best_leaf[c] = 4;
            continue;
        }
        float* v = nullptr;
        int32_t* t = nullptr;
        float* q = nullptr;
        float* dist = nullptr;
        void* ws = nullptr;
        if (cudaMalloc(&v, sizeof(float) * 3 * voff.back()) != cudaSuccess ||
            cudaMalloc(&t, sizeof(int32_t) * 3 * toff.back()) != cudaSuccess ||
            cudaMalloc(&q, sizeof(float) * 3 * nq) != cudaSuccess ||
            cudaMalloc(&dist, sizeof(float) * nq) != cudaSuccess) {
            result = CP_ERROR_OUT_OF_MEMORY;
        }
        for (size_t k = 0; k < mem.size() && result == CP_SUCCESS; ++k) {
            const int32_t m = mem[k];
            if (cudaMemcpyAsync(v + 3 * voff[k], verts + 3 * vert_offsets[m],
                                sizeof(float) * 3 * (voff[k + 1] - voff[k]), cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync(t + 3 * toff[k], tris + 3 * tri_offsets[m],
                                sizeof(int32_t) * 3 * (toff[k + 1] - toff[k]), cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
                cudaMemcpyAsync(q + 3 * qoff[k], queries + 3 * q_offsets[m],
                                sizeof(float) * 3 * (qoff[k + 1] - qoff[k]), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
                result = CP_ERROR_CUDA;
        }
        BatchEntry best = {c, qcls, branching, 4, 1e30f};
        for (int li = 0; li < 4 && result == CP_SUCCESS; ++li) {
            cp_build_opts bo;
            cp_build_opts_default(&bo);
            bo.branching = branching;
            bo.leaf_size = leaves[li];
            cp_batch* b = nullptr;
            cp_status s = cp_batch_create(v, voff.data(), t, toff.data(), (int32_t)mem.size(), &bo, st, &b);
            if (s != CP_SUCCESS) {
                result = s;
                break;
            }
            cp_query_opts qo;
            cp_query_opts_default(&qo);
            size_t wsb = 0;
            cp_batch_query_workspace_size(b, nq, &qo, &wsb);
            if (ws) cudaFree(ws);
            ws = nullptr;
            if (cudaMalloc(&ws, wsb) != cudaSuccess) {
                cp_batch_destroy(b);
                result = CP_ERROR_OUT_OF_MEMORY;
                break;
            }
            float ms = 1e30f;
            for (int rep = 0; rep < 3 && s == CP_SUCCESS; ++rep) {
                cudaEventRecord(e0, st);
                s = cp_batch_query(b, q, qoff.data(), &qo, nullptr, dist, nullptr, nullptr, ws, wsb, 0, st);
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                float tms = 0.0f;
                cudaEventElapsedTime(&tms, e0, e1);
                if (rep > 0 && tms < ms) ms = tms;  // the first run warms caches
            }
            cp_batch_destroy(b);
            if (s != CP_SUCCESS) {
                result = s;
                break;
            }
            if (ms < best.ms) best = {c, qcls, branching, leaves[li], ms};
        }
        cudaFree(ws);
        cudaFree(v);
        cudaFree(t);
        cudaFree(q);
        cudaFree(dist);
        if (result == CP_SUCCESS) {
            best_leaf[c] = best.leaf;
            found.push_back(best);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (result != CP_SUCCESS) return result;
    for (int32_t m = 0; m < nmeshes; ++m) leaf_sizes[m] = best_leaf[cls[m]];
    if (cache_path) {
        std::vector<BatchEntry> out;
        for (const BatchEntry& e : cache) {
            bool replaced = false;
            for (const BatchEntry& f : found)
                if (f.cls == e.cls && f.qcls == e.qcls && f.K == e.K) replaced = true;
            if (!replaced) out.push_back(e);
        }
        for (const BatchEntry& f : found) out.push_back(f);
        write_batch_cache(cache_path, out);
    }
    return CP_SUCCESS;
}
