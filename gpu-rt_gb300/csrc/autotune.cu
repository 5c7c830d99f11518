// autotune.cu — per-size-class choice of branching, leaf size, block size and
// short-stack depth by timing real builds and queries on the caller's data.
// The reference has no tuner; its only knobs are UI sliders that feed push
// constants (src/gpurt.cpp:283-322, src/vk/rt.h:85-102).  Results are cached
// in a plain text file, one line per (triangle class, query class, branching):
//   <tri_class> <query_class> <branching> <leaf_size> <block_size> <short_stack> <ms>
// where a class is floor(log2(count)) and short_stack 0 stands for the
// warp-packet traversal.
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
    std::ofstream f(path, std::ios::trunc);
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
