// persist.cu — a built BVH written to a file and read back, so that a later
// run can skip the build (the reference keeps nothing between runs; its only
// file output is the rendered image, src/gpurt.cpp:258-262).
//
// File layout (host byte order): a fixed header (magic "CPQBVH", format 1,
// build parameters, counts), the per-mesh vertex and triangle offsets, the
// per-mesh leaf sizes when the build had them, then every device array a
// build leaves behind, in a fixed order, as raw bytes.  Scratch (refit
// arrival counters) and the device status word are not stored.
//
// Reading validates before anything reaches the GPU: the header against the
// file's size and the library's limits, and every array that a kernel indexes
// by: triangle indices within their mesh, the sorted order a permutation with
// inv_order its inverse, keys sorted with each mesh's run at its own offsets,
// parents, children and leaf ranges in range, and each mesh's wide tree a
// tree (every node reached once, no deeper than the stored depth bound, its
// leaves inside that mesh's triangles).  A damaged or crafted file is refused
// with a message instead of making a kernel read out of bounds or loop.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "bvh.cuh"

namespace cpq {

namespace {

constexpr char kMagic[8] = {'C', 'P', 'Q', 'B', 'V', 'H', '\0', '\1'};
constexpr int64_t kMaxFileTriangles = (int64_t(1) << 27) - 1;

struct FileHeader {
    char magic[8];
    int32_t K, leaf_size, collapse, nmeshes;
    float c_node, c_tri;
    int32_t mesh_bits, morton_bits, max_wide_depth, stack_bound;
    int32_t has_mesh_leaf, reserved;
    int64_t nt, nv, num_wide, num_leaves;
};
static_assert(sizeof(FileHeader) == 88, "file header layout");

// One stored device array: its member in the Bvh, element size and count.
struct Stored {
    void** dev;
    size_t elem;
    size_t count;
};

std::vector<Stored> stored_arrays(Bvh& b) {
    const size_t n = (size_t)b.nt, nn = 2 * n - 1, nm = (size_t)b.nmeshes, w = (size_t)b.num_wide;
    const size_t K = (size_t)b.p.K, inner = n > 1 ? n - 1 : 1;
    std::vector<Stored> a = {
        {reinterpret_cast<void**>(&b.tris), 4, 3 * n},      {reinterpret_cast<void**>(&b.keys), 8, n},
        {reinterpret_cast<void**>(&b.order), 4, n},         {reinterpret_cast<void**>(&b.inv_order), 4, n},
        {reinterpret_cast<void**>(&b.left), 4, inner},      {reinterpret_cast<void**>(&b.right), 4, inner},
        {reinterpret_cast<void**>(&b.parent), 4, nn},       {reinterpret_cast<void**>(&b.first), 4, nn},
        {reinterpret_cast<void**>(&b.last), 4, nn},         {reinterpret_cast<void**>(&b.box), 4, 6 * nn},
        {reinterpret_cast<void**>(&b.cost), 4, nn},         {reinterpret_cast<void**>(&b.leaf_flag), 1, nn},
        {reinterpret_cast<void**>(&b.cluster), 1, nn},      {reinterpret_cast<void**>(&b.mesh_root), 4, nm},
        {reinterpret_cast<void**>(&b.wide_root), 4, nm},    {reinterpret_cast<void**>(&b.frame), 4, 6 * nm},
        {reinterpret_cast<void**>(&b.recs), sizeof(TriRec), n},
        {reinterpret_cast<void**>(&b.fast), sizeof(FastTri), n},
        {reinterpret_cast<void**>(&b.nodes), 32 * K, w},    {reinterpret_cast<void**>(&b.wide_src), 4, w},
        {reinterpret_cast<void**>(&b.slot_src), 4, w * K}};
    if (!b.p.mesh_leaf.empty() || b.mesh_leaf) a.push_back({reinterpret_cast<void**>(&b.mesh_leaf), 4, nm});
    return a;
}

struct FileCloser {
    void operator()(FILE* f) const {
        if (f) fclose(f);
    }
};
using File = std::unique_ptr<FILE, FileCloser>;

int ceil_log2_i(int64_t v) {
    int b = 0;
    while ((int64_t(1) << b) < v) ++b;
    return b;
}

// A child reference that a traversal may follow: an inner node or a leaf of
// at most 15 triangles inside [lo, hi).
bool ref_ok(int32_t ref, int64_t num_wide, int64_t lo, int64_t hi) {
    if (!ref_is_leaf(ref)) return ref < num_wide;
    const int64_t f = leaf_first(ref), c = leaf_count(ref);
    return c >= 1 && c <= 15 && f >= lo && f + c <= hi;
}

template <typename T>
const T* as(const std::vector<unsigned char>& v) {
    return reinterpret_cast<const T*>(v.data());
}

// Every index-bearing array of a read file, against the header's counts.
bool validate(const FileHeader& h, const std::vector<int64_t>& voff, const std::vector<int64_t>& toff,
              const std::vector<std::vector<unsigned char>>& arr, std::string* why) {
    const int64_t n = h.nt, nn = 2 * n - 1, nm = h.nmeshes, w = h.num_wide, K = h.K;
    const int shift = 3 * h.morton_bits;
    const int32_t* tris = as<int32_t>(arr[0]);
    const uint64_t* keys = as<uint64_t>(arr[1]);
    const int32_t* order = as<int32_t>(arr[2]);
    const int32_t* inv = as<int32_t>(arr[3]);
    const int32_t* left = as<int32_t>(arr[4]);
    const int32_t* right = as<int32_t>(arr[5]);
    const int32_t* parent = as<int32_t>(arr[6]);
    const int32_t* first = as<int32_t>(arr[7]);
    const int32_t* last = as<int32_t>(arr[8]);
    const int32_t* mesh_root = as<int32_t>(arr[13]);
    const int32_t* wide_root = as<int32_t>(arr[14]);
    const TriRec* recs = as<TriRec>(arr[16]);
    const FastTri* fast = as<FastTri>(arr[17]);
    const unsigned char* nodes = arr[18].data();
    const int32_t* wide_src = as<int32_t>(arr[19]);
    const int32_t* slot_src = as<int32_t>(arr[20]);
    auto bad = [&](const std::string& m) {
        *why = m;
        return false;
    };
    // triangles: local vertex indices inside their mesh
    for (int64_t m = 0; m < nm; ++m) {
        const int64_t nvm = voff[m + 1] - voff[m];
        for (int64_t t = toff[m]; t < toff[m + 1]; ++t)
            for (int k = 0; k < 3; ++k)
                if (tris[3 * t + k] < 0 || tris[3 * t + k] >= nvm)
                    return bad("triangle " + std::to_string(t) + " has a vertex index outside its mesh");
    }
    // the sorted order: a permutation, inv_order its inverse, keys sorted with
    // mesh m's triangles at sorted positions [toff[m], toff[m+1])
    for (int64_t k = 0; k < n; ++k) {
        if (order[k] < 0 || order[k] >= n || inv[order[k]] != k) return bad("order and inv_order do not match");
        if (k > 0 && keys[k] < keys[k - 1]) return bad("keys are not sorted");
    }
    for (int64_t m = 0; m < nm; ++m)
        for (int64_t k = toff[m]; k < toff[m + 1]; ++k) {
            if (nm > 1 && (int64_t)(keys[k] >> shift) != m) return bad("a key's mesh bits do not match its position");
            if (order[k] < toff[m] || order[k] >= toff[m + 1]) return bad("a sorted triangle outside its mesh");
            const int32_t local = (int32_t)(order[k] - toff[m]);
            if (__builtin_bit_cast(int32_t, fast[k].p4.w) != local || __builtin_bit_cast(int32_t, recs[k].p2.y) != local)
                return bad("a triangle record's index does not match the order");
        }
    // the binary hierarchy: inner nodes 0 .. n-2, leaves n-1 .. 2n-2
    for (int64_t i = 0; i + 1 < n; ++i)
        if (left[i] < 0 || left[i] >= nn || right[i] < 0 || right[i] >= nn) return bad("a child outside the tree");
    for (int64_t v = 0; v < nn; ++v) {
        if (parent[v] < -1 || parent[v] >= (n > 1 ? n - 1 : 0)) return bad("a parent outside the inner nodes");
        if (first[v] < 0 || first[v] >= n || last[v] < first[v] || last[v] >= n) return bad("a node range outside the triangles");
    }
    for (int64_t m = 0; m < nm; ++m)
        if (mesh_root[m] < 0 || mesh_root[m] >= nn) return bad("a mesh root outside the tree");
    for (int64_t i = 0; i < w; ++i) {
        if (wide_src[i] < 0 || wide_src[i] >= nn) return bad("a wide node's source outside the tree");
        for (int64_t s = 0; s < K; ++s)
            if (slot_src[i * K + s] < -1 || slot_src[i * K + s] >= nn) return bad("a wide slot's source outside the tree");
    }
    // each mesh's wide tree: every node reached once, at most max_wide_depth
    // levels below the root, leaves inside the mesh's sorted range
    std::vector<unsigned char> seen((size_t)w, 0);
    std::vector<std::pair<int32_t, int32_t>> stack;
    for (int64_t m = 0; m < nm; ++m) {
        const int64_t lo = toff[m], hi = toff[m + 1];
        if (!ref_ok(wide_root[m], w, lo, hi)) return bad("a mesh's wide root is not a node or leaf of that mesh");
        if (ref_is_leaf(wide_root[m])) continue;
        stack.assign(1, {wide_root[m], 0});
        while (!stack.empty()) {
            const auto [node, depth] = stack.back();
            stack.pop_back();
            if (seen[node]) return bad("a wide node is reached twice (not a tree)");
            seen[node] = 1;
            if (depth > h.max_wide_depth) return bad("the wide tree is deeper than its stored bound");
            const float* rows = reinterpret_cast<const float*>(nodes + (size_t)node * 32 * K);
            const int32_t* child = reinterpret_cast<const int32_t*>(rows + 6 * K);
            for (int64_t s = 0; s < K; ++s) {
                if (rows[s] == INFINITY) continue;  // an empty slot: its box is never entered
                if (!ref_ok(child[s], w, lo, hi)) return bad("a wide child outside its mesh's nodes or triangles");
                if (!ref_is_leaf(child[s])) stack.push_back({child[s], depth + 1});
            }
        }
    }
    return true;
}

}  // namespace

cudaError_t bvh_save(Bvh& b, const char* path, std::string* why) {
    File f(fopen(path, "wb"));
    if (!f) {
        *why = std::string("cannot open ") + path + " for writing";
        return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return e;
    FileHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kMagic, 8);
    h.K = b.p.K;
    h.leaf_size = b.p.leaf_size;
    h.collapse = b.p.collapse;
    h.nmeshes = b.nmeshes;
    h.c_node = b.p.c_node;
    h.c_tri = b.p.c_tri;
    h.mesh_bits = b.mesh_bits;
    h.morton_bits = b.morton_bits;
    h.max_wide_depth = b.max_wide_depth;
    h.stack_bound = b.stack_bound;
    h.has_mesh_leaf = b.mesh_leaf ? 1 : 0;
    h.nt = b.nt;
    h.nv = b.nv;
    h.num_wide = b.num_wide;
    h.num_leaves = b.num_leaves;
    bool ok = fwrite(&h, sizeof h, 1, f.get()) == 1 &&
              fwrite(b.h_voff.data(), 8, b.h_voff.size(), f.get()) == b.h_voff.size() &&
              fwrite(b.h_toff.data(), 8, b.h_toff.size(), f.get()) == b.h_toff.size();
    std::vector<unsigned char> host;
    for (const Stored& s : stored_arrays(b)) {
        if (!ok) break;
        host.resize(s.elem * s.count);
        e = cudaMemcpy(host.data(), *s.dev, host.size(), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return e;
        ok = fwrite(host.data(), 1, host.size(), f.get()) == host.size();
    }
    if (!ok || fflush(f.get()) != 0) {
        *why = std::string("writing ") + path + " failed";
        return cudaErrorInvalidValue;
    }
    return cudaSuccess;
}

cudaError_t bvh_load(Bvh& b, const char* path, cudaStream_t st, std::string* why, bool* bad_file) {
    *bad_file = false;
    auto refuse = [&](const std::string& m) {
        *why = m;
        *bad_file = true;
        return cudaErrorInvalidValue;
    };
    File f(fopen(path, "rb"));
    if (!f) return refuse(std::string("cannot open ") + path);
    if (fseek(f.get(), 0, SEEK_END) != 0) return refuse("cannot size the file");
    const long size = ftell(f.get());
    if (size < 0 || fseek(f.get(), 0, SEEK_SET) != 0) return refuse("cannot size the file");
    FileHeader h;
    if (fread(&h, sizeof h, 1, f.get()) != 1) return refuse("shorter than a header");
    if (std::memcmp(h.magic, kMagic, 8) != 0) return refuse("not a BVH file of this library (magic or format)");
    if (h.K != 2 && h.K != 4 && h.K != 8) return refuse("branching must be 2, 4 or 8");
    if (h.leaf_size < 1 || h.leaf_size > 15 || (h.collapse != 0 && h.collapse != 1)) return refuse("bad build options");
    if (h.nmeshes < 1 || h.nmeshes > (1 << 20)) return refuse("bad mesh count");
    if (h.nt < h.nmeshes || h.nt > kMaxFileTriangles || h.nv < h.nmeshes || h.nv > INT32_MAX * (int64_t)h.nmeshes)
        return refuse("bad triangle or vertex count");
    const int mesh_bits = h.nmeshes > 1 ? ceil_log2_i(h.nmeshes) : 0;
    const int morton_bits = (64 - mesh_bits) / 3 > 21 ? 21 : (64 - mesh_bits) / 3;
    if (h.mesh_bits != mesh_bits || h.morton_bits != morton_bits) return refuse("key layout does not match the mesh count");
    if (h.num_wide < 1 || h.num_wide > 2 * h.nt || h.num_leaves < 1 || h.num_leaves > h.nt)
        return refuse("bad node counts");
    if (h.max_wide_depth < 0 || h.max_wide_depth > 255 || h.stack_bound != (h.K - 1) * (h.max_wide_depth + 1) ||
        h.stack_bound > 256)
        return refuse("bad depth bound");
    if (h.has_mesh_leaf != 0 && h.has_mesh_leaf != 1) return refuse("bad leaf-size flag");
    const size_t nm = (size_t)h.nmeshes;
    std::vector<int64_t> voff(nm + 1), toff(nm + 1);
    if (fread(voff.data(), 8, nm + 1, f.get()) != nm + 1 || fread(toff.data(), 8, nm + 1, f.get()) != nm + 1)
        return refuse("truncated offsets");
    if (voff[0] != 0 || toff[0] != 0 || voff[nm] != h.nv || toff[nm] != h.nt) return refuse("offsets do not match the counts");
    for (size_t m = 0; m < nm; ++m)
        if (voff[m + 1] <= voff[m] || toff[m + 1] <= toff[m] || voff[m + 1] - voff[m] > INT32_MAX)
            return refuse("every mesh needs triangles and vertices");
    b = Bvh();
    b.p.K = h.K;
    b.p.leaf_size = h.leaf_size;
    b.p.collapse = h.collapse;
    b.p.c_node = h.c_node;
    b.p.c_tri = h.c_tri;
    b.nmeshes = h.nmeshes;
    b.nt = h.nt;
    b.nv = h.nv;
    b.mesh_bits = h.mesh_bits;
    b.morton_bits = h.morton_bits;
    b.num_wide = h.num_wide;
    b.num_leaves = h.num_leaves;
    b.max_wide_depth = h.max_wide_depth;
    b.stack_bound = h.stack_bound;
    b.h_voff = voff;
    b.h_toff = toff;
    if (h.has_mesh_leaf) b.p.mesh_leaf.assign(nm, 0);  // read with the arrays below
    std::vector<Stored> arrays = stored_arrays(b);
    size_t expect = 0;
    for (const Stored& s : arrays) expect += s.elem * s.count;
    if ((size_t)size != sizeof h + 16 * (nm + 1) + expect) return refuse("the file's size does not match its header");
    std::vector<std::vector<unsigned char>> host(arrays.size());
    for (size_t i = 0; i < arrays.size(); ++i) {
        host[i].resize(arrays[i].elem * arrays[i].count);
        if (fread(host[i].data(), 1, host[i].size(), f.get()) != host[i].size()) return refuse("truncated arrays");
    }
    if (h.has_mesh_leaf) {
        const int32_t* ml = as<int32_t>(host.back());
        int32_t mx = 1;
        for (size_t m = 0; m < nm; ++m) {
            if (ml[m] < 1 || ml[m] > 15) return refuse("a per-mesh leaf size outside 1..15");
            mx = ml[m] > mx ? ml[m] : mx;
        }
        if (mx != h.leaf_size) return refuse("the leaf size is not the largest per-mesh size");
        b.p.mesh_leaf.assign(ml, ml + nm);
    }
    std::string reason;
    if (!validate(h, voff, toff, host, &reason)) return refuse(reason);
    // the device copy
    cudaError_t e = cudaGetDevice(&b.device);
    for (size_t i = 0; i < arrays.size() && e == cudaSuccess; ++i) {
        if (alloc_fault()) {
            e = cudaErrorMemoryAllocation;
            break;
        }
        void* p = nullptr;
        e = cudaMalloc(&p, host[i].size());
        if (e != cudaSuccess) break;
        b.allocations.push_back(p);
        b.device_bytes += host[i].size();
        *arrays[i].dev = p;
        e = cudaMemcpyAsync(p, host[i].data(), host[i].size(), cudaMemcpyHostToDevice, st);
    }
    const size_t nn = (size_t)(2 * h.nt - 1);
    struct Extra {
        void** dev;
        size_t bytes;
    } extra[] = {{reinterpret_cast<void**>(&b.d_voff), 8 * (nm + 1)},
                 {reinterpret_cast<void**>(&b.d_toff), 8 * (nm + 1)},
                 {reinterpret_cast<void**>(&b.arrive), 4 * nn},
                 {reinterpret_cast<void**>(&b.status), 4 * 64}};
    for (const Extra& x : extra) {
        if (e != cudaSuccess) break;
        if (alloc_fault()) {
            e = cudaErrorMemoryAllocation;
            break;
        }
        void* p = nullptr;
        e = cudaMalloc(&p, x.bytes);
        if (e != cudaSuccess) break;
        b.allocations.push_back(p);
        b.device_bytes += x.bytes;
        *x.dev = p;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.d_voff, voff.data(), 8 * (nm + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.d_toff, toff.data(), 8 * (nm + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.status, 0, 4 * 64, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host copies go out of scope
    return e;
}

}  // namespace cpq
