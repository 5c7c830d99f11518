// bvh.cuh — the device-resident BVH shared by single meshes and batches.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace cpq {

struct BuildParams {
    int K = 2;              // branching
    int leaf_size = 4;      // max triangles per leaf
    int collapse = 0;       // 0 count, 1 SAH
    float c_node = 1.0f;    // SAH node-visit cost
    float c_tri = 1.0f;     // SAH triangle-test cost
    // optional, per mesh of a batch: max triangles per leaf (then leaf_size is
    // their maximum); empty: leaf_size for every mesh
    std::vector<int32_t> mesh_leaf;
};

// Everything a build leaves on the device.  A single mesh is a batch of one.
struct Bvh {
    BuildParams p;
    int32_t nmeshes = 0;
    int64_t nt = 0, nv = 0;
    int mesh_bits = 0;          // high key bits holding the mesh id
    int morton_bits = 21;       // bits per axis of the build's Morton codes
    int64_t num_wide = 0, num_leaves = 0;
    int32_t max_wide_depth = 0, stack_bound = 0;
    float build_ms = 0.0f;
    int device = 0;

    // traversal data
    void* nodes = nullptr;          // WideNode<K>[num_wide]
    TriRec* recs = nullptr;         // nt triangle records in leaf order (exact vertices)
    FastTri* fast = nullptr;        // nt distance-test records in leaf order
    int32_t* wide_root = nullptr;   // nmeshes
    float* frame = nullptr;         // nmeshes x 6: query Morton frame (lo xyz, scale xyz)

    // kept for refit and inspection
    int32_t* tris = nullptr;        // nt x 3 local indices
    int64_t* d_voff = nullptr;      // nmeshes + 1
    int64_t* d_toff = nullptr;      // nmeshes + 1
    std::vector<int64_t> h_voff, h_toff;
    uint64_t* keys = nullptr;       // nt sorted
    int32_t* order = nullptr;       // nt: sorted position -> global triangle
    int32_t* inv_order = nullptr;   // nt: global triangle -> sorted position
    int32_t* left = nullptr;        // nt - 1
    int32_t* right = nullptr;       // nt - 1
    int32_t* parent = nullptr;      // 2nt - 1
    int32_t* first = nullptr;       // 2nt - 1
    int32_t* last = nullptr;        // 2nt - 1
    float* box = nullptr;           // (2nt - 1) x 6: lo xyz, hi xyz
    float* cost = nullptr;          // 2nt - 1
    uint8_t* leaf_flag = nullptr;   // 2nt - 1
    uint8_t* cluster = nullptr;     // 2nt - 1
    uint32_t* arrive = nullptr;     // 2nt - 1 refit counters
    int32_t* mesh_root = nullptr;   // nmeshes: binary root per mesh
    int32_t* mesh_leaf = nullptr;   // nmeshes: per-mesh leaf limit, or nullptr (leaf_size)
    int32_t* wide_src = nullptr;    // num_wide
    int32_t* slot_src = nullptr;    // num_wide x K: binary node per child slot (-1 empty)
    uint32_t* status = nullptr;     // device status word (CP_DEVICE_* bits)

    std::vector<void*> allocations;
    size_t device_bytes = 0;
};

// Build.  verts: nv points at vert_stride floats; tris: local indices;
// h_voff/h_toff: host offsets (nmeshes + 1).  Synchronises the stream.
// On failure returns a CUDA error or sets *bad_input (invalid index /
// non-finite vertex) and leaves the Bvh to be released by bvh_free.
cudaError_t bvh_build(Bvh& b, const float* verts, int64_t vert_stride, const int32_t* tris,
                      const std::vector<int64_t>& h_voff, const std::vector<int64_t>& h_toff,
                      const BuildParams& p, cudaStream_t st, bool* bad_input, std::string* why);

// Move the vertices and refit every box; topology unchanged.  Asynchronous.
cudaError_t bvh_refit(Bvh& b, const float* verts, int64_t vert_stride, cudaStream_t st);

void bvh_free(Bvh& b);

// A built BVH written to a file and read back (persist.cu).  bvh_save
// synchronises the device; bvh_load validates the whole file on the host
// before any device work (*bad_file and *why on refusal) and synchronises `st`.
cudaError_t bvh_save(Bvh& b, const char* path, std::string* why);
cudaError_t bvh_load(Bvh& b, const char* path, cudaStream_t st, std::string* why, bool* bad_file);

// Query workspace and launch (query.cu).
struct QueryParams {
    int block = 256;
    int sort = 1;
    int blocks_per_sm = 0;
    int short_stack = 8;
    int traversal = 0;  // 0 auto (packet when sorted), 1 per-thread, 2 warp packet
    int seed_chunk = 1; // packet traversal: packets per claim, seeded after the first (1: no seeding)
    bool no_timing = false;  // never create timing events, even when cp_timing_enable is on
};

size_t query_workspace_bytes(const Bvh& b, int64_t nq, const QueryParams& qp);

// The visiting order of nq points (queries or ray origins): their Hilbert
// order when `sort` (else nullptr), in a workspace of
// query_workspace_bytes(b, nq, {sort}) bytes, plus the zeroed work counter of
// a persistent traversal.  `coarse` sorts only the Hilbert index's top bits
// (about 16 points per curve segment): a radix pass less, for per-thread
// walks.  `keys_out` (optional; single meshes, whose keys have at most 32
// bits) receives each point's key in input order.  Stream-ordered; no host
// synchronisation.
cudaError_t order_points(const Bvh& b, const float* points, int64_t nq, const int64_t* d_qoff,
                         bool sort, void* ws, size_t ws_bytes, cudaStream_t st, const int32_t** perm,
                         unsigned long long** counter, bool coarse = false, uint32_t* keys_out = nullptr);

// q_off: device array of nmeshes + 1 query offsets (nullptr for one mesh).
cudaError_t bvh_query(const Bvh& b, const float* queries, int64_t nq, const int64_t* d_qoff,
                      const QueryParams& qp, float* out_point, float* out_dist, int32_t* out_tri,
                      float* out_bary, void* ws, size_t ws_bytes, cudaStream_t st);

// CUDA-event timing of traversal launches (diagnostic; see cp_timing_enable).
void timing_enable(bool events, bool counters);
cudaError_t timing_read(double* ms, int64_t* launches, bool reset);
// Allocation-failure injection for tests (cp_debug_fail_allocation): true
// when the library's next device allocation is to fail.
bool alloc_fault();

// Counters of the counting packet kernel: warp node visits, leaf triangles
// (per warp leaf visit), stack pops, skipped pops, lane-triangle tests
// (active lanes x leaf triangles), triangle rounds executed and lane-node
// visits (lanes whose bound admitted the node, summed over warp visits).
constexpr int kStatCount = 7;
cudaError_t traversal_stats(unsigned long long* out, bool reset);

// Proxy triangles for the top level of an instanced scene: per instance the
// world box of its mesh in `bottom` as (lo, hi, hi); verts 2n x 3, tris n x 3.
cudaError_t instance_proxies(const Bvh& bottom, const int32_t* inst_mesh, const float* inst_fwd,
                             int32_t n, float* verts, int32_t* tris, cudaStream_t st);

// The instances of a scene on the device.  Similarity instances are walked
// through the batch's own BVHs in object space; general affine ones through
// world-space copies (`baked_bvh`, one mesh per such instance, built from
// instance_bake's output).
struct InstanceSet {
    const int32_t* mesh = nullptr;   // per instance: the batch mesh it places
    const int32_t* baked = nullptr;  // per instance: its baked copy, or -1
    const float* inv = nullptr;      // 12 per instance: object <- world, row-major 3 x 4
    const float* fwd = nullptr;      // 12 per instance: world <- object
    const float* s2 = nullptr;       // 2 per instance: squared scale, lower bound of the squared stretch
    const Bvh* baked_bvh = nullptr;  // null when every instance is a similarity
};

// World-space triangles of the baked instances: for each j < nb, instance
// baked_inst[j]'s mesh in its local triangle order at out_off[j] (host
// prefix sums copied to the device, total = out_off[nb]); verts 9 floats and
// tris 3 local indices (3i, 3i+1, 3i+2) per triangle.
cudaError_t instance_bake(const Bvh& bottom, const int32_t* baked_inst, const int32_t* inst_mesh,
                          const float* inst_fwd, const int64_t* out_off, int32_t nb, int64_t total, float* verts,
                          int32_t* tris, cudaStream_t st);

// Closest points over the instances of a batch's meshes: `top` is a BVH
// over the instances' proxies (local index = instance), `bottom` the batch.
// Workspace: query_workspace_bytes(top, nq, ...) with the same sort flag.
cudaError_t bvh_instance_query(const Bvh& top, const Bvh& bottom, const InstanceSet& is, const float* queries,
                               int64_t nq, bool sort, float* out_point, float* out_dist, int32_t* out_inst,
                               int32_t* out_tri, float* out_bary, void* ws, size_t ws_bytes, cudaStream_t st);

cudaError_t bvh_backward(const Bvh& b, const float* queries, const int32_t* tri, const float* bary,
                         const float* grad_dist, int64_t nq, float* grad_q, float* grad_verts,
                         cudaStream_t st);

}  // namespace cpq
