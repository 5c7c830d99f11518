/*
 * cpq.h — C ABI of the GB300 closest-point engine.
 *
 * Query surface: a triangle mesh goes in, a BVH is built on the GPU, a batch
 * of query points goes in, and for every point the closest point on the mesh,
 * the unsigned distance and the index of the closest triangle come out.
 *
 * The reference (TheNumbat/GPU-RT, main branch) has no library target and no
 * FFI: it is one SDL executable (CMakeLists.txt:66-70).  Its closest-point
 * work lives on a branch that is not available, so every entry point below
 * names the reference interface whose role it takes over:
 *   - mesh in + BVH built  ->  VK::Mesh (src/vk/mesh.h:14-58) and
 *                              VK::Accel(const Mesh&) (src/vk/vulkan.h:259,
 *                              src/vk/vulkan.cpp:881-936);
 *   - query                ->  trace_ray / traceRayEXT over the TLAS
 *                              (src/shaders/rt/rt.rgen:257-270), issued by
 *                              RTPipe::trace (src/vk/rt.cpp:346-394);
 *   - many meshes at once  ->  the TLAS over per-mesh BLASes
 *                              (src/vk/vulkan.cpp:777-856, src/gpurt.cpp:220-241);
 *   - destroy              ->  Drop<T> / Accel::destroy (src/vk/vulkan.h:305-336).
 *
 * Conventions
 *   - Every array argument is caller-owned DEVICE memory unless the entry
 *     point's name ends in _host.  Handles own their BVH memory.
 *   - Every call returns a cp_status and never exits the process (the
 *     reference's die() calls std::exit, src/lib/log.h:46-49).
 *     cp_last_error_string() describes the last failure of the calling thread.
 *   - Calls are asynchronous on the given stream unless documented otherwise.
 *     A NULL stream is the legacy default stream.
 *   - A built mesh is read-only for cp_query / cp_backward, so concurrent
 *     queries on different streams are safe.  cp_mesh_refit and
 *     cp_mesh_destroy need exclusive access.
 *   - Triangle indices are int32 triples into the mesh's own vertex array.
 *     Vertices are float xyz triples with a byte stride >= 12 (48 reads the
 *     reference's VK::Mesh::Vertex layout, src/vk/mesh.h:16-22, directly).
 *   - Tie rule: among triangles at exactly the same computed distance, the one
 *     with the smallest index wins, among those the traversal reaches: a
 *     box whose FP32 bound rounds to the best distance found so far is not
 *     entered, so where two triangles share the closest point (an edge or a
 *     vertex) the reported one can depend on the visiting order, which the
 *     query options (seeding, traversal kind) change; the distance and the
 *     point agree to their rounding.
 */
#ifndef GPURT_CPQ_H
#define GPURT_CPQ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define CP_API __declspec(dllexport)
#else
#define CP_API __attribute__((visibility("default")))
#endif

/* Same type as cudaStream_t; declared here so the header needs no CUDA headers. */
typedef struct CUstream_st* cp_stream_t;

typedef enum cp_status {
    CP_SUCCESS = 0,
    CP_ERROR_INVALID_VALUE = 1,   /* bad pointer, size, option or index */
    CP_ERROR_OUT_OF_MEMORY = 2,   /* a device or host allocation failed */
    CP_ERROR_CUDA = 3,            /* a CUDA runtime call failed */
    CP_ERROR_DEVICE_FAULT = 4,    /* a kernel reported an error through its status word */
    CP_ERROR_NOT_SUPPORTED = 5,   /* no GPU, or an option the library does not support */
    CP_ERROR_SCRATCH_TOO_SMALL = 6 /* a workspace or fixed scratch area is too small */
} cp_status;

/* Device status-word bits, reported by cp_mesh_device_status(). */
#define CP_DEVICE_STACK_OVERFLOW 0x1u
#define CP_DEVICE_BAD_INDEX      0x2u
#define CP_DEVICE_NONFINITE      0x4u

typedef enum cp_collapse {
    CP_COLLAPSE_COUNT = 0,  /* a subtree becomes a leaf when it holds <= leaf_size triangles */
    CP_COLLAPSE_SAH = 1     /* ... and the surface-area heuristic says a leaf is cheaper */
} cp_collapse;

typedef struct cp_build_opts {
    int32_t branching;      /* BVH width: 2, 4 or 8 */
    int32_t leaf_size;      /* maximum triangles per leaf, 1..15 */
    int32_t collapse;       /* cp_collapse */
    float sah_node_cost;    /* SAH cost of one node visit (CP_COLLAPSE_SAH) */
    float sah_tri_cost;     /* SAH cost of one point-triangle test (CP_COLLAPSE_SAH) */
} cp_build_opts;

typedef struct cp_query_opts {
    int32_t block_size;     /* traversal threads per block: 64..1024, multiple of 32; 0 = default */
    int32_t sort_queries;   /* 1: walk the queries along a Hilbert curve through their positions (outputs keep input order) */
    int32_t blocks_per_sm;  /* persistent grid = SM count x this; 0 = from occupancy */
    int32_t short_stack;    /* per-thread stack entries kept in shared memory: 4, 8 or 16; 0 = default */
    int32_t traversal;      /* CP_TRAVERSAL_*: how lanes share work */
    int32_t seed_chunk;     /* packet traversal: consecutive packets a warp claims at once, each after the
                               first starting its lanes' limits at an upper bound from the previous packet's
                               closest points: 1 (no seeding) .. 16; 0 = default (1) */
} cp_query_opts;

/* Traversal kernels.  PACKET: the 32 lanes of a warp take 32 consecutive
 * (Hilbert-ordered, so neighbouring) queries and walk one shared stack, a node
 * being visited when any lane still needs it; THREAD: every lane walks its
 * own query with its own stack.  AUTO picks PACKET when sort_queries is set. */
#define CP_TRAVERSAL_AUTO   0
#define CP_TRAVERSAL_THREAD 1
#define CP_TRAVERSAL_PACKET 2

/* Statistics of a built mesh (cp_mesh_info). */
typedef struct cp_mesh_info_t {
    int64_t num_vertices;
    int64_t num_triangles;
    int64_t num_binary_nodes;   /* 2*T - 1 */
    int64_t num_wide_nodes;
    int64_t num_leaves;         /* leaf clusters */
    int32_t branching;
    int32_t leaf_size;
    int32_t max_wide_depth;     /* edges on the longest root-to-leaf path of the wide BVH */
    int32_t stack_bound;        /* stack entries the traversal can need at most */
    int64_t device_bytes;       /* BVH + triangle memory held by the handle */
    float build_ms;             /* device time of the last build or refit (0 if not timed) */
} cp_mesh_info_t;

typedef struct cp_mesh cp_mesh;
typedef struct cp_batch cp_batch;
typedef struct cp_scene cp_scene;

/* ---- options ---------------------------------------------------------------- */

/* Binary BVH, leaf size 4, count collapse: the canonical configuration. */
CP_API void cp_build_opts_default(cp_build_opts* opts);
CP_API void cp_query_opts_default(cp_query_opts* opts);

/* ---- errors ----------------------------------------------------------------- */

/* Message of the last failed call on this thread ("" if none). */
CP_API const char* cp_last_error_string(void);
CP_API const char* cp_status_string(cp_status status);
/* Library version as an integer (major * 10000 + minor * 100 + patch). */
CP_API int32_t cp_version(void);

/* Kernels this library has launched in the process so far (all devices).
 * A diagnostic: the difference across a region counts its launches.  No
 * counterpart in the reference. */
CP_API uint64_t cp_kernel_launches(void);

/* Diagnostic timing, flags of cp_timing_enable (0 turns both off).
 * CP_TIMING_EVENTS: every traversal-kernel launch outside a stream capture
 * is bracketed by CUDA events on its own stream; cp_timing_read waits for
 * them and returns the summed device time (ms) and the number of launches
 * since the last reset.  CP_TIMING_COUNTERS: packet traversals run a
 * counting build of the kernel (a few percent slower) whose counts, summed
 * over warps, cp_traversal_stats returns in counts7: [0] warp node visits,
 * [1] leaf triangles per warp leaf visit, [2] stack pops, [3] skipped pops,
 * [4] lane-triangle tests (active lanes x leaf triangles), [5] triangle
 * rounds executed by warps, [6] lane-node visits (lanes whose bound
 * admitted the visited node); it synchronises the device.
 * No counterpart in the reference (its only timing is an FPS readout,
 * src/gpurt.cpp:275). */
#define CP_TIMING_EVENTS 1
#define CP_TIMING_COUNTERS 2
CP_API cp_status cp_timing_enable(int32_t flags);

/* Test hook (fault injection on the host): the library's next `after` device
 * allocations succeed and the one after fails as if the device were out of
 * memory — the call that made it returns CP_ERROR_OUT_OF_MEMORY, having
 * released what it held — after which the hook disarms itself; a negative
 * value disarms it at once.  Covers BVH builds, their temporaries and query
 * workspaces. */
CP_API void cp_debug_fail_allocation(int64_t after);
CP_API cp_status cp_timing_read(double* traverse_ms, int64_t* launches, int32_t reset);
CP_API cp_status cp_traversal_stats(uint64_t* counts7, int32_t reset);

/* Diagnostic: read bandwidth (GB/s) of 128-bit L2 loads over a `bytes`-sized
 * buffer, best of 5 timed launches of `reps` sweeps each.  A buffer smaller
 * than L2 (129 MB on GB300) measures L2, a larger one HBM.  Synchronous. */
CP_API cp_status cp_probe_read_bandwidth(int64_t bytes, int32_t reps, double* gbs,
                                         cp_stream_t stream);

/* ---- single mesh -------------------------------------------------------------- */

/*
 * Build a BVH over a triangle mesh.  Replaces VK::Accel(const Mesh&)
 * (src/vk/vulkan.h:259; src/vk/vulkan.cpp:881-936), which hands the mesh to
 * the Vulkan driver's closed BVH builder.  Here the build is a Morton-code
 * LBVH (63-bit codes, stable radix sort, Karras 2012 hierarchy), a bottom-up
 * bounding-box refit, a leaf collapse (count or SAH) and a collapse to
 * `branching`-wide nodes.  `verts` holds nv points of 3 floats at
 * `vert_stride_bytes` (a multiple of 4, >= 12); `tris` holds nt int32 triples.
 * opts may be NULL (defaults).  Synchronises `stream` before returning.
 */
CP_API cp_status cp_mesh_create(const float* verts, int64_t nv, int64_t vert_stride_bytes,
                                const int32_t* tris, int64_t nt, const cp_build_opts* opts,
                                cp_stream_t stream, cp_mesh** out);

/*
 * Move the vertices of a built mesh (same count, same triangles) and refit
 * every box bottom-up; the tree topology is kept.  Takes the role of the
 * reference's rebuild-on-change of its BLAS (src/gpurt.cpp:220-241).
 * Asynchronous on `stream`; no host synchronisation, so it can be captured
 * in a CUDA graph.
 */
CP_API cp_status cp_mesh_refit(cp_mesh* mesh, const float* verts, int64_t vert_stride_bytes,
                               cp_stream_t stream);

/* Free the handle and its device memory (Accel::destroy, src/vk/vulkan.h:268). */
CP_API cp_status cp_mesh_destroy(cp_mesh* mesh);

CP_API cp_status cp_mesh_info(const cp_mesh* mesh, cp_mesh_info_t* out);

/*
 * Synchronise `stream`, return the device status bits the kernels set on this
 * mesh since the last call (CP_DEVICE_*), and clear them.
 */
CP_API cp_status cp_mesh_device_status(cp_mesh* mesh, cp_stream_t stream, uint32_t* bits);

/*
 * Bytes of device workspace cp_query needs for nq queries with these options.
 */
CP_API cp_status cp_query_workspace_size(const cp_mesh* mesh, int64_t nq, const cp_query_opts* opts,
                                         size_t* bytes);

/*
 * Diagnostic: the order in which cp_query with sort_queries walks these
 * queries — perm[i] is the input index of the i-th query along the Hilbert
 * curve of the query box, keys (NULL: not written) each query's 30-bit curve
 * index in input order — so that perm sorts keys stably.  nq >= 2; device
 * arrays; asynchronous on `stream`.
 */
CP_API cp_status cp_query_order(cp_mesh* mesh, const float* queries, int64_t nq, int32_t* perm,
                                uint32_t* keys, cp_stream_t stream);

/*
 * Diagnostic: the library's radix sort (the one that orders queries and rays
 * and sorts the build's Morton keys) on caller keys — perm receives the
 * permutation that sorts keys[0..n) (key_bytes 4 or 8, device) stably on
 * bits [begin_bit, end_bit).  The keys are not modified.  Asynchronous on
 * `stream`.
 */
CP_API cp_status cp_debug_order_sort(const void* keys, int32_t key_bytes, int64_t n, int32_t begin_bit,
                                     int32_t end_bit, int32_t* perm, cp_stream_t stream);

/*
 * Closest-point query.  Replaces the per-pixel traceRayEXT over the
 * acceleration structure (src/shaders/rt/rt.rgen:257-270) with a closest-first
 * BVH descent and an exact point-triangle distance at the leaves; the
 * hit payload {barycentrics, primitive id} (src/shaders/rt/rtcommon.glsl:55-60,
 * src/shaders/rt/rt.rchit:11-16) becomes {closest point, distance, triangle,
 * barycentrics}.
 *   queries    nq x 3 floats
 *   out_point  nq x 3 floats (closest point), may be NULL
 *   out_dist   nq floats (unsigned distance), may be NULL
 *   out_tri    nq int32 (closest triangle), may be NULL
 *   out_bary   nq x 2 floats (barycentric weights of vertices 1 and 2 of the
 *              closest triangle; vertex 0 has 1 - u - v), may be NULL
 *   workspace  device memory of cp_query_workspace_size() bytes, or NULL to
 *              allocate it stream-ordered inside the call.
 * nq == 0 is a no-op.  Asynchronous on `stream`.
 */
CP_API cp_status cp_query(const cp_mesh* mesh, const float* queries, int64_t nq,
                          const cp_query_opts* opts, float* out_point, float* out_dist,
                          int32_t* out_tri, float* out_bary, void* workspace,
                          size_t workspace_bytes, cp_stream_t stream);

/*
 * cp_query with HOST arrays: copies the queries to the device, queries them
 * and copies the results back.  Up to 64M queries are ordered and traversed
 * as one set (denser sets traverse faster than chunks of them); larger calls
 * go in 64M-query chunks whose copies overlap the previous chunk's traversal
 * on a second stream.  Host arrays should be
 * pinned (cudaHostAlloc / cudaHostRegister) for full copy speed.  Synchronous:
 * the outputs are ready when it returns.
 */
CP_API cp_status cp_query_host(const cp_mesh* mesh, const float* queries, int64_t nq,
                               const cp_query_opts* opts, float* out_point, float* out_dist,
                               int32_t* out_tri, float* out_bary, cp_stream_t stream);

/*
 * cp_query_host without the wait: enqueues on `stream` the copy of the
 * queries to the device, the query (all nq as one ordered set) and the copies
 * of the results back, and returns.  The outputs are ready once the stream
 * reaches this point (synchronise it, or an event recorded after the call);
 * until then the caller must neither change the queries nor read or reuse
 * the outputs.  The host arrays must be pinned (cudaHostAlloc /
 * cudaHostRegister; anything else is refused with CP_ERROR_INVALID_VALUE, as
 * a copy from pageable memory would not be asynchronous).  Device buffers
 * come from the library's stream-ordered pool and go back to it in stream
 * order.  Calls on different streams overlap: with two streams taking
 * alternate batches, one batch's copies run while the other's kernels do, so
 * a stream of batches costs about the device time per batch.  nq up to
 * 2^31 - 1.
 */
CP_API cp_status cp_query_host_async(const cp_mesh* mesh, const float* queries, int64_t nq,
                                     const cp_query_opts* opts, float* out_point, float* out_dist,
                                     int32_t* out_tri, float* out_bary, cp_stream_t stream);

/* ---- glTF ingest (host) ---------------------------------------------------- */

/*
 * Reads a glTF 2.0 scene (.gltf with external or base64 "data:" buffers, or
 * .glb) on the host, as the reference's Scene::load / Scene::parse_mesh do
 * with tinygltf (src/scene/scene.cpp:48-315, 317-391), keeping what the
 * closest-point path needs: triangle geometry and where it is placed.
 *
 * Primitives: every meshes[i].primitives[j] in file order whose mode is
 * TRIANGLES, TRIANGLE_STRIP (triangles (k-2, k-1, k)) or TRIANGLE_FAN
 * ((0, k-1, k)), as parse_mesh converts them; other modes are skipped.
 * POSITION must be FLOAT VEC3; indices may be (U)BYTE, (U)SHORT or UINT, or
 * absent (0..count-1).  Vertices are in the mesh's own (object) space,
 * indices local to the primitive; vert_offsets / tri_offsets have
 * num_primitives + 1 entries, so the arrays feed cp_batch_create directly.
 *
 * Instances: every scene's root nodes, depth first, one instance per
 * primitive of each node's mesh, in the order Scene::load adds objects; world = parent * local with local the node's
 * "matrix" or T * R * S of its translation / rotation / scale.  (The
 * reference reads only "matrix", so it places TRS-only nodes at identity.)
 * Matrices are 4 x 4 row-major floats.
 *
 * Shading inputs (cp_gltf_shading): per vertex the NORMAL attribute,
 * aligned with the vertices and zero where a primitive has none or fewer
 * normals than positions (as parse_mesh pairs them, scene.cpp:304-307); per
 * primitive 8 floats, the material factors parse_mesh copies
 * (scene.cpp:286-299): baseColorFactor rgb, emissiveFactor rgb,
 * metallicFactor, roughnessFactor, with glTF's defaults (1, 0, 1, 1) and the
 * default material for a primitive without one.
 *
 * Texture inputs (cp_gltf_textures): per vertex TEXCOORD_0 (2 floats) and
 * TANGENT (4 floats: xyz, w), paired with the vertices as the normals are and
 * zero where absent or not FLOAT VEC2 / VEC4 (scene.cpp:188-265, 303-310); per
 * primitive the glTF texture index of its material's baseColorTexture,
 * emissiveTexture, metallicRoughnessTexture and normalTexture, -1 where
 * absent (Scene_Obj's *_tex, scene.cpp:294-302; an index past the file's
 * textures is refused); per texture its image ("source", -1 if absent or out
 * of range); per image its "uri" (empty if none) and "bufferView" (-1 if
 * none).  Image files are not decoded: a caller decodes them to RGBA8 for
 * cp_shade_scene_textures.
 *
 * Arrays returned by cp_gltf_* are owned by the handle and live until
 * cp_gltf_free.  Errors (unreadable file, malformed JSON, an accessor out of
 * its buffer, an index past its vertices) return CP_ERROR_INVALID_VALUE with
 * the reason in cp_last_error_string().  No CUDA device is needed.
 */
typedef struct cp_gltf cp_gltf;

CP_API cp_status cp_gltf_load(const char* path, cp_gltf** out);
CP_API void cp_gltf_free(cp_gltf* scene);
CP_API cp_status cp_gltf_primitives(const cp_gltf* scene, int32_t* num_primitives,
                                    const float** verts, const int32_t** tris,
                                    const int64_t** vert_offsets, const int64_t** tri_offsets);
CP_API cp_status cp_gltf_instances(const cp_gltf* scene, int32_t* num_instances,
                                   const int32_t** primitive, const float** world);
CP_API cp_status cp_gltf_shading(const cp_gltf* scene, int32_t* num_primitives, const float** normals,
                                 const float** materials);
CP_API cp_status cp_gltf_textures(const cp_gltf* scene, int32_t* num_primitives, const float** texcoords,
                                  const float** tangents, const int32_t** prim_tex, int32_t* num_textures,
                                  const int32_t** tex_image, int32_t* num_images, const char* const** image_uri,
                                  const int32_t** image_view);

/* ---- ray queries ----------------------------------------------------------- */

/*
 * Rays through the same BVH: the reference's own GPU query, `trace_ray`
 * (closest hit, src/shaders/rt/rt.rgen:257-270) and `visibility` (stop at the
 * first hit of a segment, rt.rgen:272-291), whose payload is the barycentrics,
 * the object and the primitive index (rtcommon.glsl:55-60, rt.rchit:11-16).
 * Boxes are tested by slabs (hit_bbox, rtcommon.glsl:242-251, made
 * conservative), triangles by Möller–Trumbore exactly as triangle_hit
 * (rtcommon.glsl:181-202) evaluates it in FP32.  The closest hit is the least
 * (t, triangle index) over every triangle the test accepts with t in
 * [tmin, tmax], so it does not depend on the traversal.
 */
typedef struct cp_ray_opts {
    float tmin;          /* hits count for t in [tmin, tmax] (the reference: [1e-5, 1e7]) */
    float tmax;          /* +inf allowed */
    float det_epsilon;   /* |det| <= det_epsilon is a miss; 0: only det == 0 (triangle_hit: 1e-5,
                            a scene-scale constant that rejects every triangle below ~3e-3 in size) */
    int32_t any_hit;     /* 1: stop at the first accepted hit (visibility); t and triangle are that hit's */
    int32_t sort_rays;   /* 1: walk the rays in the Hilbert order of their origins (outputs keep input order) */
    int32_t block_size;  /* threads per block: 32..256, multiple of 32; 0 = default */
} cp_ray_opts;

CP_API void cp_ray_opts_default(cp_ray_opts* opts);  /* [0, +inf], exact det test, closest hit, sorted, 256 */

CP_API cp_status cp_ray_workspace_size(const cp_mesh* mesh, int64_t n, const cp_ray_opts* opts,
                                       size_t* bytes);

/*
 * n rays (origins and directions: n x 3 floats, device; directions need not
 * be unit, t is in units of the direction's length).  tmax_per_ray (n floats,
 * may be NULL) lowers tmax per ray: segment ends, as visibility(a, b) uses.
 * Outputs (device, each may be NULL): out_t (n; +inf on a miss), out_tri (n;
 * -1 on a miss), out_uv (n x 2: weights u of vertex 1 and v of vertex 2; the
 * reference's barycentrics are (1 - u - v, u, v)).  workspace as cp_query.
 * n == 0 is a no-op.  Asynchronous on `stream`.
 */
CP_API cp_status cp_ray_query(const cp_mesh* mesh, const float* origins, const float* directions,
                              const float* tmax_per_ray, int64_t n, const cp_ray_opts* opts,
                              float* out_t, int32_t* out_tri, float* out_uv, void* workspace,
                              size_t workspace_bytes, cp_stream_t stream);

/*
 * cp_query for callers that must not allocate device memory while they run:
 * a render or simulation loop that forbids allocation after start-up (an
 * allocation can synchronise the device and stall a frame), a plugin whose
 * host owns all device memory, or code running while its own allocator holds
 * a lock.  Same arguments and results as cp_query, minus the workspace: the
 * scratch comes from a fixed 32 MiB device array inside the library
 * (cp_query_noalloc_scratch_bytes).  At most 1,048,576 queries per call with
 * sort_queries on (any count up to 2^31 - 1 with it off); a larger call
 * returns CP_ERROR_SCRATCH_TOO_SMALL with a message and launches nothing.
 * The runtime loads the array on a device lazily, at the first call made with
 * that device current, and the device holds it until the process exits: that
 * first call is the one that allocates (32 MiB) and can fail with
 * CP_ERROR_OUT_OF_MEMORY.  Make it at start-up — a call with nq == 0 (NULL
 * pointers allowed) loads the array and does nothing else — before the host
 * claims the rest of the device memory and before any stream capture.  After
 * that the call makes no cudaMalloc / cudaFree and no other allocation.  It
 * looks the array's address up on every call (cudaGetSymbolAddress), so it
 * stays valid across cudaDeviceReset.  All calls share the one array and find
 * the last call's contents in it (each call clears what must start at zero):
 * calls that overlap on the GPU (other streams, other threads) race and give
 * wrong results — keep them ordered on one stream.  This entry point has no
 * counterpart in the reference.
 */
CP_API cp_status cp_query_noalloc(const cp_mesh* mesh, const float* queries, int64_t nq,
                                  const cp_query_opts* opts, float* out_point, float* out_dist,
                                  int32_t* out_tri, float* out_bary, cp_stream_t stream);

/* Size in bytes of cp_query_noalloc's fixed scratch array. */
CP_API size_t cp_query_noalloc_scratch_bytes(void);

/*
 * Adjoint of the unsigned distance.  For each query i with upstream gradient
 * g_i = grad_dist[i], closest triangle t = tri[i] and barycentrics b = bary[i]:
 *   grad_queries[i]  = g_i (q_i - p_i) / d_i           (written; may be NULL)
 *   grad_verts[v_k] += -g_i b_k (q_i - p_i) / d_i      (accumulated atomically
 *                      for the three vertices of t; may be NULL)
 * with p_i = sum_k b_k v_k recomputed from the mesh and d_i = |q_i - p_i|;
 * d_i == 0 contributes zero.  The residual q_i - p_i is formed in float-float
 * from the triangle's vertices, so queries very close to the surface keep an
 * accurate direction.  bary may be NULL: the barycentrics of the closest point
 * on tri[i] are then recomputed exactly (float-float Voronoi regions) from
 * the query, which removes the FP32 rounding of cached weights.  The gradient with respect to the vertices
 * follows from the envelope theorem (the barycentrics are optimal, so their
 * own derivative drops out).  grad_verts is nv x 3 floats and is NOT cleared.
 * No counterpart in the reference, which has no differentiable path.
 */
CP_API cp_status cp_backward(const cp_mesh* mesh, const float* queries, const int32_t* tri,
                             const float* bary, const float* grad_dist, int64_t nq,
                             float* grad_queries, float* grad_verts, cp_stream_t stream);

/* ---- many meshes, one launch ---------------------------------------------- */

/*
 * Build one BVH per mesh for a set of meshes in one batched build: one sort
 * over (mesh id, Morton code) keys, one hierarchy and refit pass, one collapse.
 * Takes the role of the reference's BLAS-per-mesh plus TLAS build
 * (src/vk/vulkan.cpp:777-856; src/gpurt.cpp:220-241).
 *   verts          all meshes' vertices back to back, total_v x 3 floats
 *   vert_offsets   HOST array of nmeshes + 1 int64 vertex offsets
 *   tris           all meshes' triangles back to back, indices LOCAL to each mesh
 *   tri_offsets    HOST array of nmeshes + 1 int64 triangle offsets
 * Every mesh needs at least one triangle.  Synchronises `stream`.
 */
CP_API cp_status cp_batch_create(const float* verts, const int64_t* vert_offsets,
                                 const int32_t* tris, const int64_t* tri_offsets, int32_t nmeshes,
                                 const cp_build_opts* opts, cp_stream_t stream, cp_batch** out);

/* cp_batch_create with a leaf size per mesh: leaf_sizes (HOST, nmeshes values
 * in 1..15) replaces opts->leaf_size mesh by mesh, in the same single build
 * (each mesh's leaves hold at most its own count; the wide nodes and the one
 * persistent query launch are shared).  cp_batch_autotune picks them per
 * size class.  The reference's per-mesh BLAS builds take no such parameter
 * (src/vk/vulkan.cpp:881-936). */
CP_API cp_status cp_batch_create_leaves(const float* verts, const int64_t* vert_offsets,
                                        const int32_t* tris, const int64_t* tri_offsets, int32_t nmeshes,
                                        const int32_t* leaf_sizes, const cp_build_opts* opts,
                                        cp_stream_t stream, cp_batch** out);

CP_API cp_status cp_batch_destroy(cp_batch* batch);

/* Per-mesh root info: number of meshes and wide-node count of the whole batch. */
CP_API cp_status cp_batch_info(const cp_batch* batch, int32_t* nmeshes, int64_t* num_wide_nodes,
                               int64_t* num_triangles, int32_t* stack_bound);

CP_API cp_status cp_batch_query_workspace_size(const cp_batch* batch, int64_t nq,
                                               const cp_query_opts* opts, size_t* bytes);

/*
 * Query every mesh of a batch in one persistent, work-stealing launch.
 * Queries of mesh m are queries[q_offsets[m] .. q_offsets[m+1]) (q_offsets is a
 * HOST array of nmeshes + 1 int64).  out_tri holds triangle indices local to
 * each mesh.  Outputs as in cp_query.  With use_graph != 0 the launch sequence
 * is captured into a CUDA graph on first use with these pointers and sizes
 * and replayed on later calls (the workspace must then be given and stay the
 * same).
 */
CP_API cp_status cp_batch_query(cp_batch* batch, const float* queries, const int64_t* q_offsets,
                                const cp_query_opts* opts, float* out_point, float* out_dist,
                                int32_t* out_tri, float* out_bary, void* workspace,
                                size_t workspace_bytes, int32_t use_graph, cp_stream_t stream);

/* ---- instanced scenes ------------------------------------------------------ */

/*
 * A scene of instances of a batch's meshes, each placed by its own 3 x 4
 * object-to-world matrix: the reference's TLAS over transformed BLAS instances
 * (Accel::recreate(blas, T), src/vk/vulkan.cpp:777-856; one model matrix per
 * object, src/rt/rt.cpp:31-45).  A top-level BVH over the instances' world
 * boxes is built on the device; a query walks it closest first and each
 * instance's mesh BVH, and the winner is re-evaluated in float-float in world
 * space from the exact object-space triangle and the instance matrix.
 *   batch               the meshes; it must outlive the scene
 *   instance_mesh       HOST array, n_instances mesh ids in [0, nmeshes)
 *   instance_transform  HOST array, n_instances x 12 floats, row-major 3 x 4
 *                       [M | t] taking object to world coordinates
 * Any finite affine matrix is accepted (non-finite: CP_ERROR_INVALID_VALUE).
 * Similarities (rotation or reflection, uniform scale, translation: M^T M =
 * s^2 I within 1e-5 s^2) share the batch mesh's BVH, walked in object space;
 * any other matrix (non-uniform scale, shear, singular) gets a world-space
 * copy of its mesh with its own BVH, built here, whose triangles keep the
 * mesh's local indices.  Distances and points are in world units.
 * Synchronises `stream`.
 */
CP_API cp_status cp_scene_create(const cp_batch* batch, const int32_t* instance_mesh,
                                 const float* instance_transform, int32_t n_instances,
                                 cp_stream_t stream, cp_scene** out);

/*
 * New transforms for every instance (same meshes): re-derives the instance
 * frames, rebuilds the world-space copies and the top level.  Synchronises
 * `stream`.  A non-finite matrix is refused with the scene unchanged; a
 * failure after that (out of memory) leaves the scene unusable until an
 * update succeeds (cp_scene_query then returns CP_ERROR_INVALID_VALUE).
 */
CP_API cp_status cp_scene_update(cp_scene* scene, const float* instance_transform, cp_stream_t stream);

/*
 * New transforms for every instance, keeping the trees' topology: the
 * world-space copies are re-baked and the top level's instance boxes
 * recomputed, and both BVHs are refit bottom-up (boxes and triangle records)
 * instead of rebuilt — the reference's TLAS update as against its BLAS
 * rebuild (src/gpurt.h:63-65, src/gpurt.cpp:220-241).  Answers are those of a
 * rebuild; a tree refit after large motions is slower to walk.  An instance
 * that changes kind (similarity <-> general affine) changes the copies, so
 * then this rebuilds as cp_scene_update does.  Synchronises `stream`; errors
 * as cp_scene_update.
 */
CP_API cp_status cp_scene_refit(cp_scene* scene, const float* instance_transform, cp_stream_t stream);

CP_API cp_status cp_scene_destroy(cp_scene* scene);

CP_API cp_status cp_scene_query_workspace_size(const cp_scene* scene, int64_t nq,
                                               const cp_query_opts* opts, size_t* bytes);

/*
 * Closest point on the scene for each world-space query.  out_instance is the
 * instance, out_tri the triangle local to that instance's mesh, out_bary the
 * weights of its b and c vertices; any output may be NULL.  Options as in
 * cp_query (sort_queries orders the queries along a Morton curve of the
 * scene's world box; the traversal options are ignored).  Workspace as in
 * cp_query (NULL = stream-ordered pool).
 */
CP_API cp_status cp_scene_query(const cp_scene* scene, const float* queries, int64_t nq,
                                const cp_query_opts* opts, float* out_point, float* out_dist,
                                int32_t* out_instance, int32_t* out_tri, float* out_bary,
                                void* workspace, size_t workspace_bytes, cp_stream_t stream);

CP_API cp_status cp_scene_ray_workspace_size(const cp_scene* scene, int64_t n, const cp_ray_opts* opts,
                                             size_t* bytes);

/*
 * Closest (or, with opts->any_hit, some) hit of each world-space ray over the
 * scene: the reference's trace_ray / visibility against its TLAS
 * (src/shaders/rt/rt.rgen:257-291; src/vk/vulkan.cpp:777-856).  Options and
 * tmax_per_ray as in cp_ray_query.  A similarity instance is hit in object
 * space (o' = A (o - t), d' = A d: the hit parameter t is the world one), a
 * general one on its world-space copy.  Outputs (each may be NULL): t (+inf on
 * a miss), instance (-1), triangle local to the instance's mesh (-1), weights
 * (u, v) of its b and c vertices.  The closest hit is the least (t, instance,
 * triangle).
 */
CP_API cp_status cp_scene_ray_query(const cp_scene* scene, const float* origins, const float* directions,
                                    const float* tmax_per_ray, int64_t n, const cp_ray_opts* opts,
                                    float* out_t, int32_t* out_instance, int32_t* out_tri, float* out_uv,
                                    void* workspace, size_t workspace_bytes, cp_stream_t stream);

/* ---- path tracer -------------------------------------------------------------
 *
 * The reference's ray-generation shader (src/shaders/rt/rt.rgen:567-677; its
 * integrators :291-548, materials src/shaders/rt/rtcommon.glsl:253-369,
 * ReSTIR src/shaders/rt/restir.glsl:17-35) and tone mapping
 * (src/shaders/tonemap.frag) as CUDA kernels over this library's BVH, writing
 * a device image buffer instead of a swapchain image.  Replaces RTPipe::trace
 * (src/vk/rt.cpp:346-394) and the tonemap pass.  Scenes are world-space
 * triangles with per-vertex normals and a material per object: factors,
 * each of which a texture may replace, and an optional normal map
 * (cp_shade_scene_textures); an object with an emission factor above zero
 * is a light, and its triangles must be contiguous.  What GLSL leaves to the
 * implementation is fixed: sin / cos / pow / exp are the library's own
 * routines, texture() is the library's own bilinear blend of sRGB-decoded
 * texels, and the pixel seed is tea(pixel, seed) where the shader reads the
 * clock (rt.rgen:569).
 */
typedef struct cp_shade_scene cp_shade_scene;

typedef struct {
    float eye[3], right[3], up[3], fwd[3]; /* orthonormal camera frame */
    float tan_half_y;                      /* tan of half the vertical field of view */
    float aspect;                          /* width / height */
    int32_t width, height;                 /* pixels; row 0 at the top */
} cp_shade_camera;

typedef struct {
    float clear[3];             /* colour of a primary miss */
    float env[3];               /* environment light of a secondary miss */
    int32_t samples;            /* samples per pixel per frame (> 0) */
    int32_t max_depth;          /* bounces (>= 0) */
    int32_t qmc;                /* 1: Hammersley jitter over samples x max_frame */
    int32_t integrator;         /* 0 direct, 1 material sampling, 2 MIS, 3 ReSTIR direct only, 4 ReSTIR */
    int32_t brdf;               /* 0 Blinn-Phong, 1 GGX */
    int32_t use_rr;             /* Russian roulette */
    int32_t use_metalness;
    int32_t frame;              /* 0: write the frame; > 0: blend into the image by 1 / (frame + 1) */
    int32_t max_frame;
    int32_t new_samples;        /* ReSTIR light candidates per pixel */
    int32_t temporal_multiplier;
    int32_t use_temporal;       /* ReSTIR: reuse the previous frame's reservoirs */
    int32_t debug_view;         /* 1, 2, 3: the previous frame's position, normal, albedo, reprojected */
    uint32_t seed;
    int32_t use_normal_map;     /* 1: bend the shading normal by an object's normal texture */
} cp_shade_params;

/* A ReSTIR reservoir (restir.glsl:1-8), 48 bytes. */
typedef struct {
    float pos[3], normal[3], emissive[3];
    float w_sum, w;
    uint32_t n_seen;
} cp_shade_reservoir;

/* Build a scene: DEVICE arrays verts and normals (nt x 3 vertices x xyz),
 * obj (nt, the object of each triangle), albedo and emissive (nobj x 3),
 * metal_rough (nobj x 2).  The scene copies them and builds a 4-wide BVH over
 * the triangles.  Synchronises `stream`.  Replaces the scene upload and
 * acceleration-structure build of src/gpurt.cpp:220-241. */
CP_API cp_status cp_shade_scene_create(const float* verts, const float* normals, const int32_t* obj, int64_t nt,
                                       const float* albedo, const float* emissive, const float* metal_rough,
                                       int32_t nobj, cp_stream_t stream, cp_shade_scene** out);
CP_API cp_status cp_shade_scene_destroy(cp_shade_scene* scene);

/* Textures of a scene (replacing any it had): texcoords (DEVICE, nt x 3
 * vertices x (u, v), may be NULL: all zero), tangents (DEVICE, nt x 3
 * vertices x (xyz, w), the tangent being xyz * w, may be NULL: only normal
 * maps use them), ntex RGBA8 images in texels (DEVICE, concatenated, row 0
 * first, colour sRGB-encoded as in the reference's R8G8B8A8_SRGB images,
 * rt.cpp:439), their sizes tex_size (HOST, ntex x (width, height)), and
 * obj_tex (HOST, nobj x 4: for each object the texture that replaces its
 * albedo, emission, metal / roughness, or gives its normal map; -1 none)
 * (Scene_Obj's *_tex, rt.rgen:97-129).  Every index is checked on the host.
 * Sampling is the library's texture(): the four texels around
 * (u mod 1) w - 1/2, (v mod 1) h - 1/2 at level 0, decoded from sRGB,
 * blended bilinearly with repeat addressing.  Synchronises `stream`. */
CP_API cp_status cp_shade_scene_textures(cp_shade_scene* scene, const float* texcoords, const float* tangents,
                                         int32_t ntex, const int32_t* tex_size, const uint8_t* texels,
                                         const int32_t* obj_tex, cp_stream_t stream);
/* Number of lights (emissive objects with triangles). */
CP_API cp_status cp_shade_scene_lights(const cp_shade_scene* scene, int32_t* n_lights);

/* Render one frame into `image` (DEVICE, height x width x 3 floats; read when
 * params->frame > 0).  gbuf (DEVICE, height x width x 9, may be NULL)
 * receives each pixel's first hit of sample 0: position, shading normal,
 * albedo (zeros on a miss).  ReSTIR's temporal state, each may be NULL:
 * prev_pv (HOST, 16 floats, row-major world-to-clip matrix of the previous
 * frame), prev_gbuf (DEVICE, the previous frame's gbuf), prev_res (DEVICE,
 * height x width reservoirs of the previous frame), out_res (DEVICE, this
 * frame's reservoirs, written by integrators 3 and 4).  Every integrator but
 * material sampling needs a light.  Asynchronous on `stream`. */
CP_API cp_status cp_shade_render(const cp_shade_scene* scene, const cp_shade_camera* camera,
                                 const cp_shade_params* params, float* image, float* gbuf, const float* prev_pv,
                                 const float* prev_gbuf, const cp_shade_reservoir* prev_res,
                                 cp_shade_reservoir* out_res, cp_stream_t stream);

/* tonemap.frag per colour component, n values (DEVICE in and out): type 0
 * Hable's filmic curve scaled to white at 11.2, 1 exponential
 * 1 - exp(-c exposure), each followed by pow(., 1 / gamma); 2 unchanged. */
CP_API cp_status cp_shade_tonemap(int32_t type, float exposure, float gamma, int64_t n, const float* in,
                                  float* out, cp_stream_t stream);

/* ---- autotuner ------------------------------------------------------------ */

/*
 * Pick branching, leaf size, block size and traversal kernel (warp packet,
 * unseeded or seeded in chunks of 4 packets, or per-thread with a short-stack
 * depth) for a size class by timing candidate builds and queries on the given
 * mesh and queries (device arrays; pass the real query set or one of the same
 * density: packet coherence depends on it).  The size class is
 * (floor(log2(nt)), floor(log2(nq))).  The winner is written to *best_build /
 * *best_query and, when cache_path is not NULL, stored in that text file (one
 * "tri_class query_class branching leaf block stack ms seed_chunk" line per
 * class pair and branching, stack 0 = packet); a cached class is returned
 * without timing.  If best_build->branching is 2, 4 or 8 on entry, only that
 * branching is tried.  Synchronous.
 */
CP_API cp_status cp_autotune(const float* verts, int64_t nv, const int32_t* tris, int64_t nt,
                             const float* queries, int64_t nq, const char* cache_path,
                             cp_build_opts* best_build, cp_query_opts* best_query);

/* The batched form tuned per size class: meshes are grouped by
 * cp_size_class(triangles), and each class gets a leaf size in {1, 2, 4, 8}.
 * One build and one launch serve every class, so each choice is timed on the
 * whole batch (DEVICE arrays as for cp_batch_create and cp_batch_query;
 * offsets HOST): first the best uniform size, then one class at a time, most
 * queries first, tries the others, a change kept when the batch gets at least
 * 2% faster.  Writes leaf_sizes (HOST, nmeshes) for cp_batch_create_leaves,
 * and the query options (the packet traversal's defaults).  With cache_path,
 * results are read from and written to the autotuner's cache file (lines
 * marked B, keyed by triangle class, the class's mean queries per mesh and
 * branching); a batch whose classes are all there is not timed.  Synchronous. */
CP_API cp_status cp_batch_autotune(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                                   const int64_t* tri_offsets, int32_t nmeshes, const float* queries,
                                   const int64_t* q_offsets, int32_t branching, const char* cache_path,
                                   int32_t* leaf_sizes, cp_query_opts* best_query);

/* ---- saved BVHs ------------------------------------------------------------ */

/* Write a built mesh (its BVH, triangle records and the arrays refit needs) to
 * a file, and read one back as a new mesh that queries, refits and exports as
 * the original does, without a build.  The file holds raw device arrays in
 * this library's layout (host byte order), behind a header with the build's
 * parameters and counts.  cp_mesh_load checks the whole file on the host
 * before anything reaches the GPU — its size against the header, every index
 * a kernel follows, that each wide tree is a tree within its depth bound — and
 * refuses a damaged or foreign file with CP_ERROR_INVALID_VALUE and a message.
 * Both are synchronous (cp_mesh_save waits for the device).  The reference
 * keeps nothing between runs (its only file output is the image,
 * src/gpurt.cpp:258-262). */
CP_API cp_status cp_mesh_save(const cp_mesh* mesh, const char* path);
CP_API cp_status cp_mesh_load(const char* path, cp_stream_t stream, cp_mesh** out);

/* A batch (cp_batch_create*) written and read back the same way: the file
 * holds every mesh's tree, leaf size, frame and offsets; the load checks the
 * whole file on the host (each mesh's tree within its triangles) before
 * anything reaches the GPU.  cp_batch_load also reads a one-mesh file as a
 * batch of one; cp_mesh_load refuses a batch file. */
CP_API cp_status cp_batch_save(const cp_batch* batch, const char* path);
CP_API cp_status cp_batch_load(const char* path, cp_stream_t stream, cp_batch** out);

/* Size class used by the autotuner cache: floor(log2(num_triangles)). */
CP_API int32_t cp_size_class(int64_t num_triangles);

/* ---- inspection (tests compare these with the CPU restatement bit for bit) -- */

/*
 * Copy the build's intermediate arrays to HOST memory (any pointer may be
 * NULL): sorted 64-bit Morton keys and triangle order (nt each), the binary
 * hierarchy's left/right children (nt-1 each; ids >= nt-1 are leaves
 * nt-1+k for sorted position k), parent (2nt-1), the leaf-cluster flag per
 * binary node (2nt-1 bytes) and, per wide node, the binary node it was made
 * from.  Synchronous.
 */
CP_API cp_status cp_mesh_export_build(const cp_mesh* mesh, uint64_t* keys, int32_t* order,
                                      int32_t* left, int32_t* right, int32_t* parent,
                                      uint8_t* cluster, int32_t* wide_src);

/*
 * Copy the wide nodes to HOST memory: num_wide_nodes * branching * 6 floats of
 * child boxes (lo x, hi x, lo y, hi y, lo z, hi z per child), child refs and
 * child counts (num_wide_nodes * branching int32 each; count 0 = inner child,
 * count > 0 = leaf of `count` triangles starting at sorted position `ref`,
 * count -1 = empty slot).  Synchronous.
 */
CP_API cp_status cp_mesh_export_wide(const cp_mesh* mesh, float* boxes, int32_t* refs,
                                     int32_t* counts);

/* The same two exports for a batch: one build over every mesh's triangles
 * (keys carry the mesh id in their high bits, so each mesh's triangles are
 * one sorted run and one subtree).  No counterpart in the reference (its
 * acceleration structures are opaque driver objects, src/vk/vulkan.cpp:777-936). */
CP_API cp_status cp_batch_export_build(const cp_batch* batch, uint64_t* keys, int32_t* order,
                                       int32_t* left, int32_t* right, int32_t* parent,
                                       uint8_t* cluster, int32_t* wide_src);
CP_API cp_status cp_batch_export_wide(const cp_batch* batch, float* boxes, int32_t* refs,
                                      int32_t* counts);

#ifdef __cplusplus
}
#endif

#endif /* GPURT_CPQ_H */
