/*
 * cpq_oracle.h — ORACLE: test infrastructure only.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library.  It is the checker for the GPU closest-point engine,
 * never part of it.
 *
 * Parity is UNPINNED against the reference: the reference's closest-point
 * code (the FCPW-GPU branch of TheNumbat/GPU-RT, README.md:6-8) is not in the
 * mounted tree, and FCPW itself (github.com/rohan-sawhney/fcpw) is neither
 * vendored nor version-pinned.  What this file restates instead:
 *   - exact point-triangle closest point by Voronoi regions (Ericson 2005,
 *     "Real-Time Collision Detection", section 5.1.5), in FP64, with the
 *     triangle index tie rule "smallest index wins";
 *   - the Morton-code LBVH of Karras 2012 ("Maximizing Parallelism in the
 *     Construction of BVHs, Octrees, and k-d Trees"), SAH leaf collapse
 *     (MacDonald and Booth 1990; surface area as in BBox::surface_area,
 *     src/lib/bbox.h:55-59) and a fixed-depth collapse to 2/4/8-wide nodes,
 *     in FP32 with the exact operation order the GPU build uses, so codes and
 *     topology can be compared bit for bit;
 *   - the closest-first stack traversal in FP32 (the timed CPU baseline).
 * Hand-computed known answers pin the FP64 routine (tests/golden).
 */
#ifndef CPQ_ORACLE_H
#define CPQ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* FP64 closest point on triangle (a, b, c) to p.  Returns the squared
 * distance; writes the closest point and barycentrics (weights of a, b, c). */
double orc_point_tri_f64(const double* p, const double* a, const double* b, const double* c,
                         double* closest, double* bary);

/* FP64 brute force over every triangle.  out_d2 = squared distance, out_tri =
 * smallest index among exact FP64 ties, out_p (nq x 3), out_bary (nq x 3). */
void orc_brute_f64(const float* verts, int64_t nv, const int32_t* tris, int64_t nt,
                   const float* q, int64_t nq, double* out_d2, int32_t* out_tri, double* out_p,
                   double* out_bary, int nthreads);

/* Same answers as orc_brute_f64, through an FP64 bounding-volume search over
 * a balanced tree of its own (Morton order, median split); used where the
 * brute force would take too long.  Returns 0 on success. */
int orc_exact_f64(const float* verts, int64_t nv, const int32_t* tris, int64_t nt, const float* q,
                  int64_t nq, double* out_d2, int32_t* out_tri, double* out_p, double* out_bary,
                  int nthreads);

/* orc_exact_f64 with FP64 query points (central finite differences). */
int orc_exact_f64_dq(const float* verts, int64_t nv, const int32_t* tris, int64_t nt,
                     const double* q, int64_t nq, double* out_d2, int32_t* out_tri, int nthreads);

/* FP64 squared distance from query i to the given triangle tri[i] (used to
 * confirm that a differing triangle index is a tie), and optionally the
 * barycentrics (nq x 3) of the closest point on that triangle. */
void orc_point_tri_batch_f64(const float* verts, const int32_t* tris, const float* q,
                             const int32_t* tri, int64_t nq, double* out_d2, double* out_bary);

/* ---- FP32 restatement of the LBVH build and traversal ------------------------ */

typedef struct orc_tree {
    int64_t nt;           /* triangles */
    int32_t nmeshes;      /* 1 for a single mesh */
    int32_t branching;    /* K */
    int32_t leaf_size;
    int32_t collapse;
    int32_t max_wide_depth;
    int32_t stack_bound;
    int64_t num_wide;
    int64_t num_leaves;
    /* binary tree: internal 0..nt-2, leaf of sorted position k = nt-1+k */
    uint64_t* keys;       /* nt sorted keys */
    int32_t* order;       /* nt: triangle (global index) at each sorted position */
    int32_t* left;        /* nt-1 */
    int32_t* right;       /* nt-1 */
    int32_t* parent;      /* 2nt-1 */
    int32_t* first;       /* 2nt-1: first sorted position under the node */
    int32_t* last;        /* 2nt-1 */
    float* box;           /* 2nt-1 x 6: lo x, lo y, lo z, hi x, hi y, hi z */
    float* cost;          /* 2nt-1: SAH cost x half area */
    uint8_t* cluster;     /* 2nt-1: 1 if the node is a leaf of the collapsed tree */
    int32_t* mesh_root;   /* nmeshes: binary root node of each mesh */
    int32_t* wide_root;   /* nmeshes: wide root node of each mesh */
    /* wide tree, num_wide nodes */
    int32_t* wide_src;    /* binary node each wide node was made from */
    float* wide_box;      /* num_wide x 6 x K: per node, K lo x, K hi x, K lo y, K hi y, K lo z, K hi z */
    int32_t* wide_ref;    /* num_wide x K */
    int32_t* wide_count;  /* num_wide x K: 0 inner, >0 leaf, -1 empty */
    float* tri_verts;     /* nt x 9: triangle vertices in sorted order */
    int32_t* mesh_of_tri; /* nt (sorted order): mesh id */
    int32_t* tri_local;   /* nt (sorted order): triangle index local to its mesh */
} orc_tree;

/* Build over one mesh or a batch: vert_offsets / tri_offsets hold nmeshes + 1
 * entries (NULL for a single mesh); tri indices are local to each mesh.
 * Returns 0 on success. */
int orc_build(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
              const int64_t* tri_offsets, int32_t nmeshes, int64_t nv_total, int64_t nt_total,
              int32_t branching, int32_t leaf_size, int32_t collapse, float c_node, float c_tri,
              orc_tree** out);
/* orc_build with a leaf size per mesh (mesh_leaf: nmeshes values in 1..15;
 * leaf_size is then ignored), as cp_batch_create_leaves builds. */
int orc_build_leaves(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                     const int64_t* tri_offsets, int32_t nmeshes, int64_t nv_total, int64_t nt_total,
                     int32_t branching, const int32_t* mesh_leaf, int32_t collapse, float c_node, float c_tri,
                     orc_tree** out);
void orc_tree_free(orc_tree* t);

/* FP32 closest-first traversal of the wide tree (the CPU baseline).
 * q_mesh[i] gives the mesh of query i (NULL: mesh 0).  out_tri is local to
 * the mesh.  node_visits / tri_tests count per query (may be NULL).
 * Returns elapsed wall seconds. */
double orc_query_f32(const orc_tree* t, const float* q, const int32_t* q_mesh, int64_t nq,
                     float* out_d, int32_t* out_tri, float* out_p, float* out_bary,
                     int32_t* node_visits, int32_t* tri_tests, int nthreads);

/* Adjoint restated in FP64 (the analytic reference gradient): for each query,
 * grad_q = g (q - p) / d and grad_verts[v_k] += -g b_k (q - p) / d, with p and
 * d recomputed in FP64 from (tri, bary). */
void orc_backward_f64(const float* verts, int64_t nv, const int32_t* tris, const float* q,
                      const int32_t* tri, const double* bary, const double* grad_d, int64_t nq,
                      double* grad_q, double* grad_verts);

/* FP64 brute force over triangles given by FP64 vertices (geometry placed by
 * an FP64 transform, e.g. instances): out_d2, out_tri, out_p (3 per query). */
void orc_brute_f64_dv(const double* verts, const int32_t* tris, int64_t nt, const float* q, int64_t nq,
                      double* out_d2, int32_t* out_tri, double* out_p, int nthreads);

/* Rays, brute force over every triangle.  The hit test is the reference's
 * triangle_hit (Möller–Trumbore, src/shaders/rt/rtcommon.glsl:181-202): in
 * FP32 (orc_ray_brute_f32) operation for operation as the GPU evaluates it,
 * or in FP64 (orc_ray_brute_f64).  |det| <= det_eps is a miss; a hit counts
 * for t in [tmin, min(tmax, tmax_per_ray[i])] (tmax_per_ray may be NULL); the
 * answer is the least (t, triangle index).  Misses give t = +inf, tri = -1,
 * uv = (0, 0).  Returns elapsed wall seconds. */
double orc_ray_brute_f32(const float* verts, const int32_t* tris, int64_t nt, const float* orig,
                         const float* dir, const float* tmax_per_ray, int64_t n, float tmin,
                         float tmax, float det_eps, float* out_t, int32_t* out_tri, float* out_uv,
                         int nthreads);
double orc_ray_brute_f64(const float* verts, const int32_t* tris, int64_t nt, const float* orig,
                         const float* dir, const float* tmax_per_ray, int64_t n, double tmin,
                         double tmax, double det_eps, double* out_t, int32_t* out_tri,
                         double* out_uv, int nthreads);

/* FP64 closest hit of every ray over FP64 vertices (no det epsilon): the
 * truth for rays through instanced scenes, whose world vertices are the FP32
 * object vertices through FP32 matrices evaluated in FP64. */
void orc_ray_brute_f64_dv(const double* verts, const int32_t* tris, int64_t nt, const float* orig,
                          const float* dir, int64_t n, double tmin, double tmax, double* out_t,
                          int32_t* out_tri, double* out_uv, int nthreads);

#ifdef __cplusplus
}
#endif

#endif
