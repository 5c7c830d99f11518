/*
 * cpq_oracle.c — ORACLE: test infrastructure only (see cpq_oracle.h).
 *
 * Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg.  Compiled WITHOUT fast-math and with -ffp-contract=off, so every FP32
 * expression rounds exactly as written and the GPU build, which spells out
 * the same operations with round-to-nearest intrinsics, produces the same
 * Morton codes, topology and boxes bit for bit.  (The reference itself builds
 * with -ffast-math, CMakeLists.txt:78-80; the oracle must not.)
 *
 * Parity unpinned: no reference code, test or golden vector exists for this
 * path in the mounted tree (README.md:6-8 points to an absent branch).
 */
#define _POSIX_C_SOURCE 200809L
#include "cpq_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ===================================================================== */
/* small vector helpers                                                   */
/* ===================================================================== */

static inline void sub3d(double* r, const double* a, const double* b) {
    r[0] = a[0] - b[0];
    r[1] = a[1] - b[1];
    r[2] = a[2] - b[2];
}
static inline double dot3d(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* ===================================================================== */
/* FP64 exact point-triangle closest point                                */
/* ===================================================================== */

/* Closest point on segment a + t*ab, t in [0,1]. */
static double seg_f64(const double* p, const double* a, const double* ab, double* t_out) {
    double ap[3];
    sub3d(ap, p, a);
    double l = dot3d(ab, ab);
    double t = 0.0;
    if (l > 0.0) {
        t = dot3d(ap, ab) / l;
        t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
    }
    double r[3] = {ap[0] - t * ab[0], ap[1] - t * ab[1], ap[2] - t * ab[2]};
    *t_out = t;
    return dot3d(r, r);
}

/* Zero-area triangle: the closest point of the three edges (ab, bc, ac; the
 * first wins a tie). */
static double degenerate_f64(const double* p, const double* a, const double* b, const double* c,
                             double* bary) {
    double ab[3], bc[3], ac[3], t0, t1, t2;
    sub3d(ab, b, a);
    sub3d(bc, c, b);
    sub3d(ac, c, a);
    double d0 = seg_f64(p, a, ab, &t0);
    double d1 = seg_f64(p, b, bc, &t1);
    double d2 = seg_f64(p, a, ac, &t2);
    if (d0 <= d1 && d0 <= d2) {
        bary[0] = 1.0 - t0; bary[1] = t0; bary[2] = 0.0;
        return d0;
    }
    if (d1 <= d2) {
        bary[0] = 0.0; bary[1] = 1.0 - t1; bary[2] = t1;
        return d1;
    }
    bary[0] = 1.0 - t2; bary[1] = 0.0; bary[2] = t2;
    return d2;
}

/* Voronoi-region closest point (Ericson 2005, section 5.1.5): classify p
 * against the vertex, edge and face regions of the triangle with six dot
 * products, then project onto the feature that owns the region. */
double orc_point_tri_f64(const double* p, const double* a, const double* b, const double* c,
                         double* closest, double* bary) {
    double ab[3], ac[3], ap[3], n[3], w[3];
    sub3d(ab, b, a);
    sub3d(ac, c, a);
    n[0] = ab[1] * ac[2] - ab[2] * ac[1];
    n[1] = ab[2] * ac[0] - ab[0] * ac[2];
    n[2] = ab[0] * ac[1] - ab[1] * ac[0];
    double d2v;
    if (dot3d(n, n) == 0.0) {
        d2v = degenerate_f64(p, a, b, c, w);
    } else {
        sub3d(ap, p, a);
        double d1 = dot3d(ab, ap), d2 = dot3d(ac, ap);
        if (d1 <= 0.0 && d2 <= 0.0) {
            w[0] = 1; w[1] = 0; w[2] = 0;
        } else {
            double bp[3];
            sub3d(bp, p, b);
            double d3 = dot3d(ab, bp), d4 = dot3d(ac, bp);
            double vc = d1 * d4 - d3 * d2;
            double cp[3];
            sub3d(cp, p, c);
            double d5 = dot3d(ab, cp), d6 = dot3d(ac, cp);
            double vb = d5 * d2 - d1 * d6;
            double va = d3 * d6 - d5 * d4;
            if (d3 >= 0.0 && d4 <= d3) {
                w[0] = 0; w[1] = 1; w[2] = 0;
            } else if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
                double t = d1 / (d1 - d3);
                w[0] = 1.0 - t; w[1] = t; w[2] = 0;
            } else if (d6 >= 0.0 && d5 <= d6) {
                w[0] = 0; w[1] = 0; w[2] = 1;
            } else if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
                double t = d2 / (d2 - d6);
                w[0] = 1.0 - t; w[1] = 0; w[2] = t;
            } else if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0) {
                double t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
                w[0] = 0; w[1] = 1.0 - t; w[2] = t;
            } else {
                double s = va + vb + vc;
                double v = vb / s, ww = vc / s;
                w[0] = 1.0 - v - ww; w[1] = v; w[2] = ww;
            }
        }
        /* squared distance measured from the vertex that owns the region keeps
         * the difference small and exact where the feature is a vertex */
        double r[3];
        for (int k = 0; k < 3; ++k)
            r[k] = (p[k] - a[k]) - (w[1] * ab[k] + w[2] * ac[k]);
        d2v = dot3d(r, r);
    }
    for (int k = 0; k < 3; ++k) {
        double ck = a[k] + w[1] * (b[k] - a[k]) + w[2] * (c[k] - a[k]);
        if (closest) closest[k] = ck;
    }
    if (bary) {
        bary[0] = w[0];
        bary[1] = w[1];
        bary[2] = w[2];
    }
    return d2v;
}

static inline void load_tri_f64(const float* verts, const int32_t* tris, int64_t t, double* a,
                                double* b, double* c) {
    const int32_t* ix = tris + 3 * t;
    for (int k = 0; k < 3; ++k) {
        a[k] = verts[3 * (int64_t)ix[0] + k];
        b[k] = verts[3 * (int64_t)ix[1] + k];
        c[k] = verts[3 * (int64_t)ix[2] + k];
    }
}

/* ===================================================================== */
/* thread pool helper: run fn(ctx, begin, end) over [0, n) in chunks      */
/* ===================================================================== */

typedef void (*range_fn)(void* ctx, int64_t begin, int64_t end);
typedef struct {
    range_fn fn;
    void* ctx;
    int64_t n, chunk;
    atomic_llong next;
} pool_job;

static void* pool_worker(void* arg) {
    pool_job* job = (pool_job*)arg;
    for (;;) {
        int64_t b = atomic_fetch_add(&job->next, job->chunk);
        if (b >= job->n) break;
        int64_t e = b + job->chunk < job->n ? b + job->chunk : job->n;
        job->fn(job->ctx, b, e);
    }
    return NULL;
}

static void parallel_for(int64_t n, int64_t chunk, int nthreads, range_fn fn, void* ctx) {
    if (n <= 0) return;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pool_job job;
    job.fn = fn;
    job.ctx = ctx;
    job.n = n;
    job.chunk = chunk < 1 ? 1 : chunk;
    atomic_init(&job.next, 0);
    pthread_t th[256];
    int started = 0;
    for (int i = 1; i < nthreads; ++i)
        if (pthread_create(&th[started], NULL, pool_worker, &job) == 0) started++;
    pool_worker(&job);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ===================================================================== */
/* FP64 brute force                                                       */
/* ===================================================================== */

typedef struct {
    const float *verts, *q;
    const int32_t* tris;
    int64_t nt;
    double *out_d2, *out_p, *out_bary;
    int32_t* out_tri;
} brute_ctx;

static void brute_range(void* vctx, int64_t b, int64_t e) {
    brute_ctx* c = (brute_ctx*)vctx;
    for (int64_t i = b; i < e; ++i) {
        double p[3] = {c->q[3 * i], c->q[3 * i + 1], c->q[3 * i + 2]};
        double best = INFINITY, bp[3] = {0, 0, 0}, bb[3] = {0, 0, 0};
        int32_t bt = -1;
        for (int64_t t = 0; t < c->nt; ++t) {
            double A[3], B[3], C[3], cp[3], w[3];
            load_tri_f64(c->verts, c->tris, t, A, B, C);
            double d2 = orc_point_tri_f64(p, A, B, C, cp, w);
            if (d2 < best) {
                best = d2;
                bt = (int32_t)t;
                memcpy(bp, cp, sizeof bp);
                memcpy(bb, w, sizeof bb);
            }
        }
        c->out_d2[i] = best;
        c->out_tri[i] = bt;
        if (c->out_p) memcpy(c->out_p + 3 * i, bp, sizeof bp);
        if (c->out_bary) memcpy(c->out_bary + 3 * i, bb, sizeof bb);
    }
}

void orc_brute_f64(const float* verts, int64_t nv, const int32_t* tris, int64_t nt,
                   const float* q, int64_t nq, double* out_d2, int32_t* out_tri, double* out_p,
                   double* out_bary, int nthreads) {
    (void)nv;
    brute_ctx c = {verts, q, tris, nt, out_d2, out_p, out_bary, out_tri};
    parallel_for(nq, 16, nthreads, brute_range, &c);
}

void orc_point_tri_batch_f64(const float* verts, const int32_t* tris, const float* q,
                             const int32_t* tri, int64_t nq, double* out_d2, double* out_bary) {
    for (int64_t i = 0; i < nq; ++i) {
        double p[3] = {q[3 * i], q[3 * i + 1], q[3 * i + 2]};
        double A[3], B[3], C[3];
        load_tri_f64(verts, tris, tri[i], A, B, C);
        out_d2[i] = orc_point_tri_f64(p, A, B, C, NULL, out_bary ? out_bary + 3 * i : NULL);
    }
}

/* ===================================================================== */
/* FP64 exact search over a balanced tree of its own                      */
/* ===================================================================== */

typedef struct {
    uint64_t key;
    int32_t idx;
} keyidx;

static int cmp_keyidx(const void* x, const void* y) {
    const keyidx* a = (const keyidx*)x;
    const keyidx* b = (const keyidx*)y;
    if (a->key != b->key) return a->key < b->key ? -1 : 1;
    return (a->idx > b->idx) - (a->idx < b->idx);
}

static uint64_t spread3(uint64_t x) {
    /* bit k of x moves to bit 3k (x < 2^21) */
    x &= 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

typedef struct {
    double lo[3], hi[3];
    int32_t left, right; /* children, or -1 */
    int32_t begin, end;  /* sorted range for a leaf */
} xnode;

typedef struct {
    const float* verts;
    const int32_t* tris;
    int32_t* perm; /* sorted position -> triangle */
    xnode* nodes;
    int32_t count;
} xtree;

static int32_t xbuild(xtree* t, int32_t b, int32_t e) {
    int32_t id = t->count++;
    xnode* n = &t->nodes[id];
    for (int k = 0; k < 3; ++k) {
        n->lo[k] = INFINITY;
        n->hi[k] = -INFINITY;
    }
    if (e - b <= 4) {
        n->left = n->right = -1;
        n->begin = b;
        n->end = e;
        for (int32_t i = b; i < e; ++i) {
            double A[3], B[3], C[3];
            load_tri_f64(t->verts, t->tris, t->perm[i], A, B, C);
            for (int k = 0; k < 3; ++k) {
                double lo = fmin(fmin(A[k], B[k]), C[k]), hi = fmax(fmax(A[k], B[k]), C[k]);
                if (lo < n->lo[k]) n->lo[k] = lo;
                if (hi > n->hi[k]) n->hi[k] = hi;
            }
        }
        return id;
    }
    int32_t m = b + (e - b) / 2;
    int32_t l = xbuild(t, b, m);
    int32_t r = xbuild(t, m, e);
    n = &t->nodes[id];
    n->left = l;
    n->right = r;
    n->begin = b;
    n->end = e;
    for (int k = 0; k < 3; ++k) {
        n->lo[k] = fmin(t->nodes[l].lo[k], t->nodes[r].lo[k]);
        n->hi[k] = fmax(t->nodes[l].hi[k], t->nodes[r].hi[k]);
    }
    return id;
}

static inline double box_d2_f64(const double* p, const double* lo, const double* hi) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) {
        double d = lo[k] - p[k];
        double d2 = p[k] - hi[k];
        d = d > d2 ? d : d2;
        if (d > 0.0) s += d * d;
    }
    return s;
}

typedef struct {
    xtree* t;
    const float* q;
    const double* qd; /* FP64 queries (used instead of q when set) */
    double *out_d2, *out_p, *out_bary;
    int32_t* out_tri;
} exact_ctx;

static void exact_range(void* vctx, int64_t b, int64_t e) {
    exact_ctx* c = (exact_ctx*)vctx;
    const xtree* t = c->t;
    for (int64_t i = b; i < e; ++i) {
        double p[3];
        for (int k = 0; k < 3; ++k) p[k] = c->qd ? c->qd[3 * i + k] : (double)c->q[3 * i + k];
        double best = INFINITY, bp[3] = {0, 0, 0}, bb[3] = {0, 0, 0};
        int32_t bt = INT32_MAX;
        int32_t stack[128];
        double sd[128];
        int sp = 0;
        stack[sp] = 0;
        sd[sp++] = 0.0;
        while (sp > 0) {
            --sp;
            /* visit while the box may hold a closer or an equally close triangle */
            if (sd[sp] > best * (1.0 + 1e-12)) continue;
            const xnode* n = &t->nodes[stack[sp]];
            if (n->left < 0) {
                for (int32_t k = n->begin; k < n->end; ++k) {
                    int32_t tri = t->perm[k];
                    double A[3], B[3], C[3], cp[3], w[3];
                    load_tri_f64(t->verts, t->tris, tri, A, B, C);
                    double d2 = orc_point_tri_f64(p, A, B, C, cp, w);
                    if (d2 < best || (d2 == best && tri < bt)) {
                        best = d2;
                        bt = tri;
                        memcpy(bp, cp, sizeof bp);
                        memcpy(bb, w, sizeof bb);
                    }
                }
                continue;
            }
            double dl = box_d2_f64(p, t->nodes[n->left].lo, t->nodes[n->left].hi);
            double dr = box_d2_f64(p, t->nodes[n->right].lo, t->nodes[n->right].hi);
            int32_t near = n->left, far = n->right;
            if (dr < dl) {
                double tmp = dl;
                dl = dr;
                dr = tmp;
                near = n->right;
                far = n->left;
            }
            stack[sp] = far;
            sd[sp++] = dr;
            stack[sp] = near;
            sd[sp++] = dl;
        }
        c->out_d2[i] = best;
        c->out_tri[i] = bt;
        if (c->out_p) memcpy(c->out_p + 3 * i, bp, sizeof bp);
        if (c->out_bary) memcpy(c->out_bary + 3 * i, bb, sizeof bb);
    }
}

static int exact_impl(const float* verts, const int32_t* tris, int64_t nt, const float* q,
                      const double* qd, int64_t nq, double* out_d2, int32_t* out_tri, double* out_p,
                      double* out_bary, int nthreads) {
    if (nt <= 0) return 1;
    keyidx* ki = (keyidx*)malloc(sizeof(keyidx) * nt);
    xtree t;
    t.verts = verts;
    t.tris = tris;
    t.perm = (int32_t*)malloc(sizeof(int32_t) * nt);
    t.nodes = (xnode*)malloc(sizeof(xnode) * (size_t)(2 * nt + 8));
    t.count = 0;
    if (!ki || !t.perm || !t.nodes) {
        free(ki);
        free(t.perm);
        free(t.nodes);
        return 2;
    }
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < nt; ++i) {
        double A[3], B[3], C[3];
        load_tri_f64(verts, tris, i, A, B, C);
        for (int k = 0; k < 3; ++k) {
            double m = (A[k] + B[k] + C[k]) / 3.0;
            lo[k] = fmin(lo[k], m);
            hi[k] = fmax(hi[k], m);
        }
    }
    for (int64_t i = 0; i < nt; ++i) {
        double A[3], B[3], C[3];
        load_tri_f64(verts, tris, i, A, B, C);
        uint64_t code = 0;
        for (int k = 0; k < 3; ++k) {
            double m = (A[k] + B[k] + C[k]) / 3.0;
            double ext = hi[k] - lo[k];
            double f = ext > 0 ? (m - lo[k]) / ext : 0.0;
            uint64_t cell = (uint64_t)(f * 1023.0);
            code |= spread3(cell) << (2 - k);
        }
        ki[i].key = code;
        ki[i].idx = (int32_t)i;
    }
    qsort(ki, (size_t)nt, sizeof(keyidx), cmp_keyidx);
    for (int64_t i = 0; i < nt; ++i) t.perm[i] = ki[i].idx;
    free(ki);
    xbuild(&t, 0, (int32_t)nt);
    exact_ctx c = {&t, q, qd, out_d2, out_p, out_bary, out_tri};
    parallel_for(nq, 64, nthreads, exact_range, &c);
    free(t.perm);
    free(t.nodes);
    return 0;
}

int orc_exact_f64(const float* verts, int64_t nv, const int32_t* tris, int64_t nt, const float* q,
                  int64_t nq, double* out_d2, int32_t* out_tri, double* out_p, double* out_bary,
                  int nthreads) {
    (void)nv;
    return exact_impl(verts, tris, nt, q, NULL, nq, out_d2, out_tri, out_p, out_bary, nthreads);
}

int orc_exact_f64_dq(const float* verts, int64_t nv, const int32_t* tris, int64_t nt,
                     const double* q, int64_t nq, double* out_d2, int32_t* out_tri, int nthreads) {
    (void)nv;
    return exact_impl(verts, tris, nt, NULL, q, nq, out_d2, out_tri, NULL, NULL, nthreads);
}

/* ===================================================================== */
/* FP32 restatement of the GPU build                                      */
/* ===================================================================== */

/* 64-bit keys, stable LSD radix sort with 8-bit digits (payload = index). */
static void radix_sort_u64(uint64_t* keys, int32_t* vals, int64_t n) {
    uint64_t* k2 = (uint64_t*)malloc(sizeof(uint64_t) * n);
    int32_t* v2 = (int32_t*)malloc(sizeof(int32_t) * n);
    for (int pass = 0; pass < 8; ++pass) {
        int shift = pass * 8;
        int64_t cnt[256] = {0};
        for (int64_t i = 0; i < n; ++i) cnt[(keys[i] >> shift) & 255]++;
        int64_t run = 0;
        for (int d = 0; d < 256; ++d) {
            int64_t c = cnt[d];
            cnt[d] = run;
            run += c;
        }
        for (int64_t i = 0; i < n; ++i) {
            int64_t dst = cnt[(keys[i] >> shift) & 255]++;
            k2[dst] = keys[i];
            v2[dst] = vals[i];
        }
        memcpy(keys, k2, sizeof(uint64_t) * n);
        memcpy(vals, v2, sizeof(int32_t) * n);
    }
    free(k2);
    free(v2);
}

static inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

/* Length of the common prefix of the index-augmented keys at sorted
 * positions i and j (Karras 2012); -1 outside [0, n). */
static inline int delta(const uint64_t* keys, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t x = keys[i] ^ keys[j];
    if (x) return clz64(x);
    return 64 + clz32((uint32_t)i ^ (uint32_t)j);
}

static int ceil_log2(int64_t v) {
    int b = 0;
    while (((int64_t)1 << b) < v) ++b;
    return b;
}

/* Quantised Morton code of one centroid sum, bit-exact with the GPU build:
 * t = (s - lo) * scale in round-to-nearest FP32, truncated, clamped. */
static inline uint32_t quantise(float s, float lo, float scale, uint32_t maxcell) {
    float t = (s - lo) * scale;
    if (!(t < (float)maxcell)) return maxcell;
    return (uint32_t)t;
}

/* Half the surface area of a box in the reference's BBox::surface_area order
 * (src/lib/bbox.h:55-59: 2 (ex ez + ex ey + ey ez), summed left to right);
 * its factor 2 is exact, so twice this equals that function bit for bit. */
static inline float half_area(const float* b) {
    float ex = b[3] - b[0], ey = b[4] - b[1], ez = b[5] - b[2];
    float xz = ex * ez;
    float xy = ex * ey;
    float yz = ey * ez;
    float s = xz + xy;
    return s + yz;
}

void orc_tree_free(orc_tree* t) {
    if (!t) return;
    free(t->keys); free(t->order); free(t->left); free(t->right); free(t->parent);
    free(t->first); free(t->last); free(t->box); free(t->cost); free(t->cluster);
    free(t->mesh_root); free(t->wide_root); free(t->wide_src); free(t->wide_box);
    free(t->wide_ref); free(t->wide_count); free(t->tri_verts); free(t->mesh_of_tri);
    free(t->tri_local);
    free(t);
}

static int build_tree(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                      const int64_t* tri_offsets, int32_t nmeshes, int64_t nv_total, int64_t nt_total,
                      int32_t K, int32_t leaf_size, const int32_t* mesh_leaf, int32_t collapse, float c_node,
                      float c_tri, orc_tree** out);

int orc_build(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
              const int64_t* tri_offsets, int32_t nmeshes, int64_t nv_total, int64_t nt_total,
              int32_t K, int32_t leaf_size, int32_t collapse, float c_node, float c_tri,
              orc_tree** out) {
    return build_tree(verts, vert_offsets, tris, tri_offsets, nmeshes, nv_total, nt_total, K, leaf_size, NULL,
                      collapse, c_node, c_tri, out);
}

int orc_build_leaves(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                     const int64_t* tri_offsets, int32_t nmeshes, int64_t nv_total, int64_t nt_total,
                     int32_t K, const int32_t* mesh_leaf, int32_t collapse, float c_node, float c_tri,
                     orc_tree** out) {
    if (!mesh_leaf || nmeshes <= 0) return 1;
    int32_t mx = 1;
    for (int32_t m = 0; m < nmeshes; ++m) {
        if (mesh_leaf[m] < 1 || mesh_leaf[m] > 15) return 1;
        if (mesh_leaf[m] > mx) mx = mesh_leaf[m];
    }
    return build_tree(verts, vert_offsets, tris, tri_offsets, nmeshes, nv_total, nt_total, K, mx, mesh_leaf,
                      collapse, c_node, c_tri, out);
}

static int build_tree(const float* verts, const int64_t* vert_offsets, const int32_t* tris,
                      const int64_t* tri_offsets, int32_t nmeshes, int64_t nv_total, int64_t nt_total,
                      int32_t K, int32_t leaf_size, const int32_t* mesh_leaf, int32_t collapse, float c_node,
                      float c_tri, orc_tree** out) {
    (void)nv_total;
    *out = NULL;
    if (nt_total <= 0 || nmeshes <= 0) return 1;
    if (K != 2 && K != 4 && K != 8) return 1;
    if (leaf_size < 1 || leaf_size > 15) return 1;
    const int64_t n = nt_total;
    int64_t voff_single[2] = {0, nv_total};
    int64_t toff_single[2] = {0, nt_total};
    if (!vert_offsets) vert_offsets = voff_single;
    if (!tri_offsets) tri_offsets = toff_single;

    orc_tree* T = (orc_tree*)calloc(1, sizeof(orc_tree));
    T->nt = n;
    T->nmeshes = nmeshes;
    T->branching = K;
    T->leaf_size = leaf_size;
    T->collapse = collapse;
    int64_t nn = 2 * n - 1;
    T->keys = (uint64_t*)malloc(8 * n);
    T->order = (int32_t*)malloc(4 * n);
    T->left = (int32_t*)malloc(4 * (n > 1 ? n - 1 : 1));
    T->right = (int32_t*)malloc(4 * (n > 1 ? n - 1 : 1));
    T->parent = (int32_t*)malloc(4 * nn);
    T->first = (int32_t*)malloc(4 * nn);
    T->last = (int32_t*)malloc(4 * nn);
    T->box = (float*)malloc(4 * 6 * nn);
    T->cost = (float*)malloc(4 * nn);
    T->cluster = (uint8_t*)calloc(nn, 1);
    T->mesh_root = (int32_t*)malloc(4 * nmeshes);
    T->wide_root = (int32_t*)malloc(4 * nmeshes);
    T->tri_verts = (float*)malloc(4 * 9 * n);
    T->mesh_of_tri = (int32_t*)malloc(4 * n);
    T->tri_local = (int32_t*)malloc(4 * n);
    uint8_t* leaf_flag = (uint8_t*)calloc(nn, 1);
    int32_t* tri_mesh = (int32_t*)malloc(4 * n); /* global triangle -> mesh */
    if (!T->keys || !T->order || !T->parent || !T->box || !T->tri_verts || !leaf_flag || !tri_mesh) {
        orc_tree_free(T);
        free(leaf_flag);
        free(tri_mesh);
        return 2;
    }
    for (int32_t m = 0; m < nmeshes; ++m)
        for (int64_t t = tri_offsets[m]; t < tri_offsets[m + 1]; ++t) tri_mesh[t] = m;

    /* --- Morton keys of centroid sums, quantised in each mesh's own box --- */
    const int mesh_bits = nmeshes > 1 ? ceil_log2(nmeshes) : 0;
    int bits = (64 - mesh_bits) / 3;
    if (bits > 21) bits = 21;
    const uint32_t maxcell = (1u << bits) - 1u;
    const float cells = (float)(1u << bits);
    float* csum = (float*)malloc(4 * 3 * n);
    for (int64_t t = 0; t < n; ++t) {
        int32_t m = tri_mesh[t];
        const float* vb = verts + 3 * vert_offsets[m];
        const int32_t* ix = tris + 3 * t;
        for (int k = 0; k < 3; ++k) {
            float s = vb[3 * (int64_t)ix[0] + k] + vb[3 * (int64_t)ix[1] + k];
            s = s + vb[3 * (int64_t)ix[2] + k];
            csum[3 * t + k] = s;
        }
    }
    float* mlo = (float*)malloc(4 * 3 * nmeshes);
    float* mscale = (float*)malloc(4 * 3 * nmeshes);
    for (int32_t m = 0; m < nmeshes; ++m) {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t t = tri_offsets[m]; t < tri_offsets[m + 1]; ++t)
            for (int k = 0; k < 3; ++k) {
                float s = csum[3 * t + k];
                lo[k] = s < lo[k] ? s : lo[k];
                hi[k] = s > hi[k] ? s : hi[k];
            }
        /* isotropic frame: one cell size, from the largest extent */
        float emax = 0.0f;
        for (int k = 0; k < 3; ++k) {
            float e = hi[k] - lo[k];
            if (e > emax) emax = e;
        }
        float scale = emax > 0.0f ? cells / emax : 0.0f;
        if (!(scale <= FLT_MAX)) scale = 0.0f;
        for (int k = 0; k < 3; ++k) {
            mlo[3 * m + k] = lo[k];
            mscale[3 * m + k] = scale;
        }
    }
    for (int64_t t = 0; t < n; ++t) {
        int32_t m = tri_mesh[t];
        uint64_t code = 0;
        for (int k = 0; k < 3; ++k) {
            uint32_t cell = quantise(csum[3 * t + k], mlo[3 * m + k], mscale[3 * m + k], maxcell);
            code |= spread3(cell) << (2 - k);
        }
        T->keys[t] = ((uint64_t)m << (3 * bits)) | code;
        T->order[t] = (int32_t)t;
    }
    free(csum);
    free(mlo);
    free(mscale);
    radix_sort_u64(T->keys, T->order, n);
    for (int64_t k = 0; k < n; ++k) {
        int32_t t = T->order[k];
        int32_t m = tri_mesh[t];
        T->mesh_of_tri[k] = m;
        T->tri_local[k] = (int32_t)(t - tri_offsets[m]);
        const float* vb = verts + 3 * vert_offsets[m];
        const int32_t* ix = tris + 3 * (int64_t)t;
        for (int v = 0; v < 3; ++v)
            for (int c = 0; c < 3; ++c) T->tri_verts[9 * k + 3 * v + c] = vb[3 * (int64_t)ix[v] + c];
    }

    /* --- Karras hierarchy --- */
    for (int64_t i = 0; i < nn; ++i) T->parent[i] = -1;
    for (int64_t k = 0; k < n; ++k) {
        T->first[n - 1 + k] = (int32_t)k;
        T->last[n - 1 + k] = (int32_t)k;
    }
    for (int32_t m = 0; m < nmeshes; ++m) T->mesh_root[m] = -1;
    for (int32_t m = 0; m < nmeshes; ++m)
        if (tri_offsets[m + 1] - tri_offsets[m] == 1) T->mesh_root[m] = (int32_t)(n - 1 + tri_offsets[m]);
    const uint64_t* K_ = T->keys;
    for (int64_t i = 0; i + 1 < n; ++i) {
        int d = (delta(K_, n, i, i + 1) - delta(K_, n, i, i - 1)) > 0 ? 1 : -1;
        int dmin = delta(K_, n, i, i - d);
        int64_t lmax = 2;
        while (delta(K_, n, i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0;
        for (int64_t t = lmax / 2; t >= 1; t /= 2)
            if (delta(K_, n, i, i + (l + t) * d) > dmin) l += t;
        int64_t j = i + l * d;
        int dnode = delta(K_, n, i, j);
        int64_t s = 0;
        for (int64_t div = 2;; div *= 2) {
            int64_t t = (l + div - 1) / div;
            if (delta(K_, n, i, i + (s + t) * d) > dnode) s += t;
            if (t <= 1) break;
        }
        int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
        int64_t lo = i < j ? i : j, hi = i < j ? j : i;
        int32_t lc = (lo == gamma) ? (int32_t)(n - 1 + gamma) : (int32_t)gamma;
        int32_t rc = (hi == gamma + 1) ? (int32_t)(n - 1 + gamma + 1) : (int32_t)(gamma + 1);
        T->left[i] = lc;
        T->right[i] = rc;
        T->parent[lc] = (int32_t)i;
        T->parent[rc] = (int32_t)i;
        T->first[i] = (int32_t)lo;
        T->last[i] = (int32_t)hi;
        int32_t m = (int32_t)(K_[lo] >> (3 * bits));
        if ((int64_t)lo == tri_offsets[m] && (int64_t)hi == tri_offsets[m + 1] - 1) T->mesh_root[m] = (int32_t)i;
    }

    /* --- bottom-up boxes, SAH costs, leaf decisions --- */
    int32_t* arrive = (int32_t*)calloc(nn, 4);
    for (int64_t k = 0; k < n; ++k) {
        int64_t node = n - 1 + k;
        float* b = T->box + 6 * node;
        const float* tv = T->tri_verts + 9 * k;
        for (int c = 0; c < 3; ++c) {
            float lo = tv[c] < tv[3 + c] ? tv[c] : tv[3 + c];
            lo = lo < tv[6 + c] ? lo : tv[6 + c];
            float hi = tv[c] > tv[3 + c] ? tv[c] : tv[3 + c];
            hi = hi > tv[6 + c] ? hi : tv[6 + c];
            b[c] = lo;
            b[3 + c] = hi;
        }
        float A = half_area(b);
        T->cost[node] = (collapse == 1) ? (c_tri * 1.0f) * A : 0.0f;
        leaf_flag[node] = 1;
        int64_t p = T->parent[node];
        while (p >= 0) {
            if (++arrive[p] < 2) break;
            int32_t l = T->left[p], r = T->right[p];
            float* pb = T->box + 6 * p;
            const float* lb = T->box + 6 * (int64_t)l;
            const float* rb = T->box + 6 * (int64_t)r;
            for (int c = 0; c < 3; ++c) {
                pb[c] = lb[c] < rb[c] ? lb[c] : rb[c];
                pb[3 + c] = lb[3 + c] > rb[3 + c] ? lb[3 + c] : rb[3 + c];
            }
            int32_t size = T->last[p] - T->first[p] + 1;
            int same_mesh = T->mesh_of_tri[T->first[p]] == T->mesh_of_tri[T->last[p]];
            int limit = mesh_leaf ? mesh_leaf[T->mesh_of_tri[T->first[p]]] : leaf_size;
            int leafable = size <= limit && same_mesh;
            if (collapse == 1) {
                float Ap = half_area(pb);
                float split = c_node * Ap;
                split = split + T->cost[l];
                split = split + T->cost[r];
                float leafc = (c_tri * (float)size) * Ap;
                int lf = leafable && leafc <= split;
                leaf_flag[p] = (uint8_t)lf;
                T->cost[p] = lf ? leafc : split;
            } else {
                leaf_flag[p] = (uint8_t)leafable;
                T->cost[p] = 0.0f;
            }
            p = T->parent[p];
        }
    }
    free(arrive);

    /* --- clusters, depth below the mesh root, wide-root flags --- */
    int32_t* mesh_root_of_node = NULL;
    (void)mesh_root_of_node;
    const int k_levels = K == 2 ? 1 : (K == 4 ? 2 : 3);
    int32_t* wide_id = (int32_t*)malloc(4 * nn);
    int32_t* depth = (int32_t*)malloc(4 * nn);
    int64_t num_wide = 0;
    int32_t max_depth = 0;
    for (int64_t v = 0; v < nn; ++v) {
        wide_id[v] = -1;
        depth[v] = -1;
        int32_t m = T->mesh_of_tri[T->first[v]];
        if (T->mesh_of_tri[T->last[v]] != m) continue; /* above the mesh roots */
        int32_t root = T->mesh_root[m];
        /* walk up to the mesh root: depth and whether an ancestor is a leaf */
        int32_t d = 0;
        int anc_leaf = 0;
        int64_t u = v;
        while (u != root) {
            u = T->parent[u];
            ++d;
            if (leaf_flag[u]) anc_leaf = 1;
        }
        depth[v] = d;
        T->cluster[v] = (uint8_t)(leaf_flag[v] && !anc_leaf);
        int is_wide = 0;
        if (v == root) is_wide = 1;
        else if (!anc_leaf && !leaf_flag[v] && v < n - 1 && (d % k_levels) == 0) is_wide = 1;
        if (is_wide) {
            wide_id[v] = (int32_t)num_wide++;
            if (d / k_levels > max_depth) max_depth = d / k_levels;
        }
    }
    T->num_wide = num_wide;
    T->max_wide_depth = max_depth;
    T->stack_bound = (K - 1) * (max_depth + 1);
    for (int32_t m = 0; m < nmeshes; ++m) T->wide_root[m] = wide_id[T->mesh_root[m]];
    T->wide_src = (int32_t*)malloc(4 * num_wide);
    T->wide_box = (float*)malloc(4 * 6 * K * num_wide);
    T->wide_ref = (int32_t*)malloc(4 * K * num_wide);
    T->wide_count = (int32_t*)malloc(4 * K * num_wide);
    int64_t leaves = 0;
    for (int64_t v = 0; v < nn; ++v) {
        int32_t w = wide_id[v];
        if (w < 0) continue;
        T->wide_src[w] = (int32_t)v;
        int32_t slots[8];
        int ns = 0;
        if (T->cluster[v]) {
            slots[ns++] = (int32_t)v;
        } else {
            slots[ns++] = (int32_t)v;
            for (int lev = 0; lev < k_levels; ++lev) {
                int32_t nxt[8];
                int nn2 = 0;
                for (int s = 0; s < ns; ++s) {
                    int32_t x = slots[s];
                    if (x < n - 1 && !T->cluster[x]) {
                        nxt[nn2++] = T->left[x];
                        nxt[nn2++] = T->right[x];
                    } else {
                        nxt[nn2++] = x;
                    }
                }
                memcpy(slots, nxt, sizeof(int32_t) * nn2);
                ns = nn2;
            }
        }
        float* wb = T->wide_box + (int64_t)w * 6 * K;
        for (int s = 0; s < K; ++s) {
            if (s < ns) {
                int32_t x = slots[s];
                const float* b = T->box + 6 * (int64_t)x;
                wb[0 * K + s] = b[0];
                wb[1 * K + s] = b[3];
                wb[2 * K + s] = b[1];
                wb[3 * K + s] = b[4];
                wb[4 * K + s] = b[2];
                wb[5 * K + s] = b[5];
                if (T->cluster[x]) {
                    T->wide_ref[(int64_t)w * K + s] = T->first[x];
                    T->wide_count[(int64_t)w * K + s] = T->last[x] - T->first[x] + 1;
                    ++leaves;
                } else {
                    T->wide_ref[(int64_t)w * K + s] = wide_id[x];
                    T->wide_count[(int64_t)w * K + s] = 0;
                }
            } else {
                wb[0 * K + s] = INFINITY;
                wb[1 * K + s] = -INFINITY;
                wb[2 * K + s] = INFINITY;
                wb[3 * K + s] = -INFINITY;
                wb[4 * K + s] = INFINITY;
                wb[5 * K + s] = -INFINITY;
                T->wide_ref[(int64_t)w * K + s] = 0;
                T->wide_count[(int64_t)w * K + s] = -1;
            }
        }
    }
    T->num_leaves = leaves;
    free(wide_id);
    free(depth);
    free(leaf_flag);
    free(tri_mesh);
    *out = T;
    return 0;
}

/* ===================================================================== */
/* FP32 traversal (CPU baseline and canonical visit counts)               */
/* ===================================================================== */

/* FP32 point-triangle squared distance with the GPU kernel's operation
 * order: Voronoi regions, difference vector measured from the vertex that
 * owns the region.  Writes the barycentric weights of b and c. */
static float pt_tri_f32(const float* q, const float* tv, float* ov, float* ow) {
    const float *a = tv, *b = tv + 3, *c = tv + 6;
    float ab[3], ac[3], ap[3];
    for (int k = 0; k < 3; ++k) {
        ab[k] = b[k] - a[k];
        ac[k] = c[k] - a[k];
        ap[k] = q[k] - a[k];
    }
    float nx = ab[1] * ac[2] - ab[2] * ac[1];
    float ny = ab[2] * ac[0] - ab[0] * ac[2];
    float nz = ab[0] * ac[1] - ab[1] * ac[0];
    float nn = nx * nx + ny * ny + nz * nz;
    float lab = ab[0] * ab[0] + ab[1] * ab[1] + ab[2] * ab[2];
    float lac = ac[0] * ac[0] + ac[1] * ac[1] + ac[2] * ac[2];
    float v = 0.0f, w = 0.0f;
    if (!(nn > 1e-10f * (lab * lac))) {
        /* (near-)degenerate: closest of the three edges */
        float best = INFINITY;
        const float* P[3] = {a, b, a};
        const float* Q[3] = {b, c, c};
        for (int e = 0; e < 3; ++e) {
            float d[3], r[3];
            for (int k = 0; k < 3; ++k) {
                d[k] = Q[e][k] - P[e][k];
                r[k] = q[k] - P[e][k];
            }
            float l = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            float t = 0.0f;
            if (l > 0.0f) {
                t = (r[0] * d[0] + r[1] * d[1] + r[2] * d[2]) / l;
                t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
            }
            float x = r[0] - t * d[0], y = r[1] - t * d[1], z = r[2] - t * d[2];
            float d2 = x * x + y * y + z * z;
            if (d2 < best) {
                best = d2;
                if (e == 0) { v = t; w = 0.0f; }
                else if (e == 1) { v = 1.0f - t; w = t; }
                else { v = 0.0f; w = t; }
            }
        }
        *ov = v;
        *ow = w;
        return best;
    }
    float d1 = ab[0] * ap[0] + ab[1] * ap[1] + ab[2] * ap[2];
    float d2 = ac[0] * ap[0] + ac[1] * ap[1] + ac[2] * ap[2];
    float r[3];
    if (d1 <= 0.0f && d2 <= 0.0f) {
        v = 0.0f; w = 0.0f;
        r[0] = ap[0]; r[1] = ap[1]; r[2] = ap[2];
    } else {
        float bp[3] = {q[0] - b[0], q[1] - b[1], q[2] - b[2]};
        float d3 = ab[0] * bp[0] + ab[1] * bp[1] + ab[2] * bp[2];
        float d4 = ac[0] * bp[0] + ac[1] * bp[1] + ac[2] * bp[2];
        float cp[3] = {q[0] - c[0], q[1] - c[1], q[2] - c[2]};
        float d5 = ab[0] * cp[0] + ab[1] * cp[1] + ab[2] * cp[2];
        float d6 = ac[0] * cp[0] + ac[1] * cp[1] + ac[2] * cp[2];
        float vc = d1 * d4 - d3 * d2;
        float vb = d5 * d2 - d1 * d6;
        float va = d3 * d6 - d5 * d4;
        if (d3 >= 0.0f && d4 <= d3) {
            v = 1.0f; w = 0.0f;
            r[0] = bp[0]; r[1] = bp[1]; r[2] = bp[2];
        } else if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
            v = d1 / (d1 - d3); w = 0.0f;
            for (int k = 0; k < 3; ++k) r[k] = ap[k] - v * ab[k];
        } else if (d6 >= 0.0f && d5 <= d6) {
            v = 0.0f; w = 1.0f;
            r[0] = cp[0]; r[1] = cp[1]; r[2] = cp[2];
        } else if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
            v = 0.0f; w = d2 / (d2 - d6);
            for (int k = 0; k < 3; ++k) r[k] = ap[k] - w * ac[k];
        } else if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
            w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            v = 1.0f - w;
            for (int k = 0; k < 3; ++k) r[k] = bp[k] - w * (c[k] - b[k]);
        } else {
            float s = va + vb + vc;
            v = vb / s;
            w = vc / s;
            for (int k = 0; k < 3; ++k) r[k] = ap[k] - (v * ab[k] + w * ac[k]);
        }
    }
    *ov = v;
    *ow = w;
    return r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
}

typedef struct {
    const orc_tree* t;
    const float* q;
    const int32_t* q_mesh;
    float *out_d, *out_p, *out_bary;
    int32_t *out_tri, *node_visits, *tri_tests;
} query_ctx;

static inline float box_lb2_f32(const float* q, float lox, float hix, float loy, float hiy,
                                float loz, float hiz) {
    float a, b, dx, dy, dz;
    a = lox - q[0]; b = q[0] - hix; dx = a > b ? a : b; dx = dx > 0.0f ? dx : 0.0f;
    a = loy - q[1]; b = q[1] - hiy; dy = a > b ? a : b; dy = dy > 0.0f ? dy : 0.0f;
    a = loz - q[2]; b = q[2] - hiz; dz = a > b ? a : b; dz = dz > 0.0f ? dz : 0.0f;
    float s = dx * dx + dy * dy;
    return s + dz * dz;
}

static void query_range(void* vctx, int64_t b, int64_t e) {
    query_ctx* c = (query_ctx*)vctx;
    const orc_tree* t = c->t;
    const int K = t->branching;
    int32_t* st_node = (int32_t*)malloc(sizeof(int32_t) * (t->stack_bound + 8));
    float* st_lb = (float*)malloc(sizeof(float) * (t->stack_bound + 8));
    for (int64_t i = b; i < e; ++i) {
        const float* q = c->q + 3 * i;
        int32_t m = c->q_mesh ? c->q_mesh[i] : 0;
        float best = INFINITY, bv = 0.0f, bw = 0.0f;
        int32_t best_pos = -1, best_local = INT32_MAX;
        int32_t visits = 0, tests = 0;
        int sp = 0;
        int32_t node = t->wide_root[m];
        for (;;) {
            if (node >= 0) {
                ++visits;
                const float* wb = t->wide_box + (int64_t)node * 6 * K;
                const int32_t* ref = t->wide_ref + (int64_t)node * K;
                const int32_t* cnt = t->wide_count + (int64_t)node * K;
                float lb[8];
                int slot[8];
                for (int s = 0; s < K; ++s) {
                    lb[s] = cnt[s] < 0 ? INFINITY
                                       : box_lb2_f32(q, wb[s], wb[K + s], wb[2 * K + s], wb[3 * K + s],
                                                     wb[4 * K + s], wb[5 * K + s]);
                    slot[s] = s;
                }
                /* ascending by bound, slot order on ties (insertion sort) */
                for (int s = 1; s < K; ++s) {
                    float x = lb[s];
                    int xs = slot[s];
                    int j = s - 1;
                    while (j >= 0 && lb[j] > x) {
                        lb[j + 1] = lb[j];
                        slot[j + 1] = slot[j];
                        --j;
                    }
                    lb[j + 1] = x;
                    slot[j + 1] = xs;
                }
                /* leaves first, nearest first */
                for (int s = 0; s < K; ++s) {
                    int sl = slot[s];
                    if (cnt[sl] <= 0 || !(lb[s] < best)) continue;
                    for (int32_t k = ref[sl]; k < ref[sl] + cnt[sl]; ++k) {
                        float v, w;
                        ++tests;
                        float d2 = pt_tri_f32(q, t->tri_verts + 9 * (int64_t)k, &v, &w);
                        int32_t loc = t->tri_local[k];
                        if (d2 < best || (d2 == best && loc < best_local)) {
                            best = d2;
                            best_pos = k;
                            best_local = loc;
                            bv = v;
                            bw = w;
                        }
                    }
                }
                /* inner children: push the far ones (farthest first), descend the nearest */
                int32_t inner[8];
                float ilb[8];
                int ni = 0;
                for (int s = 0; s < K; ++s) {
                    int sl = slot[s];
                    if (cnt[sl] == 0 && lb[s] < best) {
                        inner[ni] = ref[sl];
                        ilb[ni] = lb[s];
                        ++ni;
                    }
                }
                if (ni > 0) {
                    for (int s = ni - 1; s >= 1; --s) {
                        st_node[sp] = inner[s];
                        st_lb[sp] = ilb[s];
                        ++sp;
                    }
                    node = inner[0];
                    continue;
                }
                node = -1;
            }
            /* pop the next entry that can still hold a closer triangle */
            while (sp > 0) {
                --sp;
                if (st_lb[sp] < best) {
                    node = st_node[sp];
                    break;
                }
            }
            if (node < 0) break;
        }
        /* final answer re-evaluated in FP64 for the winning triangle */
        if (best_pos >= 0) {
            const float* tv = t->tri_verts + 9 * (int64_t)best_pos;
            double p[3] = {q[0], q[1], q[2]};
            double A[3] = {tv[0], tv[1], tv[2]}, B[3] = {tv[3], tv[4], tv[5]}, C[3] = {tv[6], tv[7], tv[8]};
            double cp[3], w3[3];
            double d2 = orc_point_tri_f64(p, A, B, C, cp, w3);
            c->out_d[i] = (float)sqrt(d2);
            if (c->out_p)
                for (int k = 0; k < 3; ++k) c->out_p[3 * i + k] = (float)cp[k];
            if (c->out_bary) {
                c->out_bary[2 * i] = (float)w3[1];
                c->out_bary[2 * i + 1] = (float)w3[2];
            }
            (void)bv;
            (void)bw;
        }
        c->out_tri[i] = best_pos >= 0 ? best_local : -1;
        if (c->node_visits) c->node_visits[i] = visits;
        if (c->tri_tests) c->tri_tests[i] = tests;
    }
    free(st_node);
    free(st_lb);
}

double orc_query_f32(const orc_tree* t, const float* q, const int32_t* q_mesh, int64_t nq,
                     float* out_d, int32_t* out_tri, float* out_p, float* out_bary,
                     int32_t* node_visits, int32_t* tri_tests, int nthreads) {
    query_ctx c = {t, q, q_mesh, out_d, out_p, out_bary, out_tri, node_visits, tri_tests};
    double t0 = now_s();
    parallel_for(nq, 256, nthreads, query_range, &c);
    return now_s() - t0;
}

/* ===================================================================== */
/* FP64 analytic adjoint                                                  */
/* ===================================================================== */

void orc_backward_f64(const float* verts, int64_t nv, const int32_t* tris, const float* q,
                      const int32_t* tri, const double* bary, const double* grad_d, int64_t nq,
                      double* grad_q, double* grad_verts) {
    (void)nv;
    for (int64_t i = 0; i < nq; ++i) {
        double A[3], B[3], C[3];
        load_tri_f64(verts, tris, tri[i], A, B, C);
        const double* w = bary + 3 * i;
        double r[3], d2 = 0.0;
        for (int k = 0; k < 3; ++k) {
            double p = w[0] * A[k] + w[1] * B[k] + w[2] * C[k];
            r[k] = q[3 * i + k] - p;
            d2 += r[k] * r[k];
        }
        double d = sqrt(d2);
        double s = d > 0.0 ? grad_d[i] / d : 0.0;
        const int32_t* ix = tris + 3 * (int64_t)tri[i];
        for (int k = 0; k < 3; ++k) {
            double gk = s * r[k];
            if (grad_q) grad_q[3 * i + k] = gk;
            if (grad_verts)
                for (int v = 0; v < 3; ++v) grad_verts[3 * (int64_t)ix[v] + k] -= w[v] * gk;
        }
    }
}

/* ===================================================================== */
/* Rays: brute force in FP32 (the GPU's arithmetic) and FP64             */
/* ===================================================================== */

/* triangle_hit (src/shaders/rt/rtcommon.glsl:181-202) in FP32, in its own
 * evaluation order (dot = (x + y) + z; cross components as differences of
 * products); compiled without contraction, so each step rounds once. */
static int mt_f32(const float o[3], const float d[3], const float a[3], const float b[3],
                  const float c[3], float det_eps, float* t, float* u, float* v) {
    float v1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    float v2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    float p[3] = {d[1] * v2[2] - d[2] * v2[1], d[2] * v2[0] - d[0] * v2[2], d[0] * v2[1] - d[1] * v2[0]};
    float det = (v1[0] * p[0] + v1[1] * p[1]) + v1[2] * p[2];
    if (!(fabsf(det) > det_eps)) return 0;
    float inv = 1.0f / det;
    float s[3] = {o[0] - a[0], o[1] - a[1], o[2] - a[2]};
    float uu = ((s[0] * p[0] + s[1] * p[1]) + s[2] * p[2]) * inv;
    if (uu < 0.0f || uu > 1.0f) return 0;
    float q[3] = {s[1] * v1[2] - s[2] * v1[1], s[2] * v1[0] - s[0] * v1[2], s[0] * v1[1] - s[1] * v1[0]};
    float vv = ((d[0] * q[0] + d[1] * q[1]) + d[2] * q[2]) * inv;
    if (vv < 0.0f || uu + vv > 1.0f) return 0;
    *t = ((v2[0] * q[0] + v2[1] * q[1]) + v2[2] * q[2]) * inv;
    *u = uu;
    *v = vv;
    return 1;
}

static int mt_f64(const double o[3], const double d[3], const double a[3], const double b[3],
                  const double c[3], double det_eps, double* t, double* u, double* v) {
    double v1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double v2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double p[3] = {d[1] * v2[2] - d[2] * v2[1], d[2] * v2[0] - d[0] * v2[2], d[0] * v2[1] - d[1] * v2[0]};
    double det = (v1[0] * p[0] + v1[1] * p[1]) + v1[2] * p[2];
    if (!(fabs(det) > det_eps)) return 0;
    double inv = 1.0 / det;
    double s[3] = {o[0] - a[0], o[1] - a[1], o[2] - a[2]};
    double uu = ((s[0] * p[0] + s[1] * p[1]) + s[2] * p[2]) * inv;
    if (uu < 0.0 || uu > 1.0) return 0;
    double q[3] = {s[1] * v1[2] - s[2] * v1[1], s[2] * v1[0] - s[0] * v1[2], s[0] * v1[1] - s[1] * v1[0]};
    double vv = ((d[0] * q[0] + d[1] * q[1]) + d[2] * q[2]) * inv;
    if (vv < 0.0 || uu + vv > 1.0) return 0;
    *t = ((v2[0] * q[0] + v2[1] * q[1]) + v2[2] * q[2]) * inv;
    *u = uu;
    *v = vv;
    return 1;
}

typedef struct {
    const float *verts, *orig, *dir, *tmax_per;
    const int32_t* tris;
    int64_t nt;
    float tmin, tmax, eps;
    double tmin64, tmax64, eps64;
    float *t32, *uv32;
    double *t64, *uv64;
    int32_t* tri;
} ray_ctx;

static void ray32_range(void* vctx, int64_t b, int64_t e) {
    ray_ctx* c = (ray_ctx*)vctx;
    for (int64_t i = b; i < e; ++i) {
        const float* o = c->orig + 3 * i;
        const float* d = c->dir + 3 * i;
        float tmax = c->tmax;
        if (c->tmax_per && c->tmax_per[i] < tmax) tmax = c->tmax_per[i];
        float bt = INFINITY, bu = 0.0f, bv = 0.0f;
        int32_t bi = -1;
        for (int64_t k = 0; k < c->nt; ++k) {
            const int32_t* ix = c->tris + 3 * k;
            float t, u, v;
            if (!mt_f32(o, d, c->verts + 3 * (int64_t)ix[0], c->verts + 3 * (int64_t)ix[1],
                        c->verts + 3 * (int64_t)ix[2], c->eps, &t, &u, &v))
                continue;
            if (!(t >= c->tmin && t <= tmax)) continue;
            if (t < bt) {  /* triangles in index order: the first of equal t is the least index */
                bt = t;
                bu = u;
                bv = v;
                bi = (int32_t)k;
            }
        }
        c->t32[i] = bt;
        c->tri[i] = bi;
        if (c->uv32) {
            c->uv32[2 * i] = bu;
            c->uv32[2 * i + 1] = bv;
        }
    }
}

static void ray64_range(void* vctx, int64_t b, int64_t e) {
    ray_ctx* c = (ray_ctx*)vctx;
    for (int64_t i = b; i < e; ++i) {
        const double o[3] = {c->orig[3 * i], c->orig[3 * i + 1], c->orig[3 * i + 2]};
        const double d[3] = {c->dir[3 * i], c->dir[3 * i + 1], c->dir[3 * i + 2]};
        double tmax = c->tmax64;
        if (c->tmax_per && c->tmax_per[i] < tmax) tmax = c->tmax_per[i];
        double bt = INFINITY, bu = 0.0, bv = 0.0;
        int32_t bi = -1;
        for (int64_t k = 0; k < c->nt; ++k) {
            double A[3], B[3], C[3];
            load_tri_f64(c->verts, c->tris, k, A, B, C);
            double t, u, v;
            if (!mt_f64(o, d, A, B, C, c->eps64, &t, &u, &v)) continue;
            if (!(t >= c->tmin64 && t <= tmax)) continue;
            if (t < bt) {
                bt = t;
                bu = u;
                bv = v;
                bi = (int32_t)k;
            }
        }
        c->t64[i] = bt;
        c->tri[i] = bi;
        if (c->uv64) {
            c->uv64[2 * i] = bu;
            c->uv64[2 * i + 1] = bv;
        }
    }
}

double orc_ray_brute_f32(const float* verts, const int32_t* tris, int64_t nt, const float* orig,
                         const float* dir, const float* tmax_per_ray, int64_t n, float tmin,
                         float tmax, float det_eps, float* out_t, int32_t* out_tri, float* out_uv,
                         int nthreads) {
    ray_ctx c;
    memset(&c, 0, sizeof c);
    c.verts = verts;
    c.tris = tris;
    c.nt = nt;
    c.orig = orig;
    c.dir = dir;
    c.tmax_per = tmax_per_ray;
    c.tmin = tmin;
    c.tmax = tmax;
    c.eps = det_eps;
    c.t32 = out_t;
    c.uv32 = out_uv;
    c.tri = out_tri;
    double t0 = now_s();
    parallel_for(n, 16, nthreads, ray32_range, &c);
    return now_s() - t0;
}

double orc_ray_brute_f64(const float* verts, const int32_t* tris, int64_t nt, const float* orig,
                         const float* dir, const float* tmax_per_ray, int64_t n, double tmin,
                         double tmax, double det_eps, double* out_t, int32_t* out_tri,
                         double* out_uv, int nthreads) {
    ray_ctx c;
    memset(&c, 0, sizeof c);
    c.verts = verts;
    c.tris = tris;
    c.nt = nt;
    c.orig = orig;
    c.dir = dir;
    c.tmax_per = tmax_per_ray;
    c.tmin64 = tmin;
    c.tmax64 = tmax;
    c.eps64 = det_eps;
    c.t64 = out_t;
    c.uv64 = out_uv;
    c.tri = out_tri;
    double t0 = now_s();
    parallel_for(n, 16, nthreads, ray64_range, &c);
    return now_s() - t0;
}

/* ===================================================================== */
/* FP64 brute force over FP64 vertices                                    */
/* ===================================================================== */

typedef struct {
    const double* verts;
    const int32_t* tris;
    int64_t nt;
    const float* q;
    double *d2, *p;
    int32_t* tri;
} brute_dv_ctx;

static void brute_dv_range(void* vctx, int64_t b, int64_t e) {
    brute_dv_ctx* c = (brute_dv_ctx*)vctx;
    for (int64_t i = b; i < e; ++i) {
        double q[3] = {c->q[3 * i], c->q[3 * i + 1], c->q[3 * i + 2]};
        double best = INFINITY, bp[3] = {0, 0, 0};
        int32_t bt = -1;
        for (int64_t t = 0; t < c->nt; ++t) {
            const int32_t* ix = c->tris + 3 * t;
            double cp[3], w[3];
            double d2 = orc_point_tri_f64(q, c->verts + 3 * (int64_t)ix[0], c->verts + 3 * (int64_t)ix[1],
                                          c->verts + 3 * (int64_t)ix[2], cp, w);
            if (d2 < best) {
                best = d2;
                bt = (int32_t)t;
                memcpy(bp, cp, sizeof bp);
            }
        }
        c->d2[i] = best;
        c->tri[i] = bt;
        if (c->p) memcpy(c->p + 3 * i, bp, sizeof bp);
    }
}

void orc_brute_f64_dv(const double* verts, const int32_t* tris, int64_t nt, const float* q, int64_t nq,
                      double* out_d2, int32_t* out_tri, double* out_p, int nthreads) {
    brute_dv_ctx c = {verts, tris, nt, q, out_d2, out_p, out_tri};
    parallel_for(nq, 16, nthreads, brute_dv_range, &c);
}

/* FP64 closest hit over FP64 vertices (instanced scenes placed in FP64). */
typedef struct {
    const double* verts;
    const int32_t* tris;
    int64_t nt;
    const float *orig, *dir;
    double tmin, tmax;
    double *t, *uv;
    int32_t* tri;
} ray_dv_ctx;

static void ray_dv_range(void* vctx, int64_t b, int64_t e) {
    ray_dv_ctx* c = (ray_dv_ctx*)vctx;
    for (int64_t i = b; i < e; ++i) {
        const double o[3] = {c->orig[3 * i], c->orig[3 * i + 1], c->orig[3 * i + 2]};
        const double d[3] = {c->dir[3 * i], c->dir[3 * i + 1], c->dir[3 * i + 2]};
        double bt = INFINITY, bu = 0.0, bv = 0.0;
        int32_t bi = -1;
        for (int64_t k = 0; k < c->nt; ++k) {
            const int32_t* ix = c->tris + 3 * k;
            double t, u, v;
            if (!mt_f64(o, d, c->verts + 3 * (int64_t)ix[0], c->verts + 3 * (int64_t)ix[1],
                        c->verts + 3 * (int64_t)ix[2], 0.0, &t, &u, &v))
                continue;
            if (!(t >= c->tmin && t <= c->tmax)) continue;
            if (t < bt) {
                bt = t;
                bu = u;
                bv = v;
                bi = (int32_t)k;
            }
        }
        c->t[i] = bt;
        c->tri[i] = bi;
        c->uv[2 * i] = bu;
        c->uv[2 * i + 1] = bv;
    }
}

void orc_ray_brute_f64_dv(const double* verts, const int32_t* tris, int64_t nt, const float* orig,
                          const float* dir, int64_t n, double tmin, double tmax, double* out_t,
                          int32_t* out_tri, double* out_uv, int nthreads) {
    ray_dv_ctx c = {verts, tris, nt, orig, dir, tmin, tmax, out_t, out_uv, out_tri};
    parallel_for(n, 16, nthreads, ray_dv_range, &c);
}
