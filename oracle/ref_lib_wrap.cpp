// ORACLE (test infrastructure only): C entry points over the reference's own
// math headers (src/lib/mathlib.h and what it includes: bbox.h, line.h,
// vec3.h), compiled as they are from a checkout of the reference by
// oracle/make_ref_lib.py into the git-ignored oracle/_ref/.  The tests compare
// the restatement's box and SAH arithmetic and its edge projection against
// them.  Nothing in the product links this file.
#include <cstdint>

// the reference's own entry to its math library: macros, then every header in
// its order (bbox.h, line.h, mat4.h and vec3.h among them)
#include "mathlib.h"

namespace {

Vec3 v3(const float* p) { return Vec3(p[0], p[1], p[2]); }
void put(const Vec3& v, float* o) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
}
void put_box(const BBox& b, float* o) {
    put(b.min, o);
    put(b.max, o + 3);
}

}  // namespace

extern "C" {

// BBox::enclose of each triangle's three vertices, in vertex order
// (tris9: n x 9 floats); out: n x 6 (min xyz, max xyz).
void ref_bbox_triangles(int64_t n, const float* tris9, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        BBox b;
        for (int j = 0; j < 3; ++j) b.enclose(v3(tris9 + 9 * i + 3 * j));
        put_box(b, out + 6 * i);
    }
}

// BBox a.enclose(BBox b) per pair (n x 6 each).
void ref_bbox_merge(int64_t n, const float* a, const float* b, float* out) {
    for (int64_t i = 0; i < n; ++i) {
        BBox x(v3(a + 6 * i), v3(a + 6 * i + 3));
        x.enclose(BBox(v3(b + 6 * i), v3(b + 6 * i + 3)));
        put_box(x, out + 6 * i);
    }
}

// BBox::surface_area per box (n x 6).
void ref_bbox_area(int64_t n, const float* boxes, float* area) {
    for (int64_t i = 0; i < n; ++i) area[i] = BBox(v3(boxes + 6 * i), v3(boxes + 6 * i + 3)).surface_area();
}

// Line(point, dir).closest(pt) per row (each n x 3); the direction is made
// unit by the constructor, as the reference does.
void ref_line_closest(int64_t n, const float* point, const float* dir, const float* pt, float* out) {
    for (int64_t i = 0; i < n; ++i) put(Line(v3(point + 3 * i), v3(dir + 3 * i)).closest(v3(pt + 3 * i)), out + 3 * i);
}

}  // extern "C"
