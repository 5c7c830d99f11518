"""The restatement's box arithmetic against the reference's own math headers.

oracle/make_ref_lib.py compiles the reference's src/lib headers (mathlib.h
and what it includes) as they are, with a thin C wrapper
(oracle/ref_lib_wrap.cpp).  These tests require:

* every binary-node box of the restatement's build (leaf: the triangle's
  vertices; inner: the children's boxes) to equal BBox::enclose
  (src/lib/bbox.h:35-42) over the same points and boxes;
* every SAH cost of the restatement's build to equal the costs recomputed
  from BBox::surface_area (bbox.h:55-59) halved, bit for bit, for two cost
  ratios — the restatement's half area sums the products in surface_area's
  order, so twice it is that function's value exactly;
* the closest point of the restatement's FP64 point-triangle routine, for
  points in an edge's Voronoi region, to agree with Line::closest
  (src/lib/line.h:28-32) on that edge's line to FP32 rounding.

The GPU build equals the restatement bit for bit (test_gpu_parity.py), so the
GPU's boxes and SAH decisions are pinned to the reference's code through it.
Skipped where no checkout of the reference exists.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import make_ref_lib

REF = make_ref_lib.load()
pytestmark = pytest.mark.skipif(REF is None, reason="no checkout of the reference's math headers")


def _p(a):
    from ctypes import c_void_p
    return c_void_p(a.ctypes.data)


def ref_triangle_boxes(tris9):
    tris9 = np.ascontiguousarray(tris9, np.float32)
    out = np.empty((tris9.shape[0], 6), np.float32)
    REF.ref_bbox_triangles(tris9.shape[0], _p(tris9), _p(out))
    return out


def ref_merge(a, b):
    a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
    out = np.empty_like(a)
    REF.ref_bbox_merge(a.shape[0], _p(a), _p(b), _p(out))
    return out


def ref_area(boxes):
    boxes = np.ascontiguousarray(boxes, np.float32)
    out = np.empty(boxes.shape[0], np.float32)
    REF.ref_bbox_area(boxes.shape[0], _p(boxes), _p(out))
    return out


def _meshes():
    from gpurt_cpq import workloads as W

    rng = np.random.default_rng(3)
    rv = rng.normal(size=(400, 3)).astype(np.float32)
    rt = rng.integers(0, 400, (1500, 3)).astype(np.int32)
    return {"icosphere4": W.icosphere(4), "heightfield64": W.heightfield(64, seed=9), "random": (rv, rt)}


@pytest.mark.parametrize("name", ["icosphere4", "heightfield64", "random"])
@pytest.mark.parametrize("c_tri", [1.0, 0.4])
def test_boxes_and_sah_costs_match_bbox(orc, name, c_tri):
    v, t = _meshes()[name]
    leaf = 8
    T = orc.Tree(v, t, 4, leaf, 1, 1.0, c_tri)
    n = T.nt
    # leaves: the sorted triangles' boxes
    leaves = ref_triangle_boxes(v[t[T.order]].reshape(-1, 9))
    assert np.array_equal(T.box[n - 1:], leaves)  # value equality (+0 and -0 alike)
    # inner nodes: the children's boxes enclosed
    inner = np.arange(n - 1)
    assert np.array_equal(T.box[inner], ref_merge(T.box[T.left[inner]], T.box[T.right[inner]]))
    # SAH costs from the reference's surface area, halved (exact)
    half = ref_area(T.box) * np.float32(0.5)
    assert np.array_equal(T.cost[n - 1:].view(np.uint32), (np.float32(c_tri) * np.float32(1.0) * half[n - 1:]).view(np.uint32))
    cost = T.cost.copy()
    cost[:n - 1] = np.nan
    size = T.last - T.first + 1
    one = np.float32
    for p in inner[np.argsort(size[inner], kind="stable")]:  # children before parents
        a = half[p]
        split = one(1.0) * a
        split = split + cost[T.left[p]]
        split = split + cost[T.right[p]]
        leafc = (one(c_tri) * one(size[p])) * a
        cost[p] = leafc if (size[p] <= leaf and leafc <= split) else split
    assert np.array_equal(cost.view(np.uint32), T.cost.view(np.uint32))


def test_edge_projection_matches_line_closest(orc):
    """Points in the Voronoi region of a triangle's edge ab (beyond ab in the
    triangle's plane, above or below it, projecting inside the segment): the
    FP64 closest point lies on ab and equals Line(a, b - a).closest(p)."""
    rng = np.random.default_rng(8)
    n = 4000
    a = rng.normal(size=(n, 3))
    b = a + rng.normal(size=(n, 3))
    c = a + rng.normal(size=(n, 3))
    ab = b - a
    nrm = np.cross(ab, c - a)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    out = np.cross(ab, nrm)  # in the plane, perpendicular to ab
    out /= np.linalg.norm(out, axis=1, keepdims=True)
    out *= np.sign(np.einsum("ij,ij->i", out, a - c))[:, None]  # away from c
    t = rng.uniform(0.05, 0.95, n)
    q = a + t[:, None] * ab + rng.uniform(0.01, 1.0, n)[:, None] * out + rng.uniform(-1, 1, n)[:, None] * nrm
    a32, b32, c32, q32 = (x.astype(np.float32) for x in (a, b, c, q))
    want = np.empty((n, 3))
    for i in range(n):
        _, cp, w = orc.point_tri_f64(q32[i], a32[i], b32[i], c32[i])
        assert w[2] == 0.0 and 0.0 < w[1] < 1.0, "not in the edge region"
        want[i] = cp
    got = np.empty((n, 3), np.float32)
    d32 = np.ascontiguousarray(b32 - a32)
    REF.ref_line_closest(n, _p(np.ascontiguousarray(a32)), _p(d32), _p(np.ascontiguousarray(q32)), _p(got))
    scale = np.abs(np.stack([a32, b32, q32])).max(axis=(0, 2))
    err = np.linalg.norm(got.astype(np.float64) - want, axis=1) / scale
    assert err.max() < 4e-6, err.max()
