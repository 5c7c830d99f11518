"""Seeded synthetic meshes and query sets for the closest-point workloads.

No public benchmark suite or dataset is involved: the reference measures none
for this path.  Every generator is deterministic for a given seed (numpy PCG64
streams) and returns float32 vertices, int32 triangles and float32 queries.

Workloads (M = 2**20):
  small     icosphere subdivided 4x (5,120 tris, 2,562 verts, r = 1), 65,536
            queries uniform in [-2, 2]^3
  large     1024 x 1024-vertex heightfield on [0,1]^2 (2,093,058 tris):
            z = sum of 8 sinusoids, frequencies U[1, 32], amplitude 0.05/f,
            random direction and phase, plus N(0, 1e-3) jitter in z; 16 M
            queries, half at random surface points + N(0, 0.01^2) per axis,
            half uniform in [-0.1, 1.1]^2 x [-0.5, 0.5], shuffled
  torus     R = 1, r = 0.3, 500 x 200 grid (200,000 tris); 4 M queries uniform
            in [-1.5, 1.5]^3; upstream gradient N(0, 1)
  batched   256 meshes, icosphere or torus with per-vertex noise of amplitude
            0.05 along the surface normal, triangle counts log-uniform in
            [1k, 500k] (nearest icosphere level / torus grid), query counts
            log-uniform in [1k, 1M], uniform in each mesh's box scaled 1.5x
  soup      4,096 Gaussian clusters (centres U[0,1]^3, vertices N(c, 0.01^2)),
            2,048 triangles each (8 M tris); queries uniform in [0,1]^3
"""
from __future__ import annotations

import math

import numpy as np

M = 1 << 20


def icosahedron():
    phi = (1.0 + 5.0 ** 0.5) / 2.0
    v = []
    for a in (-1.0, 1.0):
        for b in (-phi, phi):
            v.append((a, b, 0.0))
            v.append((0.0, a, b))
            v.append((b, 0.0, a))
    v = np.array(v, dtype=np.float64)
    # faces: every triple of mutually adjacent vertices (edge length 2)
    d = np.linalg.norm(v[:, None, :] - v[None, :, :], axis=-1)
    adj = np.abs(d - 2.0) < 1e-9
    faces = []
    for i in range(12):
        for j in range(i + 1, 12):
            if not adj[i, j]:
                continue
            for k in range(j + 1, 12):
                if adj[i, k] and adj[j, k]:
                    a, b, c = v[i], v[j], v[k]
                    if np.dot(np.cross(b - a, c - a), a + b + c) < 0:
                        faces.append((i, k, j))
                    else:
                        faces.append((i, j, k))
    f = np.array(faces, dtype=np.int64)
    assert f.shape == (20, 3)
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


def icosphere(level: int, radius: float = 1.0):
    """Unit icosahedron subdivided `level` times (each face into 4), on a sphere."""
    v, f = icosahedron()
    for _ in range(level):
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        edges = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)])
        edges = np.sort(edges, axis=1)
        key = edges[:, 0] * (v.shape[0] + 1) + edges[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        e0, e1 = uniq // (v.shape[0] + 1), uniq % (v.shape[0] + 1)
        mid = 0.5 * (v[e0] + v[e1])
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = v.shape[0]
        v = np.concatenate([v, mid])
        nf = f.shape[0]
        ab, bc, ca = base + inv[:nf], base + inv[nf:2 * nf], base + inv[2 * nf:]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
                            np.stack([ca, bc, c], 1), np.stack([ab, bc, ca], 1)])
    return (v * radius).astype(np.float32), f.astype(np.int32)


def torus(nu: int = 500, nv: int = 200, R: float = 1.0, r: float = 0.3):
    """Torus grid: nu steps around the main ring, nv around the tube; 2*nu*nv tris."""
    u = 2.0 * np.pi * np.arange(nu) / nu
    w = 2.0 * np.pi * np.arange(nv) / nv
    U, W = np.meshgrid(u, w, indexing="ij")
    x = (R + r * np.cos(W)) * np.cos(U)
    y = (R + r * np.cos(W)) * np.sin(U)
    z = r * np.sin(W)
    verts = np.stack([x, y, z], -1).reshape(-1, 3)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    i1, j1 = (i + 1) % nu, (j + 1) % nv
    v00, v10, v11, v01 = i * nv + j, i1 * nv + j, i1 * nv + j1, i * nv + j1
    t0 = np.stack(np.broadcast_arrays(v00, v10, v11), -1).reshape(-1, 3)
    t1 = np.stack(np.broadcast_arrays(v00, v11, v01), -1).reshape(-1, 3)
    tris = np.stack([t0, t1], 1).reshape(-1, 3)
    return verts.astype(np.float32), tris.astype(np.int32)


def torus_normals(nu: int, nv: int):
    u = 2.0 * np.pi * np.arange(nu) / nu
    w = 2.0 * np.pi * np.arange(nv) / nv
    U, W = np.meshgrid(u, w, indexing="ij")
    n = np.stack([np.cos(W) * np.cos(U), np.cos(W) * np.sin(U), np.sin(W)], -1)
    return n.reshape(-1, 3)


def heightfield_params(seed: int, count: int = 8):
    rng = np.random.default_rng(seed)
    freq = rng.uniform(1.0, 32.0, count)
    theta = rng.uniform(0.0, 2.0 * np.pi, count)
    phase = rng.uniform(0.0, 2.0 * np.pi, count)
    amp = 0.05 / freq
    return freq, theta, phase, amp


def heightfield(n: int = 1024, seed: int = 1, jitter: float = 1e-3):
    """n x n vertex grid over [0,1]^2 with z = sum of 8 sinusoids + N(0, jitter) noise."""
    freq, theta, phase, amp = heightfield_params(seed)
    g = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(g, g, indexing="ij")
    Z = np.zeros_like(X)
    for f, t, p, a in zip(freq, theta, phase, amp):
        Z += a * np.sin(2.0 * np.pi * f * (X * np.cos(t) + Y * np.sin(t)) + p)
    rng = np.random.default_rng(seed + 1000)
    Z += rng.normal(0.0, jitter, Z.shape)
    verts = np.stack([X, Y, Z], -1).reshape(-1, 3)
    i = np.arange(n - 1)[:, None]
    j = np.arange(n - 1)[None, :]
    v00, v10, v11, v01 = i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1
    t0 = np.stack(np.broadcast_arrays(v00, v10, v11), -1).reshape(-1, 3)
    t1 = np.stack(np.broadcast_arrays(v00, v11, v01), -1).reshape(-1, 3)
    tris = np.stack([t0, t1], 1).reshape(-1, 3)
    return verts.astype(np.float32), tris.astype(np.int32)


def surface_points(verts: np.ndarray, tris: np.ndarray, count: int, rng) -> np.ndarray:
    """Uniform random triangles, uniform barycentric points on them."""
    t = rng.integers(0, tris.shape[0], count)
    r1 = np.sqrt(rng.random(count))
    r2 = rng.random(count)
    a, b, c = (verts[tris[t, k]].astype(np.float64) for k in range(3))
    return (1 - r1)[:, None] * a + (r1 * (1 - r2))[:, None] * b + (r1 * r2)[:, None] * c


def heightfield_queries(verts: np.ndarray, tris: np.ndarray, count: int, seed: int = 2,
                        sigma: float = 0.01) -> np.ndarray:
    rng = np.random.default_rng(seed)
    near = count // 2
    p = surface_points(verts, tris, near, rng) + rng.normal(0.0, sigma, (near, 3))
    far = count - near
    box = np.stack([rng.uniform(-0.1, 1.1, far), rng.uniform(-0.1, 1.1, far),
                    rng.uniform(-0.5, 0.5, far)], -1)
    q = np.concatenate([p, box]).astype(np.float32)
    return q[rng.permutation(count)]


def uniform_queries(count: int, lo, hi, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    lo = np.broadcast_to(np.asarray(lo, np.float64), (3,))
    hi = np.broadcast_to(np.asarray(hi, np.float64), (3,))
    return (lo + (hi - lo) * rng.random((count, 3))).astype(np.float32)


def small(seed: int = 0, nq: int = 65536):
    verts, tris = icosphere(4)
    q = uniform_queries(nq, -2.0, 2.0, seed)
    return verts, tris, q


def large(seed: int = 1, nq: int = 16 * M, n: int = 1024):
    verts, tris = heightfield(n, seed)
    q = heightfield_queries(verts, tris, nq, seed + 1)
    return verts, tris, q


def torus_workload(seed: int = 3, nq: int = 4 * M):
    verts, tris = torus(500, 200)
    q = uniform_queries(nq, -1.5, 1.5, seed)
    g = np.random.default_rng(seed + 1).normal(0.0, 1.0, nq).astype(np.float32)
    return verts, tris, q, g


def _noisy(verts: np.ndarray, normals: np.ndarray, amp: float, rng) -> np.ndarray:
    return (verts + amp * rng.uniform(-1.0, 1.0, (verts.shape[0], 1)) * normals).astype(np.float32)


def batched(seed: int = 4, nmeshes: int = 256, tri_range=(1000, 500_000), q_range=(1000, M),
            noise: float = 0.05):
    """List of meshes (verts, tris, kind) and per-mesh query arrays."""
    rng = np.random.default_rng(seed)
    levels = np.arange(3, 8)
    sphere_counts = 20 * 4 ** levels
    cache = {}
    meshes, queries = [], []
    for m in range(nmeshes):
        target = math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))
        if rng.random() < 0.5:
            lvl = int(levels[np.argmin(np.abs(np.log(sphere_counts) - math.log(target)))])
            if ("s", lvl) not in cache:
                cache[("s", lvl)] = icosphere(lvl)
            v, t = cache[("s", lvl)]
            n = v / np.linalg.norm(v, axis=1, keepdims=True)
            kind = f"icosphere{lvl}"
        else:
            nv_ = max(3, int(round(math.sqrt(target * 0.15))))
            nu_ = max(3, int(round(target / (2 * nv_))))
            v, t = torus(nu_, nv_)
            n = torus_normals(nu_, nv_)
            kind = f"torus{nu_}x{nv_}"
        v = _noisy(v, n, noise, rng)
        nq = int(round(math.exp(rng.uniform(math.log(q_range[0]), math.log(q_range[1])))))
        lo, hi = v.min(0).astype(np.float64), v.max(0).astype(np.float64)
        c, h = 0.5 * (lo + hi), 0.75 * (hi - lo)
        q = (c - h + 2 * h * rng.random((nq, 3))).astype(np.float32)
        meshes.append((v, t, kind))
        queries.append(q)
    return meshes, queries


def concat_batch(meshes, queries):
    """Back-to-back arrays and offsets for cp_batch_create / cp_batch_query."""
    voff = np.zeros(len(meshes) + 1, np.int64)
    toff = np.zeros(len(meshes) + 1, np.int64)
    qoff = np.zeros(len(meshes) + 1, np.int64)
    for i, ((v, t, _), q) in enumerate(zip(meshes, queries)):
        voff[i + 1] = voff[i] + v.shape[0]
        toff[i + 1] = toff[i] + t.shape[0]
        qoff[i + 1] = qoff[i] + q.shape[0]
    V = np.concatenate([m[0] for m in meshes])
    T = np.concatenate([m[1] for m in meshes])
    Q = np.concatenate(queries)
    return V, voff, T, toff, Q, qoff


def soup(seed: int = 5, clusters: int = 4096, per: int = 2048, sigma: float = 0.01):
    """Triangle soup: each triangle has 3 own vertices drawn around its cluster centre."""
    rng = np.random.default_rng(seed)
    centres = rng.random((clusters, 3)).astype(np.float32)
    v = rng.standard_normal((clusters, per * 3, 3), dtype=np.float32)
    v *= np.float32(sigma)
    v += centres[:, None, :]
    tris = np.arange(clusters * per * 3, dtype=np.int32).reshape(-1, 3)
    return v.reshape(-1, 3), tris


def random_rotations(n: int, rng) -> np.ndarray:
    """(n, 3, 3) rotations from uniform random unit quaternions, FP64."""
    qr = rng.normal(size=(n, 4))
    qr /= np.linalg.norm(qr, axis=1, keepdims=True)
    w, x, y, z = qr.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                     np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                     np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)


def flatten_instances(meshes, inst_mesh, T):
    """All instances' triangles in one world-space FP32 mesh."""
    wv, wt, off = [], [], 0
    for m, t in zip(inst_mesh, T):
        v, tri = meshes[m]
        t64 = t.astype(np.float64)
        wv.append((v.astype(np.float64) @ t64[:, :3].T + t64[:, 3]).astype(np.float32))
        wt.append(tri + off)
        off += v.shape[0]
    return np.concatenate(wv), np.concatenate(wt).astype(np.int32)


def instanced_scene(seed: int = 31, nq: int = 16 * M, grid: int = 16):
    """grid^3 similarity instances (random rotation, scale 0.6..1.2) of three
    meshes at pitch 3; queries half uniform over the grid, half N(0, 0.02) off
    the instances' surfaces.  Returns (meshes, inst_mesh, T (n, 3, 4) f32, q)."""
    meshes = [icosphere(4), torus(100, 40), heightfield(64, seed=3)]
    n_inst = grid ** 3
    rng = np.random.default_rng(seed)
    inst_mesh = rng.integers(0, len(meshes), n_inst).astype(np.int32)
    R = random_rotations(n_inst, rng)
    g = np.stack(np.meshgrid(*[np.arange(grid)] * 3, indexing="ij"), -1).reshape(-1, 3)
    T = np.zeros((n_inst, 3, 4))
    T[:, :, :3] = R * rng.uniform(0.6, 1.2, n_inst)[:, None, None]
    T[:, :, 3] = 3.0 * g + rng.uniform(-0.3, 0.3, (n_inst, 3))
    T = T.astype(np.float32)
    half = nq // 2
    lo, hi = np.full(3, -2.0), np.full(3, 3.0 * (grid - 1) + 2.0)
    far = rng.uniform(lo, hi, (half, 3))
    k = rng.integers(0, n_inst, nq - half)
    near = np.empty((nq - half, 3))
    for m, (v, tri) in enumerate(meshes):
        sel = np.nonzero(inst_mesh[k] == m)[0]
        p = surface_points(v, tri, len(sel), rng)
        t = T[k[sel]].astype(np.float64)
        near[sel] = np.einsum("nij,nj->ni", t[:, :, :3], p) + t[:, :, 3]
    near += rng.normal(0.0, 0.02, near.shape)
    q = np.concatenate([far, near]).astype(np.float32)
    return meshes, inst_mesh, T, q[rng.permutation(nq)]


def camera_rays(width: int, height: int, eye, yfov: float, aspect: float) -> tuple[np.ndarray, np.ndarray]:
    """Pinhole primary rays through pixel centres, looking down -z from `eye`
    (row 0 at the top): origins (n, 3) and unit directions (n, 3), float32."""
    th = np.tan(0.5 * yfov)
    i = (np.arange(width) + 0.5) / width * 2.0 - 1.0
    j = 1.0 - (np.arange(height) + 0.5) / height * 2.0
    X, Y = np.meshgrid(i * th * aspect, j * th)
    d = np.stack([X, Y, -np.ones_like(X)], -1).reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(np.asarray(eye, np.float64), d.shape)
    return np.ascontiguousarray(o, np.float32), d.astype(np.float32)


# The Cornell box's camera (media/cbox/cbox.gltf: node CamInst, camera
# "default"): eye on the +z axis, looking down -z, vertical field of view
# 0.7175 rad at 4:3; its ceiling light is instance 5.
CBOX_EYE = (0.0, 0.0, 19.992091970966317)
CBOX_YFOV = 0.7175414562225342
CBOX_ASPECT = 4.0 / 3.0
CBOX_LIGHT_INSTANCE = 5
