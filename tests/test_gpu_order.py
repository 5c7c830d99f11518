"""The library's radix sort and the query ordering built on it.

The ordering decides only the order in which queries are walked, never an
answer, but a sort that lost or duplicated an index would drop or repeat
queries (and the build's sort must be stable for bit-exact trees).  These
tests require:

* cp_debug_order_sort to return exactly numpy's stable argsort of the keys'
  bits [begin_bit, end_bit): 32- and 64-bit keys, eight- and ten-bit digits,
  one to seven passes, tile-edge sizes, and key sets with degenerate digit
  distributions (all keys equal, already sorted, reversed, a handful of
  values, a narrow band whose high digits are constant);
* cp_query_order's keys to equal a restatement of Skilling's Hilbert index
  over the FP32 query frame, its permutation to sort them stably, and
  consecutive queries along it to be close.
"""
from __future__ import annotations

import zlib
from ctypes import c_void_p

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(keys: np.ndarray, begin: int, end: int, cuda) -> np.ndarray:
    import torch

    from gpurt_cpq._lib import check, lib

    kb = keys.dtype.itemsize
    dk = torch.from_numpy(keys.view(np.int32 if kb == 4 else np.int64)).to(cuda)
    perm = torch.empty(len(keys), dtype=torch.int32, device=cuda)
    stream = c_void_p(torch.cuda.current_stream().cuda_stream)
    check(lib.cp_debug_order_sort(c_void_p(dk.data_ptr()), kb, len(keys), begin, end, c_void_p(perm.data_ptr()),
                                  stream), "cp_debug_order_sort")
    return perm.cpu().numpy()


def _want(keys: np.ndarray, begin: int, end: int) -> np.ndarray:
    k = keys.astype(np.uint64)
    mask = np.uint64((1 << (end - begin)) - 1) if end - begin < 64 else np.uint64(2**64 - 1)
    return np.argsort((k >> np.uint64(begin)) & mask, kind="stable").astype(np.int32)


def _keys(kind: str, n: int, bits: int, dtype, rng) -> np.ndarray:
    hi = 1 << bits
    if kind == "random":
        k = rng.integers(0, hi, n, dtype=np.uint64)
    elif kind == "equal":
        k = np.full(n, (hi - 1) // 3, np.uint64)
    elif kind == "sorted":
        k = np.sort(rng.integers(0, hi, n, dtype=np.uint64))
    elif kind == "reversed":
        k = np.sort(rng.integers(0, hi, n, dtype=np.uint64))[::-1].copy()
    elif kind == "few":
        k = rng.choice(rng.integers(0, hi, 5, dtype=np.uint64), n)
    else:  # "clustered": a narrow band, so the low digits vary and the high ones do not
        k = (hi // 2) + rng.integers(0, 1 << min(bits, 12), n, dtype=np.uint64)
        k = np.minimum(k, np.uint64(hi - 1))
    return k.astype(dtype)


@pytest.mark.parametrize("dtype,begin,end", [(np.uint32, 0, 30), (np.uint32, 6, 30), (np.uint32, 0, 32),
                                             (np.uint32, 0, 8), (np.uint32, 0, 16), (np.uint32, 3, 13),
                                             (np.uint64, 0, 38), (np.uint64, 0, 63), (np.uint64, 0, 64),
                                             (np.uint64, 20, 50)])
@pytest.mark.parametrize("kind", ["random", "equal", "sorted", "reversed", "few", "clustered"])
def test_order_sort_is_a_stable_argsort(cuda, dtype, begin, end, kind):
    rng = np.random.default_rng(zlib.crc32(f"{kind} {begin} {end} {dtype.__name__}".encode()))
    tile = 8192 if dtype == np.uint32 else 2048
    for n in (2, 3, 1000, tile - 1, tile, tile + 1, 3 * tile + 17, 70_001):
        keys = _keys(kind, n, end, dtype, rng)
        got = _sort(keys, begin, end, cuda)
        want = _want(keys, begin, end)
        assert np.array_equal(got, want), (kind, n, begin, end, np.nonzero(got != want)[0][:5])


def test_order_sort_large(cuda):
    """16,777,216 30-bit keys (the headline query count) and 4M 40-bit keys."""
    rng = np.random.default_rng(5)
    k32 = rng.integers(0, 1 << 30, 1 << 24, dtype=np.uint64).astype(np.uint32)
    assert np.array_equal(_sort(k32, 0, 30, cuda), _want(k32, 0, 30))
    k64 = rng.integers(0, 1 << 40, 1 << 22, dtype=np.uint64)
    assert np.array_equal(_sort(k64, 0, 40, cuda), _want(k64, 0, 40))


def _hilbert3(x, y, z, bits):
    """Skilling's 3D Hilbert index (2004, "Programming the Hilbert curve"),
    vectorised: undo the excess rotations and reflections level by level,
    Gray-decode, interleave the transposed coordinates (x's bit highest)."""
    X = [x.astype(np.uint64), y.astype(np.uint64), z.astype(np.uint64)]
    Q = 1 << (bits - 1)
    while Q > 1:
        P = np.uint64(Q - 1)
        for i in range(3):
            hi = (X[i] & np.uint64(Q)) != 0
            t = (X[0] ^ X[i]) & P
            X[0] = np.where(hi, X[0] ^ P, X[0] ^ t)
            if i:
                X[i] = np.where(hi, X[i], X[i] ^ t)
        Q >>= 1
    X[1] ^= X[0]
    X[2] ^= X[1]
    t = np.zeros_like(X[0])
    Q = 1 << (bits - 1)
    while Q > 1:
        t = np.where((X[2] & np.uint64(Q)) != 0, t ^ np.uint64(Q - 1), t)
        Q >>= 1
    X = [v ^ t for v in X]
    out = np.zeros_like(X[0])
    for b in range(bits):
        for j in range(3):
            out |= ((X[j] >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + 2 - j)
    return out


def _query_cells(q):
    """Each query's cell in the isotropic 1024^3 frame over the query box, in
    FP32 as the ordering computes it."""
    q = q.astype(np.float32)
    lo, hi = q.min(0), q.max(0)
    ext = np.float32((hi - lo).max())
    scale = np.float32(1024.0) / ext
    t = (q - lo) * scale
    return np.minimum(np.maximum(t, np.float32(0)), np.float32(1023)).astype(np.uint32)


def test_query_order_sorts_its_keys(cpq, cuda):
    import torch

    from gpurt_cpq import workloads as W

    v, t = W.heightfield(256, seed=3)
    m = cpq.Mesh(torch.from_numpy(v).to(cuda), torch.from_numpy(t).to(cuda), branching=4, leaf_size=8)
    q = np.concatenate([W.heightfield_queries(v, t, 300_000, seed=4), W.uniform_queries(100_000, -0.2, 1.2, 5)])
    perm, keys = m.query_order(torch.from_numpy(q).to(cuda))
    perm, keys = perm.cpu().numpy(), keys.cpu().numpy()
    assert keys.max() < 1 << 30
    c = _query_cells(q)
    assert np.array_equal(keys, _hilbert3(c[:, 0], c[:, 1], c[:, 2], 10).astype(np.int64))
    assert np.array_equal(np.sort(perm), np.arange(len(q)))
    assert np.array_equal(perm, np.argsort(keys, kind="stable"))
    # neighbours along the curve are close: far closer than random pairs
    walk = np.linalg.norm(np.diff(q[perm], axis=0), axis=1).mean()
    rand = np.linalg.norm(np.diff(q, axis=0), axis=1).mean()
    assert walk < 0.05 * rand, (walk, rand)
