"""Oracle for the visibility-edge hot path — TEST INFRASTRUCTURE.

A CPU (FP64, OpenMP) restatement of the reference algorithms, used only by the
tests, the smoke check and the benchmark's CPU-baseline leg to check and time
the GPU kernels. The product (visacd_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build_oracle import build as _build

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build()
        L = C.CDLL(str(path))
        P = C.c_void_p
        i32, i64 = C.c_int32, C.c_int64
        L.oracle_num_threads.restype = C.c_int
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_score_planes.argtypes = [P, i32, P, i32, P, i64, P, P, C.POINTER(i32), C.POINTER(i64)]
        L.oracle_score_planes_ref32.argtypes = [P, i32, P, i32, P, i64, P]
        L.oracle_visibility.argtypes = [P, i32, P, P, i32, P, i32, P, i32, C.c_int, i32, i32, P,
                                        C.POINTER(i64), C.POINTER(i64)]
        L.oracle_visibility.restype = i64
        L.oracle_visibility_rows.argtypes = [P, i32, P, P, i32, P, P, i32, P, i32, P,
                                             C.POINTER(i64), C.POINTER(i64)]
        L.oracle_visibility_rows.restype = i64
        L.oracle_candidate_planes.argtypes = [P, P, i64, i32, C.c_uint32, P, C.POINTER(i32)]
        L.oracle_edge_draws.argtypes = [i64, i32, C.c_uint32, P]
        L.oracle_seg_tri_batch.argtypes = [P, P, i64, P]
        L.oracle_seg_tri_batch.restype = i64
        L.oracle_candidate_planes.restype = i32
        L.oracle_sample_points.argtypes = [P, P, i32, i32, C.c_uint32, P, P, i64, P]
        L.oracle_sample_points.restype = i64
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def num_threads() -> int:
    return lib().oracle_num_threads()


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def score_planes(planes, points, edges):
    """FP64 scores, exact quantized integer scores, qexp, skipped-edge count."""
    pl = np.ascontiguousarray(planes, dtype=np.float32).reshape(-1, 4)
    pt = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    ed = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    s64 = np.zeros(len(pl), dtype=np.float64)
    q = np.zeros(len(pl), dtype=np.uint64)
    qexp = C.c_int32()
    skipped = C.c_int64()
    lib().oracle_score_planes(_p(pl), len(pl), _p(pt), len(pt), _p(ed), len(ed), _p(s64), _p(q),
                              C.byref(qexp), C.byref(skipped))
    return s64, q, qexp.value, skipped.value


def score_planes_ref32(planes, points, edges):
    """The reference kernel's FP32 arithmetic in edge order (float scores)."""
    pl = np.ascontiguousarray(planes, dtype=np.float32).reshape(-1, 4)
    pt = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
    ed = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros(len(pl), dtype=np.float32)
    lib().oracle_score_planes_ref32(_p(pl), len(pl), _p(pt), len(pt), _p(ed), len(ed), _p(out))
    return out


def visibility(pts, tris, cage_verts, cage_tris, is_new=None, use_bvh=True, rows=None):
    """Per-pair result bytes (bit0 edge, bit1 grazing), edge list, counters."""
    p = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(tris, dtype=np.uint32).reshape(-1, 3)
    cv = np.ascontiguousarray(cage_verts, dtype=np.float32).reshape(-1, 3)
    ct = np.ascontiguousarray(cage_tris, dtype=np.uint32).reshape(-1, 3)
    m = None if is_new is None else np.ascontiguousarray(is_new, dtype=np.uint8)
    n = len(p)
    r0, r1 = (0, n) if rows is None else rows
    npairs = n * (n - 1) // 2
    bits = np.zeros(npairs, dtype=np.uint8)
    ng = C.c_int64()
    npr = C.c_int64()
    ne = lib().oracle_visibility(_p(p), n, _p(m), _p(t), len(t), _p(cv), len(cv), _p(ct), len(ct),
                                 int(use_bvh), r0, r1, _p(bits), C.byref(ng), C.byref(npr))
    edges = pairs_from_linear(np.nonzero(bits & 1)[0], n)
    return bits, edges, {"n_edges": int(ne), "n_grazing": ng.value, "pairs": npr.value}


def visibility_rows(pts, tris, cage_verts, cage_tris, rows, bits=None):
    """visibility() (BVH traversal) for an explicit list of pair rows; bits, if
    given, is the n(n-1)/2 result array to write into (only those rows)."""
    p = np.ascontiguousarray(pts, dtype=np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(tris, dtype=np.uint32).reshape(-1, 3)
    cv = np.ascontiguousarray(cage_verts, dtype=np.float32).reshape(-1, 3)
    ct = np.ascontiguousarray(cage_tris, dtype=np.uint32).reshape(-1, 3)
    r = np.ascontiguousarray(rows, dtype=np.int32)
    n = len(p)
    if bits is None:
        bits = np.zeros(n * (n - 1) // 2, dtype=np.uint8)
    ng = C.c_int64()
    npr = C.c_int64()
    ne = lib().oracle_visibility_rows(_p(p), n, None, _p(t), len(t), _p(cv), _p(ct), len(ct), _p(r),
                                      len(r), _p(bits), C.byref(ng), C.byref(npr))
    return bits, {"n_edges": int(ne), "n_grazing": ng.value, "pairs": npr.value}


def pairs_from_linear(k: np.ndarray, n: int) -> np.ndarray:
    """Row-major linear pair index -> (i, j), i < j."""
    k = np.asarray(k, dtype=np.int64)
    if len(k) == 0:
        return np.zeros((0, 2), dtype=np.uint32)
    b = 2 * n - 1
    i = np.floor((b - np.sqrt(np.maximum(b * b - 8.0 * k, 0.0))) / 2).astype(np.int64)
    start = lambda r: r * (2 * n - r - 1) // 2  # noqa: E731
    i = np.clip(i, 0, n - 2)
    for _ in range(3):
        i = np.where(start(i) > k, i - 1, i)
        i = np.where((i + 1 <= n - 2) & (start(i + 1) <= k), i + 1, i)
    j = k - start(i) + i + 1
    return np.stack([i, j], axis=1).astype(np.uint32)


def linear_from_pairs(e: np.ndarray, n: int) -> np.ndarray:
    e = np.asarray(e, dtype=np.int64)
    i, j = e[:, 0], e[:, 1]
    return i * (2 * n - i - 1) // 2 + (j - i - 1)


def candidate_planes(verts, edges, num_planes: int, seed: int) -> np.ndarray:
    v = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1, 3)
    e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros((num_planes, 4), dtype=np.float64)
    n = lib().oracle_candidate_planes(_p(v), _p(e), len(e), num_planes, seed, _p(out), None)
    return out[:n]


def candidate_planes_with_draws(verts, edges, num_planes: int, seed: int):
    """candidate_planes plus the raw edge draws (5 num_planes of them) and how
    many the loop consumed."""
    v = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1, 3)
    e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros((max(num_planes, 1), 4), dtype=np.float64)
    used = C.c_int32()
    n = lib().oracle_candidate_planes(_p(v), _p(e), len(e), num_planes, seed, _p(out), C.byref(used))
    draws = np.zeros(5 * num_planes, dtype=np.int32)
    lib().oracle_edge_draws(len(e), len(draws), seed, _p(draws))
    return out[:n], draws, used.value


def seg_tri_batch(seg, tri):
    """Independent FP64 segment-triangle decisions: (hit bool[S], grazing bool[S])."""
    sg = np.ascontiguousarray(np.asarray(seg, dtype=np.float32)).reshape(-1, 6)
    tr = np.ascontiguousarray(np.asarray(tri, dtype=np.float32)).reshape(-1, 9)
    out = np.zeros(len(sg), np.uint8)
    lib().oracle_seg_tri_batch(_p(sg), _p(tr), len(sg), _p(out))
    return (out & 1).astype(bool), (out & 2).astype(bool)


def sample_points(verts, tris, res: int, seed: int):
    """Surface samples of the reference's extract_point_set (base 1, one per
    untouched triangle) on std::mt19937(seed): (xyz, triangle ids, the
    engine's next four outputs)."""
    v = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    cap = 64 * max(res, 1000) + 2 * len(t) + 16
    xyz = np.zeros((cap, 3), dtype=np.float64)
    ids = np.zeros(cap, dtype=np.int32)
    nxt = np.zeros(4, dtype=np.uint32)
    n = lib().oracle_sample_points(_p(v), _p(t), len(t), res, seed, _p(xyz), _p(ids), cap, _p(nxt))
    if n < 0:
        raise ValueError("sample capacity too small")
    return xyz[:n], ids[:n], nxt
