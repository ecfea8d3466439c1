"""Seeded synthetic meshes for tests and benchmarks (numpy only).

* torus(R, r, nu, nv, perturb, seed): nu x nv grid, each vertex's tube radius
  scaled by 1 + U(-perturb, perturb).
* icosphere(level): unit icosphere, 10 * 4^level + 2 vertices.
* displaced_blob(level, seed): icosphere with radius
  r(u) = 1 + 0.3 * sum_k a_k exp(-|u - c_k|^2 / (2 * 0.15^2)), k = 1..8,
  a_k ~ U(-1, 1), c_k uniform on the unit sphere.
* offset_cage(verts, tris, dist): every vertex moved by `dist` along its
  area-weighted normal — a quick stand-in cage for kernel-level workloads.
* segment_triangle_cases(n, graze_frac, seed): independent segment-triangle
  tests, a fraction of them built to pass within 1e-6 of a triangle edge.

All functions return (vertices float64 (n, 3), triangles int32 (m, 3)).
"""
from __future__ import annotations

import functools

import numpy as np


def torus(R: float = 1.0, r: float = 0.35, nu: int = 64, nv: int = 32, perturb: float = 0.02,
          seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    u = 2.0 * np.pi * np.arange(nu) / nu
    v = 2.0 * np.pi * np.arange(nv) / nv
    uu, vv = np.meshgrid(u, v, indexing="ij")
    rr = r * (1.0 + rng.uniform(-perturb, perturb, size=uu.shape))
    x = (R + rr * np.cos(vv)) * np.cos(uu)
    y = (R + rr * np.cos(vv)) * np.sin(uu)
    z = rr * np.sin(vv)
    verts = np.stack([x, y, z], axis=-1).reshape(-1, 3)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = (i * nv + j)
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    t1 = np.stack([a, b, c], axis=-1).reshape(-1, 3)
    t2 = np.stack([a, c, d], axis=-1).reshape(-1, 3)
    tris = np.concatenate([t1, t2], axis=0).astype(np.int32)
    return verts.astype(np.float64), tris


def _icosahedron() -> tuple[np.ndarray, np.ndarray]:
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v, f


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    v, f = _icosphere_cached(level)
    return v.copy(), f.copy()


@functools.lru_cache(maxsize=8)
def _icosphere_cached(level: int) -> tuple[np.ndarray, np.ndarray]:
    v, f = _icosahedron()
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid], axis=0)
        m = inv.reshape(3, -1).T + base  # midpoints of edges (01, 12, 20) per face
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1),
                            np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    return v, f.astype(np.int32)


def displaced_blob(level: int, seed: int, n_bumps: int = 8, amp: float = 0.3,
                   width: float = 0.15) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    v, f = icosphere(level)
    a = rng.uniform(-1.0, 1.0, size=n_bumps)
    c = rng.normal(size=(n_bumps, 3))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    d2 = ((v[:, None, :] - c[None, :, :]) ** 2).sum(-1)
    radius = 1.0 + amp * (a[None, :] * np.exp(-d2 / (2.0 * width * width))).sum(-1)
    return v * radius[:, None], f


def vertex_normals(verts: np.ndarray, tris: np.ndarray) -> np.ndarray:
    p0, p1, p2 = verts[tris[:, 0]], verts[tris[:, 1]], verts[tris[:, 2]]
    fn = np.cross(p1 - p0, p2 - p0)
    vn = np.zeros_like(verts)
    for k in range(3):
        np.add.at(vn, tris[:, k], fn)
    n = np.linalg.norm(vn, axis=1, keepdims=True)
    return vn / np.where(n > 0, n, 1.0)


def offset_cage(verts: np.ndarray, tris: np.ndarray, dist: float) -> tuple[np.ndarray, np.ndarray]:
    return verts + dist * vertex_normals(verts, tris), tris.copy()


def random_planes(n: int, seed: int, offset_range: float = 0.8) -> np.ndarray:
    """Unit normals uniform on the sphere, offsets U(-offset_range, offset_range)."""
    rng = np.random.default_rng(seed)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = rng.uniform(-offset_range, offset_range, size=n)
    return np.concatenate([nrm, d[:, None]], axis=1).astype(np.float32)


def segment_triangle_cases(n: int, graze_frac: float = 0.05, seed: int = 0):
    """n (segment, triangle) pairs in [-1, 1]^3 (float32): seg n x 6 (p, q),
    tri n x 9. A `graze_frac` share of the segments pass through a point within
    1e-6 of one of their triangle's edges (the FP32 filter cannot decide them
    and the FP64 re-check must); the rest are random."""
    rng = np.random.default_rng(seed)
    tri = rng.uniform(-1, 1, size=(n, 3, 3))
    p = rng.uniform(-1, 1, size=(n, 3))
    q = rng.uniform(-1, 1, size=(n, 3))
    g = rng.random(n) < graze_frac
    k = int(g.sum())
    e = rng.integers(0, 3, size=k)
    a = tri[g, e]
    b = tri[g, (e + 1) % 3]
    x = a + rng.uniform(0, 1, size=(k, 1)) * (b - a)
    x += 1e-6 * rng.uniform(-1, 1, size=(k, 3))
    d = rng.normal(size=(k, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p[g] = x + d * rng.uniform(0.2, 1.0, size=(k, 1))
    q[g] = x - d * rng.uniform(0.2, 1.0, size=(k, 1))
    seg = np.concatenate([p, q], axis=1).astype(np.float32)
    return seg, tri.reshape(n, 9).astype(np.float32), g
