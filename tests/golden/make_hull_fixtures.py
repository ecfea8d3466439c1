"""Generate hull fixtures from the reference's own btConvexHullComputer.

Runs the reference's Bullet hull (lib/3rd/btConvexHull, through
Mesh::compute_vch, lib/src/core.cpp:113-142, compiled in place by
oracle/build_ref.py) on point clouds on the integer grid 0..10216 with every
axis spanning the whole range: that hull maps the input box onto exactly that
grid before its integer arithmetic, so on these inputs it is exact and its
output coordinates are the input coordinates. Records each cloud, its hull
volume and its hull vertex set. The tests compare the host QuickHull (CPU) and
visacd_convex_hulls (GPU) against this file. Needs the reference tree
(development container); the fixture is committed so the GPU machine does not.

    python tests/golden/make_hull_fixtures.py
"""
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle.ref as R  # noqa: E402
from visacd_gb300 import meshgen as mg  # noqa: E402

L = 10216


def _span(p):
    """Points mapped onto the grid with every axis covering 0..L."""
    p = np.asarray(p, float)
    lo, hi = p.min(0), p.max(0)
    return np.round((p - lo) / np.where(hi > lo, hi - lo, 1.0) * L)


def clouds():
    rng = np.random.default_rng(2027)
    corners = np.array([[0, 0, 0], [L, L, L]], float)
    out = {}
    out["random_300"] = np.concatenate([corners, rng.integers(0, L + 1, (300, 3))]).astype(float)
    out["random_3000"] = np.concatenate([corners, rng.integers(0, L + 1, (3000, 3))]).astype(float)
    g = np.linspace(0, L, 7)
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    out["lattice_7"] = lat
    out["lattice_7_duplicates"] = np.concatenate([lat, lat[::5], lat[:11]])
    s = rng.normal(size=(3000, 3))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    out["sphere_3000"] = np.round((np.concatenate([s, np.eye(3), -np.eye(3)]) + 1) * (L / 2))
    v, _ = mg.displaced_blob(3, seed=4)
    out["blob_s3"] = _span(v)
    v, _ = mg.displaced_blob(4, seed=9)
    out["blob_s4"] = _span(v)
    v, _ = mg.torus(nu=48, nv=24, seed=3)
    out["torus_48x24"] = _span(v)
    # a box with many points on its faces: large coplanar facets
    f = rng.integers(0, L + 1, (600, 3)).astype(float)
    f[np.arange(600), rng.integers(0, 3, 600)] = rng.choice([0.0, L], 600)
    out["box_faces"] = np.concatenate([corners, [[0, 0, L], [0, L, 0], [L, 0, 0], [L, L, 0], [L, 0, L], [0, L, L]], f])
    out["tetrahedron"] = np.array([[0, 0, 0], [L, 0, 0], [0, L, 0], [0, 0, L]], float)
    flat = rng.integers(0, L + 1, (200, 2)).astype(float)
    flat[:2] = [[0, 0], [L, L]]
    out["flat"] = np.c_[flat, np.full(200, L / 2)]
    return out


def main():
    cases = []
    for name, p in clouds().items():
        bv, bt = R.hull_bt(p)
        vol = 0.0
        if len(bt):
            a, b, c = bv[bt[:, 0]], bv[bt[:, 1]], bv[bt[:, 2]]
            vol = float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)
        cases.append({"name": name, "points": p.astype(np.int64).tolist(), "bt_volume": vol,
                      "bt_hull_vertices": sorted(map(list, {tuple(map(int, x)) for x in bv})) if len(bt) else [],
                      "bt_triangles": int(len(bt))})
        print(f"{name}: {len(p)} points, {len(bt)} bt triangles, volume {vol:.6e}")
    out = Path(__file__).with_name("hull_bt.json")
    out.write_text(json.dumps({"grid": L, "cases": cases}, separators=(",", ":")))
    print("wrote", out, out.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
