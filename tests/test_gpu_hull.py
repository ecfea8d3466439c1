"""Convex hulls on the GPU (visacd_convex_hulls, one warp per part) against
the host QuickHull (hull.cpp), which the reference's btConvexHullComputer pins
(tests/test_hull_fixture.py): the same triangles in the same order, with and
without the orientation fix, on random, spherical, lattice, duplicate,
coplanar, collinear and tiny point sets, on mesh vertices and on clipped parts
(planar caps), one part at a time and many in one launch; and against the
btConvexHull fixture directly (hull vertex set, volume to 1e-12)."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg
from test_hull_fixture import check_against_bt, hull_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V(native):
    from visacd_gb300 import build
    build.build_host()
    import visacd_gb300.visacd as V
    return V


def _host(V, p, fix=True):
    return np.asarray(V._convex_hull(np.asarray(p, np.float64), fix)["triangles"], np.int32).reshape(-1, 3)


def _clouds():
    rng = np.random.default_rng(17)
    out = {}
    for n in (4, 5, 9, 50, 500, 5000):
        out[f"normal_{n}"] = rng.normal(size=(n, 3))
    out["cube_3000"] = rng.uniform(-1, 1, (3000, 3))
    s = rng.normal(size=(4000, 3))
    out["sphere_4000"] = s / np.linalg.norm(s, axis=1, keepdims=True)
    for lvl, seed in ((3, 1), (4, 2), (5, 3)):
        out[f"blob_s{lvl}"] = mg.displaced_blob(lvl, seed=seed)[0]
    out["torus"] = mg.torus(nu=64, nv=32, seed=1)[0]
    g = np.linspace(-1, 1, 9)
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    out["lattice_9"] = lat
    out["lattice_duplicates"] = np.concatenate([lat, lat[::7], lat[:5]])
    out["flat_xy"] = np.c_[rng.uniform(-1, 1, (400, 2)), np.zeros(400)]
    a, b = rng.normal(size=3), rng.normal(size=3)
    uv = rng.uniform(-1, 1, (300, 2))
    out["flat_tilted"] = uv[:, :1] * a + uv[:, 1:] * b + 0.25
    out["near_flat"] = np.c_[rng.uniform(-1, 1, (300, 2)), rng.normal(scale=1e-13, size=300)]
    out["collinear"] = np.outer(np.linspace(-1, 1, 40), [0.3, -0.2, 0.9])
    out["same_point"] = np.ones((20, 3))
    out["three_points"] = rng.normal(size=(3, 3))
    out["two_points"] = rng.normal(size=(2, 3))
    out["one_point"] = rng.normal(size=(1, 3))
    out["empty"] = np.zeros((0, 3))
    out["big_offset"] = rng.normal(size=(800, 3)) * 1e-3 + 1e6
    return out


def _clipped_parts(V, n_meshes=4):
    """Parts of displaced blobs cut by random planes with the host clip: planar
    caps of coplanar vertices, as the decomposition's parts have."""
    rng = np.random.default_rng(23)
    parts = []
    for s in range(n_meshes):
        v, t = mg.displaced_blob(3 + (s % 2), seed=40 + s)
        nrm = rng.normal(size=3)
        nrm /= np.linalg.norm(nrm)
        halves, _, _ = V._clip(v, t, [*nrm, rng.uniform(-0.3, 0.3)])
        for h in halves:
            hv, ht = np.asarray(h["vertices"]), np.asarray(h["triangles"])
            nrm2 = rng.normal(size=3)
            nrm2 /= np.linalg.norm(nrm2)
            quarters, _, _ = V._clip(hv, ht, [*nrm2, rng.uniform(-0.2, 0.2)])
            parts += [np.asarray(q["vertices"]) for q in quarters]
    return parts


@pytest.mark.parametrize("fix", [True, False])
def test_gpu_hull_equals_host_one_by_one(V, ctx, fix):
    for name, p in _clouds().items():
        got = ctx.convex_hulls([p], fix_normals=fix)[0]
        want = _host(V, p, fix)
        assert got.shape == want.shape and np.array_equal(got, want), (name, got.shape, want.shape)


def test_gpu_hull_equals_host_batched(V, ctx):
    clouds = list(_clouds().values()) + _clipped_parts(V)
    got = ctx.convex_hulls(clouds)
    assert len(got) == len(clouds)
    for k, (p, g) in enumerate(zip(clouds, got)):
        assert np.array_equal(g, _host(V, p)), k


def test_gpu_hull_clipped_parts(V, ctx):
    parts = _clipped_parts(V, 8)
    assert len(parts) >= 16
    for p, g in zip(parts, ctx.convex_hulls(parts)):
        assert np.array_equal(g, _host(V, p))


@pytest.mark.parametrize("case", hull_cases(), ids=lambda c: c["name"])
def test_gpu_hull_matches_btconvexhull_fixture(V, ctx, case):
    p = np.asarray(case["points"], dtype=np.float64)
    got = ctx.convex_hulls([p])[0]
    assert np.array_equal(got, _host(V, p))
    check_against_bt(V, case, got)


def test_gpu_hull_rejects_bad_arguments(native, ctx):
    p = np.random.default_rng(1).normal(size=(10, 3))
    bad = p.copy()
    bad[3, 1] = np.nan
    with pytest.raises(native.VisacdError):
        ctx.convex_hulls([p, bad])
    bad[3, 1] = np.inf
    with pytest.raises(native.VisacdError):
        ctx.convex_hulls([bad])
    assert [len(t) for t in ctx.convex_hulls([])] == []


def test_gpu_hull_batch_over_several_launches(V, ctx):
    """A batch whose work regions pass 1 GiB runs as several launches (each
    part's result lands at its own offset): 132 s5-blob point sets of 10,242
    points, four distinct orders of the same points cycled."""
    v = mg.displaced_blob(5, seed=8)[0]
    rng = np.random.default_rng(5)
    sets = [v] + [v[rng.permutation(len(v))] for _ in range(3)]
    want = [_host(V, p) for p in sets]
    got = ctx.convex_hulls([sets[k % 4] for k in range(132)])
    for k, g in enumerate(got):
        assert np.array_equal(g, want[k % 4]), k
