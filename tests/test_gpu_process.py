"""The drop-in `visacd` module end to end on the GPU: the reference's Python
surface (lib/bindings.cpp) and process() on seeded synthetic meshes."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def visacd():
    from visacd_gb300 import build
    build.build_host()
    import visacd as m
    m.config.verbose = False
    return m


def _mesh(visacd, v, t):
    m = visacd.Mesh()
    m.vertices = visacd.VecArray3d(v.tolist())
    m.triangles = visacd.make_vecarray3i(np.asarray(t, dtype=np.int32))
    return m


def test_surface_and_config(visacd):
    assert visacd.config.score_mode == "concavity"
    assert visacd.config.flat_surface_k == 2.0 and visacd.config.use_merging is False
    c = visacd.Config()
    assert c.return_parts is False and c.use_flat_surfaces is True
    m = visacd.Mesh()
    m.vertices = visacd.VecArray3d([[0, 0, 0], [1, 0, 0]])
    assert len(m.vertices) == 2 and list(m.vertices[1]) == [1.0, 0.0, 0.0]


def test_process_torus(visacd):
    v, t = mg.torus(nu=32, nv=16, seed=42)
    visacd.set_seed(42)
    r = visacd.process(_mesh(visacd, v, t), 0.04, 8)
    assert 1 <= r.num_parts <= 8 and r.num_parts == len(r.parts)
    assert np.isfinite(r.concavity) and r.concavity >= 0
    # hulls are returned in the input frame: inside the input's bounding box (+ remesh offset)
    allv = np.concatenate([np.array(list(p.vertices)) for p in r.parts])
    assert np.all(allv.min(0) > v.min(0) - 0.1) and np.all(allv.max(0) < v.max(0) + 0.1)
    # same seed, same result
    visacd.set_seed(42)
    r2 = visacd.process(_mesh(visacd, v, t), 0.04, 8)
    assert r2.num_parts == r.num_parts and r2.concavity == r.concavity


def test_process_edge_mode_and_parts(visacd):
    v, t = mg.displaced_blob(3, seed=9)
    visacd.set_seed(1)
    visacd.config.score_mode = "edge"
    visacd.config.return_parts = True
    try:
        r = visacd.process(_mesh(visacd, v, t), 0.02, 5)
    finally:
        visacd.config.score_mode = "concavity"
        visacd.config.return_parts = False
    assert 1 <= r.num_parts <= 5
    for p in r.parts:
        assert len(p.triangles) > 0


def test_gpu_concavity_metric_equals_host(visacd):
    from visacd_gb300 import visacd as V
    for seed, level in [(3, 3), (4, 4), (5, 2)]:
        v, t = mg.displaced_blob(level, seed=seed)
        V._checker_hooks(host_concavity=True)
        V.set_seed(11)
        a = V._compute_h(v, t, 0.3, 3000)
        V._checker_hooks(host_concavity=False)
        V.set_seed(11)
        b = V._compute_h(v, t, 0.3, 3000)
        assert a == b
        hv = V._convex_hull(v)
        V._checker_hooks(host_concavity=True)
        V.set_seed(5)
        a = V._compute_hb(v, t, hv["vertices"], hv["triangles"], 10000)
        V._checker_hooks(host_concavity=False)
        V.set_seed(5)
        b = V._compute_hb(v, t, hv["vertices"], hv["triangles"], 10000)
        assert a == b


def test_face_hausdorff_floor(visacd):
    """visacd_face_hausdorff_floor: exact at or above the floor, below it otherwise."""
    from visacd_gb300 import _native as N
    from visacd_gb300 import visacd as V
    ctx = N.Context(0)
    try:
        for seed, level in [(3, 3), (8, 4)]:
            v, t = mg.displaced_blob(level, seed=seed)
            hv = V._convex_hull(v)
            V.set_seed(seed)
            xa, ia = V._sample_points(v, t, 3000)
            xb, ib = V._sample_points(hv["vertices"], hv["triangles"], 3000)
            args = (v, t, xa, ia, hv["vertices"], hv["triangles"], xb, ib)
            exact = ctx.face_hausdorff(*args)
            assert exact > 0
            for f in (0.0, 0.3 * exact, exact * (1 - 1e-12), exact):
                assert ctx.face_hausdorff(*args, floor=f) == exact
            for f in (exact * (1 + 1e-12), 1.5 * exact, 10.0):
                assert ctx.face_hausdorff(*args, floor=f) < f
    finally:
        ctx.close()


def test_process_gpu_metric_equals_host_metric(visacd):
    """process() with the floored GPU metric (values evaluated largest volume
    term first) picks the same parts and returns the same concavity as with
    the exact host metric evaluated in part order."""
    from visacd_gb300 import visacd as V
    v, t = mg.displaced_blob(3, seed=21)
    out = []
    for gpu in (False, True):
        V._checker_hooks(host_concavity=not gpu)
        V.set_seed(3)
        try:
            out.append(V.process(_mesh(V, v, t), 0.02, 10))
        finally:
            V._checker_hooks(host_concavity=False)
    a, b = out
    assert a.num_parts == b.num_parts and a.concavity == b.concavity
    for pa, pb in zip(a.parts, b.parts):
        np.testing.assert_array_equal(np.array(pa.vertices), np.array(pb.vertices))


def test_face_hausdorff_batch(visacd):
    """visacd_face_hausdorff_batch: independent jobs equal single calls; with
    pruning across jobs, the jobs attaining the largest concavity keep their
    exact value, the others stay at or below theirs, and the first maximum of
    max(lower, value) is unchanged."""
    from visacd_gb300 import _native as N
    from visacd_gb300 import visacd as V
    ctx = N.Context(0)
    try:
        jobs, lower = [], []
        for seed, level in [(3, 2), (8, 3), (11, 3), (12, 2), (14, 3)]:
            v, t = mg.displaced_blob(level, seed=seed)
            hv = V._convex_hull(v)
            V.set_seed(seed)
            xa, ia = V._sample_points(v, t, 3000)
            xb, ib = V._sample_points(hv["vertices"], hv["triangles"], 3000)
            jobs.append((v, t, xa, ia, hv["vertices"], hv["triangles"], xb, ib))
            vol = abs(V._mesh_volume(hv["vertices"], hv["triangles"]) - V._mesh_volume(v, t))
            lower.append(0.3 * (3 * vol / (4 * 3.14159265)) ** (1 / 3))
        single = np.array([ctx.face_hausdorff(*j) for j in jobs])
        np.testing.assert_array_equal(ctx.face_hausdorff_batch(jobs), single)
        lower = np.array(lower)
        for low, floor in ((lower, 0.0), (np.zeros(len(jobs)), 0.0), (lower, 0.5 * single.max())):
            got = ctx.face_hausdorff_batch(jobs, lower=low, floor=floor, independent=False)
            M = max(floor, np.maximum(low, single).max())
            assert np.all(got <= single)
            for j in range(len(jobs)):
                if single[j] == M:
                    assert got[j] == single[j]
            c_true, c_got = np.maximum(low, single), np.maximum(low, got)
            if c_true.max() >= floor:
                assert c_got.max() == c_true.max() and np.argmax(c_got) == np.argmax(c_true)
    finally:
        ctx.close()
