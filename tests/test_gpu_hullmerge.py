"""Hull merging on the GPU: the hull-pair distance kernel equals the host's
exact nearest-neighbour mesh_dist bit for bit, its bounding-box cutoff only
drops pairs that are farther apart than the cutoff, and decompositions with
hull merging on take the same merges with the GPU distances as with the host
ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V(native):
    from visacd_gb300 import build
    build.build_host()
    import visacd_gb300.visacd as V
    V.config.verbose = False
    return V


def _hulls(rng, n):
    out = []
    for h in range(n):
        c = rng.uniform(-1, 1, 3)
        m = int(rng.integers(1, 700))
        out.append(c + rng.normal(scale=rng.uniform(0.01, 0.3), size=(m, 3)))
    return out


def test_hull_distances_equal_host(V, ctx):
    rng = np.random.default_rng(5)
    hulls = _hulls(rng, 24)
    hulls.append(np.zeros((0, 3)))  # an empty hull
    pairs = np.array([(a, b) for a in range(len(hulls)) for b in range(a)], np.int32)
    got = ctx.hull_distances(hulls, pairs)
    for (a, b), d in zip(pairs, got):
        ref = V._mesh_dist(hulls[a], hulls[b])
        assert d == ref, (a, b, d, ref)
    # with a cutoff: pairs closer than it keep their exact value, others get DBL_MAX
    cut = float(np.median(got[np.isfinite(got) & (got < 1e300)]))
    gc = ctx.hull_distances(hulls, pairs, cut)
    for d, dc in zip(got, gc):
        if d < cut:
            assert dc == d
        else:
            assert dc == d or dc == np.finfo(np.float64).max


@pytest.mark.parametrize("hooks", [{"host_merge": True, "host_hull": True},  # merge distances and union hulls on host
                                   {"host_merge": True, "host_hull": False},  # union hulls on the GPU
                                   {"host_merge": False, "host_hull": True}])  # distances on the GPU
def test_merging_same_with_gpu_distances_and_hulls(V, hooks):
    """process() with hull merging: the GPU hull-pair distances and the GPU
    union hulls (visacd_convex_hulls, batched per cost pass) give the same
    merges, parts and concavity as the host ones."""
    from visacd_gb300 import meshgen as mg
    v, t = mg.torus(nu=48, nv=24, seed=3)
    m = V.Mesh()
    m.vertices = V.VecArray3d([list(map(float, p)) for p in v])
    m.triangles = V.make_vecarray3i(t.astype(np.int32))
    V.config.use_merging = True
    out = []
    try:
        for h in (hooks, {"host_merge": False, "host_hull": False}):
            V._checker_hooks(**h)
            V.set_seed(11)
            out.append(V.process(m, 0.05, 12))
    finally:
        V.config.use_merging = False
        V._checker_hooks(host_merge=False, host_hull=False)
    a, b = out
    assert a.num_parts == b.num_parts and a.concavity == b.concavity
    for pa, pb in zip(a.parts, b.parts):
        np.testing.assert_array_equal(np.array(pa.vertices), np.array(pb.vertices))
        np.testing.assert_array_equal(np.array(pa.triangles), np.array(pb.triangles))
