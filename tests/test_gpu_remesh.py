"""GPU SDF remesh (visacd_sdf_remesh) against the host restatement: the same
mesh bit for bit — vertices, triangles and their order — for the scales and
levels process() uses (remesh 30 / 0.55/30, cages 40 / 0.03 and 40 / 0.02),
on closed meshes and on clipped parts."""
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


def _meshes():
    from visacd_gb300 import meshgen as mg, proposer as pp
    v, t = mg.torus(seed=2)
    yield "torus", v / np.abs(v).max(), t
    for s in (3, 11):
        yield f"blob{s}", *pp.make_blob(1_000_000 + s)[1:3]
    v, t = mg.displaced_blob(5, seed=1)
    yield "blob_s5", v / np.abs(v).max(), t


@pytest.mark.parametrize("scale,level", [(30.0, 0.55 / 30), (40.0, 0.03), (40.0, 0.02), (20.0, 0.55 / 20)])
def test_gpu_remesh_equals_host(V, scale, level):
    for name, v, t in _meshes():
        h = V._manifold_preprocess(v, t, scale, level)
        g = V._manifold_preprocess_gpu(v, t, scale, level)
        assert len(h["vertices"]) > 0, name
        np.testing.assert_array_equal(g["triangles"], h["triangles"], err_msg=name)
        np.testing.assert_array_equal(g["vertices"], h["vertices"], err_msg=name)


def test_gpu_remesh_clipped_parts(V):
    from visacd_gb300 import meshgen as mg
    v, t = mg.displaced_blob(4, seed=9)
    v = v / np.abs(v).max()
    parts, _, _ = V._clip(v, t, [0.6, 0.8, 0.0, 0.05])
    assert len(parts) == 2
    for p in parts:
        h = V._manifold_preprocess(p["vertices"], p["triangles"], 40.0, 0.02)
        g = V._manifold_preprocess_gpu(p["vertices"], p["triangles"], 40.0, 0.02)
        np.testing.assert_array_equal(g["triangles"], h["triangles"])
        np.testing.assert_array_equal(g["vertices"], h["vertices"])


def test_gpu_remesh_edge_cases(native, ctx):
    v, t = ctx.sdf_remesh(np.zeros((0, 3)), np.zeros((0, 3), np.int32), 40.0, 0.02)
    assert v.shape == (0, 3) and t.shape == (0, 3)
    with pytest.raises(native.VisacdError):
        ctx.sdf_remesh(np.zeros((3, 3)), np.array([[0, 1, 3]], np.int32), 40.0, 0.02)
    # a single triangle: a closed thin shell around it
    v, t = ctx.sdf_remesh(np.array([[0, 0, 0], [0.5, 0, 0], [0, 0.5, 0]], float), np.array([[0, 1, 2]], np.int32),
                          40.0, 0.03)
    assert len(v) > 0 and len(t) > 0
    e = np.sort(np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]), 1)
    _, cnt = np.unique(e, axis=0, return_counts=True)
    assert (cnt == 2).all()


def test_gpu_remesh_degenerate_triangles(V):
    """Zero-area and sliver triangles (no plane, near-parallel edges) in a
    closed mesh: the GPU bounds must stay conservative; same mesh as the host."""
    from visacd_gb300 import meshgen as mg
    v, t = mg.displaced_blob(3, seed=4)
    v = v / np.abs(v).max()
    n = len(v)
    # a duplicated vertex (zero-area triangles) and a sliver fan on one face
    extra_v = np.array([v[t[0, 0]], 0.5 * (v[t[1, 0]] + v[t[1, 1]]) + 1e-9], float)
    v2 = np.concatenate([v, extra_v])
    t2 = np.concatenate([t, [[t[0, 0], t[0, 1], n], [t[1, 0], t[1, 1], n + 1], [n, n + 1, t[2, 2]]]]).astype(np.int32)
    for scale, level in [(40.0, 0.02), (30.0, 0.55 / 30)]:
        h = V._manifold_preprocess(v2, t2, scale, level)
        g = V._manifold_preprocess_gpu(v2, t2, scale, level)
        np.testing.assert_array_equal(g["triangles"], h["triangles"])
        np.testing.assert_array_equal(g["vertices"], h["vertices"])
