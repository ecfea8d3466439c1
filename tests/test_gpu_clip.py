"""Per-part clipping on the GPU (visacd_clip through the C ABI and the host
assembly) against the host clip, which is itself pinned bit-exact to the
reference's clip.cpp: identical parts, maps, border points and edges."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V():
    from visacd_gb300 import build
    build.build_host()
    from visacd_gb300 import visacd
    return visacd


def _planes(rng, n):
    out = []
    for _ in range(n):
        nrm = rng.normal(size=3)
        nrm /= np.linalg.norm(nrm)
        out.append([*nrm, rng.uniform(-0.5, 0.5)])
    return out


def _same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x["vertices"], y["vertices"])
        np.testing.assert_array_equal(x["triangles"], y["triangles"])
        np.testing.assert_array_equal(x["is_new"], y["is_new"])


def test_gpu_clip_equals_host_clip(V):
    rng = np.random.default_rng(7)
    for level, seed in [(2, 1), (3, 2), (4, 3), (5, 4)]:
        v, t = mg.displaced_blob(level, seed=seed)
        for pl in _planes(rng, 4):
            a, am1, am2 = V._clip(v, t, pl)
            b, bm1, bm2 = V._clip_gpu(v, t, pl)
            np.testing.assert_array_equal(am1, bm1)
            np.testing.assert_array_equal(am2, bm2)
            _same(a, b)


def test_gpu_clip_on_plane_vertices(V):
    # planes through vertices: on-plane cases, coplanar faces, border dedup
    v, t = mg.icosphere(3)
    for pl in ([0, 0, 1, 0.0], [1, 0, 0, 0.0], [0, 1, 0, 0.5], [0.0, 0.5257311121191336, 0.85065080835204, 0.0]):
        a, am1, am2 = V._clip(v, t, pl)
        b, bm1, bm2 = V._clip_gpu(v, t, pl)
        np.testing.assert_array_equal(am1, bm1)
        _same(a, b)
    g = np.linspace(-1, 1, 9)
    xx, yy = np.meshgrid(g, g)
    grid = np.stack([xx.ravel(), yy.ravel(), np.zeros(81)], 1)
    tris = []
    for i in range(8):
        for j in range(8):
            q = i * 9 + j
            tris += [[q, q + 9, q + 10], [q, q + 10, q + 1]]
    tris = np.array(tris)
    box_v = np.concatenate([grid, grid + [0, 0, 1.0]])
    box_t = np.concatenate([tris[:, ::-1], tris + 81])
    for pl in ([0, 0, 1, 0.0], [1, 0, 0, 0.25], [0, 1, 0, 0.0]):
        a, am1, _ = V._clip(box_v, box_t, pl)
        b, bm1, _ = V._clip_gpu(box_v, box_t, pl)
        np.testing.assert_array_equal(am1, bm1)
        _same(a, b)


def test_gpu_clip_raw_outputs(ctx, V):
    v, t = mg.displaced_blob(3, seed=9)
    pl = [0.3, -0.2, 0.93, 0.05]
    r = ctx.clip(v, t, pl)
    a, m1, m2 = V._clip(v, t, pl)
    assert r["nv_pos"] == int(np.count_nonzero(m1)) and r["nv_neg"] == int(np.count_nonzero(m2))
    np.testing.assert_array_equal(r["pos_tris"], a[0]["triangles"][: r["n_pos"]])
    np.testing.assert_array_equal(r["neg_tris"], a[1]["triangles"][: r["n_neg"]])
    np.testing.assert_array_equal(r["border"], a[0]["vertices"][r["nv_pos"]:])
    assert r["n_touching"] > 0 and r["n_border_edges"] >= r["n_border"] - 2


def test_gpu_clip_both_resolver_modes(ctx, V):
    """The ordered resolver keeps its tables in shared memory up to 1024
    touching triangles and in global memory beyond: both equal the host."""
    pl = np.array([0.3, 0.5, 0.81])
    pl = list(pl / np.linalg.norm(pl)) + [0.01]
    seen = []
    for level in (5, 7):
        v, t = mg.icosphere(level)
        seen.append(ctx.clip(v, t, pl)["n_touching"])
        a, am1, am2 = V._clip(v, t, pl)
        b, bm1, bm2 = V._clip_gpu(v, t, pl)
        np.testing.assert_array_equal(am1, bm1)
        np.testing.assert_array_equal(am2, bm2)
        _same(a, b)
    assert seen[0] <= 1024 < seen[1]
