"""Plane scoring on the GPU (through the C ABI) against the FP64 oracle.

Bar: quantized integer scores bit-exact with the oracle (exact FP64 side
classification + identical FP32 length quantization), FP64 scores within 1e-5
relative of the oracle's FP64 sums, identical first-max argmax."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


def _edges_uniform(rng, n_pts, E):
    pts = rng.uniform(-1, 1, size=(n_pts, 3)).astype(np.float32)
    e = rng.integers(0, n_pts, size=(E, 2)).astype(np.uint32)
    return pts, e


def _check(ctx, orc, planes, pts, edges):
    s_gpu, st = ctx.score_planes(planes, pts, edges)
    s64, q, qexp, skipped = orc.score_planes(planes, pts, edges)
    assert st["quantum_exp"] == qexp
    assert st["skipped_edges"] == skipped
    q_gpu = np.round(np.ldexp(s_gpu, -qexp)).astype(np.uint64)
    np.testing.assert_array_equal(q_gpu, q)
    np.testing.assert_array_equal(np.ldexp(q.astype(np.float64), qexp), s_gpu)
    denom = np.maximum(np.abs(s64), 1e-30)
    nz = s64 > 0
    assert np.all(np.abs(s_gpu - s64)[nz] / denom[nz] <= REL_TOL)
    assert np.all(s_gpu[~nz] == 0)
    if len(planes):
        assert st["argmax"] == int(np.argmax(q))
    return s_gpu, st


@pytest.mark.parametrize("P,E", [(1, 1), (7, 1000), (300, 5000), (513, 20000), (2540, 70000), (5000, 3000)])
def test_random_planes_random_edges(ctx, orc, P, E):
    rng = np.random.default_rng(P * 7 + E)
    pts, edges = _edges_uniform(rng, 4096, E)
    planes = mg.random_planes(P, seed=P)
    _check(ctx, orc, planes, pts, edges)


def test_blob_edges_with_candidate_planes(ctx, orc):
    v, t = mg.displaced_blob(3, seed=11)
    cv, ct = mg.offset_cage(v, t, 0.03)
    _, edges, _ = orc.visibility(v, t, cv, ct, use_bvh=True)
    assert len(edges) > 100
    planes = orc.candidate_planes(v, edges, 2500, seed=42).astype(np.float32)
    _check(ctx, orc, planes, v.astype(np.float32), edges)


def test_band_pairs_are_decided_exactly(ctx, orc):
    """Endpoints placed within float rounding of +-1e-6 from the planes, so most
    (plane, block) pairs need the FP64 re-decision."""
    rng = np.random.default_rng(5)
    P, E = 64, 4096
    planes = mg.random_planes(P, seed=9)
    planes[:, 3] = 0.0
    pts = rng.uniform(-1, 1, size=(2 * E, 3)).astype(np.float32)
    # Project points onto plane 0 then push them +-1e-6 (+- a few ulps).
    n0 = planes[0, :3].astype(np.float64)
    d = pts.astype(np.float64) @ n0
    off = np.where(np.arange(2 * E) % 2 == 0, 1.0, -1.0) * (1e-6 + rng.integers(-3, 4, 2 * E) * 6e-8)
    pts = (pts - (d - off)[:, None] * n0[None, :]).astype(np.float32)
    edges = np.stack([np.arange(0, 2 * E, 2), np.arange(1, 2 * E, 2)], 1).astype(np.uint32)
    _, st = _check(ctx, orc, planes, pts, edges)
    assert st["band_blocks"] > 0


def test_edge_cases(ctx, orc):
    rng = np.random.default_rng(1)
    pts, edges = _edges_uniform(rng, 100, 2000)
    planes = mg.random_planes(50, seed=3)
    # empty edge list
    s, st = ctx.score_planes(planes, pts, edges[:0])
    assert np.all(s == 0) and st["argmax"] == 0
    # no planes
    s, st = ctx.score_planes(planes[:0], pts, edges)
    assert len(s) == 0 and st["argmax"] == -1
    # out-of-range indices are skipped like the reference (plane_intersections.cu:34-36)
    bad = edges.copy()
    bad[::7, 1] = 1000
    _check(ctx, orc, planes, pts, bad)
    # non-finite endpoints contribute nothing
    p2 = pts.copy()
    p2[3] = np.nan
    p2[4, 1] = np.inf
    _check(ctx, orc, planes, p2, edges)
    # degenerate (zero-length) edges and duplicated edges
    dup = np.concatenate([edges, edges[:100], np.stack([np.arange(50), np.arange(50)], 1).astype(np.uint32)])
    _check(ctx, orc, planes, pts, dup)
    # NaN plane scores zero
    pl = planes.copy()
    pl[5] = np.nan
    s, _ = _check(ctx, orc, pl, pts, edges)
    assert s[5] == 0


def test_scores_independent_of_repeat(ctx, orc):
    rng = np.random.default_rng(2)
    pts, edges = _edges_uniform(rng, 2000, 50000)
    planes = mg.random_planes(1000, seed=4)
    a, _ = ctx.score_planes(planes, pts, edges)
    b, _ = ctx.score_planes(planes, pts, edges)
    np.testing.assert_array_equal(a, b)


def test_reference_signature_entry_point(native, orc):
    rng = np.random.default_rng(8)
    pts, edges = _edges_uniform(rng, 500, 10000)
    planes = mg.random_planes(200, seed=8)
    out = native.classify_and_rate_planes(planes, pts, edges)
    s64, _, _, _ = orc.score_planes(planes, pts, edges)
    np.testing.assert_allclose(out, s64.astype(np.float32), rtol=2e-6, atol=0)


@pytest.mark.parametrize("E", [1 << 20, 1 << 22])
def test_precision_sweep_sizes(ctx, orc, E):
    """Precision-sweep shapes: endpoints U[-1,1]^3, P = 4096 planes with offsets
    U(-0.8, 0.8). The oracle runs on a 64-plane slice (the GPU runs all 4096)."""
    rng = np.random.default_rng(E)
    pts = rng.uniform(-1, 1, size=(2 * E, 3)).astype(np.float32)
    edges = np.arange(2 * E, dtype=np.uint32).reshape(E, 2)
    planes = mg.random_planes(4096, seed=E)
    s_gpu, st = ctx.score_planes(planes, pts, edges)
    sub = np.arange(0, 4096, 64)
    s64, q, qexp, _ = orc.score_planes(planes[sub], pts, edges)
    q_gpu = np.round(np.ldexp(s_gpu[sub], -qexp)).astype(np.uint64)
    np.testing.assert_array_equal(q_gpu, q)
    assert np.max(np.abs(s_gpu[sub] - s64) / s64) <= REL_TOL


def test_planes_per_thread_change_no_score(ctx):
    """Scores and the argmax are the same whatever planes each thread takes
    (forced 1, 2, 4, 8), and the autotuner picks one of them."""
    rng = np.random.default_rng(21)
    pts = rng.normal(size=(3000, 3)).astype(np.float32)
    e = rng.integers(0, 3000, size=(20000, 2)).astype(np.uint32)
    nrm = rng.normal(size=(1500, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    planes = np.concatenate([nrm, rng.uniform(-0.5, 0.5, (1500, 1))], 1).astype(np.float32)
    planes[:20, 3] = -(planes[:20, :3] @ pts[e[:20, 0]].T).diagonal()  # planes through edge endpoints
    ref = None
    try:
        for k in (1, 2, 4, 8):
            ctx.set_score_k(k)
            s, st = ctx.score_planes(planes, pts, e)
            if ref is None:
                ref = (s, st["argmax"])
            np.testing.assert_array_equal(s, ref[0])
            assert st["argmax"] == ref[1]
    finally:
        ctx.set_score_k(0)
    best, ms = ctx.autotune_scoring(planes, pts, e)
    assert best in (1, 2, 4, 8) and len(ms) == 4 and all(m > 0 for m in ms)
    s, _ = ctx.score_planes(planes, pts, e)
    np.testing.assert_array_equal(s, ref[0])
