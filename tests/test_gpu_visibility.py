"""Visibility on the GPU (LBVH + traversal, through the C ABI) against the FP64
oracle: identical edge sets except for pairs the oracle marks as grazing
(within 1e-6 of a decision boundary); the grazing count is reported."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _compare(ctx, orc, v, t, cv, ct, is_new=None, brute=False):
    sb = ctx.bvh(v, t)
    cb = ctx.bvh(cv, ct)
    e_gpu, st = ctx.visibility(v, sb, cb, is_new=is_new)
    bits, e_orc, ost = orc.visibility(v, t, cv, ct, is_new=is_new, use_bvh=not brute)
    n = len(v)
    assert np.all(e_gpu[:, 0] < e_gpu[:, 1]) if len(e_gpu) else True
    k_gpu = orc.linear_from_pairs(e_gpu, n) if len(e_gpu) else np.zeros(0, np.int64)
    assert np.all(np.diff(k_gpu) > 0), "edges must be in row-major order"
    gpu_bits = np.zeros(n * (n - 1) // 2, dtype=bool)
    gpu_bits[k_gpu] = True
    orc_edge = (bits & 1).astype(bool)
    grazing = (bits & 2).astype(bool)
    diff = gpu_bits != orc_edge
    assert not np.any(diff & ~grazing), f"{int(np.sum(diff & ~grazing))} non-grazing pairs differ"
    assert st["pairs_tested"] == ost["pairs"]
    return e_gpu, st, ost, int(np.sum(diff))


def test_blob_level2_bruteforce(ctx, orc):
    v, t = mg.displaced_blob(2, seed=3)
    cv, ct = mg.offset_cage(v, t, 0.03)
    e, st, ost, nd = _compare(ctx, orc, v, t, cv, ct, brute=True)
    assert len(e) > 10


@pytest.mark.parametrize("seed", [1, 2])
def test_blob_level3(ctx, orc, seed):
    v, t = mg.displaced_blob(3, seed=seed)
    cv, ct = mg.offset_cage(v, t, 0.03)
    _compare(ctx, orc, v, t, cv, ct)


def test_torus_small(ctx, orc):
    v, t = mg.torus(nu=32, nv=16, seed=42)
    cv, ct = mg.offset_cage(v, t, 0.03)
    e, st, ost, nd = _compare(ctx, orc, v, t, cv, ct)
    assert len(e) > 100


def test_masked_pairs(ctx, orc):
    v, t = mg.displaced_blob(3, seed=7)
    cv, ct = mg.offset_cage(v, t, 0.03)
    rng = np.random.default_rng(0)
    m = (rng.random(len(v)) < 0.1).astype(np.uint8)
    e, st, ost, nd = _compare(ctx, orc, v, t, cv, ct, is_new=m)
    assert np.all(m[e[:, 0]] | m[e[:, 1]])


def test_mask_all_and_none(ctx, orc):
    v, t = mg.displaced_blob(2, seed=5)
    cv, ct = mg.offset_cage(v, t, 0.03)
    e_all, _, _, _ = _compare(ctx, orc, v, t, cv, ct, is_new=np.ones(len(v), np.uint8))
    e_ref, _, _, _ = _compare(ctx, orc, v, t, cv, ct)
    np.testing.assert_array_equal(e_all, e_ref)
    e_none, st, _, _ = _compare(ctx, orc, v, t, cv, ct, is_new=np.zeros(len(v), np.uint8))
    assert len(e_none) == 0 and st["pairs_tested"] == 0


def test_tiny_inputs(ctx, orc):
    # two points, one triangle part, tetrahedral cage
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    t = np.array([[0, 1, 2]], np.int32)
    cv = np.array([[-5, -5, -5], [5, -5, -5], [0, 5, -5], [0, 0, 5]], np.float64)
    ct = np.array([[0, 2, 1], [0, 1, 3], [1, 2, 3], [2, 0, 3]], np.int32)
    _compare(ctx, orc, v, t, cv, ct, brute=True)
    # empty cage: nothing can hit it -> no edges
    sb, cb = ctx.bvh(v, t), ctx.bvh(np.zeros((0, 3)), np.zeros((0, 3), np.int32))
    e, st = ctx.visibility(v, sb, cb)
    assert len(e) == 0
    # single point
    sb1 = ctx.bvh(v[:1], np.zeros((0, 3), np.int32))
    e, st = ctx.visibility(v[:1], sb1, cb)
    assert len(e) == 0


def test_duplicate_vertices_are_not_edges(ctx, orc):
    v, t = mg.displaced_blob(2, seed=9)
    v = np.concatenate([v, v[:5]])  # 5 coincident copies (unreferenced)
    cv, ct = mg.offset_cage(*mg.displaced_blob(2, seed=9), 0.03)
    e, st, ost, nd = _compare(ctx, orc, v, t, cv, ct)
    assert st["degenerate"] >= 5


def test_bad_triangle_index_rejected(ctx, native):
    v = np.zeros((3, 3))
    with pytest.raises(native.VisacdError):
        ctx.bvh(v, np.array([[0, 1, 7]], np.int32))


def test_compute_intersection_matrix_one_call(ctx, orc):
    v, t = mg.displaced_blob(2, seed=4)
    cv, ct = mg.offset_cage(v, t, 0.03)
    e1, st1 = ctx.compute_intersection_matrix(v, t, cv, ct)
    e2, st2, _, _ = _compare(ctx, orc, v, t, cv, ct)
    np.testing.assert_array_equal(e1, e2)


def test_every_launch_shape_gives_the_same_edges(ctx, native, orc):
    v, t = mg.displaced_blob(3, seed=21)
    cv, ct = mg.offset_cage(v, t, 0.03)
    sb, cb = ctx.bvh(v, t), ctx.bvh(cv, ct)
    ref, _ = ctx.visibility(v, sb, cb)
    m = (np.arange(len(v)) % 5 == 0).astype(np.uint8)
    ref_m, _ = ctx.visibility(v, sb, cb, is_new=m)
    for var in range(native.lib().visacd_vis_variant_count()):
        ctx.set_vis_variant(var)
        e, _ = ctx.visibility(v, sb, cb)
        np.testing.assert_array_equal(e, ref)
        e, _ = ctx.visibility(v, sb, cb, is_new=m)
        np.testing.assert_array_equal(e, ref_m)
    ctx.set_vis_variant(-1)
    best, ms = ctx.autotune_visibility(v, sb, cb)
    assert 0 <= best < len(ms) and all(x > 0 for x in ms)
    e, _ = ctx.visibility(v, sb, cb)
    np.testing.assert_array_equal(e, ref)


def test_bvh_depth(ctx):
    """The tree depth reported by the build (root height in edges, taken in the
    bottom-up fit): within [ceil(log2 n), n - 1], exact for small trees."""
    import math
    from visacd_gb300 import meshgen as mg
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32)
    b = ctx.bvh(tri, np.array([[0, 1, 2], [1, 3, 2]], np.int32))
    assert b.info() == (2, 1)
    b.close()
    for level in (2, 4):
        v, t = mg.displaced_blob(level, seed=1)
        b = ctx.bvh(v, t)
        nt, depth = b.info()
        assert nt == len(t) and math.ceil(math.log2(nt)) <= depth <= nt - 1
        b.close()


def test_torus_64x32_all_pairs(ctx, orc):
    """The small plain-method workload: seeded torus R = 1, r = 0.35, 64 x 32
    grid with radial perturbation U(-0.02, 0.02) r (2048 vertices, all
    2,096,128 pairs) against its 0.03 offset cage. Every pair outside the
    grazing band matches the FP64 oracle."""
    v, t = mg.torus(nu=64, nv=32, seed=42)
    cv, ct = mg.offset_cage(v, t, 0.03)
    e, st, ost, nd = _compare(ctx, orc, v, t, cv, ct)
    assert ost["pairs"] == 2096128
    assert nd <= ost["n_grazing"]
    cleared, reads = ctx.vis_trace_counts()
    print(f"torus 64x32: {len(e)} edges, {ost['n_grazing']} grazing pairs, {nd} differ (all grazing); "
          f"{cleared} segments cleared by the free-space walk ({reads} grid reads)")


def test_blob_s5_all_pairs(ctx, orc):
    """The large concave blob: icosphere subdivision 5 (10242 vertices, 20480
    triangles) with 8 seeded Gaussian bumps, all 52,444,161 pairs against its
    0.03 offset cage (the benchmark's workload and seed). Every pair outside
    the grazing band matches the FP64 oracle."""
    v, t = mg.displaced_blob(5, seed=2026)
    cv, ct = mg.offset_cage(v, t, 0.03)
    e, st, ost, nd = _compare(ctx, orc, v, t, cv, ct)
    assert ost["pairs"] == 52444161
    assert nd <= ost["n_grazing"]
    cleared, reads = ctx.vis_trace_counts()
    assert cleared > 0
    print(f"blob s5: {len(e)} edges, {ost['n_grazing']} grazing pairs, {nd} differ (all grazing); "
          f"{cleared} segments cleared by the free-space walk ({reads} grid reads)")


@pytest.mark.parametrize("case", ["blob_s5", "torus_64x32", "blob_s4_masked", "tiny_cage_gap"])
def test_free_space_walk_changes_nothing(ctx, case):
    """The cage's free-space walk only skips segments that cannot hit the cage:
    the edges and the pair, hit and degenerate counts are the same with and
    without it; only the BVH work (node visits, triangle tests, FP64
    re-decisions) shrinks."""
    is_new = None
    if case == "blob_s5":
        v, t = mg.displaced_blob(5, seed=2026)
        cv, ct = mg.offset_cage(v, t, 0.03)
    elif case == "torus_64x32":
        v, t = mg.torus(nu=64, nv=32, seed=42)
        cv, ct = mg.offset_cage(v, t, 0.03)
    elif case == "blob_s4_masked":  # 1/3 of the vertices new: about 2.4M pairs
        v, t = mg.displaced_blob(4, seed=7)
        v = np.concatenate([v, v * 0.999])  # two shells: many pairs graze or cross
        t = np.concatenate([t, t[:, ::-1] + len(v) // 2])
        cv, ct = mg.offset_cage(v[: len(v) // 2], t[: len(t) // 2], 0.03)
        is_new = (np.arange(len(v)) % 3 == 0).astype(np.uint8)
    else:  # a cage 1e-4 off the part: few segments are cleared
        v, t = mg.displaced_blob(4, seed=3)
        cv, ct = mg.offset_cage(v, t, 1e-4)
    sb, cb = ctx.bvh(v, t), ctx.bvh(cv, ct)
    try:
        ctx.set_vis_trace(False)
        e0, s0 = ctx.visibility(v, sb, cb, is_new=is_new)
        ctx.set_vis_trace(True)
        e1, s1 = ctx.visibility(v, sb, cb, is_new=is_new)
    finally:
        ctx.set_vis_trace(True)
    cleared, reads = ctx.vis_trace_counts()
    np.testing.assert_array_equal(e0, e1)
    for k in ("pairs_tested", "n_edges", "self_hits", "cage_hits", "degenerate"):
        assert s0[k] == s1[k], k
    # Cleared segments skip their cage triangle tests (and those tests' FP64
    # re-decisions).
    assert s1["fp64_rechecks"] <= s0["fp64_rechecks"] and s1["tri_tests"] <= s0["tri_tests"]
    # The share cleared depends on the shape: most chords of the blob stay far
    # from its cage; the torus's run close to its tube.
    # Calls below 2^22 pairs (the torus) do not walk.
    least = {"blob_s5": 0.9, "torus_64x32": 0.0, "blob_s4_masked": 0.3, "tiny_cage_gap": 0.0}[case]
    if least > 0:
        assert cleared > least * s1["pairs_tested"]
        assert s1["node_visits"] < s0["node_visits"]
    print(f"{case}: {s1['pairs_tested']} pairs, {cleared} cleared, {reads} grid reads, "
          f"node visits {s0['node_visits']} -> {s1['node_visits']}")


def test_bvh_depth_on_clustered_and_degenerate_meshes(ctx, orc):
    """Meshes that stress the Morton hierarchy stay within the 64-entry
    traversal stack and give the oracle's edges: a cluster of tiny triangles
    next to a far one (Morton codes crowd into few cells), many coincident
    triangles (equal codes), and a long thin strip."""
    rng = np.random.default_rng(5)
    # 1) 4000 tiny triangles packed within 1e-4 of the origin plus one far one.
    c = rng.normal(size=(4000, 1, 3)) * 1e-4
    tri = c + rng.normal(size=(4000, 3, 3)) * 1e-6
    far = np.array([[[50, 50, 50], [51, 50, 50], [50, 51, 50]]], np.float64)
    v1 = np.concatenate([tri, far]).reshape(-1, 3)
    t1 = np.arange(len(v1), dtype=np.int32).reshape(-1, 3)
    # 2) 3000 copies of one triangle (all Morton codes equal).
    v2 = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64), (3000, 1))
    t2 = np.arange(len(v2), dtype=np.int32).reshape(-1, 3)
    # 3) a 1 x 1e-5 strip of 4096 triangles.
    xs = np.linspace(0, 1, 2049)
    v3 = np.concatenate([np.stack([xs, np.zeros_like(xs), np.zeros_like(xs)], 1),
                         np.stack([xs, np.full_like(xs, 1e-5), np.zeros_like(xs)], 1)])
    i = np.arange(2048)
    t3 = np.concatenate([np.stack([i, i + 1, 2049 + i], 1),
                         np.stack([i + 1, 2050 + i, 2049 + i], 1)]).astype(np.int32)
    for v, t in [(v1, t1), (v2, t2), (v3, t3)]:
        b = ctx.bvh(v, t)
        nt, depth = b.info()
        assert nt == len(t) and depth <= 64, f"depth {depth} for {nt} triangles"
        b.close()
    # The strip as a part inside a box cage: visibility runs and matches.
    cv = np.array([[-1, -1, -1], [2, -1, -1], [2, 2, -1], [-1, 2, -1],
                   [-1, -1, 1], [2, -1, 1], [2, 2, 1], [-1, 2, 1]], np.float64)
    ct = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                   [1, 2, 6], [1, 6, 5], [2, 3, 7], [2, 7, 6], [3, 0, 4], [3, 4, 7]], np.int32)
    _compare(ctx, orc, v3[::8], np.zeros((0, 3), np.int32), cv, ct)


def test_visibility_batch_equals_per_part_calls(ctx, orc):
    """Several parts of uneven size in one call (one persistent launch over
    all parts' work items): unmasked, masked and tiny parts give the edges of
    one call per part, in part order."""
    rng = np.random.default_rng(3)
    parts = []
    for level, seed, masked in [(3, 1, False), (2, 2, True), (3, 3, True), (2, 4, False)]:
        v, t = mg.displaced_blob(level, seed=seed)
        cv, ct = mg.offset_cage(v, t, 0.03)
        m = (rng.random(len(v)) < 0.15).astype(np.uint8) if masked else None
        parts.append((v, ctx.bvh(v, t), ctx.bvh(cv, ct), m))
    tiny = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    parts.append((tiny[:1], ctx.bvh(tiny[:1], np.zeros((0, 3), np.int32)), parts[0][2], None))
    got, st = ctx.visibility_batch(parts)
    assert len(got) == len(parts)
    pairs = 0
    for (v, sb, cb, m), e in zip(parts, got):
        want, s1 = ctx.visibility(v, sb, cb, is_new=m)
        np.testing.assert_array_equal(e, want)
        pairs += s1["pairs_tested"]
    assert st["pairs_tested"] == pairs
    # the batch is what the oracle gives for a masked part too
    v, sb, cb, m = parts[1]
    t = mg.displaced_blob(2, seed=2)[1]
    bits, _, _ = orc.visibility(v, t, *mg.offset_cage(v, t, 0.03), is_new=m)
    k = orc.linear_from_pairs(got[1], len(v)) if len(got[1]) else np.zeros(0, np.int64)
    gb = np.zeros(len(bits), bool)
    gb[k] = True
    assert not np.any((gb != (bits & 1).astype(bool)) & ~(bits & 2).astype(bool))


@pytest.mark.parametrize("case", ["far_translated", "cage_inside_part", "degenerate_cage", "single_far_triangle"])
def test_free_space_walk_edge_cases(ctx, case):
    """Cages the free-space grid cannot serve, or serves oddly, still give the
    same edges as the traversal alone: coordinates far from the origin (the
    grid is refused: its margin would not cover the rounding), a cage smaller
    than the part (walks start outside the grid), degenerate cage triangles
    (their distance bound falls back to the triangle's box), and a cage of one
    far triangle (a tiny grid the segments never enter)."""
    v, t = mg.displaced_blob(4, seed=9)
    v = np.concatenate([v, v * 0.98])  # 5124 vertices: 13.1M pairs, above the walk's 2^22
    t = np.concatenate([t, t[:, ::-1] + len(v) // 2])
    cv, ct = mg.offset_cage(v[: len(v) // 2], t[: len(t) // 2], 0.03)
    if case == "far_translated":
        v = v + 1.0e5
        cv = cv + 1.0e5
    elif case == "cage_inside_part":
        cv = cv * 0.5
    elif case == "degenerate_cage":
        ct = ct.copy()
        ct[::3, 1] = ct[::3, 0]  # every third triangle collapsed to an edge
    else:
        cv = np.array([[10.0, 10.0, 10.0], [10.1, 10.0, 10.0], [10.0, 10.1, 10.0]])
        ct = np.array([[0, 1, 2]])
    sb, cb = ctx.bvh(v, t), ctx.bvh(cv, ct)
    try:
        ctx.set_vis_trace(False)
        e0, s0 = ctx.visibility(v, sb, cb)
        ctx.set_vis_trace(True)
        e1, s1 = ctx.visibility(v, sb, cb)
    finally:
        ctx.set_vis_trace(True)
    cleared, reads = ctx.vis_trace_counts()
    np.testing.assert_array_equal(e0, e1)
    for k in ("pairs_tested", "n_edges", "self_hits", "cage_hits", "degenerate"):
        assert s0[k] == s1[k], k
    if case == "far_translated":
        assert cleared == 0 and reads == 0  # no grid
    if case == "degenerate_cage":
        assert cleared > 0.5 * s1["pairs_tested"]
    print(f"{case}: {s1['pairs_tested']} pairs, {len(e1)} edges, {cleared} cleared, {reads} grid reads")


def test_free_space_grid_reused_for_the_next_cage(ctx):
    """A context keeps the last grid's 3D array for the next grid of the same
    size: a cage moved by a small offset (same extent, same grid size, other
    bounds) built after the first cage's BVH is gone must walk on its own
    bounds, so its edges equal those with the walk off."""
    v, t = mg.displaced_blob(5, seed=2026)
    cv, ct = mg.offset_cage(v, t, 0.03)
    sb = ctx.bvh(v, t)
    out = []
    for shift in (0.0, 0.02):
        cb = ctx.bvh(cv + np.array([shift, -shift, 0.5 * shift]), ct)
        ctx.set_vis_trace(True)
        e1, s1 = ctx.visibility(v, sb, cb)
        cleared, _ = ctx.vis_trace_counts()
        ctx.set_vis_trace(False)
        e0, s0 = ctx.visibility(v, sb, cb)
        ctx.set_vis_trace(True)
        np.testing.assert_array_equal(e0, e1)
        assert s0["n_edges"] == s1["n_edges"] and cleared > 0
        out.append(len(e1))
        cb.close()
    assert out[0] != out[1]  # the moved cage gives other edges
