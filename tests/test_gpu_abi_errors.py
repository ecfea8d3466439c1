"""Argument checking of the newer C entry points: bad sizes and indices come
back as VISACD_ERR_INVALID_ARG with a message (no kernel runs on them), and
empty inputs are valid no-ops."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_hull_distances_bad_pairs(native, ctx):
    hulls = [np.zeros((3, 3)), np.ones((2, 3))]
    with pytest.raises(native.VisacdError):
        ctx.hull_distances(hulls, np.array([[0, 2]], np.int32))
    assert len(ctx.hull_distances(hulls, np.zeros((0, 2), np.int32))) == 0


def test_segment_triangle_empty(ctx):
    hit, n64 = ctx.segment_triangle_tests(np.zeros((0, 6), np.float32), np.zeros((0, 9), np.float32))
    assert hit.shape == (0,) and n64 == 0


def test_face_hausdorff_empty_rejected(native, ctx):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    t = np.array([[0, 1, 2]], np.int32)
    with pytest.raises(native.VisacdError):
        ctx.face_hausdorff(v, t, np.zeros((0, 3)), np.zeros(0, np.int32), v, t, v, np.zeros(3, np.int32))


def test_proposer_bad_parameter_count(native, ctx):
    with pytest.raises(ValueError):
        native.PlaneProposer(ctx, params=np.zeros(10, np.float32))


def test_process_batch_needs_one_seed_per_mesh(native):
    from visacd_gb300 import build
    build.build_host()
    import visacd_gb300.visacd as V
    m = V.Mesh()
    with pytest.raises(RuntimeError):
        V.process_batch(V.MeshList([m, m]), 0.05, 4, [1], 1)


def test_learned_mode_without_weights_fails_loudly(native):
    from visacd_gb300 import build, meshgen as mg
    build.build_host()
    import visacd_gb300.visacd as V
    v, t = mg.torus(nu=24, nv=12, seed=1)
    m = V.Mesh()
    m.vertices = V.VecArray3d(v.tolist())
    m.triangles = V.make_vecarray3i(t.astype(np.int32))
    old_mode, old_path = V.config.plane_proposer, V.config.proposer_weights
    V.config.verbose = False
    V.config.plane_proposer = "learned"
    V.config.proposer_weights = "/nonexistent/weights.bin"
    try:
        with pytest.raises(RuntimeError):
            V.process(m, 0.01, 4)
    finally:
        V.config.plane_proposer, V.config.proposer_weights = old_mode, old_path
    with pytest.raises(RuntimeError):
        V.config.plane_proposer = "nonsense"
        try:
            V.process(m, 0.01, 4)
        finally:
            V.config.plane_proposer = old_mode


def test_face_hausdorff_batch_bad_indices(native, ctx):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    t = np.array([[0, 1, 2]], np.int32)
    x = v.copy()
    ok = (v, t, x, np.zeros(3, np.int32), v, t, x, np.zeros(3, np.int32))
    assert len(ctx.face_hausdorff_batch([ok])) == 1
    with pytest.raises(native.VisacdError):
        ctx.face_hausdorff_batch([(v, t, x, np.array([0, 1, 0], np.int32), v, t, x, np.zeros(3, np.int32))])
    with pytest.raises(native.VisacdError):
        ctx.face_hausdorff_batch([(v, np.array([[0, 1, 3]], np.int32), x, np.zeros(3, np.int32), v, t, x,
                                   np.zeros(3, np.int32))])
    assert len(ctx.face_hausdorff_batch([])) == 0


def test_clip_bad_triangle_index(native, ctx):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    with pytest.raises(native.VisacdError):
        ctx.clip(v, np.array([[0, 1, -1]], np.int32), [1.0, 0.0, 0.0, -0.5])


def test_throughput_probes(ctx):
    """The in-process roofline denominators: the FP32 FMA rate and the texture
    fetch rates (coherent blocks faster than one line per lane)."""
    assert ctx.fp32_peak_tflops() > 1.0
    coherent, divergent = ctx.tex_peak_gfetch()
    assert coherent > divergent > 1.0
