"""Precision form: FP32 segment-triangle filter + FP64 re-decision against the
FP64 oracle on 200k independent tests, 5 % built to graze a triangle edge
within 1e-6. Every decision must equal the oracle's (the FP32 bound is
rigorous and the FP64 formula is the oracle's), and the grazing tests must be
the ones sent to FP64."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def test_segment_triangle_decisions_equal_fp64(ctx, orc):
    seg, tri, built = mg.segment_triangle_cases(200_000, 0.05, seed=4)
    hit, n64 = ctx.segment_triangle_tests(seg, tri)
    ref, grazing = orc.seg_tri_batch(seg, tri)
    np.testing.assert_array_equal(hit, ref)
    assert grazing[built].mean() > 0.5          # the construction grazes
    assert n64 >= int(grazing.sum())            # every grazing decision went to FP64
    assert n64 < 0.2 * len(seg)                 # and the filter decides the bulk in FP32


def test_segment_triangle_edge_cases(ctx, orc):
    # degenerate triangle, zero-length segment, segment ending on the triangle, t below tmin
    seg = np.array([[0, 0, 1, 0, 0, -1], [0.2, 0.2, 0, 0.2, 0.2, 0], [0.1, 0.1, 1, 0.1, 0.1, 0],
                    [0.1, 0.1, 0.0005, 0.1, 0.1, -1]], np.float32)
    tri = np.array([[0, 0, 0, 1, 1, 1, 2, 2, 2], [0, 0, 0, 1, 0, 0, 0, 1, 0], [0, 0, 0, 1, 0, 0, 0, 1, 0],
                    [0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    hit, _ = ctx.segment_triangle_tests(seg, tri)
    ref, _ = orc.seg_tri_batch(seg, tri)
    np.testing.assert_array_equal(hit, ref)
