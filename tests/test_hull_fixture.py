"""The host QuickHull (hull.cpp) against the reference's btConvexHullComputer
(lib/3rd/btConvexHull via Mesh::compute_vch, lib/src/core.cpp:113-142), through
the committed fixture tests/golden/hull_bt.json (made by make_hull_fixtures.py
from the reference compiled in place): on integer-grid clouds where that hull
is exact, the same hull vertex set and the same volume to 1e-12. The GPU hull
(visacd_convex_hulls) is compared with the same fixture and with this host
hull in tests/test_gpu_hull.py."""
import json
from pathlib import Path

import numpy as np
import pytest

FIXTURE = Path(__file__).resolve().parent / "golden" / "hull_bt.json"


@pytest.fixture(scope="module")
def V():
    from visacd_gb300 import build
    build.build_host()
    import visacd_gb300.visacd as V
    return V


def hull_cases():
    return json.loads(FIXTURE.read_text())["cases"]


def check_against_bt(V, case, tris):
    p = np.asarray(case["points"], dtype=np.float64)
    t = np.asarray(tris).reshape(-1, 3)
    ours = set(map(tuple, p[np.unique(t)].astype(np.int64))) if len(t) else set()
    assert ours == set(map(tuple, case["bt_hull_vertices"])), case["name"]
    vol = V._mesh_volume(p, t) if len(t) else 0.0
    ref = case["bt_volume"]
    assert abs(vol - ref) <= 1e-12 * max(1.0, abs(ref)), (case["name"], vol, ref)


@pytest.mark.parametrize("case", hull_cases(), ids=lambda c: c["name"])
def test_host_hull_matches_btconvexhull_fixture(V, case):
    h = V._convex_hull(np.asarray(case["points"], dtype=np.float64))
    check_against_bt(V, case, h["triangles"])
