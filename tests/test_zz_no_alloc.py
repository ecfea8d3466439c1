"""The allocation-free scoring entry point (visacd_score_planes_noalloc).

It serves callers that cannot allocate device memory from inside the library —
code running under a fixed, pre-reserved memory budget or a latency-bound loop
that must not hit cudaMalloc. Its scratch is a static device array, so the
test checks, through the C ABI, that two calls in a row (different sizes; the
second must not see the first call's leftovers) give the same scores and argmax
as visacd_score_planes, and that sizes above the limits are refused.
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

CAPACITY = 4  # VISACD_ERR_CAPACITY


def _inputs(seed, P, E, n_pts=3000):
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-1, 1, size=(n_pts, 3)).astype(np.float32)
    edges = rng.integers(0, n_pts, size=(E, 2)).astype(np.uint32)
    planes = mg.random_planes(P, seed=seed)
    return planes, pts, edges


def _noalloc(lib, torch, planes, pts, edges):
    dev = torch.device("cuda", 0)
    d_pl = torch.from_numpy(planes).to(dev)
    d_pt = torch.from_numpy(pts).to(dev)
    d_ed = torch.from_numpy(edges.view(np.int32)).to(dev)
    d_sc = torch.full((max(len(planes), 1),), -1.0, dtype=torch.float64, device=dev)
    d_am = torch.full((1,), -7, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.visacd_score_planes_noalloc(
        C.c_void_p(d_pl.data_ptr()), len(planes), C.c_void_p(d_pt.data_ptr()), len(pts),
        C.c_void_p(d_ed.data_ptr()), len(edges), C.c_void_p(d_sc.data_ptr()),
        C.c_void_p(d_am.data_ptr()), C.c_void_p(stream.cuda_stream))
    stream.synchronize()
    return rc, d_sc.cpu().numpy()[: len(planes)], int(d_am.cpu().item())


def test_noalloc_matches_allocating_entry_point_twice(ctx, native):
    torch = pytest.importorskip("torch")
    lib = native.lib()
    for seed, P, E in [(1, 4096, 65536), (2, 700, 20000)]:
        planes, pts, edges = _inputs(seed, P, E)
        ref, st = ctx.score_planes(planes, pts, edges)
        rc, got, am = _noalloc(lib, torch, planes, pts, edges)
        assert rc == 0, lib.visacd_last_error()
        np.testing.assert_array_equal(got, ref)
        assert am == st["argmax"]


def test_noalloc_rejects_sizes_beyond_limit(native):
    torch = pytest.importorskip("torch")
    lib = native.lib()
    planes, pts, edges = _inputs(3, 16, 65537)
    rc, _, _ = _noalloc(lib, torch, planes, pts, edges)
    assert rc == CAPACITY
    assert b"65536" in lib.visacd_last_error()
    planes, pts, edges = _inputs(4, 4097, 100)
    rc, _, _ = _noalloc(lib, torch, planes, pts, edges)
    assert rc == CAPACITY
    assert b"4096" in lib.visacd_last_error()
