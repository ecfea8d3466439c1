"""Candidate split planes and the split search on the GPU (through the C ABI)
against the oracle's restatement of get_candidate_planes
(lib/src/process.cpp:28-72), which the CPU suite pins bit for bit against the
reference compiled in place: the same planes in the same order, bit for bit,
and the same number of draws consumed; the split search picks the oracle's
first maximum (flat planes' scores times flat_k)."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _blob_edges(orc, level=3, seed=2):
    v, t = mg.displaced_blob(level, seed=seed)
    _, e, _ = orc.visibility(v, t, *mg.offset_cage(v, t, 0.03))
    return v, e


def _near_duplicates():
    # nearly parallel edges with close midpoints: many candidates are dropped
    # as similar (normals within 5 degrees and offsets within 1e-3)
    rng = np.random.default_rng(4)
    n = 300
    v = np.stack([rng.uniform(0, 0.05, n), rng.uniform(-2e-3, 2e-3, n), rng.uniform(-2e-3, 2e-3, n)], 1)
    i = rng.integers(0, n, 4000)
    j = rng.integers(0, n, 4000)
    keep = i != j
    e = np.stack([np.minimum(i, j), np.maximum(i, j)], 1)[keep].astype(np.uint32)
    return v, e


@pytest.mark.parametrize("case", ["blob", "near_duplicates", "few_edges", "degenerate"])
@pytest.mark.parametrize("seed", [0, 42])
def test_candidate_planes_bit_exact(ctx, orc, case, seed):
    if case == "blob":
        v, e = _blob_edges(orc)
    elif case == "near_duplicates":
        v, e = _near_duplicates()
    elif case == "few_edges":  # every draw repeats one of three edges
        v, e = _blob_edges(orc)
        e = e[:3]
    else:  # coincident endpoints are skipped but still consume their draw
        v, e = _blob_edges(orc, 2, 5)
        v = np.concatenate([v, v[e[:40, 0]]])
        extra = np.stack([e[:40, 0], len(v) - 40 + np.arange(40)], 1).astype(np.uint32)
        e = np.concatenate([extra, e[:200]])
    kept = {}
    for num in (2500, 64):
        want, draws, used = orc.candidate_planes_with_draws(v, e, num, seed)
        got, got_used = ctx.candidate_planes(v, e, draws, num)
        np.testing.assert_array_equal(got, want)
        assert got_used == used
        kept[num] = len(want)
    if case == "near_duplicates":  # many draws dropped as similar
        assert 0 < kept[2500] < 2500


def test_candidate_planes_edge_cases(ctx, orc):
    v, e = _blob_edges(orc, 2, 1)
    got, used = ctx.candidate_planes(v, e, np.zeros(0, np.int32), 0)
    assert len(got) == 0 and used == 0
    got, used = ctx.candidate_planes(v, np.zeros((0, 2), np.uint32), np.zeros(0, np.int32), 10)
    assert len(got) == 0
    native = pytest.importorskip("visacd_gb300._native")
    with pytest.raises(native.VisacdError):
        ctx.candidate_planes(v, e, np.array([len(e)], np.int32), 10)  # draw outside [0, E)


@pytest.mark.parametrize("flat_k", [2.0, 1.0])
def test_split_search_picks_the_first_maximum(ctx, orc, flat_k):
    v, e = _blob_edges(orc, 3, 8)
    want, draws, used = orc.candidate_planes_with_draws(v, e, 2500, 7)
    rng = np.random.default_rng(1)
    nrm = rng.normal(size=(6, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    flat = np.concatenate([nrm, rng.uniform(-0.3, 0.3, (6, 1))], 1)
    flat = np.concatenate([flat, want[:2]])  # ties between a flat plane and a candidate
    planes = np.concatenate([want, flat])
    s64, _ = ctx.score_planes(planes.astype(np.float32), v.astype(np.float32), e)
    # the reference compares float scores; flat ones times flat_k in double
    s = s64.astype(np.float32)
    s[len(want):] = (s[len(want):].astype(np.float64) * flat_k).astype(np.float32)
    best = int(np.argmax(s))
    plane, info = ctx.split_search(v, e, draws, 2500, flat, flat_k)
    assert info["best_index"] == best
    assert info["n_candidates"] == len(want) and info["draws_used"] == used
    np.testing.assert_array_equal(plane, planes[best])
    assert info["best_score"] == float(s[best])
    # without flat planes, and with no scoreable edge
    plane, info = ctx.split_search(v, e, draws, 2500)
    assert info["best_index"] == int(np.argmax(s[: len(want)]))
    plane, info = ctx.split_search(v, np.zeros((0, 2), np.uint32), np.zeros(0, np.int32), 2500, flat, flat_k)
    assert info["n_candidates"] == 0
