"""The learned split search in one call (visacd_learned_split_search, through
the C ABI) against the composition of the separately checked calls: the
proposer's planes (visacd_lp_propose), the host statement of the refinement,
the probe candidates (visacd_candidate_planes, pinned against the oracle's
get_candidate_planes, lib/src/process.cpp:28-72), the exact scores
(visacd_score_planes) and the decision restated here. Bit for bit: the number
of refined and probe planes, the draws used, the fallback decision, the first
maximum, its plane and every reported score."""
from pathlib import Path

import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

WEIGHTS = Path(__file__).resolve().parents[1] / "visacd_gb300" / "proposer_weights.bin"


@pytest.fixture(scope="module")
def V(native):
    from visacd_gb300 import build
    build.build_host()
    import visacd_gb300.visacd as V
    return V


@pytest.fixture(scope="module")
def proposers(native, ctx):
    trained = native.PlaneProposer(ctx, params=np.fromfile(WEIGHTS, dtype=np.float32))
    untrained = native.PlaneProposer(ctx, seed=3)
    yield {"trained": trained, "untrained": untrained}
    trained.close()
    untrained.close()


def _frame(v):
    lo, hi = v.min(0), v.max(0)
    center = (0.5 * (lo + hi)).astype(np.float32)
    half = 0.5 * float((hi - lo).max())
    return center, (half if half > 0 else 1.0)


def _compose(ctx, lp, V, v, e, k, draws, probe, flat, flat_k, tol):
    """The split search from its parts, as the host ran it before it was one call."""
    center, half = _frame(v)
    prop = lp.propose(v.astype(np.float32), e, center, half)
    ref = V._refine_proposals(v, e, prop, k).reshape(-1, 4)
    pr, used = ctx.candidate_planes(v, e, draws, probe)
    pr = pr.reshape(-1, 4)
    planes = np.concatenate([prop, ref, pr, flat.reshape(-1, 4)])
    s, _ = ctx.score_planes(planes.astype(np.float32), v.astype(np.float32), e)
    n_prop = 16 + len(ref)
    s = s.astype(np.float64)
    s[n_prop + len(pr):] *= flat_k
    best_prop = s[:n_prop].max()
    best_probe = max(0.0, s[n_prop:n_prop + len(pr)].max()) if len(pr) else 0.0
    best = int(np.argmax(s))
    return {"best_index": best, "n_refined": len(ref), "n_probe": len(pr), "draws_used": used,
            "fallback": int(best_prop < (1.0 - tol) * best_probe), "best_score": s[best],
            "best_proposal_score": best_prop, "best_probe_score": best_probe}, planes[best], center, half


def _check(ctx, orc, lp, V, v, e, k=32, probe=64, seed=0, flat=None, flat_k=2.0, tol=0.01):
    flat = np.zeros((0, 4)) if flat is None else flat
    _, draws, _ = orc.candidate_planes_with_draws(v, e, probe, seed)
    want, want_plane, center, half = _compose(ctx, lp, V, v, e, k, draws, probe, flat, flat_k, tol)
    plane, info = lp.split_search(v, e, center, half, half, k, draws, probe, flat, flat_k, tol)
    assert info == want
    np.testing.assert_array_equal(plane, want_plane)
    return info


def _blob_edges(orc, level=3, seed=2):
    v, t = mg.displaced_blob(level, seed=seed)
    _, e, _ = orc.visibility(v, t, *mg.offset_cage(v, t, 0.03))
    return v, e


def _flat(seed, n=6):
    rng = np.random.default_rng(seed)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return np.concatenate([nrm, rng.uniform(-0.3, 0.3, (n, 1))], 1)


@pytest.mark.parametrize("which", ["trained", "untrained"])
@pytest.mark.parametrize("k", [32, 8, 1, 0])
def test_learned_split_equals_composition(ctx, orc, V, proposers, which, k):
    v, e = _blob_edges(orc, 3, 2)
    info = _check(ctx, orc, proposers[which], V, v, e, k=k, seed=k, flat=_flat(k))
    assert info["n_refined"] <= 16 * k


@pytest.mark.parametrize("seed", [1, 5, 9])
def test_learned_split_blobs_and_flat_k(ctx, orc, V, proposers, seed):
    v, e = _blob_edges(orc, 3, seed)
    lp = proposers["trained"]
    _check(ctx, orc, lp, V, v, e, seed=seed, flat=_flat(seed), flat_k=1.0)
    _check(ctx, orc, lp, V, v, e, seed=seed + 1, probe=0)  # proposals and refinement alone


def test_learned_split_fallback_decision(ctx, orc, V, proposers):
    v, e = _blob_edges(orc, 3, 4)
    lp = proposers["untrained"]
    assert _check(ctx, orc, lp, V, v, e, seed=2, tol=-1.0)["fallback"] == 1  # below 2 x the probe's best
    assert _check(ctx, orc, lp, V, v, e, seed=2, tol=1.0)["fallback"] == 0   # never
    _check(ctx, orc, lp, V, v, e, seed=2, tol=0.01)


def test_learned_split_few_and_degenerate_edges(ctx, orc, V, proposers):
    lp = proposers["trained"]
    v, e = _blob_edges(orc, 2, 5)
    # fewer bisectors than refine_k: every one is kept
    info = _check(ctx, orc, lp, V, v, e[:20], seed=3)
    assert info["n_refined"] == 20
    # coincident endpoints have no bisector but their draws still count
    v2 = np.concatenate([v, v[e[:40, 0]]])
    extra = np.stack([e[:40, 0], len(v) - 40 + np.arange(40)], 1).astype(np.uint32)
    e2 = np.concatenate([extra, e[:300]])
    info = _check(ctx, orc, lp, V, v2, e2, seed=4)
    assert info["n_refined"] <= 300


def test_learned_split_many_edges(ctx, orc, V, proposers):
    # more edges than one refinement block covers: several blocks per proposal
    v, _ = mg.displaced_blob(5, seed=3)
    rng = np.random.default_rng(11)
    i = rng.integers(0, len(v), 400_000)
    j = rng.integers(0, len(v), 400_000)
    keep = i != j
    e = np.stack([np.minimum(i, j), np.maximum(i, j)], 1)[keep].astype(np.uint32)
    _check(ctx, orc, proposers["trained"], V, v, e, seed=6, flat=_flat(6))


def test_learned_split_rejects_bad_arguments(ctx, orc, native, proposers):
    v, e = _blob_edges(orc, 2, 1)
    lp = proposers["trained"]
    center, half = _frame(v)
    draws = np.zeros(5, np.int32)
    with pytest.raises(native.VisacdError):
        lp.split_search(v, e, center, half, half, 33, draws, 1)  # refine_k above 32
    with pytest.raises(native.VisacdError):
        lp.split_search(v, np.zeros((0, 2), np.uint32), center, half, half, 8, draws[:0], 1)
    with pytest.raises(native.VisacdError):
        lp.split_search(v, e, center, 0.0, half, 8, draws, 1)
    with pytest.raises(native.VisacdError):
        lp.split_search(v, e, center, half, half, 8, np.array([len(e)], np.int32), 1)


def test_proposer_outlives_its_context(native, orc):
    """Destroying the context first releases the proposer's device memory;
    later calls fail cleanly and destroying the proposer still works."""
    c2 = native.Context(0)
    lp = native.PlaneProposer(c2, seed=1)
    v, e = _blob_edges(orc, 2, 1)
    center, half = _frame(v)
    lp.propose(v.astype(np.float32), e, center, half)
    c2.close()
    with pytest.raises(native.VisacdError):
        lp.propose(v.astype(np.float32), e, center, half)
    with pytest.raises(native.VisacdError):
        lp.split_search(v, e, center, half, half, 8, np.zeros(5, np.int32), 1)
    lp.close()
