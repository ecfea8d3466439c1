"""Decomposition with the learned proposer and the batched driver.

* process_batch: mesh i decomposed by a worker thread with its own GPU
  context and engine equals set_seed(seeds[i]); process(mesh_i) exactly.
* learned mode: the trained proposer (committed weights) decomposes held-out
  blobs, the exact scoring kernel ranks its proposals, and the trained network
  beats an untrained one on the share of splits that need the fallback and on
  the proposal quality against the exhaustive search, and beats the method
  without the network (a random draw of as many candidates) at equal cost."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mesh(V, v, t):
    m = V.Mesh()
    m.vertices = V.VecArray3d([list(map(float, p)) for p in v])
    m.triangles = V.make_vecarray3i(np.ascontiguousarray(t, dtype=np.int32))
    return m


def _parts_equal(a, b):
    assert a.num_parts == b.num_parts
    assert a.concavity == b.concavity
    for pa, pb in zip(a.parts, b.parts):
        np.testing.assert_array_equal(np.array(pa.vertices), np.array(pb.vertices))
        np.testing.assert_array_equal(np.array(pa.triangles), np.array(pb.triangles))


@pytest.fixture(scope="module")
def V(native):
    from visacd_gb300 import build
    build.build_host()
    import visacd_gb300.visacd as V
    V.config.verbose = False
    return V


def test_process_batch_equals_sequential(V):
    from visacd_gb300 import meshgen as mg, proposer as pp
    meshes = [_mesh(V, *mg.torus(nu=32, nv=16, seed=1)), _mesh(V, *pp.make_blob(1_000_001)[1:3]),
              _mesh(V, *pp.make_blob(1_000_002)[1:3])]
    seeds = [42, 7, 9]
    for mode in ("exhaustive", "learned"):
        V.config.plane_proposer = mode
        try:
            seq = []
            for m, s in zip(meshes, seeds):
                V.set_seed(s)
                seq.append(V.process(m, 0.04, 8))
            got = V.process_batch(V.MeshList(meshes), 0.04, 8, seeds, 3)
            assert len(got) == len(seq)
            for a, b in zip(got, seq):
                _parts_equal(a, b)
        finally:
            V.config.plane_proposer = "exhaustive"


def test_learned_process_runs_and_uses_proposals(V):
    from visacd_gb300 import proposer as pp
    _, v, t, _, _ = pp.make_blob(1_000_010)
    V.config.plane_proposer = "learned"
    try:
        V._reset_counters()
        V.set_seed(3)
        r = V.process(_mesh(V, v, t), 0.02, 16)
        st = V._stage_times()
    finally:
        V.config.plane_proposer = "exhaustive"
    assert r.num_parts >= 2 and np.isfinite(r.concavity)
    # one proposer call per split of a part that has visibility edges
    assert 0 < st["lp_calls"] <= st["iterations"]
    assert st["lp_fallbacks"] < st["lp_calls"]


def test_network_gains_over_the_method_without_it(native, ctx):
    """What the trained network adds: with the same number of exactly scored
    planes per split (16 proposals + their refinement + the 64-plane probe),
    the learned rule without its fallback picks better planes than the
    reference's random draw of that many candidates (the method without the
    network), on held-out blobs, both against the full 2500-candidate search."""
    from visacd_gb300 import proposer as pp
    trained = native.PlaneProposer(ctx, params=pp.load_params())
    held = list(range(pp.HELDOUT_SEED0 + 600, pp.HELDOUT_SEED0 + 648))
    st, _ = pp.evaluate(ctx, trained, held)
    print({k: round(v, 4) for k, v in st.items()})
    assert st["mean_learned_no_fallback_ratio"] > st["mean_no_network_same_budget_ratio"], st
    assert st["frac_learned_no_fallback_within_1pct"] > st["frac_no_network_same_budget_within_1pct"] + 0.1, st


def test_trained_proposer_beats_untrained(native, ctx):
    from visacd_gb300 import proposer as pp
    trained = native.PlaneProposer(ctx, params=pp.load_params())
    untrained = native.PlaneProposer(ctx, seed=12345)
    held = list(range(pp.HELDOUT_SEED0 + 500, pp.HELDOUT_SEED0 + 548))
    st, _ = pp.evaluate(ctx, trained, held)
    su, _ = pp.evaluate(ctx, untrained, held)
    assert st["mean_raw_proposal_ratio"] > su["mean_raw_proposal_ratio"] + 0.1, (st, su)
    assert st["fallback_rate"] < 0.5 * su["fallback_rate"], (st, su)
    assert st["mean_chosen_ratio"] > 0.99, st
