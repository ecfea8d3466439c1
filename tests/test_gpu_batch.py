"""Batched visibility + scoring (one graph-captured launch sequence over many
parts of uneven size) against per-part calls of the single-part entry points:
identical edge lists, scores and argmax, before and after graph replay."""
import numpy as np
import pytest

from visacd_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _part(seed, level):
    v, t = mg.displaced_blob(level, seed=seed)
    cv, ct = mg.offset_cage(v, t, 0.03)
    rng = np.random.default_rng(seed)
    nrm = rng.normal(size=(512, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    proj = v @ nrm.T
    d = -rng.uniform(proj.min(0), proj.max(0))
    planes = np.concatenate([nrm, d[:, None]], 1).astype(np.float32)
    return v.astype(np.float32), t, cv, ct, planes


def test_batch_equals_per_part_calls(ctx, native):
    rng = np.random.default_rng(0)
    levels = [2, 3, 2, 3, 1, 2, 3, 2]
    parts, bvhs = [], []
    for k, lv in enumerate(levels):
        v, t, cv, ct, pl = _part(100 + k, lv)
        sb, cb = ctx.bvh(v, t), ctx.bvh(cv, ct)
        bvhs += [sb, cb]
        parts.append((v, sb, cb, pl))
    batch = native.Batch(ctx, parts)
    for use_graph in (False, True, True):
        batch.run(use_graph)
        ne, scores, am, edges = batch.results(with_edges=True)
        eo = so = 0
        for k, (v, sb, cb, pl) in enumerate(parts):
            e_ref, _ = ctx.visibility(v, sb, cb)
            assert ne[k] == len(e_ref)
            np.testing.assert_array_equal(edges[eo:eo + ne[k]], e_ref)
            s_ref, st = ctx.score_planes(pl, v, e_ref)
            np.testing.assert_array_equal(scores[so:so + len(pl)], s_ref)
            if len(e_ref):
                assert am[k] == st["argmax"]
            eo += ne[k]
            so += len(pl)
    batch.close()
