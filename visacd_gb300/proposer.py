"""Training data, training loop and evaluation of the learned plane proposer.

The network and its kernels live in csrc/gpu/learned.cu (C ABI visacd_lp_*);
this module drives them from Python:

* `make_blob(seed)`: a seeded displaced icosphere (subdivision 3 or 4) in the
  [-1, 1] frame the decomposition works in, with a 0.03 offset cage.
* `label_blob(...)`: its visibility edges (GPU), the reference's candidate
  draw (2500 planes, `set_seed(seed)` first) scored exhaustively on the GPU,
  the top-L planes as labels (weights = score / best score, in the blob's
  bounding-box frame), and the network features of the sampled edges.
* `train(...)`: Adam over shuffled mini-batches with a cosine learning rate,
  all forward / backward / update work in the project's kernels.
* `evaluate(...)`: on held-out blobs, the best proposal's exact score against
  the exhaustive best, and what the probe-and-fallback rule would do.

Command line (needs a GPU):

    python -m visacd_gb300.proposer train --blobs 20000 --out visacd_gb300/proposer_weights.bin
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import time
from pathlib import Path

import numpy as np

from . import meshgen as mg

WEIGHTS = Path(__file__).resolve().parent / "proposer_weights.bin"
LABELS = 8
TRAIN_SEED0 = 0
HELDOUT_SEED0 = 1_000_000


def make_blob(seed: int):
    """Seeded blob (subdivision 3 or 4) normalised like process() does, and its
    offset cage."""
    rng = np.random.default_rng([seed, 77])
    level = int(rng.integers(3, 5))
    v, t = mg.displaced_blob(level, seed=seed)
    lo, hi = v.min(axis=0), v.max(axis=0)
    v = 2.0 * (v - 0.5 * (lo + hi)) / float((hi - lo).max())
    cv, ct = mg.offset_cage(v, t, 0.03)
    return seed, v, t, cv, ct


def part_frame(v: np.ndarray):
    lo, hi = v.min(axis=0), v.max(axis=0)
    half = 0.5 * float((hi - lo).max())
    return 0.5 * (lo + hi), (half if half > 0 else 1.0)


def exhaustive(ctx, v, edges, seed: int):
    """The reference's split search on one part: candidate draw after
    set_seed(seed), exact scores. Returns (planes P x 4, scores P)."""
    import visacd_gb300.visacd as V
    V.set_seed(seed)
    planes = np.asarray(V._candidate_planes(v, edges, 2500), dtype=np.float64).reshape(-1, 4)
    if len(planes) == 0:
        return planes, np.zeros(0)
    scores, _ = ctx.score_planes(planes, v, edges)
    return planes, scores


def visibility(ctx, v, t, cv, ct):
    sb, cb = ctx.bvh(v, t), ctx.bvh(cv, ct)
    try:
        edges, _ = ctx.visibility(v, sb, cb)
    finally:
        sb.close()
        cb.close()
    return edges


def to_frame(planes: np.ndarray, center, half: float) -> np.ndarray:
    """Planes n.x + d = 0 in the input frame -> n.x' + d' = 0 with x' = (x - c) / h."""
    p = np.array(planes, dtype=np.float64).reshape(-1, 4)
    p[:, 3] = (p[:, :3] @ np.asarray(center, dtype=np.float64) + p[:, 3]) / half
    return p


def label_blob(ctx, lp, seed, v, t, cv, ct, L: int = LABELS):
    edges = visibility(ctx, v, t, cv, ct)
    if len(edges) < 4:
        return None
    planes, scores = exhaustive(ctx, v, edges, seed)
    if len(planes) == 0 or scores.max() <= 0:
        return None
    order = np.argsort(-scores, kind="stable")[:L]
    c, h = part_frame(v)
    lab = np.zeros((L, 4), np.float32)
    w = np.zeros(L, np.float32)
    lab[: len(order)] = to_frame(planes[order], c, h)
    w[: len(order)] = scores[order] / scores[order[0]]
    feats = lp.features(v, edges, c, h)
    return feats, lab, w


def build_dataset(ctx, lp, seeds, workers: int = 16, log=print):
    feats, labels, weights, used = [], [], [], []
    t0 = time.time()
    with mp.get_context("spawn").Pool(workers) as pool:
        for k, (seed, v, t, cv, ct) in enumerate(pool.imap(make_blob, seeds, chunksize=32)):
            r = label_blob(ctx, lp, seed, v, t, cv, ct)
            if r is not None:
                feats.append(r[0])
                labels.append(r[1])
                weights.append(r[2])
                used.append(seed)
            if log and (k + 1) % 2000 == 0:
                log(f"  labelled {k + 1}/{len(seeds)} blobs ({time.time() - t0:.1f} s)")
    return np.stack(feats), np.stack(labels), np.stack(weights), np.array(used)


def train(ctx, feats, labels, weights, epochs: int = 30, batch: int = 64, lr: float = 2e-3,
          seed: int = 0, log=print):
    from ._native import PlaneProposer
    lp = PlaneProposer(ctx, seed=seed)
    rng = np.random.default_rng(seed)
    n = len(feats)
    steps = epochs * (n // batch)
    history = []
    step = 0
    t0 = time.time()
    for ep in range(epochs):
        perm = rng.permutation(n)
        tot, cnt = 0.0, 0
        for b in range(n // batch):
            idx = np.sort(perm[b * batch:(b + 1) * batch])
            cur = lr * 0.5 * (1.0 + np.cos(np.pi * step / max(steps, 1)))
            tot += lp.train_step(feats[idx], labels[idx], weights[idx], cur)
            cnt += 1
            step += 1
        history.append(tot / max(cnt, 1))
        if log:
            log(f"  epoch {ep + 1}/{epochs}: loss {history[-1]:.4f} ({time.time() - t0:.1f} s)")
    return lp, history


def bisector_planes(v, edges) -> np.ndarray:
    """Perpendicular-bisector plane of every edge (the reference's candidate
    form, lib/src/process.cpp:45-53): n = unit(p2 - p1), d = -n . midpoint."""
    p1 = v[edges[:, 0].astype(np.int64)]
    p2 = v[edges[:, 1].astype(np.int64)]
    n = p2 - p1
    ln = np.linalg.norm(n, axis=1)
    ok = ln >= 1e-6
    n = n[ok] / ln[ok, None]
    m = 0.5 * (p1[ok] + p2[ok])
    return np.concatenate([n, -(n * m).sum(axis=1, keepdims=True)], axis=1)


def refine(prop: np.ndarray, bis: np.ndarray, per: int = 8, half: float = 1.0) -> np.ndarray:
    """For each proposal, the `per` bisector planes nearest to it under the
    training distance (normal sign folded; offsets in units of the part's
    half-extent)."""
    if len(bis) == 0:
        return np.zeros((0, 4))
    c = prop[:, :3] @ bis[:, :3].T
    s = np.where(c >= 0, 1.0, -1.0)
    D = 2 - 2 * np.abs(c) + ((s * prop[:, 3:4] - bis[None, :, 3]) / half) ** 2
    k = min(per, len(bis))
    idx = np.unique(np.argpartition(D, k - 1, axis=1)[:, :k].reshape(-1))
    return bis[idx]


def evaluate(ctx, lp, seeds, probe: int = 64, tol: float = 0.01, per: int = 8):
    """Per held-out blob: exhaustive best score, best proposal score, best probe
    score (the reference's draw limited to `probe` planes after
    set_seed(seed + 1)), the score of the plane the learned rule picks, and the
    method without the network at the same budget: the reference's draw of as
    many planes as the learned rule scores (proposals + refined + probe), after
    set_seed(seed + 2)."""
    import visacd_gb300.visacd as V
    rows = []
    for seed in seeds:
        _, v, t, cv, ct = make_blob(seed)
        edges = visibility(ctx, v, t, cv, ct)
        if len(edges) < 4:
            continue
        planes, scores = exhaustive(ctx, v, edges, seed)
        if len(planes) == 0 or scores.max() <= 0:
            continue
        c, h = part_frame(v)
        prop = lp.propose(v, edges, c, h)
        ps, _ = ctx.score_planes(prop, v, edges)
        ref = refine(prop, bisector_planes(v, edges), per, h)
        rs, _ = ctx.score_planes(ref, v, edges) if len(ref) else (np.zeros(1), None)
        raw = float(ps.max())
        ps = np.concatenate([ps, rs])
        V.set_seed(seed + 1)
        pr = np.asarray(V._candidate_planes(v, edges, probe), dtype=np.float64).reshape(-1, 4)
        qs, _ = ctx.score_planes(pr, v, edges) if len(pr) else (np.zeros(1), None)
        budget = len(prop) + len(ref) + len(pr)
        V.set_seed(seed + 2)
        nn = np.asarray(V._candidate_planes(v, edges, budget), dtype=np.float64).reshape(-1, 4)
        ns, _ = ctx.score_planes(nn, v, edges) if len(nn) else (np.zeros(1), None)
        best, bp, bq = float(scores.max()), float(ps.max()), float(qs.max())
        fallback = bp < (1.0 - tol) * bq
        chosen = best if fallback else max(bp, bq)
        rows.append({"seed": int(seed), "edges": int(len(edges)), "exhaustive": best, "raw": raw,
                     "refined_planes": int(len(ref)), "proposal": bp,
                     "probe": bq, "fallback": bool(fallback), "chosen": chosen,
                     "learned_no_fallback": max(bp, bq), "budget": int(budget),
                     "no_network": float(ns.max())})
    r = np.array([[x["proposal"] / x["exhaustive"], x["probe"] / x["exhaustive"],
                   x["chosen"] / x["exhaustive"], x["fallback"], x["raw"] / x["exhaustive"],
                   x["refined_planes"], x["learned_no_fallback"] / x["exhaustive"],
                   x["no_network"] / x["exhaustive"], x["budget"]] for x in rows])
    summary = {
        "blobs": len(rows),
        "mean_raw_proposal_ratio": float(r[:, 4].mean()),
        "mean_refined_planes": float(r[:, 5].mean()),
        "mean_proposal_ratio": float(r[:, 0].mean()),
        "frac_proposal_within_1pct": float((r[:, 0] >= 0.99).mean()),
        "mean_probe_ratio": float(r[:, 1].mean()),
        "fallback_rate": float(r[:, 3].mean()),
        "mean_chosen_ratio": float(r[:, 2].mean()),
        "frac_chosen_within_1pct": float((r[:, 2] >= 0.99).mean()),
        "mean_planes_scored": float(r[:, 8].mean()),
        "mean_learned_no_fallback_ratio": float(r[:, 6].mean()),
        "frac_learned_no_fallback_within_1pct": float((r[:, 6] >= 0.99).mean()),
        "mean_no_network_same_budget_ratio": float(r[:, 7].mean()),
        "frac_no_network_same_budget_within_1pct": float((r[:, 7] >= 0.99).mean()),
    }
    return summary, rows


def save(lp, path: Path = WEIGHTS) -> None:
    lp.params().astype("<f4").tofile(str(path))


def load_params(path: Path = WEIGHTS) -> np.ndarray:
    return np.fromfile(str(path), dtype="<f4")


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--blobs", type=int, default=20000)
    tr.add_argument("--heldout", type=int, default=256)
    tr.add_argument("--epochs", type=int, default=30)
    tr.add_argument("--batch", type=int, default=64)
    tr.add_argument("--lr", type=float, default=2e-3)
    tr.add_argument("--workers", type=int, default=16)
    tr.add_argument("--out", type=Path, default=WEIGHTS)
    tr.add_argument("--report", type=Path, default=None)
    args = ap.parse_args(argv)

    from ._native import Context, PlaneProposer
    t_all = time.time()
    ctx = Context(0)
    feat_lp = PlaneProposer(ctx, seed=0)
    print(f"labelling {args.blobs} training blobs")
    t0 = time.time()
    feats, labels, weights, used = build_dataset(ctx, feat_lp, list(range(TRAIN_SEED0, TRAIN_SEED0 + args.blobs)),
                                                 workers=args.workers)
    t_data = time.time() - t0
    print(f"dataset: {len(used)} blobs with edges ({t_data:.1f} s)")
    t0 = time.time()
    lp, history = train(ctx, feats, labels, weights, epochs=args.epochs, batch=args.batch, lr=args.lr)
    t_train = time.time() - t0
    save(lp, args.out)
    held = list(range(HELDOUT_SEED0, HELDOUT_SEED0 + args.heldout))
    summary, _ = evaluate(ctx, lp, held)
    untrained, _ = evaluate(ctx, PlaneProposer(ctx, seed=12345), held)
    report = {
        "command": "python -m visacd_gb300.proposer train " + " ".join(
            f"--{k} {v}" for k, v in [("blobs", args.blobs), ("heldout", args.heldout), ("epochs", args.epochs),
                                     ("batch", args.batch), ("lr", args.lr)]),
        "train_blobs": int(len(used)), "dataset_s": t_data, "train_s": t_train,
        "loss_history": history, "heldout_trained": summary, "heldout_untrained": untrained,
        "total_s": time.time() - t_all,
    }
    print(json.dumps(report, indent=1))
    if args.report:
        args.report.write_text(json.dumps(report, indent=1))


if __name__ == "__main__":
    main()
