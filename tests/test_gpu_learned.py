"""The learned proposer's tensor-core kernels against the CPU oracle:
features, forward planes, loss and every parameter gradient (BF16 storage
emulated by the oracle, so the remaining difference is FP32 vs FP64
accumulation), and a short training run that must lower the loss."""
import numpy as np
import pytest

from oracle import learned_ref as lr

pytestmark = pytest.mark.gpu

# Relative L2 tolerance per parameter block for GPU vs oracle gradients: FP32
# accumulation against FP64 can flip a BF16 rounding of a stored activation or
# gradient (one BF16 ulp = 2^-8 relative); measured errors are far below this.
GRAD_RTOL = 2e-2


def _case(seed, B, L=8):
    rng = np.random.default_rng(seed)
    feats = np.empty((B, lr.POINTS, lr.FEATS), dtype=np.float32)
    feats[..., :3] = rng.uniform(-1, 1, size=(B, lr.POINTS, 3))
    d = rng.normal(size=(B, lr.POINTS, 3))
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    feats[..., 3:6] = d
    feats[..., 6] = rng.uniform(0.05, 1.5, size=(B, lr.POINTS))
    n = rng.normal(size=(B, L, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    labels = np.concatenate([n, rng.uniform(-0.6, 0.6, size=(B, L, 1))], axis=-1).astype(np.float32)
    w = rng.uniform(0.3, 1.0, size=(B, L)).astype(np.float32)
    w[:, -2:] = 0
    return feats, labels, w


def test_features_match_oracle(native, ctx):
    from visacd_gb300 import meshgen as mg
    lp = native.PlaneProposer(ctx, seed=1)
    v, t = mg.displaced_blob(3, seed=5)
    rng = np.random.default_rng(0)
    for E in (1, 100, 2048, 9000):
        e = np.sort(rng.integers(0, len(v), size=(E, 2)), axis=1).astype(np.uint32)
        e = e[e[:, 0] != e[:, 1]]
        c = v.mean(axis=0)
        got = lp.features(v, e, c, 1.3)
        ref = lr.features(v, e, c, 1.3)
        np.testing.assert_allclose(got, ref, rtol=2e-6, atol=2e-6)


def test_forward_and_gradients_match_oracle(native, ctx):
    params = lr.init_params(3)
    lp = native.PlaneProposer(ctx, params=params)
    np.testing.assert_array_equal(lp.params(), params)
    feats, labels, w = _case(7, B=3)
    loss, g = lp.grads(feats, labels, w)
    rloss, rg, Z6 = lr.forward_backward(params, feats, labels, w, emulate_bf16=True)
    assert abs(loss - rloss) <= 1e-3 * abs(rloss)
    planes = lp.forward(feats)
    np.testing.assert_allclose(planes, lr.planes_from_head(Z6), atol=2e-3)
    errs = {}
    for l in range(6):
        for name, lo, n in (("W", lr.WOFF[l], lr.K[l] * lr.N[l]), ("b", lr.BOFF[l], lr.N[l])):
            a, b = g[lo:lo + n], rg[lo:lo + n]
            errs[f"{name}{l + 1}"] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
    assert max(errs.values()) < GRAD_RTOL, errs
    # the exact FP64 network (no BF16 rounding) agrees to BF16 precision
    _, g64, _ = lr.forward_backward(params, feats, labels, w, emulate_bf16=False)
    cos = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
    assert cos > 0.99


def test_training_lowers_loss_and_is_deterministic(native, ctx):
    feats, labels, w = _case(11, B=16)
    runs = []
    for _ in range(2):
        lp = native.PlaneProposer(ctx, seed=4)
        first = lp.train_step(feats, labels, w, 3e-3)
        for _ in range(60):
            last = lp.train_step(feats, labels, w, 3e-3)
        runs.append((first, last, lp.params()))
    assert runs[0][1] < 0.6 * runs[0][0], runs[0][:2]
    np.testing.assert_array_equal(runs[0][2], runs[1][2])


def test_tcgen05_forward_matches_mma_sync(native, ctx):
    """The tcgen05 (tensor-memory) forward of the per-edge layers against the
    mma.sync one: same BF16 operands, FP32 accumulation in another order, so
    the planes and every gradient agree to BF16 rounding."""
    params = lr.init_params(5)
    feats, labels, w = _case(13, B=3)
    a = native.PlaneProposer(ctx, params=params)
    a.set_tcgen05(False)
    b = native.PlaneProposer(ctx, params=params)
    b.set_tcgen05(True)
    pa, pb = a.forward(feats), b.forward(feats)
    np.testing.assert_allclose(pb, pa, atol=2e-2)
    la, ga = a.grads(feats, labels, w)
    lb, gb = b.grads(feats, labels, w)
    assert abs(la - lb) <= 1e-2 * abs(la)
    assert np.linalg.norm(ga - gb) <= 2e-2 * np.linalg.norm(ga)
    # and the oracle (BF16-emulated) agrees with the tcgen05 path as with mma.sync
    rloss, rg, _ = lr.forward_backward(params, feats, labels, w, emulate_bf16=True)
    assert abs(lb - rloss) <= 1e-2 * abs(rloss)
