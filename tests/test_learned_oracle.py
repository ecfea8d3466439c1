"""The learned proposer's CPU oracle checked against central finite
differences (float64, no BF16 rounding), and its feature restatement checked
on edge cases. CPU only."""
import numpy as np

from oracle import learned_ref as lr


def _case(seed=0, B=2, L=5):
    rng = np.random.default_rng(seed)
    params = lr.init_params(seed)
    feats = rng.uniform(-1, 1, size=(B, lr.POINTS, lr.FEATS)).astype(np.float32)
    n = rng.normal(size=(B, L, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    labels = np.concatenate([n, rng.uniform(-0.5, 0.5, size=(B, L, 1))], axis=-1).astype(np.float32)
    w = rng.uniform(0.2, 1.0, size=(B, L)).astype(np.float32)
    w[0, -1] = 0.0  # an unused slot
    return params.astype(np.float64), feats, labels, w


def test_oracle_gradient_matches_finite_differences():
    params, feats, labels, w = _case()
    loss, g, _ = lr.forward_backward(params, feats, labels, w, emulate_bf16=False)
    assert np.isfinite(loss) and loss > 0
    rng = np.random.default_rng(1)
    # a few entries of every weight and bias block
    picks = []
    for l in range(6):
        picks += list(rng.integers(lr.WOFF[l], lr.WOFF[l] + lr.K[l] * lr.N[l], size=6))
        picks += list(rng.integers(lr.BOFF[l], lr.BOFF[l] + lr.N[l], size=3))
    h = 1e-6
    bad = []
    for i in picks:
        if i >= lr.WOFF[0] and i < lr.WOFF[0] + lr.K[0] * lr.N[0] and (i - lr.WOFF[0]) % lr.K[0] >= lr.FEATS:
            continue  # padded input columns: zero gradient by construction
        p1 = params.copy()
        p1[i] += h
        p2 = params.copy()
        p2[i] -= h
        l1 = lr.forward_backward(p1, feats, labels, w, emulate_bf16=False, backward=False)[0]
        l2 = lr.forward_backward(p2, feats, labels, w, emulate_bf16=False, backward=False)[0]
        fd = (l1 - l2) / (2 * h)
        if abs(fd - g[i]) > 1e-5 + 1e-3 * abs(fd):
            bad.append((int(i), fd, g[i]))
    assert not bad, bad


def test_oracle_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0])
    r = lr.bf16(x)
    assert r[0] == 1.0
    # ties go to even mantissa; 1 + 2^-8 is halfway between 1 and 1 + 2^-7
    assert r[1] == 1.0
    assert r[2] == 1.0
    assert r[3] == 1.0 + 2 ** -7
    assert r[4] == -2.5 and r[5] == 0.0


def test_features_sampling_and_canonical_direction():
    pts = np.array([[0, 0, 0], [2, 0, 0], [0, -3, 0], [1, 1, 1]], dtype=np.float32)
    edges = np.array([[0, 1], [0, 2], [1, 3]], dtype=np.uint32)
    f = lr.features(pts, edges, center=[0, 0, 0], scale=2.0)
    assert f.shape == (lr.POINTS, lr.FEATS)
    # E < 2048: sample s takes edge s mod E
    np.testing.assert_allclose(f[0], [0.5, 0, 0, 1, 0, 0, 1.0])
    np.testing.assert_allclose(f[1], [0, -0.75, 0, 0, 1, 0, 1.5])   # direction (0,-1,0) flipped
    np.testing.assert_allclose(f[3], f[0])
    big = np.stack([np.arange(5000), np.arange(5000) + 1], axis=1).astype(np.uint32)
    P = np.random.default_rng(0).uniform(-1, 1, size=(5001, 3)).astype(np.float32)
    g = lr.features(P, big, [0, 0, 0], 1.0)
    # E >= 2048: sample s takes edge floor(s * E / 2048)
    e7 = big[(7 * 5000) // 2048]
    np.testing.assert_allclose(g[7, :3], 0.5 * (P[e7[0]] + P[e7[1]]), rtol=1e-6)
