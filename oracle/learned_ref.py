"""CPU oracle of the learned plane proposer (test infrastructure only).

numpy float64 restatement of the network, loss and backward pass that
visacd_gb300/csrc/gpu/learned.cu runs on the tensor cores. The proposer has
no counterpart in the reference: this module is the gradient check of the
project's own kernels. Parity anchor: the formulas here are checked against
central finite differences (tests/test_learned_oracle.py); the GPU is then
checked against this module.

With `emulate_bf16=True` every tensor the GPU stores in BF16 (weights, input,
activations, back-propagated gradients) is rounded to BF16 (round to nearest
even) at the same point, so the remaining GPU/oracle difference is FP32 vs
FP64 accumulation. With `emulate_bf16=False` it is the exact FP64 network.
"""
from __future__ import annotations

import numpy as np

POINTS, FEATS, IN, PLANES = 2048, 7, 16, 16
K = [16, 64, 128, 256, 128, 64]
N = [64, 128, 256, 128, 64, 64]
LAMBDA = 0.1


def offsets():
    w, b, at = [], [], 0
    for k, n in zip(K, N):
        w.append(at)
        at += k * n
        b.append(at)
        at += n
    return w, b, at


WOFF, BOFF, TOTAL = offsets()


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to BF16 (nearest even) through float32, returned as float64."""
    f = np.asarray(x, dtype=np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray):
    p = np.asarray(params, dtype=np.float64)
    Ws = [p[WOFF[l]:WOFF[l] + K[l] * N[l]].reshape(N[l], K[l]) for l in range(6)]
    bs = [p[BOFF[l]:BOFF[l] + N[l]] for l in range(6)]
    return Ws, bs


def features(points, edges, center, scale) -> np.ndarray:
    """Features of the 2048 sampled edges (float32 arithmetic, learned.cu's
    lp_features_kernel)."""
    pts = np.asarray(points, dtype=np.float32).reshape(-1, 3)
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    E = len(e)
    s = np.arange(POINTS, dtype=np.int64)
    idx = (s * E) // POINTS if E >= POINTS else s % E
    p, q = pts[e[idx, 0]], pts[e[idx, 1]]
    c = np.asarray(center, dtype=np.float32)
    inv = np.float32(1.0) / np.float32(scale)
    mid = (np.float32(0.5) * (p + q) - c) * inv
    d = q - p
    ln = np.sqrt((d * d).sum(axis=1, dtype=np.float32)).astype(np.float32)
    u = np.where(ln[:, None] > 0, d / np.where(ln > 0, ln, 1)[:, None], 0).astype(np.float32)
    a = np.abs(u)
    pick = np.where((a[:, 0] >= a[:, 1]) & (a[:, 0] >= a[:, 2]), 0, np.where(a[:, 1] >= a[:, 2], 1, 2))
    big = u[np.arange(POINTS), pick]
    u = np.where(big[:, None] < 0, -u, u)
    return np.concatenate([mid, u, (ln * inv)[:, None]], axis=1).astype(np.float32)


def _loss_grad(Z, labels, lw):
    """Set loss per part and its gradient w.r.t. the head output Z [B x 64]."""
    B = Z.shape[0]
    dZ = np.zeros_like(Z)
    losses = np.zeros(B)
    for b in range(B):
        z = Z[b].reshape(PLANES, 4)
        n_raw, d = z[:, :3], z[:, 3]
        r = np.sqrt((n_raw ** 2).sum(axis=1)) + 1e-12
        nh = n_raw / r[:, None]
        lab, w = labels[b], lw[b]
        gn = np.zeros((PLANES, 3))
        gd = np.zeros(PLANES)
        valid = w > 0
        wsum = w.sum()
        inv_w = 1.0 / wsum if wsum > 0 else 0.0
        c = nh @ lab[:, :3].T                      # [q, l]
        Dp = 2 - 2 * c + (d[:, None] - lab[None, :, 3]) ** 2
        Dm = 2 + 2 * c + (-d[:, None] - lab[None, :, 3]) ** 2
        D = np.where(Dp <= Dm, Dp, Dm)
        S = np.where(Dp <= Dm, 1.0, -1.0)
        total = 0.0

        def add(q, l, coef):
            gn[q] += coef * (-2 * S[q, l] * lab[l, :3])
            gd[q] += coef * 2 * (d[q] - S[q, l] * lab[l, 3])

        for l in range(lab.shape[0]):
            if not valid[l]:
                continue
            q = int(np.argmin(D[:, l]))
            total += w[l] * inv_w * D[q, l]
            add(q, l, w[l] * inv_w)
        if valid.any():
            Dv = np.where(valid[None, :], D, np.inf)
            for q in range(PLANES):
                l = int(np.argmin(Dv[q]))
                total += LAMBDA / PLANES * D[q, l]
                add(q, l, LAMBDA / PLANES)
        losses[b] = total
        dotg = (nh * gn).sum(axis=1)
        dn = (gn - nh * dotg[:, None]) / r[:, None]
        dZ[b] = np.concatenate([dn, gd[:, None]], axis=1).reshape(-1) / B
    return losses, dZ


def forward_backward(params, feats, labels, lw, emulate_bf16: bool = True, backward: bool = True):
    """Returns (mean loss, gradient vector (TOTAL,), head output Z [B x 64])."""
    rnd = bf16 if emulate_bf16 else (lambda x: np.asarray(x, dtype=np.float64))
    Ws, bs = unpack(params)
    Wb = [rnd(W) for W in Ws]
    f = np.asarray(feats, dtype=np.float64).reshape(-1, POINTS, FEATS)
    B = f.shape[0]
    X0 = np.zeros((B * POINTS, IN))
    X0[:, :FEATS] = rnd(f.reshape(-1, FEATS))
    relu = lambda x: np.where(x > 0, x, 0.0)
    A1 = rnd(relu(X0 @ Wb[0].T + bs[0]))
    A2 = rnd(relu(A1 @ Wb[1].T + bs[1]))
    A3 = rnd(relu(A2 @ Wb[2].T + bs[2]))
    A3b = A3.reshape(B, POINTS, 256)
    arg = A3b.argmax(axis=1)                      # first maximum
    G = A3b.max(axis=1)
    A4 = rnd(relu(G @ Wb[3].T + bs[3]))
    A5 = rnd(relu(A4 @ Wb[4].T + bs[4]))
    Z6 = A5 @ Wb[5].T + bs[5]
    lab = np.asarray(labels, dtype=np.float64).reshape(B, -1, 4)
    w = np.asarray(lw, dtype=np.float64).reshape(B, -1)
    losses, dZ6 = _loss_grad(Z6, lab, w)
    if not backward:
        return losses.mean(), None, Z6
    g = np.zeros(TOTAL)

    def put(l, dW, db):
        g[WOFF[l]:WOFF[l] + dW.size] = dW.reshape(-1)
        g[BOFF[l]:BOFF[l] + db.size] = db

    dZ6 = rnd(dZ6)
    put(5, dZ6.T @ A5, dZ6.sum(axis=0))
    dZ5 = rnd((dZ6 @ Wb[5]) * (A5 > 0))
    put(4, dZ5.T @ A4, dZ5.sum(axis=0))
    dZ4 = rnd((dZ5 @ Wb[4]) * (A4 > 0))
    put(3, dZ4.T @ G, dZ4.sum(axis=0))
    dG = dZ4 @ Wb[3]
    mask = G > 0
    dZ3 = np.zeros((B, POINTS, 256))
    bi, ci = np.nonzero(mask)
    dZ3[bi, arg[bi, ci], ci] = rnd(dG[bi, ci])
    dZ3 = dZ3.reshape(-1, 256)
    put(2, dZ3.T @ A2, (dG * mask).sum(axis=0))
    dZ2 = rnd((dZ3 @ Wb[2]) * (A2 > 0))
    put(1, dZ2.T @ A1, dZ2.sum(axis=0))
    dZ1 = rnd((dZ2 @ Wb[1]) * (A1 > 0))
    put(0, dZ1.T @ X0, dZ1.sum(axis=0))
    return losses.mean(), g, Z6


def planes_from_head(Z6) -> np.ndarray:
    z = np.asarray(Z6, dtype=np.float64).reshape(-1, PLANES, 4)
    n = z[..., :3]
    r = np.sqrt((n ** 2).sum(axis=-1, keepdims=True)) + 1e-12
    return np.concatenate([n / r, z[..., 3:]], axis=-1)


def init_params(seed: int = 0) -> np.ndarray:
    """A seeded He-uniform initialisation (numpy generator; for tests)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(TOTAL, dtype=np.float32)
    fan = [FEATS, 64, 128, 256, 128, 64]
    for l in range(6):
        a = np.sqrt(6.0 / fan[l])
        W = rng.uniform(-a, a, size=(N[l], K[l])).astype(np.float32)
        W[:, fan[l]:] = 0
        p[WOFF[l]:WOFF[l] + W.size] = W.reshape(-1)
        p[BOFF[l]:BOFF[l] + N[l]] = rng.uniform(-0.1, 0.1, size=N[l])
    return p
