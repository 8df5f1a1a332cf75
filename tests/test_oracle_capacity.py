"""CPU checks of the oracle's restatement of the capacity network (no GPU).

The oracle's backward is checked against central finite differences of its own forward in
float64 (no BF16 rounding), and its BF16 mode against an independent numpy forward pass, so the
oracle that the GPU gradients are compared with is itself pinned.
"""
import numpy as np

import oracle as O


def _bf16(x):
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _setup(seed=0, n=64):
    rng = np.random.default_rng(seed)
    P = (rng.normal(size=O.CAP_PARAMS) * 0.2).astype(np.float32)
    P[-1] = 1.5
    F = rng.random((n, O.CAP_FEATURES)).astype(np.float32) * 3
    T = (rng.random(n) * 3).astype(np.float32)
    return P, F, T


def test_backward_matches_finite_differences():
    P, F, T = _setup()
    g, _, _ = O.cap_forward_backward(P, F, T, 24, 5, 11, mode=-1)
    rng = np.random.default_rng(1)
    idx = np.concatenate([rng.integers(0, O.CAP_PARAMS, 40), [O.CAP_PARAMS - 1]])
    for i in idx:
        a, b = P.copy(), P.copy()
        a[i] += np.float32(3e-5)
        b[i] -= np.float32(3e-5)
        _, la, _ = O.cap_forward_backward(a, F, T, 24, 5, 11, mode=-1)
        _, lb, _ = O.cap_forward_backward(b, F, T, 24, 5, 11, mode=-1)
        fd = (la - lb) / (float(a[i]) - float(b[i]))
        assert abs(fd - g[i]) <= 1e-5 + 1e-3 * abs(g[i]), (i, fd, g[i])


def test_bf16_forward_matches_numpy():
    P, F, T = _setup(2, 32)
    _, _, y = O.cap_forward_backward(P, F, T, 32, 0, 1, mode=1)
    W1 = _bf16(P[:2048]).reshape(64, 32).astype(np.float64)
    b1 = P[2048:2112].astype(np.float64)
    W2 = _bf16(P[2112:6208]).reshape(64, 64).astype(np.float64)
    b2 = P[6208:6272].astype(np.float64)
    W3 = _bf16(P[6272:6336]).astype(np.float64)
    b3 = float(P[6336])
    x = _bf16(F).astype(np.float64)
    h1 = _bf16(np.maximum(x @ W1.T + b1, 0)).astype(np.float64)
    h2 = np.maximum(h1 @ W2.T + b2, 0)
    z = h2 @ W3 + b3
    want = np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z)))
    np.testing.assert_allclose(y, want, rtol=2e-3, atol=2e-3)
