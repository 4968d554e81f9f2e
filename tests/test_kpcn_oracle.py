"""The FP64 denoiser oracle (oracle/kpcn_ref.py): its backward pass against central finite
differences of its own exact (unrounded) forward pass, and the BF16 rounding helper."""
from __future__ import annotations

import numpy as np
import pytest

K = pytest.importorskip("kpcn_ref")


def _batch(rng, N=1, H=16, W=16):
    rgb = rng.gamma(0.7, 0.6, size=(N, H, W, 3))
    g = np.zeros((N, H, W, 8))
    n = rng.normal(size=(N, H, W, 3))
    g[..., 0:3] = n / np.linalg.norm(n, axis=-1, keepdims=True)
    g[..., 3] = rng.uniform(1, 5, size=(N, H, W))
    g[..., 4:7] = rng.uniform(0.1, 0.9, size=(N, H, W, 3))
    tgt = rng.gamma(2.0, 0.2, size=(N, H, W, 3))
    return rgb, g, tgt


def _params(rng):
    p = []
    for ci, co, _ in K.SPECS:
        p.append(rng.normal(0, np.sqrt(2.0 / (9 * ci)), size=9 * ci * co))
        p.append(rng.normal(0, 0.05, size=co))
    return np.concatenate(p)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -3.14159, 0.0, 1e-40])
    r = K.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0            # tie to even
    assert r[2] == 1.0 + 2 ** -7
    assert r[3] == 1.0 + 2 ** -6                  # tie to even (up)
    assert abs(r[4] + 3.140625) < 1e-12


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    rgb, g, tgt = _batch(rng)
    p = _params(rng)
    net = K.Net(p, rounded=False)
    net.forward(rgb, g)
    net.loss(tgt)
    grad = net.backward()

    def L(q):
        n2 = K.Net(q, rounded=False)
        n2.forward(rgb, g)
        return n2.loss(tgt)

    sl = []
    off = 0
    for ci, co, _ in K.SPECS:
        sl.append((off, off + 9 * ci * co, off + 9 * ci * co + co))
        off += 9 * ci * co + co
    idx = []
    for layer in (0, 4, 9, 10, 16, 18):
        a, b, c = sl[layer]
        idx += list(rng.integers(a, b, size=3)) + [int(rng.integers(b, c))]
    eps = 1e-5
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = L(q)
        q[i] -= 2 * eps
        lm = L(q)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-4 * max(1e-3, abs(fd)) + 1e-8, (i, fd, grad[i])
