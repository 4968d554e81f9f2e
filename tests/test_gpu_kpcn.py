"""The denoiser's BF16 tensor-core training kernels against the FP64 oracle (oracle/kpcn_ref.py,
itself checked by finite differences in test_kpcn_oracle.py).

The oracle rounds to BF16 at the same points as the CUDA path, so the two differ only by FP32
versus FP64 accumulation (and the rare BF16 rounding or ReLU decision that this flips).
Tolerances: loss within 1e-3 relative; every layer's weight and bias gradient within 2e-2
relative L2 error with cosine similarity >= 0.999; forward output within 1e-3 * max(1, |x|).

The gradient check uses targets far above any output (20 + noisy), so the L1 loss's sign is the
same everywhere: with targets near the output, a pixel whose sign differs between FP32 and FP64
changes the summed gradients by a few percent, which says nothing about the kernels."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
K = pytest.importorskip("kpcn_ref")


def _batch(rng, N, H, W):
    rgb = rng.gamma(0.7, 0.6, size=(N, H, W, 3)).astype(np.float32)
    g = np.zeros((N, H, W, 8), np.float32)
    n = rng.normal(size=(N, H, W, 3))
    g[..., 0:3] = n / np.linalg.norm(n, axis=-1, keepdims=True)
    g[..., 3] = rng.uniform(1, 5, size=(N, H, W))
    g[..., 3][rng.uniform(size=(N, H, W)) < 0.1] = K.INF
    g[..., 4:7] = rng.uniform(0.1, 0.9, size=(N, H, W, 3))
    tgt = rng.gamma(2.0, 0.2, size=(N, H, W, 3)).astype(np.float32)
    return rgb, g, tgt


def _cuda(*arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def test_gradients_match_oracle(ctx):
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(7)
    rgb, g, _ = _batch(rng, 2, 32, 48)
    tgt = (20.0 + rgb).astype(np.float32)
    net = D.Denoiser(seed=3)
    p = net.params
    loss = net.train_step(*_cuda(rgb, g, tgt), update=False)
    grads = net.grads()
    o = K.Net(p)
    o.forward(rgb, g)
    lo = o.loss(tgt.astype(np.float64))
    go = o.backward()
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    for name, ws, bs, _ in D.layer_slices():
        for sl in (ws, bs):
            a, b = grads[sl].astype(np.float64), go[sl]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
            assert rel < 2e-2 and cos > 0.999, (name, rel, cos)


def test_denoise_matches_oracle_forward(ctx):
    """Any image size (padded to multiples of 16 inside), batch of 2."""
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(9)
    rgb, g, _ = _batch(rng, 2, 37, 45)
    net = D.Denoiser(seed=5)
    out = net.denoise(*_cuda(rgb, g)).cpu().numpy()
    want = K.Net(net.params).forward(rgb, g)
    err = np.abs(out - want) / np.maximum(1.0, np.abs(want))
    assert err.max() < 1e-3, err.max()
    assert out.shape == rgb.shape


def test_training_fits_a_batch(ctx):
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(11)
    rgb, g, _ = _batch(rng, 4, 64, 64)
    # target: the input itself, which the predicted kernels reach by peaking at the centre tap
    # (the initial kernels are close to a uniform 5x5 box)
    t = _cuda(rgb, g, rgb)
    net = D.Denoiser(seed=1)
    first = net.train_step(*t, lr=2e-3)
    for _ in range(80):
        last = net.train_step(*t, lr=2e-3)
    assert last < 0.5 * first, (first, last)


def test_save_load_roundtrip(ctx, tmp_path):
    from cudapathtracing_gb300 import denoiser as D
    a, b = D.Denoiser(seed=1), D.Denoiser(seed=2)
    assert not np.array_equal(a.params, b.params)
    a.save(str(tmp_path / "w.npz"))
    b.load(str(tmp_path / "w.npz"))
    assert np.array_equal(a.params, b.params)
