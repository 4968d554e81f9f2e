"""The denoiser's BF16 tensor-core training kernels against the FP64 oracle (oracle/kpcn_ref.py,
itself checked by finite differences in test_kpcn_oracle.py).

The oracle rounds to BF16 at the same points as the CUDA path.  Each layer is checked on the
library's own inputs to that layer ("teacher forcing", Net.use_activations): run freely, two
correct BF16 networks drift apart by rounding steps, and a pre-activation within a step of zero
takes the other side of a ReLU, which moves a layer's summed gradient by sqrt(flipped fraction)
and says nothing about the kernels.  Tolerances:
  forward   every convolution output within one BF16 step (2^-7 relative) of the oracle's, at
            least 99% of them identical; logits (FP32) within 1e-4 relative; pooling exact
  backward  loss within 1e-3 relative; every layer's weight and bias gradient within 1e-2
            relative L2 error, cosine similarity >= 0.9999
  inference end-to-end output within 1e-3 * max(1, |x|) of the free-running oracle."""
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
    g[..., 7] = rng.gamma(0.5, 0.02, size=(N, H, W))   # variance of the pixel mean
    tgt = rng.gamma(2.0, 0.2, size=(N, H, W, 3)).astype(np.float32)
    return rgb, g, tgt


def _cuda(*arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


NAMES = ["X0", "A0a", "cat0", "p1", "A1a", "cat1", "p2", "A2a", "cat2", "p3", "A3a", "cat3", "p4", "A4a", "A4b",
         "D3a", "D3b", "D2a", "D2b", "D1a", "D1b", "D0a", "D0b", "logits"]


def _run(net, rgb, g, tgt):
    loss = net.train_step(*_cuda(rgb, g, tgt), update=False)
    ex = {n: net.export(n) for n in NAMES}
    o = K.Net(net.params)
    o.use_activations(ex, rgb, g)
    return loss, ex, o


BACKENDS = pytest.mark.parametrize("backend", [0, 1, 2], ids=["mma_sync", "tcgen05", "tcgen05_ws"])


# Engine 2 switches to row tiles (k_conv3x3_rows) where the padded width is a multiple of 128:
# a 256-wide batch runs levels 0-1 on row tiles and levels 2-4 on im2col tiles.
ROW_SHAPE = (1, 32, 256)


@BACKENDS
def test_forward_layers_match_oracle(ctx, backend):
    _forward_layers(backend, (2, 32, 48))


def test_forward_layers_match_oracle_row_tiles(ctx):
    _forward_layers(2, ROW_SHAPE)


def _forward_layers(backend, shape):
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(7)
    rgb, g, tgt = _batch(rng, *shape)
    net = D.Denoiser(seed=3)
    net.set_backend(backend)
    _, ex, o = _run(net, rgb, g, tgt)
    net.check()
    skip = {"A0b": ("cat0", 64), "A1b": ("cat1", 96), "A2b": ("cat2", 128), "A3b": ("cat3", 160)}
    for name, (want, _) in o.layer_outputs().items():
        if name in skip:
            got = o.a[skip[name][0]][..., skip[name][1]:]
        else:
            got = o.a[name]
        if name == "logits":
            assert np.abs(got - want).max() <= 1e-4 * max(1.0, np.abs(want).max()), name
            continue
        d = np.abs(got - want)
        assert (d <= 2.0 ** -7 * np.abs(want) + 1e-6).all(), (name, d.max())
        assert (got == want).mean() >= 0.99, (name, (got == want).mean())


@BACKENDS
def test_gradients_match_oracle(ctx, backend):
    _gradients(backend, (2, 32, 48))


def test_gradients_match_oracle_row_tiles(ctx):
    _gradients(2, ROW_SHAPE)


def _gradients(backend, shape):
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(7)
    rgb, g, tgt = _batch(rng, *shape)
    net = D.Denoiser(seed=3)
    net.set_backend(backend)
    loss, ex, o = _run(net, rgb, g, tgt)
    net.check()
    grads = net.grads()
    lo = o.loss(tgt.astype(np.float64))
    go = o.backward()
    assert abs(loss - lo) <= 1e-3 * lo, (loss, lo)
    table, bad = [], []
    for name, ws, bs, _ in D.layer_slices():
        for part, sl in (("W", ws), ("b", bs)):
            a, b = grads[sl].astype(np.float64), go[sl]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
            table.append(f"{name}.{part} rel {rel:.2e} cos {cos:.6f}")
            if not (rel < 1e-2 and cos > 0.9999):
                bad.append(table[-1])
    print("\n".join(table))
    assert not bad, bad


@BACKENDS
def test_denoise_matches_oracle_forward(ctx, backend):
    """Any image size (padded to multiples of 16 inside), batch of 2."""
    _denoise(backend, (2, 37, 45))


def test_denoise_matches_oracle_forward_row_tiles(ctx):
    """Padded to 32 x 256: row tiles with zero rows and columns of padding."""
    _denoise(2, (1, 21, 250))


def _denoise(backend, shape):
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(9)
    rgb, g, _ = _batch(rng, *shape)
    net = D.Denoiser(seed=5)
    net.set_backend(backend)
    out = net.denoise(*_cuda(rgb, g)).cpu().numpy()
    net.check()
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


def test_trained_denoiser_gain(ctx):
    """The committed weights on a held-out scene (not in the training seeds) at 4 spp: the
    denoiser's display-space RMSE against a 2048-spp render is well below the plain render's and
    below the reference's own joint-bilateral filter's."""
    import os
    import torch
    from cudapathtracing_gb300 import api, training as T
    from cudapathtracing_gb300.denoiser import Denoiser
    if not os.path.exists(T.DEFAULT_WEIGHTS):
        pytest.skip("no trained weights in the tree")
    from cudapathtracing_gb300 import procedural as P
    net = Denoiser()
    net.load(T.DEFAULT_WEIGHTS)
    sc = api.Scene(ctx, P.random_scene(T.EVAL_SEED0, width=128)).init()
    ref, _, _ = T.render(ctx, sc, 2048, seed=1, gbuf=False)
    rgb, gb, _ = T.render(ctx, sc, 4, seed=2)
    den = net.denoise(rgb, gb)[0]
    bil = api.filter_bilateral(ctx, rgb, gb)
    torch.cuda.synchronize()
    e_plain, e_bil, e_den = T.rmse(rgb, ref), T.rmse(bil, ref), T.rmse(den, ref)
    print(f"RMSE plain {e_plain:.4f} bilateral {e_bil:.4f} denoised {e_den:.4f}")
    assert e_den < 0.5 * e_plain and e_den < e_bil, (e_plain, e_bil, e_den)


def test_denoise_unaligned_gbuffer(ctx):
    """A G-buffer that does not start on a 16-byte boundary (read with scalar loads) gives the
    same output as an aligned copy (read as float4 pairs)."""
    import torch
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(11)
    rgb, g, _ = _batch(rng, 1, 32, 48)
    net = D.Denoiser(seed=5)
    r_t, g_t = _cuda(rgb, g)
    want = net.denoise(r_t, g_t)
    buf = torch.empty(g_t.numel() + 1, device="cuda")
    buf[1:] = g_t.flatten()
    g_u = buf[1:].view(g_t.shape)
    assert g_u.data_ptr() % 16 != 0
    got = net.denoise(r_t, g_u)
    net.check()
    assert torch.equal(got, want)


def test_fused_apply_matches_training_path_and_logits_not_exported(ctx):
    """At inference the default engine applies the predicted kernels inside the logits
    convolution (no logits stored); the training pass stores the logits and applies them with a
    separate kernel.  On the same weights and inputs both give the same output up to FP32
    summation order, and exporting "logits" after the fused pass is refused, not stale."""
    from cudapathtracing_gb300 import denoiser as D
    rng = np.random.default_rng(13)
    rgb, g, tgt = _batch(rng, 1, 32, 256)   # padded width 256: row tiles, the fused epilogue
    net = D.Denoiser(seed=5)
    r_t, g_t, t_t = _cuda(rgb, g, tgt)
    net.train_step(r_t, g_t, t_t, update=False)
    unfused = net.export("out").reshape(rgb.shape)
    fused = net.denoise(r_t, g_t).cpu().numpy()
    net.check()
    err = np.abs(fused - unfused) / np.maximum(1.0, np.abs(unfused))
    assert err.max() < 1e-5, err.max()
    with pytest.raises(Exception, match="logits"):
        net.export("logits")


def test_barrier_wait_limit_reports_timeout(ctx):
    """The bounded mbarrier wait of the tensor-core kernels gives up on a barrier that nothing
    arrives on and sets the error word: cpt_denoiser_check reports CPT_ERR_TIMEOUT once, then the
    denoiser checks clean and still matches the oracle."""
    from cudapathtracing_gb300 import denoiser as D, _lib
    net = D.Denoiser(seed=5)
    _lib.check(_lib.lib().cpt_denoiser_wait_selftest(net.h), "cpt_denoiser_wait_selftest")
    with pytest.raises(_lib.CptError) as e:
        net.check()
    assert e.value.status == 4
    net.check()
    rng = np.random.default_rng(9)
    rgb, g, _ = _batch(rng, 1, 16, 32)
    out = net.denoise(*_cuda(rgb, g)).cpu().numpy()
    net.check()
    want = K.Net(net.params).forward(rgb, g)
    assert (np.abs(out - want) / np.maximum(1.0, np.abs(want))).max() < 1e-3


def _disp(x):
    return np.minimum(np.sqrt(np.maximum(x, 0.0)), 1.0)


def _drmse(a, b):
    return float(np.sqrt(((_disp(a) - _disp(b)) ** 2).mean()))


def _band_pair(ctx, oracle_mod, k, rows, spp, seed):
    import torch
    from cudapathtracing_gb300 import abi, api, procedural as P, training as T
    d = P.random_scene(T.EVAL_SEED0 + k, width=512)
    s = api.Scene(ctx, d).init()
    prm = dict(spp=spp, **T.RENDER)
    out = []
    for sd in (seed, seed + 1000):
        rgb = torch.zeros((s.height, s.width, 3), device="cuda")
        s.render(integrator=abi.INTEGRATOR_WAVEFRONT, rows=rows, rgb=rgb, seed=sd, **prm)
        torch.cuda.synchronize()
        out.append(rgb.cpu().numpy()[rows[0]:rows[1]].astype(np.float64))
    s.close()
    o = oracle_mod.OracleScene(d).render(abi.render_params(row_begin=rows[0], row_end=rows[1], seed=seed, **prm))
    return out[0], out[1], o["rgb"][rows[0]:rows[1]]


@pytest.mark.parametrize("k", range(8))
def test_denoise_eval_renders_follow_the_fp64_oracle(ctx, oracle_mod, k):
    """The wall-time-to-RMSE evaluation (bench.py denoise, training.evaluate) renders every held-out
    512x512 scene with the library, the high-spp reference included.  On the same PCG32 streams the
    library follows the FP64 oracle's sample paths; where FP32 and FP64 round a path apart (near-
    specular GGX down to roughness 0.05, glass, volumes) the two renders hold different samples of
    the same estimator.  Check on a 4-row band at 256 spp with the evaluation's estimator and
    integrator: the display-space RMSE between the library's render and the oracle's (same seed) is
    below 0.3 of the RMSE between two library renders of different seeds (independent noise)."""
    g, g2, o = _band_pair(ctx, oracle_mod, k, (200, 204), 256, 18)
    assert np.isfinite(g).all()
    same, indep = _drmse(g, o), _drmse(g, g2)
    match = (np.abs(g - o) <= 2e-3 * np.maximum(1.0, np.abs(o))).all(-1).mean()
    print(f"scene {k}: pixels within 2e-3 {match:.4f}; display RMSE vs oracle {same:.2e}, between seeds {indep:.2e}")
    assert same < 0.3 * indep, (same, indep)


def test_denoise_eval_reference_vs_fp64_oracle_at_16384_spp(ctx, oracle_mod):
    """The evaluation's reference itself: one row of held-out scene 0 (near-specular GGX and glass,
    where paths part most) at the reference's 16384 spp and seed, library against FP64 oracle.  Their
    display-space RMSE bounds (triangle inequality) how far an RMSE reported against the library's
    reference can be from the RMSE against the oracle's render: below 2e-3, a fifth of the 0.01
    target."""
    g, _, o = _band_pair(ctx, oracle_mod, 0, (256, 257), 16384, 18)
    d = _drmse(g, o)
    print(f"display RMSE, library vs FP64 oracle at 16384 spp: {d:.2e}")
    assert d < 2e-3, d
