"""cpt_filter_bilateral / cpt_filter_temporal (FP32, device) against the FP64 oracle
(oracle/filters.py, pinned to the reference's kernels in test_filters.py).

Tolerance: |gpu - oracle| <= 2e-4 * max(1, |oracle|) per channel.  Bilateral: every pixel.
Temporal: the FP32 reprojection may land on the neighbouring source pixel where the projected
coordinate is within rounding of a pixel edge, so >= 99% of pixels must match."""
from __future__ import annotations

import numpy as np
import pytest

from cudapathtracing_gb300 import abi, api, procedural as P

filters = pytest.importorskip("filters")
pytestmark = pytest.mark.gpu

TOL = 2e-4


def _render(ctx, width=64, spp=2):
    import torch
    d = P.cornell_box(width=width)
    s = api.Scene(ctx, d).init()
    H = s.height
    rgb = torch.zeros((H, width, 3), device="cuda")
    gb = torch.zeros((H, width, 8), device="cuda")
    s.render(spp=spp, seed=4, estimator=abi.ESTIMATOR_CONFIG, max_depth=8, rr_depth=3, rr_prob=0.8, rgb=rgb, gbuffer=gb)
    torch.cuda.synchronize()
    return d, s, rgb, gb


def _close(a, b):
    return (np.abs(a - b) <= TOL * np.maximum(1.0, np.abs(b))).all(-1)


@pytest.mark.parametrize("prm", [abi.filter_params(), abi.filter_params(4.0, 0.5, 0.3, 0.5, 6)])
def test_bilateral_matches_oracle(ctx, prm):
    import torch
    d, s, rgb, gb = _render(ctx)
    out = api.filter_bilateral(ctx, rgb, gb, params=prm)
    torch.cuda.synchronize()
    g4 = gb.cpu().numpy()[..., :4].astype(np.float64)
    want = filters.bilateral(rgb.cpu().numpy(), g4, prm.sigma_g, prm.sigma_r, prm.sigma_n, prm.sigma_d, prm.radius)
    got = out.cpu().numpy()
    ok = _close(got, want)
    assert ok.all(), (ok.mean(), np.abs(got - want).max())
    # the filter reduces the noise of a 2-spp render (variance of neighbouring-pixel differences)
    r = rgb.cpu().numpy()
    assert np.abs(np.diff(got, axis=1)).mean() < 0.7 * np.abs(np.diff(r, axis=1)).mean()


def test_temporal_matches_oracle(ctx):
    import torch
    d, s, rgb, gb = _render(ctx)
    cam = d.camera
    H = s.height
    rng = np.random.default_rng(1)
    prev = torch.from_numpy(rng.uniform(size=(H, cam.width, 3)).astype(np.float32)).cuda()
    prev_cam = abi.Camera(width=cam.width, aspect_ratio=cam.aspect_ratio,
                          look_from=tuple(np.asarray(cam.look_from) + [0.05, 0.02, 0.0]),
                          look_at=tuple(cam.look_at), vfov_deg=cam.vfov_deg)
    cur = rgb.clone()
    api.filter_temporal(ctx, cur, prev, gb, cam, prev_cam, alpha=0.1)
    torch.cuda.synchronize()
    g4 = gb.cpu().numpy()[..., :4].astype(np.float64)
    pos = filters.positions_from_depth(g4, cam.width, cam.aspect_ratio, cam.look_from, cam.look_at, cam.vfov_deg)
    want = filters.temporal(rgb.cpu().numpy().astype(np.float64), prev.cpu().numpy().astype(np.float64), pos,
                            cam.width, prev_cam.look_from, prev_cam.look_at, prev_cam.vfov_deg, 0.1)
    ok = _close(cur.cpu().numpy(), want)
    assert ok.mean() >= 0.99, ok.mean()


def test_filter_argument_errors(ctx):
    import torch
    d, s, rgb, gb = _render(ctx, width=32, spp=1)
    with pytest.raises(Exception):
        api.filter_bilateral(ctx, rgb, gb, out=rgb)
    with pytest.raises(Exception):
        api.filter_bilateral(ctx, rgb, gb, params=abi.filter_params(sigma_r=0.0))
    other = abi.Camera(width=16, aspect_ratio=1.0)
    with pytest.raises(Exception):
        api.filter_temporal(ctx, rgb, rgb.clone(), gb, d.camera, other)
