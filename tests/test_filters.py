"""The FP64 filter oracle (oracle/filters.py) pinned against the reference's own gaussianSeparate
and addPrevious kernels, run as host loops from oracle/_ref (skipped where the reference is not
mounted)."""
from __future__ import annotations

import numpy as np
import pytest

from cudapathtracing_gb300 import abi

filters = pytest.importorskip("filters")


def _gbuf(rng, H, W, miss_frac=0.1):
    n = rng.normal(size=(H, W, 3))
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    # piecewise-smooth normals and depths so that the edge-stopping terms matter
    n[:, W // 2:] = n[0, 0]
    d = 2.0 + rng.uniform(0, 0.5, size=(H, W))
    d[H // 3:, :] += 3.0
    miss = rng.uniform(size=(H, W)) < miss_frac
    d[miss] = filters.INF
    n[miss] = 0.0
    return np.concatenate([n, d[..., None]], -1)


@pytest.fixture
def ref(oracle_mod):
    if oracle_mod.ref_lib() is None or not hasattr(oracle_mod.ref_lib(), "ref_gaussian_separate"):
        pytest.skip("oracle/_ref not built here")
    return oracle_mod


@pytest.mark.parametrize("sigmas", [(8.0, 5.0, 0.1, 0.2), (3.0, 0.2, 0.5, 1.0)])
def test_bilateral_oracle_matches_reference(ref, sigmas):
    rng = np.random.default_rng(3)
    H, W = 23, 41
    rgb = rng.gamma(0.6, 0.5, size=(H, W, 3))
    g = _gbuf(rng, H, W)
    want = ref.ref_bilateral(rgb, g, *sigmas)
    got = filters.bilateral(rgb, g, *sigmas, radius=16)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-13)
    assert np.abs(got - rgb).max() > 1e-3   # it filtered something


def test_temporal_oracle_matches_reference(ref):
    rng = np.random.default_rng(5)
    cam = abi.Camera(width=48, aspect_ratio=48 / 32, look_from=(0.3, 0.5, 4.0), look_at=(0.0, 0.2, 0.0), vfov_deg=40.0)
    H = filters.camera_height(cam.width, cam.aspect_ratio)
    rgb = rng.uniform(size=(H, cam.width, 3))
    prev = rng.uniform(size=(H, cam.width, 3))
    g = _gbuf(rng, H, cam.width, miss_frac=0.15)
    pos = filters.positions_from_depth(g, cam.width, cam.aspect_ratio, cam.look_from, cam.look_at, cam.vfov_deg)
    pre_from, pre_at = (0.6, 0.4, 4.1), (0.05, 0.2, 0.0)
    for moving, alpha in [(0, 0.1), (1, 0.4)]:
        want = ref.ref_temporal(rgb, prev, pos, cam, pre_from, pre_at, moving)
        got = filters.temporal(rgb, prev, pos, cam.width, pre_from, pre_at, cam.vfov_deg, alpha)
        assert np.allclose(got, want, rtol=1e-12, atol=1e-13)
    _, _, ok = filters.reproject(pos, cam.width, H, pre_from, pre_at, cam.vfov_deg)
    assert 0.3 < ok.mean() < 1.0   # both valid reprojections and fallbacks are exercised
