"""Image writers of the headless renderer (no GPU)."""
from __future__ import annotations

import numpy as np

from cudapathtracing_gb300 import imageio


def test_ppm_uses_the_reference_display_transform_and_row_order(tmp_path):
    rgb = np.zeros((3, 4, 3), np.float32)
    rgb[0, 0] = (1.0, 0.25, 4.0)      # bottom-left pixel
    rgb[2, 3] = (0.0, 0.01, -1.0)     # top-right pixel
    p = str(tmp_path / "a.ppm")
    imageio.write_ppm(p, rgb)
    raw = open(p, "rb").read()
    assert raw.startswith(b"P6\n4 3\n255\n")
    back = imageio.read_ppm(p)
    assert back.shape == (3, 4, 3)
    assert tuple(back[0, 0]) == (254, 127, 254)   # 254.99*sqrt(x), clamped
    assert tuple(back[2, 3]) == (0, 25, 0)
    # the file's first pixel is the top-left one
    assert tuple(np.frombuffer(raw[11:14], np.uint8)) == tuple(back[2, 0])


def test_pfm_roundtrip(tmp_path):
    rgb = np.random.default_rng(0).normal(size=(5, 7, 3)).astype(np.float32)
    p = str(tmp_path / "a.pfm")
    imageio.write_pfm(p, rgb)
    assert np.array_equal(imageio.read_pfm(p), rgb)
