"""Seeded workload generators: sizes and determinism."""
from __future__ import annotations

import hashlib

import numpy as np

from cudapathtracing_gb300 import procedural as P


def _h(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def test_icosphere_counts():
    v, f = P.icosphere(3)
    assert f.shape == (1280, 3) and v.shape == (642, 3)
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
    # closed manifold: every edge is shared by exactly two faces
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, counts = np.unique(e, axis=0, return_counts=True)
    assert (counts == 2).all()


def test_cornell_box_layout():
    d = P.cornell_box()
    assert d.num_triangles == 34 and len(d.lights) == 1 and d.num_prims == 35
    assert d.camera.width == 512 and d.camera.height == 512
    alb = np.array([m["color"] for m in d.materials])
    assert (alb >= 0.1).all() and (alb <= 0.8).all()


def test_generators_are_deterministic():
    a = P.uniform_rays(1000, seed=1)
    b = P.uniform_rays(1000, seed=1)
    assert _h(a) == _h(b)
    d = a["direction"].astype(np.float64)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    assert (np.abs(a["origin"]) <= 2.0).all()
    assert _h(P.displaced_icosphere(2)) == _h(P.displaced_icosphere(2))


def test_camera_height_rule():
    from cudapathtracing_gb300.abi import Camera
    assert Camera(1920, 16.0 / 9.0).height == 1080
    assert Camera(800, 16.0 / 9.0).height == 450
    assert Camera(10, 100.0).height == 1


def test_pcg32_jump_ahead_matches_stepping():
    """advance(n) equals n draws (config-estimator sample streams start k * 2^32 draws ahead)."""
    streams = np.arange(5, dtype=np.uint64) * np.uint64(7919)
    for n in (0, 1, 2, 7, 64, 1000):
        a = P.PCG32Streams(11, streams)
        b = P.PCG32Streams(11, streams)
        for _ in range(n):
            a.next()
        b.advance(n)
        assert np.array_equal(a.state, b.state)
        assert np.array_equal(a.next(), b.next())
    # jumps compose: 3 * 2^32 in one step or in three
    a = P.PCG32Streams(3, streams).advance(3 << 32)
    b = P.PCG32Streams(3, streams).advance(1 << 32).advance(1 << 32).advance(1 << 32)
    assert np.array_equal(a.state, b.state)
