"""Autotuner host logic (no GPU): coordinate descent, margin rule, cache round trip and keys."""
from __future__ import annotations

import types

import pytest

from cudapathtracing_gb300 import abi, autotune as T


def fake_measure(best):
    """Score = 100 + bonus per knob value equal to `best`; deterministic."""
    def m(cfg):
        return 100.0 + sum(10.0 for k, v in best.items() if cfg[k] == v)
    return m


def test_descent_finds_separable_optimum_and_never_loses_to_defaults():
    target = {"slots": 1 << 22, "block_trace": 64, "short_stack": 24}
    best, score, dscore, trials = T.coordinate_descent(
        T.KNOBS[abi.INTEGRATOR_WAVEFRONT], fake_measure(target))
    for k, v in target.items():
        assert best[k] == v
    assert score >= dscore
    assert trials[0]["config"] == T.DEFAULTS


def test_margin_keeps_incumbent_on_ties():
    best, score, dscore, _ = T.coordinate_descent(T.KNOBS[abi.INTEGRATOR_WAVEFRONT], lambda cfg: 50.0)
    assert best == T.DEFAULTS and score == dscore


def test_noisy_gain_below_margin_is_ignored():
    def m(cfg):
        return 100.0 * (1.01 if cfg["slots"] == 1 << 20 else 1.0)
    best, _, _, _ = T.coordinate_descent(["slots"], m, margin=0.02)
    assert best["slots"] == T.DEFAULTS["slots"]


def test_cache_round_trip_and_key_stability(tmp_path):
    path = str(tmp_path / "tune.json")
    ch = T.Choice(knobs=dict(T.DEFAULTS, render_block=(32, 4)), score=700.0, default_score=650.0)
    T.save_cache(path, {"k": ch.to_json()})
    back = T.Choice.from_json(T.load_cache(path)["k"])
    assert back.knobs == ch.knobs and back.score == 700.0
    scene = types.SimpleNamespace(num_triangles=10, num_spheres=1, num_lights=2, width=64, height=48)
    dev = {"name": "GPU", "sms": 152}
    prm = dict(estimator=abi.ESTIMATOR_CONFIG, max_depth=8, rr_depth=3)
    k1 = T.workload_key(dev, scene, prm, abi.INTEGRATOR_WAVEFRONT)
    assert k1 == T.workload_key(dev, scene, dict(prm), abi.INTEGRATOR_WAVEFRONT)
    assert k1 != T.workload_key(dev, scene, prm, abi.INTEGRATOR_MEGAKERNEL)
    assert k1 != T.workload_key(dev, scene, prm, abi.INTEGRATOR_WAVEFRONT, probe_spp=2)   # timed at other spp
    scene.width = 65
    assert k1 != T.workload_key(dev, scene, prm, abi.INTEGRATOR_WAVEFRONT)
    assert T.load_cache(str(tmp_path / "missing.json")) == {}
