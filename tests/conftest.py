"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on a CPU-only host."""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
SCENES = os.path.join(GOLDEN, "scenes")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; calls libcpt.so through its C ABI")


def pytest_collection_modifyitems(config, items):
    have_gpu = None
    for item in items:
        if "gpu" in item.keywords:
            if have_gpu is None:
                import torch
                have_gpu = torch.cuda.is_available()
            if not have_gpu:
                item.add_marker(pytest.mark.skip(reason="no CUDA device"))


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"])
    return oracle


@pytest.fixture(scope="session")
def cptlib():
    from cudapathtracing_gb300 import build
    build.build()
    from cudapathtracing_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def ctx(cptlib):
    from cudapathtracing_gb300 import api
    c = api.Context(0)
    yield c
    c.close()


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name))


def outward_f32(lo: np.ndarray, hi: np.ndarray):
    """FP32 boxes rounded outwards from FP64 ones (min down, max up)."""
    flo = lo.astype(np.float32)
    fhi = hi.astype(np.float32)
    flo = np.where(flo.astype(np.float64) > lo, np.nextafter(flo, np.float32(-np.inf)), flo)
    fhi = np.where(fhi.astype(np.float64) < hi, np.nextafter(fhi, np.float32(np.inf)), fhi)
    return flo, fhi


def check_rgba8(gpu_rgba8, ref_rgba8, gpu_rgb, ref_rgb, equal_frac=0.98):
    """The 8-bit display image (sqrt gamma, x254.99, clamp; Render.cu:229-260) of an FP32 render
    against the FP64 one: at least `equal_frac` of the bytes are equal, and every byte of a pixel
    whose radiance agrees to 1e-4 (the same path, FP32 rounding only) is within one step, since
    rounding can only move a value across one quantisation boundary.  Pixels whose path diverged
    (an edge hit or a roulette draw at its threshold) are bounded by the radiance tolerance."""
    g8 = gpu_rgba8.astype(np.int32)
    r8 = ref_rgba8.astype(np.int32)
    same = (np.abs(gpu_rgb.astype(np.float64) - ref_rgb) <= 1e-4 * np.maximum(1.0, np.abs(ref_rgb))).all(-1)
    d = np.abs(g8 - r8)[..., :3]
    eq = (d == 0).mean()
    print(f"rgba8: {eq:.5f} of bytes equal; max step on same-path pixels {d[same].max() if same.any() else 0}")
    assert eq >= equal_frac, eq
    assert (d[same] <= 1).all(), int(d[same].max())
    assert same.mean() >= 0.9, same.mean()
