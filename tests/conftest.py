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
