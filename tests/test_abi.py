"""libcpt.so loads on a CPU-only host and exports exactly what include/cpt.h declares."""
from __future__ import annotations

import ctypes as C

from cudapathtracing_gb300 import _lib, abi


def test_library_exports_every_declared_symbol(cptlib):
    declared = _lib.declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(cptlib, name), name


def test_abi_version_and_layouts(cptlib):
    assert cptlib.cpt_abi_version() == 1
    assert C.sizeof(abi.cpt_ray) == 32 and C.sizeof(abi.cpt_hit) == 16
    assert C.sizeof(abi.cpt_light) == 96 and C.sizeof(abi.cpt_sphere) == 40
    assert C.sizeof(abi.cpt_material) == 72


def test_errors_are_statuses_not_exits(cptlib):
    # NULL arguments come back as CPT_ERR_INVALID_ARGUMENT with a message, never a crash.
    assert cptlib.cpt_scene_create(None, None, None) == 1
    assert b"null" in cptlib.cpt_last_error_string().lower()
    assert cptlib.cpt_render(None, None, None, None, None) == 1
    assert cptlib.cpt_lbvh_scratch_bytes(1000) > 1000 * 40
