"""libcpt.so loads on a CPU-only host and exports exactly what include/cpt.h declares."""
from __future__ import annotations

import ctypes as C
import os

import pytest

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


def test_cpp_wrapper_header_compiles_and_links(tmp_path):
    """include/cpt.hpp (the reference-named C++ classes) compiles against cpt.h and links with
    libcpt.so; the program only queries the ABI version (no GPU needed)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "use.cpp"
    src.write_text(
        '#include "cpt.hpp"\n#include <cstdio>\n'
        'int main() { static_assert(sizeof(cpt::Scene) == sizeof(void*), "handle");\n'
        '  std::printf("%d\\n", cpt_abi_version()); return 0; }\n')
    lib = os.path.join(root, "cudapathtracing_gb300", "_build")
    exe = tmp_path / "use"
    r = subprocess.run([gxx, "-std=c++17", "-I" + os.path.join(root, "include"), str(src), "-L" + lib, "-lcpt",
                        "-Wl,-rpath," + lib, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip().isdigit()
