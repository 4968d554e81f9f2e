"""Scene builders shared by the tests (the golden fixtures were generated from the same
builders by tests/golden/make_golden.py)."""
from __future__ import annotations

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

from make_golden import degenerate_scene, mixed_scene, textured_scene  # noqa: E402,F401

from cudapathtracing_gb300 import api, procedural as P  # noqa: E402

SCENES = os.path.join(ROOT, "tests", "golden", "scenes")


def ini_desc(name: str):
    p = api.IniParser()
    p.Parse(os.path.join(SCENES, name + ".ini"))
    return p.to_scene_desc()


def by_name(name: str):
    if name == "cornell":
        return P.cornell_box(width=48)
    if name == "degenerate":
        return degenerate_scene()
    if name == "mixed":
        return mixed_scene()
    if name == "ico3":
        return P.icosphere_scene(level=3)
    if name == "textured":
        return textured_scene()
    return ini_desc(name)
