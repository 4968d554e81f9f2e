"""The FP64 oracle against the golden vectors produced by the reference's own code, and
(where the reference is mounted and compiled into oracle/_ref) against the reference live."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden
from cudapathtracing_gb300 import abi, procedural as P
import scenes

LBVH_CASES = ["cornell", "degenerate", "mixed", "ico3", "volume_glass", "glossy"]


def test_pcg32_known_answer():
    # pcg32-demo (O'Neill): pcg32_srandom_r(42, 54), first six outputs
    g = P.PCG32Streams(42, np.array([54], dtype=np.uint64))
    got = [int(g.next()[0]) for _ in range(6)]
    assert got == [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]


@pytest.mark.parametrize("name", LBVH_CASES)
def test_oracle_lbvh_matches_reference(oracle_mod, cptlib, name):
    o = oracle_mod.OracleScene(scenes.by_name(name))
    L = o.lbvh()
    G = golden(f"lbvh_{name}.npz")
    for k in ("keys", "order", "child_a", "child_b", "node_boxes", "leaf_boxes"):
        assert np.array_equal(L[k], G[k]), k


@pytest.mark.parametrize("name", ["ico3", "mixed"])
def test_oracle_hits_match_reference(oracle_mod, name):
    d = scenes.by_name(name)
    rays = P.uniform_rays(4096, seed=1) if name == "ico3" else P.uniform_rays(4096, seed=3, box=3.0)
    ids, t, _, _ = oracle_mod.OracleScene(d).trace(P.rays_as_f64(rays))
    G = golden(f"hits_{name}.npz")
    assert np.array_equal(ids, G["ids"])
    assert np.array_equal(t, G["t"])
    assert (ids >= 0).mean() > 0.1


@pytest.mark.parametrize("name", ["cornell", "mixed", "volume_glass", "glossy"])
def test_oracle_render_matches_reference(oracle_mod, cptlib, name):
    G = golden(f"render_{name}.npz")
    r = oracle_mod.OracleScene(scenes.by_name(name)).render(abi.render_params(spp=int(G["spp"]), seed=0))
    assert np.array_equal(r["rgb"], G["rgb"])
    assert np.array_equal(r["rgba8"], G["rgba8"])


def test_oracle_against_live_reference(oracle_mod):
    """Random scenes: LBVH, hits and a render, oracle vs the reference's compiled code."""
    if oracle_mod.ref_lib() is None:
        pytest.skip("oracle/_ref not built (reference not mounted)")
    for seed in (21, 22, 23):
        d = scenes.mixed_scene(seed)
        o, r = oracle_mod.OracleScene(d), oracle_mod.RefScene(d)
        Lo, Lr = o.lbvh(), r.lbvh()
        for k in Lo:
            assert np.array_equal(Lo[k], Lr[k]), (seed, k)
        rays = P.rays_as_f64(P.uniform_rays(2048, seed=seed, box=3.0))
        io, to, _, _ = o.trace(rays)
        ir, tr = r.trace(rays)
        assert np.array_equal(io, ir) and np.array_equal(to, tr)
        ro = o.render(abi.render_params(spp=2, seed=seed))
        rr = r.render(2, seed=seed)
        assert np.array_equal(ro["rgb"], rr["rgb"]) and np.array_equal(ro["rgba8"], rr["rgba8"])


@pytest.mark.parametrize("name", ["cornell", "mixed"])
def test_oracle_pick_and_material_edit_match_reference(oracle_mod, name):
    """getObject at every pixel, then changeMaterial edits (a range over lights, spheres and
    triangles; a range from the picked primitive) and a STATIC render: the restated oracle equals
    the reference's own kernels bit for bit (tests/golden/pick_*.npz)."""
    G = golden(f"pick_{name}.npz")
    o = oracle_mod.OracleScene(scenes.by_name(name))
    picks = np.array([[o.pick(x, y) for x in range(o.width)] for y in range(o.height)], np.int32)
    assert np.array_equal(picks, G["picks"])
    for first, end, ax, ay, glass in G["edits"]:
        o.set_material(int(first), int(end), ax, ay, bool(glass))
    r = o.render(abi.render_params(spp=int(G["spp"]), seed=0))
    assert np.array_equal(r["rgb"], G["rgb"])
    assert np.array_equal(r["rgba8"], G["rgba8"])


def test_oracle_pick_against_live_reference(oracle_mod):
    lib = oracle_mod.ref_lib()
    if lib is None or not hasattr(lib, "ref_pick"):
        pytest.skip("oracle/_ref not built (reference not mounted)")
    for seed in (21, 22):
        d = scenes.mixed_scene(seed)
        o, r = oracle_mod.OracleScene(d), oracle_mod.RefScene(d)
        for y in range(0, o.height, 3):
            for x in range(o.width):
                assert o.pick(x, y) == r.pick(x, y), (seed, x, y)
        for rr in (o, r):
            rr.set_material(3, 200, 0.15, 0.45, True)
        a = o.render(abi.render_params(spp=2, seed=seed))
        b = r.render(2, seed=seed)
        assert np.array_equal(a["rgb"], b["rgb"])


def test_oracle_single_and_empty_scenes(oracle_mod):
    d = abi.SceneDesc()
    d.add_material((1, 1, 1))
    d.spheres.append(dict(center=(0.0, 0.0, 0.0), radius=1.0, material=0))
    d.camera = abi.Camera(8, 1.0, (0, 0, 5), (0, 0, 0), 40.0, (0.1, 0.2, 0.3))
    o = oracle_mod.OracleScene(d)
    ids, t, _, _ = o.trace(np.array([[0, 0, 5, 0.001, 0, 0, -1, 999999.0]], np.float64))
    assert ids[0] == 0 and abs(t[0] - 4.0) < 1e-12
    e = abi.SceneDesc()
    e.camera = d.camera
    r = oracle_mod.OracleScene(e).render(abi.render_params(spp=1))
    assert np.allclose(r["rgb"], np.array([0.1, 0.2, 0.3]))


def test_oracle_textures_and_sky_match_reference(oracle_mod):
    """Textured triangles (UVs partly outside [0, 1]) and an equirectangular sky image: the
    restated texel and sky lookups (HitRecord.cuh:38-49, Camera.cuh:50-63) equal the reference's
    own code bit for bit (tests/golden/render_textured.npz)."""
    G = golden("render_textured.npz")
    r = oracle_mod.OracleScene(scenes.by_name("textured")).render(abi.render_params(spp=int(G["spp"]), seed=0))
    assert np.array_equal(r["rgb"], G["rgb"])
    assert np.array_equal(r["rgba8"], G["rgba8"])
    if oracle_mod.ref_lib() is not None:
        rr = oracle_mod.RefScene(scenes.by_name("textured")).render(int(G["spp"]), seed=0)
        assert np.array_equal(rr["rgb"], G["rgb"])
