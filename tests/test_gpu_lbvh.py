"""LBVH on the GPU against the reference (golden vectors) and the oracle: Morton keys, sort
order and topology bit-exact; FP32 boxes equal to the reference's FP64 boxes rounded outwards."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import SCENES, golden, outward_f32
from cudapathtracing_gb300 import abi, api, procedural as P
import scenes

pytestmark = pytest.mark.gpu

CASES = ["cornell", "degenerate", "mixed", "ico3", "volume_glass", "glossy"]


def make_scene(ctx, name):
    if name in ("volume_glass", "glossy"):
        return api.Scene(ctx, ini_path=os.path.join(SCENES, name + ".ini")).init()
    return api.Scene(ctx, scenes.by_name(name)).init()


def assert_lbvh_equal(L, G):
    for k in ("keys", "order", "child_a", "child_b"):
        assert np.array_equal(L[k], G[k]), k
    for k in ("node_boxes", "leaf_boxes"):
        lo, hi = outward_f32(G[k][:, :3], G[k][:, 3:])
        assert np.array_equal(L[k][:, :3], lo), k
        assert np.array_equal(L[k][:, 3:], hi), k


@pytest.mark.parametrize("name", CASES)
def test_lbvh_matches_reference_golden(ctx, name):
    s = make_scene(ctx, name)
    assert_lbvh_equal(s.export_lbvh(), golden(f"lbvh_{name}.npz"))


def test_lbvh_full_size_icosphere_vs_oracle(ctx, oracle_mod):
    """1,310,720-triangle displaced icosphere: bit-exact against the oracle at full size."""
    d = P.icosphere_scene(level=8)
    s = api.Scene(ctx, d).init()
    assert s.num_prims == 1310720
    assert_lbvh_equal(s.export_lbvh(), oracle_mod.OracleScene(d).lbvh())
    st = s.buildBVH()
    assert st.num_prims == 1310720 and st.ms_total > 0


def test_lbvh_spheres_scene_vs_oracle(ctx, oracle_mod):
    """The 1080p wavefront scene (200 level-5 spheres, 4,096,014 triangles + 2 lights)."""
    d = P.spheres_scene()
    s = api.Scene(ctx, d).init()
    L = s.export_lbvh()
    O = oracle_mod.OracleScene(d).lbvh()
    assert_lbvh_equal(L, O)
    # size-independent properties: order is a permutation, keys strictly increase
    assert np.array_equal(np.sort(L["order"]), np.arange(s.num_prims, dtype=np.uint32))
    assert (L["keys"][1:] > L["keys"][:-1]).all()


@pytest.mark.parametrize("n", [1, 2, 3, 5, 33, 4097, 4096 * 3 + 17])
def test_lbvh_small_and_ragged_sizes(ctx, oracle_mod, n):
    d = abi.SceneDesc()
    d.add_material((0.5, 0.5, 0.5))
    g = P.PCG32Streams(n, np.arange(n, dtype=np.uint64))
    c = np.stack([g.uniform() * 4 - 2 for _ in range(3)], 1)
    e = np.stack([g.uniform() * 0.2 for _ in range(6)], 1)
    d.tri_vertices = np.concatenate([c, c + e[:, :3], c + e[:, 3:]], 1).astype(np.float32)
    d.tri_material = np.zeros(n, np.uint32)
    d.bounds_min, d.bounds_max = (-2.0,) * 3, (2.2,) * 3
    d.camera = abi.Camera(8, 1.0, (0, 0, 5), (0, 0, 0), 40.0)
    s = api.Scene(ctx, d).init()
    assert_lbvh_equal(s.export_lbvh(), oracle_mod.OracleScene(d).lbvh())


def test_empty_scene_renders_background(ctx):
    d = abi.SceneDesc()
    d.add_material((1, 1, 1))
    d.camera = abi.Camera(16, 1.0, (0, 0, 5), (0, 0, 0), 40.0, (0.25, 0.5, 0.75))
    s = api.Scene(ctx, d).init()
    r = s.render(spp=2)
    assert np.allclose(r["rgb"], np.array([0.25, 0.5, 0.75], np.float32))
    hits = s.trace(P.uniform_rays(64))
    assert (hits["prim"] == -1).all()


def test_low_level_device_build_matches_scene_build(ctx):
    """cpt_lbvh_build_device on caller-owned torch buffers (Device::buildBVH's shape)."""
    import torch
    d = P.icosphere_scene(level=3)
    G = golden("lbvh_ico3.npz")
    n = d.num_triangles
    dev = torch.device("cuda:0")
    tri = torch.from_numpy(d.tri_vertices).to(dev)
    out = dict(keys=torch.zeros(n, dtype=torch.int64, device=dev), order=torch.zeros(n, dtype=torch.int32, device=dev),
               children=torch.zeros((n - 1, 2), dtype=torch.int32, device=dev),
               node_range=torch.zeros((n - 1, 2), dtype=torch.int32, device=dev),
               node_boxes=torch.zeros((n - 1, 8), dtype=torch.float32, device=dev),
               leaf_boxes=torch.zeros((n, 8), dtype=torch.float32, device=dev))
    scratch = torch.zeros(api.Device.scratch_bytes(n), dtype=torch.uint8, device=dev)
    api.Device.buildBVH(None, None, tri, d.bounds_min, d.bounds_max, out, scratch)
    torch.cuda.synchronize()
    assert np.array_equal(out["keys"].cpu().numpy().view(np.uint64), G["keys"])
    assert np.array_equal(out["order"].cpu().numpy().view(np.uint32), G["order"])
    ch = out["children"].cpu().numpy()
    assert np.array_equal(ch[:, 0], G["child_a"]) and np.array_equal(ch[:, 1], G["child_b"])
    lo, hi = outward_f32(G["node_boxes"][:, :3], G["node_boxes"][:, 3:])
    nb = out["node_boxes"].cpu().numpy()
    assert np.array_equal(nb[:, 0:3], lo) and np.array_equal(nb[:, 4:7], hi)
    # every internal node's range covers exactly its two children
    rg = out["node_range"].cpu().numpy()
    assert (rg[:, 0] <= rg[:, 1]).all() and rg[0, 0] == 0 and rg[0, 1] == n - 1


def _expected_refit(L):
    """Node boxes recomputed bottom-up from the exported leaf boxes over the same topology."""
    ni = L["child_a"].shape[0]
    box = np.zeros((ni, 6), np.float32)
    done = np.zeros(ni, bool)
    stack = [0]
    while stack:
        nd = stack[-1]
        kids = (L["child_a"][nd], L["child_b"][nd])
        pending = [k for k in kids if k >= 0 and not done[k]]
        if pending:
            stack.extend(pending)
            continue
        bs = [L["leaf_boxes"][~k] if k < 0 else box[k] for k in kids]
        box[nd, :3] = np.minimum(bs[0][:3], bs[1][:3])
        box[nd, 3:] = np.maximum(bs[0][3:], bs[1][3:])
        done[nd] = True
        stack.pop()
    return box


def test_update_refit_and_rebuild(ctx, oracle_mod):
    """Scene::Update: moved vertices, then (a) refit keeping the topology and (b) a full rebuild."""
    d = P.icosphere_scene(level=4)
    s = api.Scene(ctx, d).init()
    before = s.export_lbvh()
    moved = (d.tri_vertices.astype(np.float64) * 1.05 + 0.01).astype(np.float32)
    s.Update(moved, rebuild=False)
    L = s.export_lbvh()
    for k in ("keys", "order", "child_a", "child_b"):
        assert np.array_equal(L[k], before[k])
    assert np.array_equal(L["node_boxes"], _expected_refit(L))
    s.Update(moved, rebuild=True)
    d2 = P.icosphere_scene(level=4)
    d2.tri_vertices = moved
    assert_lbvh_equal(s.export_lbvh(), oracle_mod.OracleScene(d2).lbvh())
