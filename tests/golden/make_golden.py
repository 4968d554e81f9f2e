"""Generates the golden fixtures in tests/golden/ from the reference's OWN code.

The reference's path (BVH.cuh, Hittable.cuh, Material.cuh, Camera.*, Render.cu,
IniParser.cpp) is compiled as host C++ by oracle/Makefile into oracle/_ref/libcpt_ref.so
(only possible where the reference is mounted).  This script runs it on small seeded
inputs and stores its outputs; the tests then check the restated oracle and the CUDA
library against these vectors on any machine.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

from cudapathtracing_gb300 import abi, procedural as P  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
SCENES = os.path.join(HERE, "scenes")


def degenerate_scene(n: int = 64) -> abi.SceneDesc:
    """n triangles sharing one centroid cell: keys differ only in the index word."""
    d = abi.SceneDesc()
    d.add_material((0.5, 0.5, 0.5))
    g = P.PCG32Streams(7, np.arange(n, dtype=np.uint64))
    tri = np.zeros((n, 9))
    for k in range(9):
        tri[:, k] = 0.25 + 1e-4 * g.uniform()
    d.tri_vertices = tri.astype(np.float32)
    d.tri_material = np.zeros(n, np.uint32)
    d.camera = abi.Camera(16, 1.0, (0, 0, 3), (0, 0, 0), 40.0, (0, 0, 0))
    return d


def mixed_scene(seed: int = 11) -> abi.SceneDesc:
    """Random triangles, spheres and lights (all three primitive kinds in one tree)."""
    d = abi.SceneDesc()
    for m in range(3):
        d.add_material((0.3 + 0.2 * m, 0.6, 0.8 - 0.2 * m), 0.2 + 0.2 * m, 0.3, abi.M_OPAQUE)
    g = P.PCG32Streams(seed, np.arange(300, dtype=np.uint64))
    c = np.stack([g.uniform() * 6 - 3 for _ in range(3)], 1)
    e = np.stack([g.uniform() * 0.6 - 0.3 for _ in range(6)], 1)
    tri = np.concatenate([c, c + e[:, :3], c + e[:, 3:]], 1)
    d.tri_vertices = tri.astype(np.float32)
    d.tri_material = (np.arange(300) % 3).astype(np.uint32)
    for k in range(4):
        d.spheres.append(dict(center=(k - 1.5, 0.5 * k, -1.0), radius=0.3 + 0.1 * k, material=k % 3))
    d.lights.append(dict(center=(0.0, 4.0, 0.0), normal=(0.0, -1.0, 0.2), width=1.5, height=0.7,
                         color=(8.0, 8.0, 8.0), visible=1))
    d.lights.append(dict(center=(2.0, 1.0, 3.0), normal=(-1.0, 0.0, -1.0), width=0.5, height=0.5,
                         color=(4.0, 2.0, 1.0), visible=1))
    pts = tri.reshape(-1, 3)
    d.bounds_min = tuple(pts.min(0))
    d.bounds_max = tuple(pts.max(0))
    d.camera = abi.Camera(32, 1.0, (0.0, 1.0, 9.0), (0.0, 0.0, 0.0), 50.0, (0.2, 0.2, 0.25))
    return d


# Material edits of the pick fixtures (changeMaterial, Render.cu:498-522): (first, end, alphaX,
# alphaY, glass).  A first of None means "the primitive picked at the image centre".
PICK_EDITS = [(0, 10, 0.3, 0.1, True), (None, 40, 0.05, 0.6, False)]


def pick_edits(center_pick: int):
    out = []
    for first, n, ax, ay, glass in PICK_EDITS:
        f = center_pick if first is None else first
        out.append((f, f + n if first is None else n, ax, ay, glass))
    return out


def pick_fixture(name: str, desc: abi.SceneDesc, spp: int = 4) -> None:
    """getObject at every pixel, then the edits above and a STATIC render of the edited scene."""
    ref = O.RefScene(desc)
    W, H = ref.width, ref.height
    picks = np.array([[ref.pick(x, y) for x in range(W)] for y in range(H)], np.int32)
    edits = pick_edits(int(picks[H // 2, W // 2]))
    for e in edits:
        ref.set_material(*e)
    r = ref.render(spp, seed=0)
    np.savez_compressed(os.path.join(HERE, f"pick_{name}.npz"), picks=picks, edits=np.array(edits, np.float64),
                        rgb=r["rgb"], rgba8=r["rgba8"], spp=spp)


def textured_scene(width: int = 48) -> abi.SceneDesc:
    """Two textured quads (UVs partly outside [0, 1], so the texel indices clamp), one untextured
    triangle, spheres of three materials, one light, and an equirectangular sky image."""
    d = abi.SceneDesc()
    g = P.PCG32Streams(5, np.arange(4096, dtype=np.uint64))

    def image(h, w):
        a = np.zeros((h, w, 3), np.uint8)
        for c in range(3):
            a[..., c] = (g.next()[: h * w].reshape(h, w) >> np.uint32(24)).astype(np.uint8)
        return a

    t_floor = d.add_texture(image(24, 32))
    t_wall = d.add_texture(image(40, 16))
    m_floor = d.add_material((0.7, 0.7, 0.7), 0.4, 0.4, abi.M_OPAQUE, texture=t_floor)
    m_wall = d.add_material((0.5, 0.5, 0.5), 0.2, 0.6, abi.M_OPAQUE, texture=t_wall)
    m_plain = d.add_material((0.8, 0.3, 0.2), 0.3, 0.3, abi.M_OPAQUE)
    m_glass = d.add_material((1.0, 1.0, 1.0), 0.1, 0.1, abi.M_SPECULAR_DIELECTRIC)
    tris = [((-3, -1, 3), (3, -1, 3), (-3, -1, -3)), ((3, -1, 3), (3, -1, -3), (-3, -1, -3)),     # floor
            ((-3, -1, -3), (3, -1, -3), (-3, 2, -3)), ((3, -1, -3), (3, 2, -3), (-3, 2, -3)),     # wall
            ((1.5, -1, 1.0), (2.5, -1, 0.5), (2.0, 0.5, 0.8))]                                    # plain
    uvs = [((0, 0), (1, 0), (0, 1)), ((1, 0), (1, 1), (0, 1)),
           ((-0.2, 0), (1.3, 0), (-0.2, 1.1)), ((1.3, 0), (1.3, 1.1), (-0.2, 1.1)),
           ((0, 0), (0, 0), (0, 0))]
    d.tri_vertices = np.array([sum(map(list, t), []) for t in tris], np.float32)
    d.tri_uvs = np.array([sum(map(list, u), []) for u in uvs], np.float32)
    d.tri_material = np.array([m_floor, m_floor, m_wall, m_wall, m_plain], np.uint32)
    d.spheres = [dict(center=(-1.0, -0.4, 0.5), radius=0.6, material=m_glass),
                 dict(center=(0.6, -0.5, -0.8), radius=0.5, material=m_plain),
                 dict(center=(-1.8, 0.3, -1.6), radius=0.4, material=m_floor)]
    d.lights.append(dict(center=(0.0, 2.5, 0.5), normal=(0.0, -1.0, 0.0), width=1.5, height=1.0,
                         color=(6.0, 6.0, 6.0), visible=1))
    d.sky = image(16, 32)
    pts = d.tri_vertices.reshape(-1, 3).astype(np.float64)
    d.bounds_min, d.bounds_max = tuple(pts.min(0)), tuple(pts.max(0))
    d.camera = abi.Camera(width, 1.0, (0.5, 1.2, 6.0), (0.0, 0.0, 0.0), 60.0, (0.1, 0.1, 0.1))
    return d


def lbvh_fixture(name: str, ref: O.RefScene) -> None:
    L = ref.lbvh()
    np.savez_compressed(os.path.join(HERE, f"lbvh_{name}.npz"), **{k: L[k] for k in
                                                                   ("keys", "order", "child_a", "child_b",
                                                                    "node_boxes", "leaf_boxes")})


def main() -> None:
    if O.ref_lib() is None:
        O.build(ref=True)
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref is not built: the reference is not mounted here")

    # LBVH keys, order, topology and FP64 boxes
    cornell = P.cornell_box(width=48)
    lbvh_fixture("cornell", O.RefScene(cornell))
    lbvh_fixture("degenerate", O.RefScene(degenerate_scene()))
    mixed = mixed_scene()
    lbvh_fixture("mixed", O.RefScene(mixed))
    ico = P.icosphere_scene(level=3)
    ref_ico = O.RefScene(ico)
    lbvh_fixture("ico3", ref_ico)
    for ini in ("volume_glass", "glossy"):
        lbvh_fixture(ini, O.RefScene(ini_path=os.path.join(SCENES, ini + ".ini")))

    # closest hits (traverseIterative)
    rays = P.uniform_rays(4096, seed=1)
    ids, t = ref_ico.trace(P.rays_as_f64(rays))
    np.savez_compressed(os.path.join(HERE, "hits_ico3.npz"), ids=ids, t=t)
    rays_m = P.uniform_rays(4096, seed=3, box=3.0)
    ids, t = O.RefScene(mixed).trace(P.rays_as_f64(rays_m))
    np.savez_compressed(os.path.join(HERE, "hits_mixed.npz"), ids=ids, t=t)

    # renders (STATIC mode, PCG32 seed 0)
    for name, ref, spp in (("cornell", O.RefScene(cornell), 4), ("mixed", O.RefScene(mixed), 4),
                           ("volume_glass", O.RefScene(ini_path=os.path.join(SCENES, "volume_glass.ini")), 4),
                           ("glossy", O.RefScene(ini_path=os.path.join(SCENES, "glossy.ini")), 4)):
        r = ref.render(spp, seed=0)
        np.savez_compressed(os.path.join(HERE, f"render_{name}.npz"), rgb=r["rgb"], rgba8=r["rgba8"], spp=spp)

    # textures and the sky image (HitRecord::sampleTexture, Camera::getSkyBox)
    r = O.RefScene(textured_scene()).render(8, seed=0)
    np.savez_compressed(os.path.join(HERE, "render_textured.npz"), rgb=r["rgb"], rgba8=r["rgba8"], spp=8)

    # picking and material edits (getObject / changeMaterial)
    pick_fixture("cornell", cornell)
    pick_fixture("mixed", mixed)

    # the reference's INI parser, flattened
    for ini in ("volume_glass", "glossy", "parser_edge"):
        np.save(os.path.join(HERE, f"ini_{ini}.npy"), O.ref_ini_dump(os.path.join(SCENES, ini + ".ini")))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
