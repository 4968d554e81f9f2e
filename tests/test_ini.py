"""The native INI parser (through the C ABI, no GPU) against the reference's IniParser."""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from conftest import SCENES, golden
from cudapathtracing_gb300 import _lib, abi, api

import oracle as _oracle

_REF_DIR = _oracle.reference_dir()
REF_INI = os.path.join(_REF_DIR, "scene_ini") if _REF_DIR else ""


def _unflatten(v):
    """ref_ini_dump layout -> dict (see oracle/ref_harness.cpp)."""
    v = list(v)
    out = {}
    out["camera"] = v[:12]
    i = 12
    for sec, width in (("lights", 12), ("spheres", 10), ("floors", 18), ("meshes", 11)):
        n = int(v[i]); i += 1
        out[sec] = [v[i + k * width:i + (k + 1) * width] for k in range(n)]
        i += n * width
    out["cloth"] = v[i]
    return out


def _ref_type(t):
    return abi.M_OPAQUE if t == abi.M_LAMBERTIAN else t


def compare_with_dump(path, dump):
    p = api.IniParser()
    p.Parse(path)
    d = p.to_scene_desc()
    ref = _unflatten(dump)
    cam = ref["camera"]
    assert np.allclose(d.camera.background, cam[0:3], rtol=0, atol=0)
    assert d.camera.width == int(cam[3]) and d.camera.aspect_ratio == cam[4]
    assert tuple(d.camera.look_from) == tuple(cam[5:8]) and tuple(d.camera.look_at) == tuple(cam[8:11])
    assert d.camera.vfov_deg == cam[11]
    assert len(d.lights) == len(ref["lights"])
    for L, R in zip(d.lights, ref["lights"]):
        assert tuple(L["center"]) == tuple(R[0:3]) and L["width"] == R[3] and L["height"] == R[4]
        assert tuple(L["normal"]) == tuple(R[5:8]) and tuple(L["color"]) == tuple(R[8:11])
        assert L["visible"] == int(R[11])
    assert len(d.spheres) == len(ref["spheres"])
    for S, R in zip(d.spheres, ref["spheres"]):
        m = d.materials[S["material"]]
        assert tuple(S["center"]) == tuple(R[0:3]) and S["radius"] == R[3]
        assert tuple(m["color"]) == tuple(R[4:7]) and (m["alpha_x"], m["alpha_y"]) == (R[7], R[8])
        assert _ref_type(m["type"]) == int(R[9])
    # floors become triangles (lt, lb, rt), (rt, lb, rb) after the spheres' triangles (none)
    nf = len(ref["floors"])
    tri = d.tri_vertices if d.tri_vertices is not None else np.zeros((0, 9))
    assert tri.shape[0] >= 2 * nf
    for k, R in enumerate(ref["floors"]):
        lt, rt, lb, rb = R[0:3], R[3:6], R[6:9], R[9:12]
        assert np.array_equal(tri[2 * k], np.array(lt + lb + rt))
        assert np.array_equal(tri[2 * k + 1], np.array(rt + lb + rb))
        m = d.materials[d.tri_material[2 * k]]
        assert tuple(m["color"]) == tuple(R[12:15]) and (m["alpha_x"], m["alpha_y"]) == (R[15], R[16])
        assert _ref_type(m["type"]) == int(R[17])
    return d


@pytest.mark.parametrize("name", ["volume_glass", "glossy", "parser_edge"])
def test_ini_matches_reference_parser(cptlib, name):
    compare_with_dump(os.path.join(SCENES, name + ".ini"), golden(f"ini_{name}.npy"))


def test_ini_edge_cases(cptlib):
    d = compare_with_dump(os.path.join(SCENES, "parser_edge.ini"), golden("ini_parser_edge.npy"))
    # "type=Volume\r" (CRLF) does not match and falls back to Opaque, as in the reference
    assert d.materials[d.spheres[0]["material"]]["type"] == abi.M_OPAQUE
    # extension keys are read; the missing mesh leaves an empty mesh but a material
    fm = d.materials[d.tri_material[0]]
    assert fm["type"] == abi.M_LAMBERTIAN and fm["eta"] == 1.4 and fm["sigma_t"] == 2.0 and fm["albedo"] == 0.5
    assert d.camera.width == 40 and d.camera.height == 20


def test_ini_bad_number_is_a_parse_error(cptlib, tmp_path):
    p = tmp_path / "bad.ini"
    p.write_text("[Sphere]\nradius=abc\n")
    with pytest.raises(_lib.CptError) as e:
        api.IniParser().Parse(str(p))
    assert e.value.status == 6
    with pytest.raises(_lib.CptError) as e:
        api.IniParser().Parse(str(tmp_path / "missing.ini"))
    assert e.value.status == 9


def test_ini_obj_mesh_bounds_and_transform(cptlib, tmp_path):
    obj = tmp_path / "quad.obj"
    obj.write_text("v -1 0 -1\nv 1 0 -1\nv 1 0 1\nv -1 0 1\nf 1 2 3 4\n")
    ini = tmp_path / "m.ini"
    ini.write_text(f"[Camera]\nwidth=16\n[Mesh]\npath={obj}\ncenter=(0,5,0)\nscale=2\nrotation=90\n")
    p = api.IniParser()
    p.Parse(str(ini))
    d = p.to_scene_desc()
    assert d.tri_vertices.shape == (2, 9)
    # bounds are taken after rotate+scale and before the translation (ObjLoader.cuh:107-112)
    assert np.allclose(d.bounds_min, (-2, 0, -2)) and np.allclose(d.bounds_max, (2, 0, 2))
    assert np.allclose(d.tri_vertices[:, 1::3], 5.0)


@pytest.mark.skipif(not os.path.isdir(REF_INI), reason="reference scene files not mounted")
def test_reference_scene_files_parse_identically(oracle_mod, cptlib):
    if oracle_mod.ref_lib() is None:
        pytest.skip("oracle/_ref not built")
    for path in sorted(glob.glob(os.path.join(REF_INI, "*.ini"))):
        compare_with_dump(path, oracle_mod.ref_ini_dump(path))


def _ppm(path, rgb):
    h, w, _ = rgb.shape
    path.write_bytes(f"P6\n# test image\n{w} {h}\n255\n".encode() + rgb.astype(np.uint8).tobytes())


def test_ini_obj_texcoords_normals_textures_and_sky(cptlib, tmp_path):
    """vt per corner ((0, 0) without one), vn only with usingNV=1 (the reference's loader flag,
    which its Scene::init leaves off), texture= and skyBox= images (binary PPM), and the
    fallbacks of an unreadable image: untextured mesh, background sky."""
    obj = tmp_path / "quad.obj"
    obj.write_text("v -1 0 -1\nv 1 0 -1\nv 1 0 1\nv -1 0 1\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0.25 0.75\n"
                   "vn 0 1 0\nvn 0.6 0.8 0\nf 1/1/1 2/2/2 3/3/1 4/4/2\nf 1//1 3//2 4//1\n")
    tex = np.arange(4 * 6 * 3, dtype=np.uint8).reshape(4, 6, 3)
    sky = (np.arange(2 * 8 * 3, dtype=np.uint8) * 3).reshape(2, 8, 3)
    _ppm(tmp_path / "t.ppm", tex)
    _ppm(tmp_path / "sky.ppm", sky)
    ini = tmp_path / "m.ini"
    ini.write_text(f"[Camera]\nwidth=16\nskyBox={tmp_path / 'sky.ppm'}\n"
                   f"[Floor]\nlt=(-1,0,1)\nrt=(1,0,1)\nlb=(-1,0,-1)\nrb=(1,0,-1)\n"
                   f"[Mesh]\npath={obj}\ntexture={tmp_path / 't.ppm'}\nusingNV=1\n"
                   f"[Mesh]\npath={obj}\ntexture={tmp_path / 'missing.ppm'}\n")
    p = api.IniParser()
    p.Parse(str(ini))
    d = p.to_scene_desc()
    assert d.tri_vertices.shape == (2 + 3 + 3, 9)
    uv = d.tri_uvs.reshape(-1, 3, 2)
    assert np.array_equal(uv[:2], np.zeros((2, 3, 2)))                      # floor: no texcoords
    assert np.allclose(uv[2], [[0, 0], [1, 0], [1, 1]])                       # fan (1, 2, 3)
    assert np.allclose(uv[3], [[0, 0], [1, 1], [0.25, 0.75]])                 # fan (1, 3, 4)
    assert np.allclose(uv[4], 0.0)                                            # f 1//1 ...: no vt
    n = d.tri_normals.reshape(-1, 3, 3)
    assert np.allclose(n[2], [[0, 1, 0], [0.6, 0.8, 0], [0, 1, 0]])          # usingNV=1
    assert np.allclose(n[4], [[0, 1, 0], [0.6, 0.8, 0], [0, 1, 0]])
    assert np.array_equal(n[5:], np.zeros((3, 3, 3)))                         # second mesh: flat
    assert len(d.textures) == 1 and np.array_equal(d.textures[0], tex)
    m1, m2 = d.materials[d.tri_material[2]], d.materials[d.tri_material[5]]
    assert m1["texture"] == 1 and m2["texture"] == 0                          # unreadable image: colour
    assert np.array_equal(d.sky, sky)
