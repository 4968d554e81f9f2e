"""The reference-named C++ wrappers (include/cpt.hpp) driving the GPU from a C++ program, the way
the reference's main.cu drives its Scene and render kernel (main.cu:13-80):

* an INI scene loaded with cpt::Scene(ctx, path) and rendered with cpt::render (STATIC mode,
  reference estimator) against the reference's own render of that file (tests/golden);
* a scene assembled with cpt::SceneBuilder (addOneLight / addOneSphere / addFloor, cpt::Material,
  cpt::Hittable, cpt::Camera) against the FP64 oracle of the same scene built in Python, and the
  camera's getSampleRay against cpt_pick.

Image tolerance as in test_gpu_render.py."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, SCENES, check_rgba8, golden
from cudapathtracing_gb300 import abi, api
from test_gpu_render import compare

pytestmark = pytest.mark.gpu

PROGRAM = r'''
#include "cpt.hpp"
#include <cstdio>
#include <cstring>
#include <vector>

static void save(const char* path, const std::vector<float>& rgb, const std::vector<uint8_t>& rgba, long rays)
{
    FILE* f = std::fopen(path, "wb");
    std::fwrite(&rays, sizeof rays, 1, f);
    std::fwrite(rgb.data(), sizeof(float), rgb.size(), f);
    std::fwrite(rgba.data(), 1, rgba.size(), f);
    std::fclose(f);
}

int main(int argc, char** argv)
{
    try {
        cpt::Context ctx(0);
        if (!std::strcmp(argv[1], "ini")) {             // Scene::init(IniParser) + render<<<>>>
            cpt::Scene scene(ctx, argv[2]);
            cpt_camera cam;
            uint32_t nl, ns, nt;
            cpt::check(cpt_scene_info(scene.get(), &nl, &ns, &nt, &cam), "cpt_scene_info");
            std::vector<float> rgb(3 * (size_t)cam.width * cam.height);
            std::vector<uint8_t> rgba(4 * (size_t)cam.width * cam.height);
            cpt_render_stats st = cpt::render(scene, rgb.data(), rgba.data(), std::atoi(argv[3]), 0);
            save(argv[4], rgb, rgba, (long)st.rays);
            return 0;
        }
        // a scene assembled object by object (Scene::addOneLight / addOneSphere / addFloor)
        cpt::Camera cam(40, 1.0, {0.05, 0.05, 0.1}, {0.0, 1.0, 6.0}, {0.0, 0.0, 0.0}, 55.0);
        cpt::SceneBuilder b(cam);
        b.addOneSphere({-0.8, 0.0, 0.0}, 0.7, cpt::Material({0.8, 0.4, 0.2}, 0.3, 0.3, cpt::M_OPAQUE));
        b.add(cpt::Hittable::Sphere({0.9, -0.2, 0.5}, 0.5, cpt::Material({1.0, 1.0, 1.0}, 0.1, 0.1,
                                                                         cpt::M_SPECULAR_DIELECTRIC)));
        b.addFloor({-3, -1, 3}, {3, -1, 3}, {-3, -1, -3}, {3, -1, -3}, cpt::Material({0.6, 0.6, 0.6}, 0.5, 0.5,
                                                                                     cpt::M_LAMBERTIAN));
        b.add(cpt::Hittable::Triangle({-2, -1, -2}, {2, -1, -2}, {0, 2, -2}, cpt::Material({0.2, 0.7, 0.3}, 0.4,
                                                                                          0.2, cpt::M_OPAQUE)));
        b.addOneLight({0.0, 3.0, 0.0}, 2.0, 1.5, {0.0, -1.0, 0.0}, {8.0, 8.0, 8.0});   // added last, placed first
        cpt::Scene scene(ctx, b.desc());
        cpt_render_params p{};
        p.spp = 8;
        p.estimator = CPT_ESTIMATOR_CONFIG;
        p.integrator = std::atoi(argv[2]);
        p.max_depth = 8;
        p.rr_depth = 3;
        p.rr_prob = 0.8f;
        p.seed = 7;
        std::vector<float> rgb(3 * (size_t)cam.width * cam.height);
        std::vector<uint8_t> rgba(4 * (size_t)cam.width * cam.height);
        cpt_render_stats st = cpt::render(scene, p, rgb.data(), rgba.data());
        save(argv[3], rgb, rgba, (long)st.rays);
        // getSampleRay through the wrappers against cpt_pick (both: the pixel-centre ray)
        for (int y = 0; y < cam.height; y += 3)
            for (int x = 0; x < cam.width; x += 3) {
                cpt_ray r = cam.getSampleRay(x, y);
                cpt_hit h;
                scene.trace(&r, 1, &h, false);
                if (h.prim != scene.pick(x, y)) { std::printf("pick mismatch %d %d\n", x, y); return 3; }
            }
        return 0;
    } catch (const cpt::Error& e) {
        std::printf("error %d: %s\n", (int)e.status, e.what());
        return 2;
    }
}
'''


@pytest.fixture(scope="module")
def program(tmp_path_factory, cptlib):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    d = tmp_path_factory.mktemp("cpp")
    src = d / "main.cpp"
    src.write_text(PROGRAM)
    lib = os.path.join(ROOT, "cudapathtracing_gb300", "_build")
    exe = d / "main"
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), str(src),
                        "-L" + lib, "-lcpt", "-Wl,-rpath," + lib, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe, d


def _load(path, h, w):
    raw = open(path, "rb").read()
    rays = int(np.frombuffer(raw[:8], np.int64)[0])
    rgb = np.frombuffer(raw[8:8 + 12 * h * w], np.float32).reshape(h, w, 3)
    rgba = np.frombuffer(raw[8 + 12 * h * w:], np.uint8).reshape(h, w, 4)
    return rgb, rgba, rays


def test_cpp_program_renders_ini_like_the_reference(program):
    exe, d = program
    G = golden("render_glossy.npz")
    out = d / "glossy.bin"
    r = subprocess.run([str(exe), "ini", os.path.join(SCENES, "glossy.ini"), str(int(G["spp"])), str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    H, W, _ = G["rgb"].shape
    rgb, rgba, rays = _load(out, H, W)
    assert rays > 0
    compare(rgb, G["rgb"])
    check_rgba8(rgba, G["rgba8"], rgb, G["rgb"])


def _builder_desc():
    """The C++ program's SceneBuilder scene, in the C ABI's order (light, spheres, triangles)."""
    d = abi.SceneDesc()
    d.lights.append(dict(center=(0.0, 3.0, 0.0), normal=(0.0, -1.0, 0.0), width=2.0, height=1.5,
                         color=(8.0, 8.0, 8.0), visible=1))
    m0 = d.add_material((0.8, 0.4, 0.2), 0.3, 0.3, abi.M_OPAQUE)
    m1 = d.add_material((1.0, 1.0, 1.0), 0.1, 0.1, abi.M_SPECULAR_DIELECTRIC)
    m2 = d.add_material((0.6, 0.6, 0.6), 0.5, 0.5, abi.M_LAMBERTIAN)
    m3 = d.add_material((0.2, 0.7, 0.3), 0.4, 0.2, abi.M_OPAQUE)
    d.spheres = [dict(center=(-0.8, 0.0, 0.0), radius=0.7, material=m0),
                 dict(center=(0.9, -0.2, 0.5), radius=0.5, material=m1)]
    lt, rt, lb, rb = (-3, -1, 3), (3, -1, 3), (-3, -1, -3), (3, -1, -3)
    tris = [lt + lb + rt, rt + lb + rb, (-2, -1, -2, 2, -1, -2, 0, 2, -2)]
    d.tri_vertices = np.array(tris, np.float64)
    d.tri_material = np.array([m2, m2, m3], np.uint32)
    d.camera = abi.Camera(40, 1.0, (0.0, 1.0, 6.0), (0.0, 0.0, 0.0), 55.0, (0.05, 0.05, 0.1))
    return d


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT],
                         ids=["megakernel", "wavefront"])
def test_cpp_scene_builder_vs_oracle(program, oracle_mod, integrator):
    exe, d = program
    out = d / f"builder{integrator}.bin"
    r = subprocess.run([str(exe), "builder", str(integrator), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    desc = _builder_desc()
    rgb, _, rays = _load(out, desc.camera.height, desc.camera.width)
    prm = dict(spp=8, estimator=abi.ESTIMATOR_CONFIG, max_depth=8, rr_depth=3, rr_prob=0.8, seed=7)
    o = oracle_mod.OracleScene(desc).render(abi.render_params(**prm))
    compare(rgb, o["rgb"])
    assert abs(rays - o["rays"]) <= 0.01 * o["rays"]
