"""The FP32 megakernel against the FP64 reference (golden, reference estimator) and the
FP64 oracle (config estimator) on the same seeds.

Tolerance (FP32 vs FP64, same PCG32 streams and draw order): a pixel matches when every
channel satisfies |gpu - ref| <= 2e-3 * max(1, ref).  Paths are identical up to rounding
except where a rounding difference flips a discrete event (an edge hit, a total internal
reflection test, a Russian-roulette draw right at its threshold), so a small fraction of
pixels may differ: at least 99% must match and the image means must agree within 0.5%."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import SCENES, check_rgba8, golden
from cudapathtracing_gb300 import abi, api, procedural as P
import scenes

pytestmark = pytest.mark.gpu

PIX_TOL = 2e-3
MATCH_FRAC = 0.99
MEAN_TOL = 5e-3


def compare(gpu_rgb, ref_rgb, match_frac=MATCH_FRAC, mean_tol=MEAN_TOL):
    g = gpu_rgb.astype(np.float64)
    r = ref_rgb
    ok = (np.abs(g - r) <= PIX_TOL * np.maximum(1.0, np.abs(r))).all(-1)
    frac = ok.mean()
    assert np.isfinite(g).all(), "non-finite pixels"
    mrel = abs(g.mean() - r.mean()) / max(r.mean(), 1e-9)
    print(f"match {frac:.5f}  mean rel {mrel:.2e}  max abs {np.abs(g - r).max():.3e}")
    assert frac >= match_frac, frac
    assert mrel <= mean_tol, mrel


def make_scene(ctx, name):
    if name in ("volume_glass", "glossy"):
        return api.Scene(ctx, ini_path=os.path.join(SCENES, name + ".ini")).init()
    return api.Scene(ctx, scenes.by_name(name)).init()


@pytest.mark.parametrize("name", ["cornell", "mixed", "volume_glass", "glossy"])
def test_reference_estimator_matches_reference_golden(ctx, name):
    G = golden(f"render_{name}.npz")
    s = make_scene(ctx, name)
    r = s.render(spp=int(G["spp"]), seed=0)
    compare(r["rgb"], G["rgb"])
    check_rgba8(r["rgba8"], G["rgba8"], r["rgb"], G["rgb"])
    assert r["rays"] > 0


def test_reference_estimator_cornell_512_vs_oracle(ctx, oracle_mod):
    """The small config at full size: 512x512 Cornell box, 16 spp."""
    d = P.cornell_box(width=512)
    s = api.Scene(ctx, d).init()
    r = s.render(spp=16, seed=0)
    o = oracle_mod.OracleScene(d).render(abi.render_params(spp=16, seed=0))
    compare(r["rgb"], o["rgb"])
    # the kernels count every closest-hit query the oracle traces (up to diverged paths)
    assert abs(r["rays"] - o["rays"]) / o["rays"] < 0.01


def config_scene(name):
    if name == "spheres":
        return P.spheres_scene(num_spheres=12, level=3, width=96)
    if name == "cornell":
        return P.cornell_box(width=96)
    return scenes.ini_desc(name)


def config_params(name, spp=8):
    return dict(spp=spp, estimator=abi.ESTIMATOR_CONFIG, max_depth=8 if name == "cornell" else 16,
                rr_depth=3, rr_prob=0.8, seed=5)


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT])
@pytest.mark.parametrize("name", ["cornell", "volume_glass", "glossy", "spheres"])
def test_config_estimator_vs_oracle(ctx, oracle_mod, name, integrator):
    d = config_scene(name)
    s = api.Scene(ctx, d).init()
    prm = config_params(name)
    r = s.render(integrator=integrator, **prm)
    o = oracle_mod.OracleScene(d).render(abi.render_params(**prm))
    compare(r["rgb"], o["rgb"])
    assert abs(r["rays"] - o["rays"]) / o["rays"] < 0.01


@pytest.mark.parametrize("width", [2, 8, "2q"])
@pytest.mark.parametrize("slots,graph", [(1 << 20, 1), (1024, 1), (1536, 0)])
@pytest.mark.parametrize("name", ["cornell", "volume_glass", "spheres"])
def test_wavefront_matches_megakernel(ctx, name, slots, graph, width):
    """Same estimator, same PCG32 streams and draw order: the two integrators trace the same
    paths.  With fewer slots than pixels the slots take new pixels as they finish.  "2q": BVH2 with
    32-byte quantised nodes."""
    d = config_scene(name)
    ctx.set_bvh_width(2 if width == "2q" else width)
    ctx.set_bvh_compression(width == "2q")
    try:
        s = api.Scene(ctx, d).init()
    finally:
        ctx.set_bvh_width(2)
        ctx.set_bvh_compression(False)
    prm = config_params(name, spp=6)
    mk = s.render(integrator=abi.INTEGRATOR_MEGAKERNEL, **prm)
    ctx.set_wavefront(slots, 128, 128, graph)
    try:
        wf = s.render(integrator=abi.INTEGRATOR_WAVEFRONT, **prm)
    finally:
        ctx.set_wavefront(1 << 21, 128, 128, 1)
    exact = (wf["rgb"] == mk["rgb"]).all(-1).mean()
    print(f"wavefront == megakernel on {exact:.5f} of pixels; rays {wf['rays']} vs {mk['rays']}")
    compare(wf["rgb"], mk["rgb"].astype(np.float64), match_frac=0.999, mean_tol=1e-3)
    assert abs(wf["rays"] - mk["rays"]) <= 1e-3 * mk["rays"]


def test_wavefront_tuning_limits(ctx):
    """Block sizes above the kernels' launch bounds are refused before any launch."""
    for bt, bs in [(512, 128), (128, 512), (96, 48)]:
        with pytest.raises(Exception):
            ctx.set_wavefront(1 << 20, bt, bs, 1)
    with pytest.raises(Exception):
        ctx.set_render_block(32, 32)
    ctx.set_wavefront(1 << 21, 256, 256, 1)
    d = P.cornell_box(width=32)
    s = api.Scene(ctx, d).init()
    try:
        r = s.render(integrator=abi.INTEGRATOR_WAVEFRONT, **config_params("cornell", spp=2))
    finally:
        ctx.set_wavefront(1 << 21, 128, 128, 1)
    assert r["rays"] > 0


def test_wavefront_gbuffer_and_rows(ctx):
    import torch
    d = P.cornell_box(width=40)
    s = api.Scene(ctx, d).init()
    prm = dict(spp=3, estimator=abi.ESTIMATOR_CONFIG, max_depth=6, rr_depth=2, rr_prob=0.75, seed=9)
    gm = torch.zeros((40, 40, 8), device="cuda")
    gw = torch.zeros((40, 40, 8), device="cuda")
    rm = torch.zeros((40, 40, 3), device="cuda")
    rw = torch.zeros((40, 40, 3), device="cuda")
    s.render(integrator=abi.INTEGRATOR_MEGAKERNEL, rgb=rm, gbuffer=gm, **prm)
    s.render(integrator=abi.INTEGRATOR_WAVEFRONT, rgb=rw, gbuffer=gw, rows=(0, 17), **prm)
    s.render(integrator=abi.INTEGRATOR_WAVEFRONT, rgb=rw, gbuffer=gw, rows=(17, 40), **prm)
    torch.cuda.synchronize()
    assert torch.allclose(gm, gw, atol=1e-5)
    assert torch.allclose(rm, rw, rtol=2e-3, atol=2e-3)
    with pytest.raises(Exception):
        s.render(integrator=abi.INTEGRATOR_WAVEFRONT, spp=1, estimator=abi.ESTIMATOR_REFERENCE)


def test_accumulate_and_row_ranges(ctx):
    d = P.cornell_box(width=64)
    s = api.Scene(ctx, d).init()
    full = s.render(spp=2, seed=3)["rgb"]
    part = np.zeros_like(full)
    s.render(spp=2, seed=3, rows=(0, 20), rgb=part)
    s.render(spp=2, seed=3, rows=(20, 64), rgb=part)
    assert np.array_equal(part, full)
    acc = full.copy()
    s.render(spp=2, seed=3, rgb=acc, flags=abi.RENDER_ACCUMULATE)
    assert np.allclose(acc, 2 * full)


def test_gbuffer_and_device_outputs(ctx):
    import torch
    d = P.cornell_box(width=32)
    s = api.Scene(ctx, d).init()
    host = s.render(spp=1, seed=1, estimator=abi.ESTIMATOR_CONFIG, max_depth=4, rr_depth=8, rr_prob=1.0)
    rgb = torch.zeros((32, 32, 3), device="cuda")
    gb = torch.zeros((32, 32, 8), device="cuda")
    s.render(spp=1, seed=1, estimator=abi.ESTIMATOR_CONFIG, max_depth=4, rr_depth=8, rr_prob=1.0, rgb=rgb, gbuffer=gb)
    torch.cuda.synchronize()
    assert np.array_equal(rgb.cpu().numpy(), host["rgb"])
    n = gb[..., :3].cpu().numpy()
    hitmask = gb[..., 3].cpu().numpy() < 999999.0
    assert hitmask.mean() > 0.9
    assert np.allclose(np.linalg.norm(n[hitmask], axis=-1), 1.0, atol=1e-4)


def test_autotuner_cache_reproducible(ctx, tmp_path):
    """Tuning picks a configuration no slower than the defaults on its probe (margin rule), stores
    it, and a second tuner with the same cache and probe applies the same choice without timing
    (a choice timed at another probe spp is a different cache entry)."""
    from cudapathtracing_gb300 import autotune
    d = P.cornell_box(width=48)
    s = api.Scene(ctx, d).init()
    prm = config_params("cornell", spp=2)
    path = str(tmp_path / "tune.json")
    try:
        t1 = autotune.Autotuner(ctx, cache_path=path, probe_spp=2, repeats=1)
        ch = t1.tune(s, prm, abi.INTEGRATOR_WAVEFRONT)
        assert ch.trials and ch.trials[0]["config"]["slots"] == autotune.DEFAULTS["slots"]
        assert ch.score >= ch.default_score
        ch2 = autotune.Autotuner(ctx, cache_path=path, probe_spp=2).tune(s, prm, abi.INTEGRATOR_WAVEFRONT)
        assert ch2.knobs == ch.knobs and ch2.score == ch.score   # from the cache, not re-timed
        r = s.render(integrator=abi.INTEGRATOR_WAVEFRONT, **prm)
        assert r["rays"] > 0
    finally:
        autotune.Autotuner(ctx, cache_path=path).apply(autotune.DEFAULTS, s)


@pytest.mark.parametrize("name", ["cornell", "mixed"])
def test_pick_and_material_edit_vs_reference_golden(ctx, oracle_mod, name):
    """cpt_pick at every pixel against the reference's getObject (Render.cu:485-496): equal except
    documented near ties and edge grazes (classified as for closest-hit queries), and equal to a
    closest-hit query along the same pixel-centre ray.  Then the fixture's changeMaterial edits
    (Render.cu:498-522) through cpt_scene_set_material and a render of the edited scene against
    the reference's render of its own edited scene (reference estimator, image tolerance above)."""
    import filters
    from test_gpu_trace import classify
    G = golden(f"pick_{name}.npz")
    d = scenes.by_name(name)
    s = api.Scene(ctx, d).init()
    H, W = G["picks"].shape
    assert (s.height, s.width) == (H, W)
    picks = np.array([[s.pick(x, y) for x in range(W)] for y in range(H)], np.int32)
    cam = d.camera
    dirs = filters.camera_rays(cam.width, cam.aspect_ratio, cam.look_from, cam.look_at, cam.vfov_deg)
    rays = np.zeros(H * W, abi.RAY_DTYPE)
    rays["origin"] = cam.look_from
    rays["direction"] = dirs.reshape(-1, 3)
    rays["tmin"], rays["tmax"] = 0.001, 999999.0
    hits = s.trace(rays)
    assert np.array_equal(picks.reshape(-1), hits["prim"])
    o = oracle_mod.OracleScene(d)
    ids, t, _, _ = o.trace(P.rays_as_f64(rays))
    nbad, unexplained = classify(o, rays, hits, G["picks"].reshape(-1), t)
    print(f"{name}: {nbad} of {H * W} picks differ, all explained" if not unexplained else unexplained)
    assert not unexplained, (nbad, unexplained[:10])
    assert nbad <= 0.01 * H * W   # shared edges of the axis-aligned quads under pixel centres
    assert s.pick(-1, 0) == -1 and s.pick(0, 10 ** 6) == -1
    for first, end, ax, ay, glass in G["edits"]:
        s.set_material(int(first), int(end), ax, ay, bool(glass))
    r = s.render(spp=int(G["spp"]), seed=0)
    compare(r["rgb"], G["rgb"])
    check_rgba8(r["rgba8"], G["rgba8"], r["rgb"], G["rgb"])


def test_material_edit_keeps_colours_and_other_primitives(ctx, oracle_mod):
    """An edit over primitives of different materials keeps each one's colour; primitives
    outside the range keep their material (the config estimator's view of both)."""
    d = P.cornell_box(width=32)
    s = api.Scene(ctx, d).init()
    prm = dict(spp=2, estimator=abi.ESTIMATOR_CONFIG, max_depth=4, rr_depth=4, rr_prob=1.0, seed=2)
    o = oracle_mod.OracleScene(d)
    # walls 0-4 (two triangles each) have five different albedos; edit floor..back (3 materials)
    first, end = len(d.lights), len(d.lights) + 6
    s.set_material(first, end, 0.2, 0.2, False)
    o.set_material(first, end, 0.2, 0.2, False)
    r = s.render(**prm)
    ref = o.render(abi.render_params(**prm))
    compare(r["rgb"], ref["rgb"])


def test_row_bands_of_ranks_reassemble_the_frame(ctx):
    """The multi-GPU row partition (shard.render_band), run rank by rank on one GPU: the bands
    together are the single-rank frame (pixels are independent)."""
    import torch
    from cudapathtracing_gb300 import shard
    d = P.cornell_box(width=48)
    s = api.Scene(ctx, d).init()
    prm = dict(spp=2, seed=4, estimator=abi.ESTIMATOR_CONFIG, max_depth=8, rr_depth=3, rr_prob=0.8,
               integrator=abi.INTEGRATOR_WAVEFRONT)
    full = torch.zeros((s.height, s.width, 3), device="cuda")
    s.render(rgb=full, **prm)
    world = 3
    rgb = torch.zeros_like(full)
    bands = [shard.render_band(s, r, world, rgb, **prm)[0] for r in range(world)]
    torch.cuda.synchronize()
    assert torch.equal(torch.cat(bands, 0), full)


def test_device_loop_limits_report_timeout(ctx):
    """The bounds that replace the reference's unbounded bounce loop and its exit(99)
    (Render.cu:58, Device.cuh:9-19) trip on purpose: a per-sample trip limit of 1 stops every path
    at its second loop trip, and a single wavefront replay (8 iterations) cannot drain depth-16
    paths with no Russian roulette.  Each render returns CPT_ERR_TIMEOUT through the C ABI, the
    error word is cleared, and the same context and scene render normally afterwards."""
    from cudapathtracing_gb300._lib import CptError
    d = P.cornell_box(width=32)
    s = api.Scene(ctx, d).init()
    cfg = dict(spp=2, estimator=abi.ESTIMATOR_CONFIG, max_depth=16, rr_depth=16, rr_prob=1.0, seed=3)
    try:
        ctx.set_loop_limits(1, 1 << 20)
        for kw in (dict(spp=2, seed=0), dict(integrator=abi.INTEGRATOR_MEGAKERNEL, **cfg),
                   dict(integrator=abi.INTEGRATOR_WAVEFRONT, **cfg)):
            with pytest.raises(CptError) as e:
                s.render(**kw)
            assert e.value.status == 4, e.value
        ctx.set_loop_limits(1 << 16, 1)
        with pytest.raises(CptError) as e:
            s.render(integrator=abi.INTEGRATOR_WAVEFRONT, **cfg)
        assert e.value.status == 4 and "drain" in str(e.value)
        with pytest.raises(CptError):
            ctx.set_loop_limits(0, 1)
    finally:
        ctx.set_loop_limits()
    for integ in (abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT):
        r = s.render(integrator=integ, **cfg)
        assert r["rays"] > 0 and np.isfinite(r["rgb"]).all()


def test_textures_and_sky_match_reference_golden(ctx):
    """Textured triangles and the equirectangular sky (HitRecord::sampleTexture, HitRecord.cuh:38-49;
    Camera::getSkyBox, Camera.cuh:50-63) against the reference's own render of the same scene."""
    G = golden("render_textured.npz")
    s = api.Scene(ctx, scenes.by_name("textured")).init()
    r = s.render(spp=int(G["spp"]), seed=0)
    compare(r["rgb"], G["rgb"])
    check_rgba8(r["rgba8"], G["rgba8"], r["rgb"], G["rgb"])


@pytest.mark.parametrize("width", [2, 8])
@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT],
                         ids=["megakernel", "wavefront"])
def test_textures_and_sky_config_estimator_vs_oracle(ctx, oracle_mod, integrator, width):
    d = scenes.by_name("textured")
    ctx.set_bvh_width(width)
    try:
        s = api.Scene(ctx, d).init()
    finally:
        ctx.set_bvh_width(2)
    prm = dict(spp=8, estimator=abi.ESTIMATOR_CONFIG, max_depth=8, rr_depth=3, rr_prob=0.8, seed=4)
    r = s.render(integrator=integrator, **prm)
    o = oracle_mod.OracleScene(d).render(abi.render_params(**prm))
    compare(r["rgb"], o["rgb"])
    assert abs(r["rays"] - o["rays"]) / o["rays"] < 0.01


def test_texture_arguments_are_checked(ctx):
    from cudapathtracing_gb300._lib import CptError
    d = scenes.by_name("textured")
    d.materials[0]["texture"] = len(d.textures) + 1
    with pytest.raises(CptError):
        api.Scene(ctx, d)


def test_ini_textured_mesh_and_sky_vs_oracle(ctx, oracle_mod, tmp_path):
    """An INI scene through cpt_scene_load_ini: an OBJ mesh with texture coordinates, a PPM
    texture and a PPM sky box, rendered on the GPU and by the oracle from the parsed scene."""
    rng = np.random.default_rng(3)
    tex = rng.integers(0, 256, size=(12, 20, 3), dtype=np.uint8)
    sky = rng.integers(0, 256, size=(8, 16, 3), dtype=np.uint8)
    for name, img in (("t.ppm", tex), ("sky.ppm", sky)):
        h, w, _ = img.shape
        (tmp_path / name).write_bytes(f"P6\n{w} {h}\n255\n".encode() + img.tobytes())
    (tmp_path / "quad.obj").write_text("v -2 0 -2\nv 2 0 -2\nv 2 0 2\nv -2 0 2\nvt -0.1 0\nvt 1.2 0\nvt 1 1\n"
                                       "vt 0 1.1\nf 1/1 2/2 3/3 4/4\n")
    ini = tmp_path / "scene.ini"
    ini.write_text(f"[Camera]\nwidth=40\naspectRatio=1.0\nlookFrom=(0, 3, 5)\nlookAt=(0, 0, 0)\nvFov=60\n"
                   f"skyBox={tmp_path / 'sky.ppm'}\n"
                   f"[Light]\ncenter=(0, 4, 0)\nwidth=2\nheight=2\nnormal=(0, -1, 0)\ncolor=(2550, 2550, 2550)\n"
                   f"[Sphere]\ncenter=(0, 0.8, 0)\nradius=0.8\ncolor=(200, 120, 80)\n"
                   f"[Mesh]\npath={tmp_path / 'quad.obj'}\ntexture={tmp_path / 't.ppm'}\ncenter=(0, -0.2, 0)\n")
    s = api.Scene(ctx, ini_path=str(ini)).init()
    p = api.IniParser()
    p.Parse(str(ini))
    d = p.to_scene_desc()
    assert len(d.textures) == 1 and d.sky is not None and d.tri_uvs is not None
    o = oracle_mod.OracleScene(d)
    for prm in (dict(spp=4, seed=1), dict(spp=4, estimator=abi.ESTIMATOR_CONFIG, max_depth=6, rr_depth=3,
                                          rr_prob=0.8, seed=2)):
        r = s.render(**prm)
        ref = o.render(abi.render_params(**prm))
        compare(r["rgb"], ref["rgb"])


@pytest.mark.parametrize("width", [2, 8])
@pytest.mark.parametrize("name", ["volume_glass", "glossy", "spheres", "textured"])
def test_wavefront_material_sort_gives_the_same_image(ctx, name, width):
    """Shading the paths binned by material changes only the order in which slots are shaded;
    every path draws from its own sample stream and group sums are added in group order, so the
    image, the G-buffer and the ray count are identical to the unsorted wavefront's."""
    import torch
    d = scenes.by_name(name) if name == "textured" else config_scene(name)
    ctx.set_bvh_width(width)
    try:
        s = api.Scene(ctx, d).init()
    finally:
        ctx.set_bvh_width(2)
    prm = config_params(name, spp=6)
    out = {}
    for sort in (False, True):
        ctx.set_material_sort(sort)
        try:
            rgb = torch.zeros((s.height, s.width, 3), device="cuda")
            gb = torch.zeros((s.height, s.width, 8), device="cuda")
            r = s.render(integrator=abi.INTEGRATOR_WAVEFRONT, rgb=rgb, gbuffer=gb, **prm)
            out[sort] = (rgb.cpu().numpy(), gb.cpu().numpy(), r["rays"])
        finally:
            ctx.set_material_sort(False)
    assert np.array_equal(out[False][0], out[True][0])
    assert np.array_equal(out[False][1], out[True][1])
    assert out[False][2] == out[True][2]


@pytest.mark.parametrize("width", [2, 8])
@pytest.mark.parametrize("slots,sort", [(1 << 21, 0), (1024, 0), (1536, 1)])
def test_render_batch_equals_single_renders(ctx, width, slots, sort):
    """cpt_render_batch runs several jobs (four scenes, image sizes, spp, depths, seeds, a row band)
    in one wavefront.  Paths of all jobs share the slots, but each pixel draws its own streams, so
    every job's image, display bytes and G-buffer are bit for bit those of its own wavefront
    render, and the batch traces the sum of their rays.  With fewer slots than items, slots move
    between jobs as they finish."""
    import torch
    ctx.set_bvh_width(width)
    try:
        scs = [api.Scene(ctx, d).init() for d in (config_scene("cornell"), scenes.by_name("textured"),
                                                   config_scene("spheres"), config_scene("volume_glass"))]
    finally:
        ctx.set_bvh_width(2)
    prms = [dict(spp=6, max_depth=8, rr_depth=3, rr_prob=0.8, seed=5),
            dict(spp=3, max_depth=5, rr_depth=2, rr_prob=0.7, seed=1),
            dict(spp=9, max_depth=16, rr_depth=3, rr_prob=0.8, seed=11, rows=(10, 50)),
            dict(spp=17, max_depth=12, rr_depth=4, rr_prob=0.9, seed=2)]

    def outs(sc):
        return (torch.zeros((sc.height, sc.width, 3), device="cuda"),
                torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda"),
                torch.zeros((sc.height, sc.width, 8), device="cuda"))
    ctx.set_wavefront(slots, 128, 128, 1)
    ctx.set_material_sort(bool(sort))
    try:
        single, rays = [], 0
        for sc, p in zip(scs, prms):
            o = outs(sc)
            r = sc.render(integrator=abi.INTEGRATOR_WAVEFRONT, estimator=abi.ESTIMATOR_CONFIG, rgb=o[0], rgba8=o[1],
                          gbuffer=o[2], **p)
            single.append(o)
            rays += r["rays"]
        bo = [outs(sc) for sc in scs]
        jobs = [dict(scene=sc, rgb=o[0], rgba8=o[1], gbuffer=o[2], **p) for sc, o, p in zip(scs, bo, prms)]
        b = api.render_batch(ctx, jobs)
    finally:
        ctx.set_wavefront(1 << 21, 128, 128, 1)
        ctx.set_material_sort(False)
    torch.cuda.synchronize()
    for k, (a, o) in enumerate(zip(single, bo)):
        for x, y in zip(a, o):
            assert torch.equal(x, y), k
    assert b["rays"] == rays
    # host outputs through the same call
    h = api.render_batch(ctx, [dict(scene=scs[0], **prms[0])])
    assert np.array_equal(h["jobs"][0]["rgb"], single[0][0].cpu().numpy())


def test_render_batch_arguments(ctx):
    from cudapathtracing_gb300._lib import CptError
    a = api.Scene(ctx, config_scene("cornell")).init()
    ctx.set_bvh_width(8)
    try:
        b = api.Scene(ctx, config_scene("cornell")).init()
    finally:
        ctx.set_bvh_width(2)
    with pytest.raises(CptError):   # different traversal layouts
        api.render_batch(ctx, [dict(scene=a, spp=1), dict(scene=b, spp=1)])
    with pytest.raises(CptError):   # bad row range
        api.render_batch(ctx, [dict(scene=a, spp=1, rows=(5, 10 ** 6))])
    assert api.render_batch(ctx, [])["rays"] == 0


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT],
                         ids=["megakernel", "wavefront"])
@pytest.mark.parametrize("spp", [1, 6, 24])
def test_gbuffer_sample_variance_vs_oracle(ctx, oracle_mod, integrator, spp):
    """G-buffer channel 7 (config estimator): the variance of the pixel mean's luminance from the
    renderer's own samples, against the FP64 oracle on the pixels whose samples follow the same paths
    (every channel of the mean within eps = 1e-4 * max(1, ref)).

    Tolerance: var = (sum Y_i^2 - (sum Y_i)^2 / n) / (n (n - 1)).  Moving one sample's luminance by
    delta moves var by 2 (Y_i - mean) delta / (n (n - 1)); with |delta| <= n eps (the mean's bound) and
    |Y_i - mean| <= sqrt(n (n - 1) var), the change is at most 2 eps sqrt(n var / (n - 1)) (n = 1:
    var = Y^2, change 2 eps sqrt(var)).  On top: 1e-3 relative and the FP32 cancellation in
    sum(Y^2) - (sum Y)^2 / n, bounded by 1e-6 * mean^2.  At one sample the G-buffer must also equal the
    squared luminance of the renderer's own pixel on every pixel (FP32 rounding only)."""
    import torch
    d = config_scene("volume_glass")
    s = api.Scene(ctx, d).init()
    prm = dict(spp=spp, estimator=abi.ESTIMATOR_CONFIG, max_depth=12, rr_depth=3, rr_prob=0.8, seed=6)
    rgb = torch.zeros((s.height, s.width, 3), device="cuda")
    gb = torch.zeros((s.height, s.width, 8), device="cuda")
    s.render(integrator=integrator, rgb=rgb, gbuffer=gb, **prm)
    torch.cuda.synchronize()
    o = oracle_mod.OracleScene(d).render(abi.render_params(**prm), gbuffer=True)
    g = gb.cpu().numpy()[..., 7].astype(np.float64)
    r = rgb.cpu().numpy().astype(np.float64)
    ov = o["gbuffer"][..., 7]
    eps = 1e-4 * np.maximum(1.0, o["rgb"]).max(-1)
    same = (np.abs(r - o["rgb"]) <= eps[..., None]).all(-1)
    lum = 0.2126 * o["rgb"][..., 0] + 0.7152 * o["rgb"][..., 1] + 0.0722 * o["rgb"][..., 2]
    path_tol = 2.0 * eps * np.sqrt(ov * spp / max(spp - 1, 1))
    ok = np.abs(g - ov) <= 1e-3 * ov + path_tol + 1e-6 * lum * lum + 1e-12
    assert same.mean() > 0.9
    if spp == 1:
        y = 0.2126 * r[..., 0] + 0.7152 * r[..., 1] + 0.0722 * r[..., 2]
        assert np.allclose(g, y * y, rtol=1e-5, atol=1e-12)
    assert ok[same].all(), (np.abs(g - ov)[same & ~ok][:5], ov[same & ~ok][:5])
    assert (g >= 0).all() and np.isfinite(g).all()
    assert (ov > 0).mean() > 0.5
