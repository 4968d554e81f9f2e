"""Image and ray-count parity against the FP64 oracle at the configurations bench.py times.

* 1080p spheres workload (200 displaced level-5 icospheres, 4,096,014 primitives, config
  estimator: depth <= 16, Russian roulette from depth 3 with survival 0.8), a band of 16 full
  rows at 4 spp with the bench's first timed seed; both integrators and both traversal layouts
  (BVH2 and the 8-wide BVH).  The band is rendered through cpt_render's row range, which the
  oracle accepts too, so the frame's own pixels, streams and draw order are compared.
* The small configuration exactly as stated: 512x512 Cornell box with Lambertian albedos,
  16 spp, maximum depth 8 (no Russian roulette), PCG32 seed 0, config estimator.

Tolerance (FP32 kernels against the FP64 oracle on the same PCG32 streams): a pixel matches
when every channel is within 2e-3 * max(1, ref); at least 99% of pixels must match, image
means within 0.5%, every pixel finite; ray counts (closest-hit and shadow queries) within 1%."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import check_rgba8
from cudapathtracing_gb300 import abi, api, procedural as P

pytestmark = pytest.mark.gpu

PIX_TOL = 2e-3
MATCH_FRAC = 0.99
MEAN_TOL = 5e-3
RAY_TOL = 0.01

BAND = (520, 536)   # rows (row 0 at the bottom) through spheres, ground and the volume box
SPHERES_PRM = dict(spp=4, estimator=abi.ESTIMATOR_CONFIG, max_depth=16, rr_depth=3, rr_prob=0.8, seed=3)
CORNELL_PRM = dict(spp=16, estimator=abi.ESTIMATOR_CONFIG, max_depth=8, rr_depth=8, rr_prob=1.0, seed=0)


def compare(gpu_rgb, ref_rgb):
    g = gpu_rgb.astype(np.float64)
    r = ref_rgb
    assert np.isfinite(g).all(), "non-finite pixels"
    ok = (np.abs(g - r) <= PIX_TOL * np.maximum(1.0, np.abs(r))).all(-1)
    frac = ok.mean()
    mrel = abs(g.mean() - r.mean()) / max(r.mean(), 1e-9)
    print(f"match {frac:.5f}  mean rel {mrel:.2e}  max abs {np.abs(g - r).max():.3e}")
    assert frac >= MATCH_FRAC, frac
    assert mrel <= MEAN_TOL, mrel


@pytest.fixture(scope="module")
def spheres(ctx, oracle_mod):
    d = P.spheres_scene()
    o = oracle_mod.OracleScene(d)
    prm = abi.render_params(row_begin=BAND[0], row_end=BAND[1], **SPHERES_PRM)
    ref = o.render(prm)
    scenes = {}
    yield d, ref, scenes
    for s in scenes.values():
        s.close()


@pytest.mark.parametrize("width", [2, 8, "2q"])
@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT],
                         ids=["megakernel", "wavefront"])
def test_spheres_1080p_band_vs_oracle(ctx, spheres, integrator, width):
    """Traversal layouts: BVH2 (64-byte nodes), the 8-wide BVH, and BVH2 with 32-byte quantised
    nodes ("2q")."""
    d, ref, scenes = spheres
    if width not in scenes:
        ctx.set_bvh_width(2 if width == "2q" else width)
        ctx.set_bvh_compression(width == "2q")
        try:
            scenes[width] = api.Scene(ctx, d).init()
        finally:
            ctx.set_bvh_width(2)
            ctx.set_bvh_compression(False)
    s = scenes[width]
    assert s.num_prims == d.num_prims == 4096016   # 4,096,014 triangles + 2 lights
    r = s.render(integrator=integrator, rows=BAND, **SPHERES_PRM)
    band = slice(BAND[0], BAND[1])
    compare(r["rgb"][band], ref["rgb"][band])
    assert abs(r["rays"] - ref["rays"]) <= RAY_TOL * ref["rays"], (r["rays"], ref["rays"])
    # rows outside the band are not written
    assert not r["rgb"][:BAND[0]].any() and not r["rgb"][BAND[1]:].any()


@pytest.fixture(scope="module")
def cornell(oracle_mod):
    d = P.cornell_box(width=512, lambertian=True, seed=0)
    return d, oracle_mod.OracleScene(d).render(abi.render_params(**CORNELL_PRM))


@pytest.mark.parametrize("integrator", [abi.INTEGRATOR_MEGAKERNEL, abi.INTEGRATOR_WAVEFRONT],
                         ids=["megakernel", "wavefront"])
def test_cornell_512_as_stated_vs_oracle(ctx, cornell, integrator):
    d, o = cornell
    s = api.Scene(ctx, d).init()
    r = s.render(integrator=integrator, **CORNELL_PRM)
    compare(r["rgb"], o["rgb"])
    assert abs(r["rays"] - o["rays"]) <= RAY_TOL * o["rays"], (r["rays"], o["rays"])
    check_rgba8(r["rgba8"], o["rgba8"], r["rgb"], o["rgb"])
    s.close()
