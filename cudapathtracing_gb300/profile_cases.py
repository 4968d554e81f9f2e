"""Small, self-contained invocations of each kernel family, sized for per-kernel ncu captures
(a few hundred MB on the device, a handful of launches of the kernel of interest).

    python -m cudapathtracing_gb300.profile_cases render  [--integrator wavefront|megakernel] [--layout bvh2|bvh2q|bvh8]
    python -m cudapathtracing_gb300.profile_cases trace   [--layout ...] [--rays N]
    python -m cudapathtracing_gb300.profile_cases build   [--layout ...]
    python -m cudapathtracing_gb300.profile_cases filter

render   the 1080p spheres scene (200 displaced level-5 icospheres, 4,096,014 triangles, config
         estimator: depth <= 16, Russian roulette from depth 3 with survival 0.8) at --spp samples,
         --frames frames (seeds 0, 1, ...), into a device image
trace    closest-hit queries of --rays uniformly distributed random rays (bench's microbench rays)
         against the displaced level-8 icosphere (1,310,720 triangles), twice
build    two LBVH builds of the level-8 icosphere (prep, radix sort, emission, refit, layout)
filter   a 2-spp wavefront render of a 20-sphere scene with its G-buffer, then one joint-bilateral
         and one temporal filter pass

The denoiser's kernels have their own driver: python -m cudapathtracing_gb300.denoiser."""
from __future__ import annotations

import argparse

import numpy as np

from . import abi, api, procedural as P

LAYOUTS = {"bvh2": (2, False), "bvh2q": (2, True), "bvh8": (8, False)}


def _context(layout: str) -> api.Context:
    ctx = api.Context(0)
    width, comp = LAYOUTS[layout]
    ctx.set_bvh_width(width)
    ctx.set_bvh_compression(comp)
    return ctx


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(prog="python -m cudapathtracing_gb300.profile_cases")
    ap.add_argument("case", choices=["render", "trace", "build", "filter"])
    ap.add_argument("--layout", default="bvh2", choices=sorted(LAYOUTS))
    ap.add_argument("--integrator", default="wavefront", choices=["wavefront", "megakernel"])
    ap.add_argument("--spp", type=int, default=1)
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--rays", type=int, default=2_000_000)
    a = ap.parse_args(argv)
    import torch
    ctx = _context(a.layout)
    if a.case == "render":
        s = api.Scene(ctx, P.spheres_scene()).init()
        rgb = torch.zeros((s.height, s.width, 3), device="cuda")
        integ = abi.INTEGRATOR_MEGAKERNEL if a.integrator == "megakernel" else abi.INTEGRATOR_WAVEFRONT
        for i in range(a.frames):
            r = s.render(spp=a.spp, seed=i, estimator=abi.ESTIMATOR_CONFIG, integrator=integ, max_depth=16,
                         rr_depth=3, rr_prob=0.8, rgb=rgb)
        print(f"render {a.integrator} {a.layout}: {a.frames} frames, {r['rays']} rays in the last")
    elif a.case == "trace":
        s = api.Scene(ctx, P.icosphere_scene(level=8)).init()
        n = a.rays
        rays = torch.from_numpy(P.uniform_rays(n, seed=1).view(np.float32).reshape(n, 8)).cuda()
        hits = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        for _ in range(2):
            s.trace(rays, hits)
        print(f"trace {a.layout}: {n} rays, {int((hits[:, 1].view(torch.int32) >= 0).sum())} hits")
    elif a.case == "build":
        s = api.Scene(ctx, P.icosphere_scene(level=8))
        for _ in range(2):
            st = s.buildBVH()
        print(f"build {a.layout}: {st.ms_total:.3f} ms")
    else:
        d = P.spheres_scene(num_spheres=20, level=4)
        s = api.Scene(ctx, d).init()
        rgb = torch.zeros((s.height, s.width, 3), device="cuda")
        gb = torch.zeros((s.height, s.width, 8), device="cuda")
        s.render(spp=2, seed=0, estimator=abi.ESTIMATOR_CONFIG, integrator=abi.INTEGRATOR_WAVEFRONT, max_depth=8,
                 rr_depth=3, rr_prob=0.8, rgb=rgb, gbuffer=gb)
        out = api.filter_bilateral(ctx, rgb, gb)
        api.filter_temporal(ctx, out, rgb, gb, d.camera, d.camera, 0.1)
        print("filter: done")
    torch.cuda.synchronize()


if __name__ == "__main__":
    main()
