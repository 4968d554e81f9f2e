"""Headless renderer: the reference's main.cu loop (main.cu:13-50, 78-80) without a window.

    python -m cudapathtracing_gb300.cli scene.ini --spp 64 --out img.ppm [--pfm img.pfm]
        [--estimator reference|config] [--integrator megakernel|wavefront] [--denoise | --bilateral]
"""
from __future__ import annotations

import argparse
import time

from . import abi, api, imageio


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("scene", help="INI scene file (IniParser format)")
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--estimator", choices=["reference", "config"], default="reference")
    ap.add_argument("--integrator", choices=["megakernel", "wavefront"], default=None,
                    help="default: wavefront for the config estimator, megakernel for the reference one")
    ap.add_argument("--max-depth", type=int, default=16)
    ap.add_argument("--rr-depth", type=int, default=3)
    ap.add_argument("--rr-prob", type=float, default=0.8)
    ap.add_argument("--denoise", action="store_true", help="apply the learned denoiser (trained weights)")
    ap.add_argument("--bilateral", action="store_true", help="apply the reference's joint-bilateral filter")
    ap.add_argument("--out", default="render.ppm")
    ap.add_argument("--pfm", default=None)
    a = ap.parse_args(argv)
    import torch
    est = abi.ESTIMATOR_CONFIG if a.estimator == "config" else abi.ESTIMATOR_REFERENCE
    integ = a.integrator or ("wavefront" if est == abi.ESTIMATOR_CONFIG else "megakernel")
    ctx = api.Context(0)
    t0 = time.perf_counter()
    scene = api.Scene(ctx, ini_path=a.scene).init()
    H, W = scene.height, scene.width
    rgb = torch.zeros((H, W, 3), device="cuda")
    gb = torch.zeros((H, W, 8), device="cuda")
    r = scene.render(spp=a.spp, seed=a.seed, estimator=est, max_depth=a.max_depth, rr_depth=a.rr_depth,
                     rr_prob=a.rr_prob, rgb=rgb, gbuffer=gb,
                     integrator=abi.INTEGRATOR_WAVEFRONT if integ == "wavefront" else abi.INTEGRATOR_MEGAKERNEL)
    if a.denoise:
        from . import training
        from .denoiser import Denoiser
        den = Denoiser()
        den.load(training.DEFAULT_WEIGHTS)
        rgb = den.denoise(rgb, gb)[0]
    elif a.bilateral:
        rgb = api.filter_bilateral(ctx, rgb, gb)
    img = rgb.cpu().numpy()
    imageio.write_ppm(a.out, img)
    if a.pfm:
        imageio.write_pfm(a.pfm, img)
    print(f"{W}x{H}, {a.spp} spp, {r['rays']} rays, render {r['ms']:.1f} ms, total {time.perf_counter() - t0:.2f} s "
          f"-> {a.out}")


if __name__ == "__main__":
    main()
