"""Training data, training loop and evaluation for the kernel-predicting denoiser.

Data: seeded random scenes (procedural.random_scene), each rendered by the library at 1, 4, 16, 64,
128, 256 and 512 spp (the inputs, with their G-buffers, whose channel 7 is the renderer's own
variance of the pixel mean) and at 4096 spp with another seed (the target).
Training: Adam on random batches of crops through cpt_denoiser_train_step.  Evaluation: RMSE in
display space (sqrt, clamped to [0, 1], per channel over all pixels, as pic2RGBW shows images,
Render.cu:462-481) against a high-spp render of a held-out scene, for the plain render, the
reference's bilateral filter and the denoiser, and the wall time each needs to reach a target RMSE.

    python -m cudapathtracing_gb300.training --scenes 2000 --steps 40000 --batch 16 --out weights.npz
"""
from __future__ import annotations

import argparse
import math
import os
import time

import numpy as np

from . import abi, api, procedural as P
from .denoiser import Denoiser

RENDER = dict(estimator=abi.ESTIMATOR_CONFIG, max_depth=16, rr_depth=3, rr_prob=0.8)
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "kpcn.npz")
TRAIN_SEED0 = 1000        # training scenes: seeds TRAIN_SEED0 ...
EVAL_SEED0 = 900000       # held-out scenes


def render(ctx, scene, spp: int, seed: int, integrator=abi.INTEGRATOR_WAVEFRONT, gbuf: bool = True):
    """(rgb [H, W, 3], gbuf [H, W, 8] or None, device ms) as device tensors."""
    import torch
    H, W = scene.height, scene.width
    rgb = torch.zeros((H, W, 3), device="cuda")
    gb = torch.zeros((H, W, 8), device="cuda") if gbuf else None
    r = scene.render(spp=spp, seed=seed, integrator=integrator, rgb=rgb, gbuffer=gb, **RENDER)
    return rgb, gb, r["ms"]


def make_dataset(ctx, n_scenes: int, size: int = 256, spp_in=(1, 4, 16, 64, 128, 256, 512), spp_ref: int = 4096,
                 seed0: int = TRAIN_SEED0, log=print):
    """Stacked device tensors noisy [M, S, S, 3], gbuf [M, S, S, 8], target [M, S, S, 3] with
    M = n_scenes * len(spp_in) (one target per scene, shared by its inputs)."""
    import torch
    noisy, gbufs, targets = [], [], []
    t0 = time.time()
    for i in range(n_scenes):
        desc = P.random_scene(seed0 + i, width=size)
        sc = api.Scene(ctx, desc).init()
        tgt, _, _ = render(ctx, sc, spp_ref, seed=7919 + i, gbuf=False)
        for k, spp in enumerate(spp_in):
            rgb, gb, _ = render(ctx, sc, spp, seed=104729 * (k + 1) + i)
            noisy.append(rgb)
            gbufs.append(gb)
            targets.append(tgt)
        sc.close()
        if log and (i + 1) % 64 == 0:
            log(f"  dataset: {i + 1}/{n_scenes} scenes, {time.time() - t0:.1f} s")
    return torch.stack(noisy), torch.stack(gbufs), torch.stack(targets)


def display(x):
    """pic2RGBW's transform (Render.cu:462-481) before quantisation: sqrt, clamped to [0, 1]."""
    return x.clamp(min=0.0).sqrt().clamp(max=1.0)


def rmse(a, b) -> float:
    return float(((display(a) - display(b)) ** 2).mean().sqrt())


def train(net: Denoiser, data, steps: int, batch: int = 8, lr: float = 1e-3, lr_min: float = 1e-5, seed: int = 0,
          log=print, log_every: int = 250):
    """Adam with a cosine learning-rate schedule on random batches; returns the loss history."""
    import torch
    noisy, gbuf, target = data
    M = noisy.shape[0]
    rng = np.random.default_rng(seed)
    hist = []
    t0 = time.time()
    for s in range(steps):
        idx = torch.from_numpy(rng.integers(0, M, size=batch)).cuda()
        cur = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * s / max(1, steps)))
        loss = net.train_step(noisy[idx].contiguous(), gbuf[idx].contiguous(), target[idx].contiguous(), lr=cur)
        hist.append(loss)
        if log and (s + 1) % log_every == 0:
            log(f"  step {s + 1}/{steps}  loss {np.mean(hist[-log_every:]):.5f}  lr {cur:.2e}  "
                f"{time.time() - t0:.1f} s")
    return hist


# spp ladder of the wall-time-to-RMSE comparison: geometric, ratio 2^(1/4) (about 1.19), so the
# spp at which a method first reaches the target is resolved to within 19 %.
LADDER = tuple(sorted({max(1, int(round(2 ** (k / 4)))) for k in range(0, 45)}))


def evaluate(ctx, net: Denoiser, desc, ref_spp: int = 16384, plain_spps=LADDER,
             denoise_spps=tuple(x for x in LADDER if x <= 512), target_rmse: float = 0.01, seed: int = 17):
    """RMSE and wall time of plain, bilateral-filtered and denoised renders against a high-spp
    reference (another seed), and the time each needs to reach target_rmse (None if it does not):
    the smallest spp of the geometric ladder at which it does.  The ladder stops once both the
    plain and the denoised render have reached the target.  Times are device milliseconds of the
    render (and of the filter / denoiser) at that spp."""
    import torch
    sc = api.Scene(ctx, desc).init()
    ref, _, ref_ms = render(ctx, sc, ref_spp, seed=seed + 1, gbuf=False)
    rows = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plain_done = den_done = False
    for spp in sorted(set(plain_spps) | set(denoise_spps)):
        if plain_done and (den_done or spp > max(denoise_spps)):
            break
        rgb, gb, ms = render(ctx, sc, spp, seed=seed)
        row = {"spp": spp, "render_ms": ms, "plain": rmse(rgb, ref)}
        ev0.record()
        bil = api.filter_bilateral(ctx, rgb, gb)
        ev1.record()
        torch.cuda.synchronize()
        row["bilateral"], row["bilateral_ms"] = rmse(bil, ref), ev0.elapsed_time(ev1)
        if spp in denoise_spps:
            net.denoise(rgb, gb)   # warm (allocation for this size)
            torch.cuda.synchronize()
            ev0.record()
            den = net.denoise(rgb, gb)
            ev1.record()
            torch.cuda.synchronize()
            row["denoised"], row["denoise_ms"] = rmse(den[0], ref), ev0.elapsed_time(ev1)
            den_done = den_done or row["denoised"] <= target_rmse
        plain_done = plain_done or row["plain"] <= target_rmse
        rows.append(row)
    sc.close()

    def first(key, extra):
        for r in rows:
            if key in r and r[key] <= target_rmse:
                return r["spp"], r["render_ms"] + (r[extra] if extra else 0.0)
        return None, None

    ps, pt = first("plain", None)
    ds, dt = first("denoised", "denoise_ms")
    return {"rows": rows, "ref_spp": ref_spp, "ref_ms": ref_ms, "target_rmse": target_rmse,
            "plain_spp": ps, "plain_ms": pt, "denoised_spp": ds, "denoised_ms": dt,
            "speedup": (pt / dt) if (pt and dt) else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=2000)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--spp-ref", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=40000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--eval-size", type=int, default=512)
    ap.add_argument("--eval-scenes", type=int, default=8)
    ap.add_argument("--eval-ref-spp", type=int, default=16384)
    ap.add_argument("--eval-only", action="store_true", help="evaluate the weights in --out, no training")
    args = ap.parse_args()
    import torch
    ctx = api.Context()
    net = Denoiser(seed=args.seed)
    if args.eval_only:
        net.load(args.out)
    else:
        t0 = time.time()
        data = make_dataset(ctx, args.scenes, args.size, spp_ref=args.spp_ref)
        torch.cuda.synchronize()
        print(f"dataset {tuple(data[0].shape)} in {time.time() - t0:.1f} s", flush=True)
        t1 = time.time()
        hist = train(net, data, args.steps, args.batch, args.lr, seed=args.seed)
        torch.cuda.synchronize()
        print(f"trained {args.steps} steps in {time.time() - t1:.1f} s; final loss {np.mean(hist[-100:]):.5f}",
              flush=True)
        del data
        os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
        net.save(args.out)
    for k in range(args.eval_scenes):
        res = evaluate(ctx, net, P.random_scene(EVAL_SEED0 + k, width=args.eval_size), ref_spp=args.eval_ref_spp)
        print(f"held-out scene {k}: plain reaches {res['target_rmse']} at {res['plain_spp']} spp "
              f"({res['plain_ms']} ms), denoised at {res['denoised_spp']} spp ({res['denoised_ms']} ms), "
              f"speedup {res['speedup']}", flush=True)
        for r in res["rows"]:
            print("   ", {k2: (round(v, 4) if isinstance(v, float) else v) for k2, v in r.items()}, flush=True)


if __name__ == "__main__":
    main()
