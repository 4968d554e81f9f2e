"""Autotuner for the render launch shapes, with a reproducible choice cache.

Knobs (all set through the C ABI on the context):
  megakernel   thread-block shape (block_x, block_y)
  wavefront    path slots (the wavefront size), trace / shade block sizes, traversal short-stack
               depth (entries kept in shared memory), material sort of the shade queue
  both         BVH layout width (2 or 8) and BVH2 node compression (64-byte FP32 or 32-byte
               quantised nodes); changing either rebuilds the scene's trace layout

Tuning is coordinate descent from the defaults: each knob in turn is swept with the others held
at their best values so far, every candidate is rendered `repeats` times on the caller's own
scene at a probe spp, and the candidate is scored by device-side Mrays/s (the library's ray
counter over its CUDA-event render time).  A candidate replaces the incumbent only if it is
faster by more than `margin`, so the result is never slower than the defaults on the probe.

The choice is stored in a JSON cache keyed by the device (name, SM count) and the workload
signature (primitive counts, image size, integrator, estimator, depth settings); a later call
with the same key applies the cached choice without timing, so repeated runs are reproducible.
"""
from __future__ import annotations

import hashlib
import json
import os
from dataclasses import asdict, dataclass, field

from . import abi

DEFAULTS = {
    "render_block": (16, 8),
    "slots": 1 << 21,
    "block_trace": 128,
    "block_shade": 128,
    "short_stack": 16,
    "bvh_width": 2,
    "bvh_compression": 0,
    "material_sort": 0,
}

CANDIDATES = {
    "render_block": [(16, 8), (32, 4), (8, 8), (8, 16), (32, 8), (16, 16)],
    "slots": [1 << 19, 1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24],
    "block_trace": [64, 128, 256],
    "block_shade": [64, 128, 256],
    "short_stack": [8, 16, 24, 32],
    "bvh_width": [2, 8],
    "bvh_compression": [0, 1],
    "material_sort": [0, 1],
}

KNOBS = {
    abi.INTEGRATOR_MEGAKERNEL: ["bvh_width", "bvh_compression", "render_block"],
    abi.INTEGRATOR_WAVEFRONT: ["bvh_width", "bvh_compression", "slots", "block_trace", "short_stack", "block_shade",
                               "material_sort"],
}


def default_cache_path() -> str:
    base = os.environ.get("CPT_TUNE_CACHE")
    if base:
        return base
    return os.path.join(os.path.expanduser("~"), ".cache", "cudapathtracing_gb300", "tune.json")


@dataclass
class Choice:
    knobs: dict
    score: float                     # Mrays/s of the choice on the probe
    default_score: float             # Mrays/s of the defaults on the probe
    trials: list = field(default_factory=list)

    def to_json(self) -> dict:
        d = asdict(self)
        d["knobs"] = {k: list(v) if isinstance(v, tuple) else v for k, v in self.knobs.items()}
        return d

    @staticmethod
    def from_json(d: dict) -> "Choice":
        knobs = dict(DEFAULTS)   # knobs added after a cache entry was written take their defaults
        knobs.update({k: tuple(v) if isinstance(v, list) else v for k, v in d["knobs"].items()})
        return Choice(knobs=knobs, score=d["score"], default_score=d["default_score"], trials=d.get("trials", []))


def workload_key(device: dict, scene, params: dict, integrator: int, probe_spp: int = 0) -> str:
    """scene: anything with num_triangles, num_spheres, num_lights, width, height (api.Scene).
    probe_spp: the samples per pixel the choice was timed at (the best slot count depends on the
    number of items, which grows with it)."""
    sig = {
        "device": device,
        "triangles": int(scene.num_triangles),
        "spheres": int(scene.num_spheres),
        "lights": int(scene.num_lights),
        "image": [int(scene.width), int(scene.height)],
        "integrator": int(integrator),
        "estimator": int(params.get("estimator", abi.ESTIMATOR_REFERENCE)),
        "max_depth": int(params.get("max_depth", 0)),
        "rr_depth": int(params.get("rr_depth", 0)),
        "probe_spp": int(probe_spp),
    }
    return hashlib.sha1(json.dumps(sig, sort_keys=True).encode()).hexdigest()[:16]


def load_cache(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(path: str, cache: dict) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def coordinate_descent(knobs: list, measure, margin: float = 0.02, candidates: dict | None = None,
                       start: dict | None = None):
    """Generic descent: measure(config) -> score (higher is better).  Returns (best, best_score,
    default_score, trials).  Pure host logic (unit-tested without a GPU)."""
    candidates = candidates or CANDIDATES
    best = dict(start or DEFAULTS)
    trials = []
    best_score = measure(dict(best))
    default_score = best_score
    trials.append({"config": dict(best), "score": best_score})
    for k in knobs:
        for v in candidates[k]:
            if v == best[k]:
                continue
            cfg = dict(best)
            cfg[k] = v
            sc = measure(cfg)
            trials.append({"config": cfg, "score": sc})
            if sc > best_score * (1.0 + margin):
                best, best_score = cfg, sc
    return best, best_score, default_score, trials


class Autotuner:
    """Tunes a Context for one scene and render configuration (see the module docstring)."""

    def __init__(self, ctx, cache_path: str | None = None, probe_spp: int = 4, repeats: int = 2,
                 margin: float = 0.02):
        self.ctx = ctx
        self.cache_path = cache_path or default_cache_path()
        self.probe_spp = probe_spp
        self.repeats = repeats
        self.margin = margin

    def device_info(self) -> dict:
        import torch
        p = torch.cuda.get_device_properties(self.ctx.device)
        return {"name": p.name, "sms": int(p.multi_processor_count)}

    def apply(self, knobs: dict, scene=None) -> None:
        c = self.ctx
        bx, by = knobs["render_block"]
        c.set_render_block(int(bx), int(by))
        c.set_wavefront(int(knobs["slots"]), int(knobs["block_trace"]), int(knobs["block_shade"]), 1)
        c.set_short_stack(int(knobs["short_stack"]))
        c.set_material_sort(bool(knobs.get("material_sort", 0)))
        layout = (int(knobs["bvh_width"]), int(knobs.get("bvh_compression", 0)))
        c.set_bvh_width(layout[0])
        c.set_bvh_compression(bool(layout[1]))
        if scene is not None and getattr(scene, "_tuned_layout", None) != layout:
            scene.buildBVH()
            scene._tuned_layout = layout

    def _measure(self, scene, params: dict, integrator: int, knobs: dict) -> float:
        import torch
        self.apply(knobs, scene)
        rgb = torch.zeros((scene.height, scene.width, 3), device="cuda")
        prm = dict(params)
        prm["spp"] = self.probe_spp
        scene.render(rgb=rgb, integrator=integrator, **prm)   # warm-up (graph capture, caches)
        rays, ms = 0, 0.0
        for i in range(self.repeats):
            prm["seed"] = int(params.get("seed", 0)) + 1 + i
            r = scene.render(rgb=rgb, integrator=integrator, **prm)
            rays += r["rays"]
            ms += r["ms"]
        return rays / max(ms, 1e-6) / 1e3   # Mrays/s

    def tune(self, scene, params: dict, integrator: int = abi.INTEGRATOR_WAVEFRONT, retune: bool = False) -> Choice:
        """Returns the choice for this workload (from the cache unless retune) and applies it."""
        key = workload_key(self.device_info(), scene, params, integrator, self.probe_spp)
        cache = load_cache(self.cache_path)
        if key in cache and not retune:
            ch = Choice.from_json(cache[key])
            self.apply(ch.knobs, scene)
            return ch
        best, score, dscore, trials = coordinate_descent(
            KNOBS[integrator], lambda cfg: self._measure(scene, params, integrator, cfg), self.margin)
        ch = Choice(knobs=best, score=score, default_score=dscore, trials=trials)
        cache = load_cache(self.cache_path)
        cache[key] = ch.to_json()
        save_cache(self.cache_path, cache)
        self.apply(best, scene)
        return ch
