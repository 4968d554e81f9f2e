"""TEST INFRASTRUCTURE ONLY — measures, with the oracle, the traversal work that defines
the algorithmic bytes per ray of the bench's roofline, and writes it to
cudapathtracing_gb300/workload_constants.json.

For each workload, every closest-hit query made by an oracle render of a sample of the
workload's pixels is re-run through an ordered, tMax-pruned traversal of the binary LBVH
with the reference's topology, counting internal-node visits (V_int) and primitive tests
(V_leaf).  Bytes per ray = 32 (ray) + 16 (hit) + V_int * (2 * 24 + 8) + V_leaf * 36.

    python oracle/visit_counts.py
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from cudapathtracing_gb300 import abi, procedural as P  # noqa: E402

OUT = os.path.join(ROOT, "cudapathtracing_gb300", "workload_constants.json")


def bytes_per_ray(v_int: float, v_leaf: float) -> float:
    return 32 + 16 + v_int * (2 * 24 + 8) + v_leaf * 36


def sample_rows(height: int, count: int) -> list:
    step = max(1, height // count)
    return [(r, r + 1) for r in range(step // 2, height, step)][:count]


def render_counts(o, params_kw, rows):
    q = vi = vl = 0
    for r0, r1 in rows:
        a, b, c = o.render_visit_counts(abi.render_params(row_begin=r0, row_end=r1, **params_kw))
        q, vi, vl = q + a, vi + b, vl + c
    return q, vi, vl


def main():
    O.build(ref=False)
    out = {}
    t0 = time.time()
    d = P.spheres_scene()
    o = O.OracleScene(d)
    kw = dict(spp=1, estimator=abi.ESTIMATOR_CONFIG, max_depth=16, rr_depth=3, rr_prob=0.8, seed=0)
    rows = sample_rows(d.camera.height, 12)
    q, vi, vl = render_counts(o, kw, rows)
    out["spheres_1080p"] = dict(queries=q, v_int=vi / q, v_leaf=vl / q, bytes_per_ray=bytes_per_ray(vi / q, vl / q),
                                sample=f"{len(rows)} rows x 1920 px x 1 spp, config estimator, seed 0")
    print("spheres", out["spheres_1080p"], f"{time.time() - t0:.1f}s")
    d = P.icosphere_scene(level=8)
    o = O.OracleScene(d)
    rays = P.uniform_rays(200_000, seed=1, first=0)
    vi, vl = o.trace_counts(P.rays_as_f64(rays))
    n = rays.shape[0]
    out["icosphere_10M"] = dict(queries=n, v_int=vi / n, v_leaf=vl / n, bytes_per_ray=bytes_per_ray(vi / n, vl / n),
                                sample="rays 0..199,999 of the 10M set (PCG32 seed 1)")
    print("icosphere", out["icosphere_10M"])
    d = P.cornell_box(width=512)
    o = O.OracleScene(d)
    q, vi, vl = render_counts(o, dict(spp=16, estimator=abi.ESTIMATOR_REFERENCE, seed=0), sample_rows(512, 16))
    out["cornell_512"] = dict(queries=q, v_int=vi / q, v_leaf=vl / q, bytes_per_ray=bytes_per_ray(vi / q, vl / q),
                              sample="16 rows x 512 px x 16 spp, reference estimator, seed 0")
    print("cornell", out["cornell_512"])
    out["_definition"] = ("bytes/ray = 32 (ray) + 16 (hit) + V_int*(2*24+8) + V_leaf*36; V_int, V_leaf: ordered "
                          "tMax-pruned traversal of the reference-topology binary LBVH, counted by the FP64 oracle")
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
