"""Render serving loop: Poisson-arriving jobs, admission by HBM budget, concurrent lanes, and
wavefronts batched across jobs.

A job is a seeded scene of the icosphere type (procedural.random_scene) at one resolution and
spp, optionally denoised.  Jobs arrive as a Poisson process; the scheduler admits them in arrival
order while the device memory they need (scene + BVH + image and wavefront buffers, estimated by
job_bytes) fits in the HBM budget next to the jobs already running, and hands each admitted job
to a free lane.  A lane is a host thread with its own library context and CUDA stream, so jobs
on different lanes overlap on the GPU; a job's scene, BVH and accumulation buffers stay on the
device for its whole life (uploaded once, rendered into device buffers, denoised in place).

With batch > 1 a free lane takes up to `batch` queued jobs that fit the budget together and runs
them as one batch: their scenes are uploaded and built, then one cpt_render_batch renders all of
them in a single wavefront (paths of every job share the path slots and persistent kernels, so a
few small jobs fill the GPU together), then each job is denoised.  A batch's rays are recorded on
each of its jobs as batch_rays and counted once in the summary.

The scheduler is plain host logic over an executor interface (run(job, lane) -> rays, and
run_batch(jobs, lane) -> rays for batches), so its admission, ordering, batching and failure
handling are tested without a GPU (tests/test_serve.py, with a fake executor that can fail or
report out-of-memory on demand).

    python -m cudapathtracing_gb300.serve --jobs 24 --rate 20 --lanes 3 --batch 4
"""
from __future__ import annotations

import argparse
import heapq
import threading
import time
from dataclasses import dataclass, field

import numpy as np

RESOLUTIONS = (256, 512, 1024, 2048)
SPPS = (1, 4, 16, 64, 256)


@dataclass(order=True)
class Job:
    arrival: float
    jid: int
    seed: int = field(compare=False)
    size: int = field(compare=False)
    spp: int = field(compare=False)
    denoise: bool = field(compare=False)
    max_level: int = field(compare=False, default=6)
    # filled by the scheduler
    bytes: int = field(compare=False, default=0)
    start: float = field(compare=False, default=0.0)
    end: float = field(compare=False, default=0.0)
    rays: int = field(compare=False, default=0)
    batch: int = field(compare=False, default=-1)      # batch number (-1: rendered alone)
    status: str = field(compare=False, default="queued")
    error: str = field(compare=False, default="")


def poisson_jobs(n: int, rate: float = 20.0, seed: int = 3, denoise_frac: float = 0.5, max_level: int = 6,
                 sizes=RESOLUTIONS, spps=SPPS):
    """n jobs drawn from numpy's generator seeded by `seed`: exponential inter-arrival times with
    the given rate, resolution uniform over `sizes` (square), spp uniform over `spps`, and the
    denoiser on with odds denoise_frac."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    return [Job(arrival=float(t[i]), jid=i, seed=int(3_000_000 + i), size=int(rng.choice(sizes)),
                spp=int(rng.choice(spps)), denoise=bool(rng.uniform() < denoise_frac), max_level=max_level)
            for i in range(n)]


def job_bytes(num_triangles: int, size: int, spp: int, slots: int = 1 << 21) -> int:
    """Device memory of one job: triangles, BVH nodes and leaf records, build scratch (~300 B per
    triangle), the image, G-buffer and denoiser activations (~700 B per pixel), and the wavefront
    state (slots and per-item group sums)."""
    px = size * size
    groups = max(1, (spp + 7) // 8)
    items = px * groups
    return int(300 * num_triangles + 700 * px + 200 * min(slots, items) + 16 * items)


class Scheduler:
    """Admission by HBM budget (FIFO: a job that does not fit waits, and so do the jobs behind
    it), up to `lanes` batches at once, each of up to `batch` jobs.  executor.run(job, lane)
    returns the rays traced or raises; executor.run_batch(jobs, lane) does the same for a batch
    of two or more jobs (its rays are the whole batch's).  MemoryError from the executor puts
    the jobs back at the head of the queue until other jobs free memory (or fails them when
    nothing else is running); any other exception fails every job of the batch."""

    def __init__(self, executor, budget_bytes: int, lanes: int = 2, clock=time.perf_counter, batch: int = 1,
                 batch_samples: int | None = None):
        self.ex = executor
        self.budget = budget_bytes
        self.lanes = lanes
        self.batch = max(1, int(batch))
        # a batch grows while its jobs' samples (pixels x spp) stay within batch_samples, so small
        # jobs are batched together and a large one (which fills the GPU alone) is not joined by
        # small ones that would then wait for it
        self.batch_samples = batch_samples
        self.clock = clock
        self.in_use = 0
        self.peak = 0
        self.batches = 0
        self.lock = threading.Condition()
        self.free_lanes = list(range(lanes))

    def _admit(self, job, need_lane: bool = True) -> bool:
        if job.bytes > self.budget:
            job.status, job.error = "rejected", "larger than the HBM budget"
            return True
        if self.in_use + job.bytes <= self.budget and (self.free_lanes or not need_lane):
            self.in_use += job.bytes
            self.peak = max(self.peak, self.in_use)
            return True
        return False

    def run(self, jobs, realtime: bool = True):
        """Runs all jobs; with realtime the jobs are released at their arrival times."""
        pending = sorted(jobs)
        done, oom, queue, threads = [], [], [], []
        running = [0]
        t0 = self.clock()

        def worker(batch, lane):
            failed_oom = False
            try:
                if len(batch) == 1:
                    rays = [int(self.ex.run(batch[0], lane))]
                else:
                    total = int(self.ex.run_batch(batch, lane))
                    rays = [total] * len(batch)
                for job, r in zip(batch, rays):
                    job.rays = r
                    job.status = "done"
            except MemoryError as e:
                failed_oom = True
                for job in batch:
                    job.status, job.error = "oom", str(e)
            except Exception as e:   # a failed batch frees its budget and its lane
                for job in batch:
                    job.status, job.error = "failed", f"{type(e).__name__}: {e}"
            end = self.clock() - t0
            with self.lock:
                for job in batch:
                    job.end = end
                    self.in_use -= job.bytes
                running[0] -= 1
                self.free_lanes.append(lane)
                (oom if failed_oom else done).extend(batch)
                self.lock.notify_all()

        i = 0
        with self.lock:
            while len(done) < len(jobs):
                now = self.clock() - t0
                while i < len(pending) and (not realtime or pending[i].arrival <= now):
                    job = pending[i]
                    job.bytes = job.bytes or self.ex.estimate(job)
                    heapq.heappush(queue, job)
                    i += 1
                # a job the executor could not fit goes back to the head of the queue while
                # others run (their memory will come back); alone, it fails
                while oom:
                    job = oom.pop()
                    if running[0] == 0 and not queue:
                        job.status = "failed"
                        done.append(job)
                    else:
                        job.status = "queued"
                        heapq.heappush(queue, job)
                while queue and self.free_lanes:
                    batch = []
                    work = 0
                    while queue and len(batch) < self.batch:
                        job = queue[0]
                        w = job.size * job.size * job.spp
                        if batch and self.batch_samples is not None and work + w > self.batch_samples:
                            break
                        if not self._admit(job, need_lane=not batch):
                            break
                        heapq.heappop(queue)
                        if job.status == "rejected":
                            job.end = self.clock() - t0
                            done.append(job)
                            continue
                        batch.append(job)
                        work += w
                    if not batch:
                        break
                    lane = self.free_lanes.pop(0)
                    bid = -1
                    if len(batch) > 1:
                        bid = self.batches
                        self.batches += 1
                    for job in batch:
                        job.status = "running"
                        job.start = self.clock() - t0
                        job.batch = bid
                    running[0] += 1
                    th = threading.Thread(target=worker, args=(batch, lane), daemon=True)
                    threads.append(th)
                    th.start()
                if len(done) >= len(jobs):
                    break
                timeout = 0.05
                if realtime and i < len(pending):
                    timeout = min(timeout, max(0.0, pending[i].arrival - (self.clock() - t0)))
                self.lock.wait(timeout=timeout)
        for th in threads:
            th.join()
        return sorted(done, key=lambda j: j.jid)


def summary(jobs, wall: float) -> dict:
    ok = [j for j in jobs if j.status == "done"]
    lat = np.array([j.end - j.arrival for j in ok]) if ok else np.zeros(1)
    batched = {j.batch: j.rays for j in ok if j.batch >= 0}   # a batch's rays once
    rays = sum(j.rays for j in ok if j.batch < 0) + sum(batched.values())
    return {"jobs": len(jobs), "done": len(ok), "failed": sum(j.status == "failed" for j in jobs),
            "rejected": sum(j.status == "rejected" for j in jobs),
            "latency_p50_s": round(float(np.percentile(lat, 50)), 4),
            "latency_p99_s": round(float(np.percentile(lat, 99)), 4),
            "latency_mean_s": round(float(lat.mean()), 4), "wall_s": round(wall, 3),
            "mrays_per_s": round(rays / max(wall, 1e-9) / 1e6, 1), "rays": int(rays),
            "batches": len(batched), "jobs_in_batches": sum(j.batch >= 0 for j in ok)}


class GpuExecutor:
    """Runs jobs on the library: one context, CUDA stream and denoiser per lane."""

    def __init__(self, lanes: int, device: int = 0, weights: str | None = None):
        import torch
        from . import api
        from .denoiser import Denoiser
        self.ctx = [api.Context(device) for _ in range(lanes)]
        self.streams = [torch.cuda.Stream(device) for _ in range(lanes)]
        self.den = []
        for _ in range(lanes):
            d = Denoiser(device)
            if weights:
                d.load(weights)
            self.den.append(d)
        self.descs = {}

    def prepare(self, jobs):
        """Builds the scene descriptions on the host before the clock starts."""
        from . import procedural as P
        for j in jobs:
            self.descs[j.jid] = P.random_scene(j.seed, width=j.size, max_level=j.max_level)

    def estimate(self, job) -> int:
        return job_bytes(self.descs[job.jid].num_triangles, job.size, job.spp)

    def run(self, job, lane) -> int:
        import torch
        from . import abi, api
        from .training import RENDER
        st = self.streams[lane]
        with torch.cuda.stream(st):
            sc = api.Scene(self.ctx[lane], self.descs[job.jid])
            sc.buildBVH(st.cuda_stream)
            rgb = torch.zeros((sc.height, sc.width, 3), device="cuda")
            gb = torch.zeros((sc.height, sc.width, 8), device="cuda") if job.denoise else None
            r = sc.render(spp=job.spp, seed=job.seed, integrator=abi.INTEGRATOR_WAVEFRONT, rgb=rgb, gbuffer=gb,
                          stream=st.cuda_stream, **RENDER)
            if job.denoise:
                self.den[lane].denoise(rgb, gb, stream=C_stream(st))
            st.synchronize()
            sc.close()
        return r["rays"]


    def run_batch(self, jobs, lane) -> int:
        """The jobs' scenes uploaded and built on the lane's stream, one cpt_render_batch over all
        of them (one wavefront), then each denoised; returns the batch's rays."""
        import torch
        from . import api
        from .training import RENDER
        st = self.streams[lane]
        scenes, outs = [], []
        try:
            with torch.cuda.stream(st):
                for job in jobs:
                    sc = api.Scene(self.ctx[lane], self.descs[job.jid])
                    sc.buildBVH(st.cuda_stream)
                    scenes.append(sc)
                    outs.append((torch.zeros((sc.height, sc.width, 3), device="cuda"),
                                 torch.zeros((sc.height, sc.width, 8), device="cuda") if job.denoise else None))
                prm = {k: v for k, v in RENDER.items() if k not in ("estimator", "integrator")}
                r = api.render_batch(self.ctx[lane], [dict(scene=sc, spp=job.spp, seed=job.seed, rgb=o[0],
                                                           gbuffer=o[1], **prm)
                                                      for sc, job, o in zip(scenes, jobs, outs)],
                                     stream=st.cuda_stream)
                for job, o in zip(jobs, outs):
                    if job.denoise:
                        self.den[lane].denoise(o[0], o[1], stream=C_stream(st))
                st.synchronize()
        finally:
            for sc in scenes:
                sc.close()
        return r["rays"]


def C_stream(st):
    import ctypes
    return ctypes.c_void_p(st.cuda_stream)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=24)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--lanes", type=int, default=3)
    ap.add_argument("--budget-gb", type=float, default=64.0)
    ap.add_argument("--max-level", type=int, default=6)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--batch", type=int, default=1, help="jobs per wavefront (cross-job batching)")
    ap.add_argument("--batch-samples", type=float, default=16.0,
                    help="a batch grows while its samples (pixels x spp) stay within this many million")
    ap.add_argument("--sizes", default="256,512,1024,2048", help="job resolutions (square)")
    ap.add_argument("--spps", default="1,4,16,64,256", help="job sample counts")
    args = ap.parse_args()
    import json
    from .training import DEFAULT_WEIGHTS
    jobs = poisson_jobs(args.jobs, args.rate, args.seed, max_level=args.max_level,
                        sizes=tuple(int(x) for x in args.sizes.split(",")),
                        spps=tuple(int(x) for x in args.spps.split(",")))
    ex = GpuExecutor(args.lanes, weights=DEFAULT_WEIGHTS)
    ex.prepare(jobs)
    # warm-up: one small job per lane (graph capture, denoiser allocation)
    for lane in range(args.lanes):
        w = Job(0.0, -1 - lane, seed=1, size=256, spp=1, denoise=True)
        ex.descs[w.jid] = ex.descs[jobs[0].jid]
        ex.run(w, lane)
    sched = Scheduler(ex, int(args.budget_gb * (1 << 30)), args.lanes, batch=args.batch,
                      batch_samples=int(args.batch_samples * 1e6))
    t0 = time.perf_counter()
    done = sched.run(jobs)
    wall = time.perf_counter() - t0
    res = summary(done, wall)
    offered = sum(j.size * j.size * j.spp for j in jobs) / max(jobs[-1].arrival, 1e-9)
    res.update({"rate_per_s": args.rate, "lanes": args.lanes, "batch": args.batch,
                "batch_msamples": args.batch_samples, "sizes": args.sizes, "spps": args.spps,
                "budget_gb": args.budget_gb,
                "peak_admitted_gb": round(sched.peak / (1 << 30), 2),
                "offered_samples_per_s": round(offered / 1e6, 1), "offered_unit": "M samples/s"})
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
