"""Serving-loop scheduler on the host (no GPU): HBM-budget admission, FIFO order, lane limits,
and failure injection (a job that raises, a job the executor reports out of memory)."""
from __future__ import annotations

import threading
import time

from cudapathtracing_gb300 import serve as S


class FakeExecutor:
    def __init__(self, bytes_of, fail=(), oom_once=(), dur=0.01):
        self.bytes_of, self.fail, self.oom_once, self.dur = bytes_of, set(fail), set(oom_once), dur
        self.lock = threading.Lock()
        self.active, self.peak_active, self.order = 0, 0, []
        self.in_use = 0
        self.budget_seen = 0

    def estimate(self, job):
        return self.bytes_of(job)

    def run(self, job, lane):
        with self.lock:
            self.active += 1
            self.peak_active = max(self.peak_active, self.active)
            self.order.append(job.jid)
        try:
            if job.jid in self.oom_once:
                self.oom_once.discard(job.jid)
                raise MemoryError("injected: allocation failed")
            time.sleep(self.dur)
            if job.jid in self.fail:
                raise RuntimeError("injected failure")
            return 1000 * (job.jid + 1)
        finally:
            with self.lock:
                self.active -= 1


    def run_batch(self, jobs, lane):
        with self.lock:
            self.batches = getattr(self, "batches", []) + [[j.jid for j in jobs]]
        return sum(self.run(j, lane) for j in jobs)


def _jobs(n, size=256, spp=4):
    return [S.Job(arrival=0.001 * i, jid=i, seed=i, size=size, spp=spp, denoise=False) for i in range(n)]


def test_budget_and_lanes_are_never_exceeded():
    ex = FakeExecutor(lambda j: 40 if j.jid % 2 else 70)
    sch = S.Scheduler(ex, budget_bytes=100, lanes=3)
    done = sch.run(_jobs(12), realtime=False)
    assert all(j.status == "done" for j in done)
    assert sch.peak <= 100
    assert ex.peak_active <= 3
    assert ex.order == sorted(ex.order)          # FIFO admission
    assert sum(j.rays for j in done) == sum(1000 * (i + 1) for i in range(12))


def test_failures_free_their_budget_and_lane():
    ex = FakeExecutor(lambda j: 60, fail={2, 5})
    sch = S.Scheduler(ex, budget_bytes=100, lanes=2)
    done = sch.run(_jobs(8), realtime=False)
    st = {j.jid: j.status for j in done}
    assert st[2] == "failed" and st[5] == "failed"
    assert sum(s == "done" for s in st.values()) == 6
    assert sch.in_use == 0


def test_oom_is_retried_and_oversized_jobs_rejected():
    ex = FakeExecutor(lambda j: 500 if j.jid == 3 else 30, oom_once={1})
    sch = S.Scheduler(ex, budget_bytes=100, lanes=2)
    done = sch.run(_jobs(6), realtime=False)
    st = {j.jid: j.status for j in done}
    assert st[3] == "rejected"
    assert st[1] == "done"                         # retried after the injected out-of-memory
    assert ex.order.count(1) == 2


def test_realtime_latencies_and_summary():
    ex = FakeExecutor(lambda j: 10, dur=0.02)
    jobs = S.poisson_jobs(10, rate=100.0, seed=1)
    sch = S.Scheduler(ex, budget_bytes=100, lanes=2)
    t0 = time.perf_counter()
    done = sch.run(jobs, realtime=True)
    wall = time.perf_counter() - t0
    assert all(j.end >= j.arrival for j in done)
    res = S.summary(done, wall)
    assert res["done"] == 10 and res["latency_p99_s"] >= res["latency_p50_s"] > 0


def test_poisson_jobs_and_memory_estimate():
    jobs = S.poisson_jobs(200, rate=20.0, seed=3)
    gaps = [b.arrival - a.arrival for a, b in zip(jobs, jobs[1:])]
    assert 0.03 < sum(gaps) / len(gaps) < 0.07       # mean 1 / 20 s
    assert {j.size for j in jobs} <= set(S.RESOLUTIONS) and {j.spp for j in jobs} <= set(S.SPPS)
    assert S.job_bytes(2_000_000, 2048, 256) > S.job_bytes(50_000, 256, 1) > 0


def test_batches_of_jobs_share_a_lane():
    """With batch=3 a free lane takes up to three queued jobs that fit the budget together; the
    batch's rays are counted once, FIFO order and the budget hold, and a failure or an
    out-of-memory report applies to the whole batch."""
    ex = FakeExecutor(lambda j: 20)
    sch = S.Scheduler(ex, budget_bytes=100, lanes=2, batch=3)
    done = sch.run(_jobs(11), realtime=False)
    assert all(j.status == "done" for j in done)
    assert ex.batches and all(2 <= len(b) <= 3 for b in ex.batches)
    assert sum(len(b) for b in ex.batches) + sum(j.batch < 0 for j in done) == 11
    assert sch.peak <= 100
    assert all(b == list(range(b[0], b[0] + len(b))) for b in ex.batches)   # FIFO: consecutive arrivals
    res = S.summary(done, 1.0)
    assert res["rays"] == sum(1000 * (i + 1) for i in range(11))
    assert res["batches"] == len(ex.batches)

    ex = FakeExecutor(lambda j: 20, fail={4}, oom_once={1})
    sch = S.Scheduler(ex, budget_bytes=100, lanes=1, batch=2)
    done = sch.run(_jobs(6), realtime=False)
    st = {j.jid: j.status for j in done}
    partner = [b for b in ex.batches if 4 in b][0]
    assert all(st[k] == "failed" for k in partner)          # the failing job's batch fails
    assert st[1] == "done" and sch.in_use == 0               # the out-of-memory batch was retried


def test_batch_sample_cap_keeps_large_jobs_alone():
    ex = FakeExecutor(lambda j: 10)
    jobs = [S.Job(arrival=0.0, jid=i, seed=i, size=(2048 if i in (2, 5) else 256), spp=4, denoise=False)
            for i in range(8)]
    sch = S.Scheduler(ex, budget_bytes=1000, lanes=1, batch=4, batch_samples=4 * 256 * 256 * 4)
    done = sch.run(jobs, realtime=False)
    assert all(j.status == "done" for j in done)
    by = {j.jid: j.batch for j in done}
    assert by[2] == -1 and by[5] == -1                    # over the cap: rendered alone
    assert all(len(b) <= 4 and 2 not in b and 5 not in b for b in ex.batches)
