"""The serving loop end to end on the GPU: small seeded jobs on two lanes, all complete, rays are
counted, and the admitted memory never exceeds the budget."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_serving_loop_small_jobs(ctx):
    from cudapathtracing_gb300 import serve as S
    jobs = [S.Job(arrival=0.01 * i, jid=i, seed=5000 + i, size=(64, 128)[i % 2], spp=(1, 4)[i % 2],
                  denoise=bool(i % 3 == 0), max_level=4) for i in range(6)]
    ex = S.GpuExecutor(lanes=2)
    ex.prepare(jobs)
    budget = 4 * max(ex.estimate(j) for j in jobs)
    sch = S.Scheduler(ex, budget, lanes=2)
    done = sch.run(jobs)
    assert [j.status for j in done] == ["done"] * 6, [(j.status, j.error) for j in done]
    assert all(j.rays > 0 for j in done)
    assert sch.peak <= budget
    res = S.summary(done, max(j.end for j in done))
    assert res["mrays_per_s"] > 0


def test_serving_loop_batches_jobs_into_one_wavefront(ctx):
    """Cross-job batching on the GPU: up to three jobs (different scenes, sizes and spp, some
    denoised) rendered per cpt_render_batch call; every job completes and the batches' rays add
    up to the rays of the same jobs rendered one by one."""
    from cudapathtracing_gb300 import serve as S
    jobs = [S.Job(arrival=0.0, jid=i, seed=6000 + i, size=(64, 96, 128)[i % 3], spp=(1, 4, 2)[i % 3],
                  denoise=bool(i % 2), max_level=4) for i in range(7)]
    ex = S.GpuExecutor(lanes=1)
    ex.prepare(jobs)
    single = sum(ex.run(j, 0) for j in jobs)
    sch = S.Scheduler(ex, 10 * max(ex.estimate(j) for j in jobs), lanes=1, batch=3)
    done = sch.run(jobs, realtime=False)
    assert [j.status for j in done] == ["done"] * 7, [(j.status, j.error) for j in done]
    assert sch.batches >= 2
    res = S.summary(done, 1.0)
    assert res["rays"] == single
