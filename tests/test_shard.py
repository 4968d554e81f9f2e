"""Row sharding across ranks on the CPU (gloo, world size 2 and 3): the bands cover the image,
and gathering the ranks' bands reproduces the image a single rank renders."""
from __future__ import annotations

import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from cudapathtracing_gb300 import shard


def test_row_ranges_cover_and_balance():
    for H in (1, 7, 270, 1080):
        for world in (1, 2, 3, 8):
            rr = shard.row_ranges(H, world)
            assert rr[0][0] == 0 and rr[-1][1] == H
            assert all(a1 == b0 for (_, b0), (a1, _) in zip(rr, rr[1:]))
            sizes = [b - a for a, b in rr]
            assert max(sizes) - min(sizes) <= 1


def _fake_frame(H, W):
    """Stands in for a render: a deterministic function of the pixel's row and column."""
    y = torch.arange(H, dtype=torch.float32)[:, None, None]
    x = torch.arange(W, dtype=torch.float32)[None, :, None]
    c = torch.arange(3, dtype=torch.float32)[None, None, :]
    return torch.sin(0.1 * y + 0.01 * x) + c


def _worker(rank, world, port, H, W, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b = shard.row_ranges(H, world)[rank]
        band = _fake_frame(H, W)[a:b].clone()
        full = shard.gather_rows(band, H, rank, world)
        if rank == 0:
            q.put(bool(torch.equal(full, _fake_frame(H, W))))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,H", [(2, 37), (3, 64)])
def test_gather_rows_reassembles_the_frame(world, H):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + world * 7 + H
    procs = [ctx.Process(target=_worker, args=(r, world, port, H, 19, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=10) is True
