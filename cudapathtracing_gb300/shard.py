"""Image sharding across ranks (one process per GPU).

The path shards with no data-path exchange: pixels are independent and every rank holds the whole
scene and BVH.  A frame is split into horizontal bands of rows (cpt_render's row range), each rank
renders its band into its own buffer, and the only exchange is one gather of the bands into the
full image on the destination rank.  Bands are balanced to within one row.
"""
from __future__ import annotations


def row_ranges(height: int, world: int):
    """[(row_begin, row_end)] for each rank, contiguous, covering [0, height)."""
    base, extra = divmod(height, world)
    out, r = [], 0
    for k in range(world):
        n = base + (1 if k < extra else 0)
        out.append((r, r + n))
        r += n
    return out


def gather_rows(band, height: int, rank: int, world: int, group=None, dst: int = 0):
    """Gathers every rank's band ([rows, W, C] tensor for its row range) into the full [height, W,
    C] image on rank `dst` (returned there; None elsewhere).  Bands are padded to the largest band
    for the collective and cut back afterwards."""
    import torch
    import torch.distributed as dist
    ranges = row_ranges(height, world)
    rows = max(b - a for a, b in ranges)
    pad = torch.zeros((rows,) + tuple(band.shape[1:]), dtype=band.dtype, device=band.device)
    pad[: band.shape[0]] = band
    parts = [torch.empty_like(pad) for _ in range(world)] if rank == dst else None
    dist.gather(pad, parts, dst=dst, group=group)
    if rank != dst:
        return None
    return torch.cat([p[: b - a] for p, (a, b) in zip(parts, ranges)], 0)


def render_band(scene, rank: int, world: int, rgb, **params):
    """Renders this rank's rows of the scene's view into rgb (the full-size device image buffer);
    returns the band (a view of rgb) and the render statistics."""
    a, b = row_ranges(scene.height, world)[rank]
    r = scene.render(rgb=rgb, rows=(a, b), **params)
    return rgb[a:b], r
