"""The atomic-free refit's index arithmetic (csrc/lbvh.cu pyramid_up, refit_from_leaves and
range_union) restated in Python over integers, with min as the union, against brute force.

* The pyramid: level l + 1 holds ceil(size(l) / 4) unions of four consecutive boxes of level l,
  built four levels per launch by blocks of 256 threads (shuffles for levels +1 and +2, warp 0 over
  shared memory for +3 and +4), launches chained from the last level written.
* The range walk: a node's union over [lo, hi) from at most three boxes at each end per level and
  at most six at the level where the walk stops.

The GPU side is checked bit for bit by the LBVH parity tests (node boxes equal the oracle's)."""
from __future__ import annotations

import numpy as np
import pytest

T = 256
EMPTY = np.iinfo(np.int64).max


def _shfl_min(v, o):
    lanes = np.arange(v.size)
    src = (lanes & ~31) | ((lanes & 31) ^ o)
    return np.minimum(v, v[src])


def _pyramid_up(vals, n, depth):
    """Levels +1 .. +depth above a level of n values (vals padded to whole blocks)."""
    nb = vals.size // T
    sizes = [(n + 3) // 4]
    for _ in range(3):
        sizes.append((sizes[-1] + 3) // 4)
    outs = [np.full(s, -1, np.int64) for s in sizes]
    i = np.arange(vals.size)
    t = i % T
    v = _shfl_min(_shfl_min(vals, 1), 2)
    m = ((t & 3) == 0) & ((i >> 2) < sizes[0])
    outs[0][(i >> 2)[m]] = v[m]
    if depth > 1:
        v = _shfl_min(_shfl_min(v, 4), 8)
        m = ((t & 15) == 0) & ((i >> 4) < sizes[1])
        outs[1][(i >> 4)[m]] = v[m]
    if depth > 2:
        for b in range(nb):
            w = np.full(32, EMPTY, np.int64)
            w[:16] = v[b * T:(b + 1) * T:16]
            w = _shfl_min(_shfl_min(w, 1), 2)
            for lane in range(0, 16, 4):
                j3 = b * 4 + (lane >> 2)
                if j3 < sizes[2]:
                    outs[2][j3] = w[lane]
            if depth > 3:
                w = _shfl_min(_shfl_min(w, 4), 8)
                if b < sizes[3]:
                    outs[3][b] = w[0]
    return outs[:depth]


def _build(leaves):
    n = leaves.size
    count, m = 0, n
    while m > 1:
        m = (m + 3) // 4
        count += 1
    levels, cur, l = [], leaves, 0
    while l < count:
        depth = min(4, count - l)
        nb = (cur.size + T - 1) // T
        vals = np.full(nb * T, EMPTY, np.int64)
        vals[:cur.size] = cur
        got = _pyramid_up(vals, cur.size, depth)
        levels += got
        cur, l = got[-1], l + depth
    return levels, count


def _range_union(leaves, levels, count, lo, hi):
    a, best, l = leaves, EMPTY, 0
    while True:
        lo_up, hi_dn = (lo + 3) & ~3, hi & ~3
        if l == count or lo_up >= hi_dn:
            assert hi - lo <= 6
            for j in range(6):
                if lo + j < hi:
                    best = min(best, a[lo + j])
            return best
        for j in range(3):
            if lo + j < lo_up:
                best = min(best, a[lo + j])
            if hi_dn + j < hi:
                best = min(best, a[hi_dn + j])
        lo, hi = lo_up >> 2, hi_dn >> 2
        a, l = levels[l], l + 1


@pytest.mark.parametrize("n", [2, 3, 5, 16, 17, 255, 256, 257, 1025, 4097, 65537])
def test_pyramid_levels_and_range_unions(n):
    rng = np.random.default_rng(n)
    leaves = rng.integers(0, 10 ** 9, n)
    levels, count = _build(leaves)
    # every level against its definition
    cur = leaves
    for lv in levels:
        m = (cur.size + 3) // 4
        pad = np.full(4 * m, EMPTY, np.int64)
        pad[:cur.size] = cur
        ref = pad.reshape(m, 4).min(1)
        assert np.array_equal(lv, ref)
        cur = ref
    assert levels[-1].size == 1
    queries = [(0, n), (n - 1, n), (0, 1)] + [tuple(sorted(rng.integers(0, n + 1, 2))) for _ in range(400)]
    for lo, hi in queries:
        if hi > lo:
            assert _range_union(leaves, levels, count, int(lo), int(hi)) == leaves[lo:hi].min()
