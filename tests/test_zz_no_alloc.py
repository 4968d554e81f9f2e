"""cpt_lbvh_build_device_static: the LBVH build whose scratch is a fixed array inside the
library, for callers that cannot allocate device memory (a host that has handed all of its
HBM to its own pools, or code where an allocation is not allowed).  Through the C ABI it must
produce exactly what the allocating entry point cpt_lbvh_build_device produces, on two calls
in a row that share the one scratch array, and reject builds above its stated maximum.

This file is collected last so that a failure here does not hide the other tests' results."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import outward_f32
from cudapathtracing_gb300 import _lib, abi, procedural as P

pytestmark = pytest.mark.gpu

MAX_PRIMS = 65536


def _bind(lib):
    f = lib.cpt_lbvh_build_device_static
    f.restype = C.c_int
    f.argtypes = [C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_double),
                  C.POINTER(C.c_double)] + [C.c_void_p] * 7
    return f


def _inputs(seed: int, n_tri: int, n_sph: int):
    """Random triangles plus spheres as extra primitives (centre, box rounded outwards)."""
    g = P.PCG32Streams(seed, np.arange(max(n_tri, n_sph), dtype=np.uint64))
    c = np.stack([g.uniform()[:n_tri] * 6 - 3 for _ in range(3)], 1)
    e = np.stack([g.uniform()[:n_tri] * 0.3 for _ in range(6)], 1)
    tri = np.concatenate([c, c + e[:, :3], c + e[:, 3:]], 1).astype(np.float32)
    ctr = np.stack([np.linspace(-2, 2, n_sph), np.full(n_sph, 0.5), np.linspace(1, -1, n_sph)], 1)
    rad = np.linspace(0.2, 0.6, n_sph)
    lo = (ctr - rad[:, None]).astype(np.float32)
    hi = (ctr + rad[:, None]).astype(np.float32)
    lo = np.where(lo.astype(np.float64) > ctr - rad[:, None], np.nextafter(lo, np.float32(-np.inf)), lo)
    hi = np.where(hi.astype(np.float64) < ctr + rad[:, None], np.nextafter(hi, np.float32(np.inf)), hi)
    boxes = np.zeros((n_sph, 8), np.float32)
    boxes[:, 0:3], boxes[:, 4:7] = lo, hi
    pts = tri.reshape(-1, 3).astype(np.float64)
    return ctr, boxes, tri, tuple(pts.min(0)), tuple(pts.max(0))


def _outputs(torch, n):
    dev = "cuda"
    return dict(keys=torch.full((n,), -1, dtype=torch.int64, device=dev),
                order=torch.full((n,), -1, dtype=torch.int32, device=dev),
                children=torch.full((n - 1, 2), 7, dtype=torch.int32, device=dev),
                node_range=torch.full((n - 1, 2), 7, dtype=torch.int32, device=dev),
                node_boxes=torch.full((n - 1, 8), 7.0, dtype=torch.float32, device=dev),
                leaf_boxes=torch.full((n, 8), 7.0, dtype=torch.float32, device=dev))


def _args(torch, ctr, boxes, tri, bmin, bmax, out):
    dc = torch.from_numpy(ctr).cuda()
    db = torch.from_numpy(boxes).cuda()
    dt = torch.from_numpy(tri).cuda()
    keep = (dc, db, dt)
    head = [ctr.shape[0], dc.data_ptr(), db.data_ptr(), tri.shape[0], dt.data_ptr(), (C.c_double * 3)(*bmin),
            (C.c_double * 3)(*bmax)]
    tail = [out[k].data_ptr() for k in ("keys", "order", "children", "node_range", "node_boxes", "leaf_boxes")]
    return keep, head, tail


def _host(out):
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("calls", [[(31, 1280, 4), (32, 5000, 9)]])
def test_static_scratch_build_matches_allocating_build(calls):
    import torch
    lib = _lib.lib()
    static_build = _bind(lib)
    for seed, n_tri, n_sph in calls:   # two calls in a row share the static scratch
        ctr, boxes, tri, bmin, bmax = _inputs(seed, n_tri, n_sph)
        n = n_tri + n_sph
        ref_out = _outputs(torch, n)
        keep, head, tail = _args(torch, ctr, boxes, tri, bmin, bmax, ref_out)
        scratch = torch.zeros(int(lib.cpt_lbvh_scratch_bytes(n)), dtype=torch.uint8, device="cuda")
        st = lib.cpt_lbvh_build_device(*head, *tail, scratch.data_ptr(), scratch.numel(), None)
        assert st == 0, lib.cpt_last_error_string()
        new_out = _outputs(torch, n)
        _, head2, tail2 = _args(torch, ctr, boxes, tri, bmin, bmax, new_out)
        st = static_build(*head2, *tail2, None)
        assert st == 0, lib.cpt_last_error_string()
        torch.cuda.synchronize()
        a, b = _host(ref_out), _host(new_out)
        for k in a:   # integer outputs and FP32 boxes: identical bits (exact tolerance)
            assert np.array_equal(a[k], b[k]), (seed, k)
        assert np.array_equal(np.sort(b["order"]), np.arange(n, dtype=np.int32))
        del keep


def test_static_scratch_rejects_builds_above_its_maximum():
    import torch
    lib = _lib.lib()
    static_build = _bind(lib)
    n = MAX_PRIMS + 1
    tri = torch.zeros((n, 9), dtype=torch.float32, device="cuda")
    out = _outputs(torch, n)
    st = static_build(0, None, None, n, tri.data_ptr(), (C.c_double * 3)(0, 0, 0), (C.c_double * 3)(1, 1, 1),
                      *[out[k].data_ptr() for k in ("keys", "order", "children", "node_range", "node_boxes",
                                                     "leaf_boxes")], None)
    assert st == 1
    assert b"65536" in lib.cpt_last_error_string()
    torch.cuda.synchronize()
    assert (out["order"] == -1).all()   # nothing was written


def test_static_scratch_at_its_maximum_matches_oracle_and_allocates_nothing(oracle_mod):
    """Exactly CPT_LBVH_STATIC_MAX_PRIMS primitives (the size the 3 MiB array is sized for):
    keys, order and topology bit-exact against the FP64 oracle's LBVH and boxes equal to its
    boxes rounded outwards.  After a warm-up call (which may load the kernels' code), a second
    call must leave the device's free memory and the caching allocator's reservation unchanged."""
    import torch
    lib = _lib.lib()
    static_build = _bind(lib)
    n_sph = 6
    n_tri = MAX_PRIMS - n_sph
    ctr, boxes, tri, bmin, bmax = _inputs(41, n_tri, n_sph)
    out = _outputs(torch, MAX_PRIMS)
    keep, head, tail = _args(torch, ctr, boxes, tri, bmin, bmax, out)
    st = static_build(*head, *tail, None)   # warm-up
    assert st == 0, lib.cpt_last_error_string()
    torch.cuda.synchronize()
    free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
    st = static_build(*head, *tail, None)
    assert st == 0, lib.cpt_last_error_string()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_reserved() == reserved0
    got = _host(out)
    del keep

    d = abi.SceneDesc()
    m = d.add_material((0.5, 0.5, 0.5))
    d.spheres = [dict(center=tuple(c), radius=float(r), material=m)
                 for c, r in zip(ctr, np.linspace(0.2, 0.6, n_sph))]
    d.tri_vertices = tri
    d.tri_material = np.zeros(n_tri, np.uint32)
    d.bounds_min, d.bounds_max = bmin, bmax
    d.camera = abi.Camera(8, 1.0, (0, 0, 5), (0, 0, 0), 40.0)
    G = oracle_mod.OracleScene(d).lbvh()
    assert np.array_equal(got["keys"].view(np.uint64), G["keys"])
    assert np.array_equal(got["order"].view(np.uint32), G["order"])
    assert np.array_equal(got["children"][:, 0], G["child_a"])
    assert np.array_equal(got["children"][:, 1], G["child_b"])
    for k, gk in (("node_boxes", "node_boxes"), ("leaf_boxes", "leaf_boxes")):
        lo, hi = outward_f32(G[gk][:, :3], G[gk][:, 3:])
        assert np.array_equal(got[k][:, 0:3], lo), k
        assert np.array_equal(got[k][:, 4:7], hi), k
