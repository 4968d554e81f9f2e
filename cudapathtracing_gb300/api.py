"""Host API over libcpt.so, named after the reference's interfaces.

  IniParser.Parse(path)           — IniParser::Parse (IniParser.cpp:3) + Scene::init assembly
  Context(device)                 — the reference's Device ctor (Device.cuh:161), minus its
                                    fixed 2,000,000-object pool
  Scene(ctx, desc).init()         — Scene::init (Scene.cuh:72): upload + LBVH build
  Scene.buildBVH() / .refit()     — Device::buildBVH (Device.cuh:169) / refit only
  Scene.Update(vertices)          — Scene::Update (Scene.cuh:147): new vertices, rebuild
  Scene.render(...)               — render (Render.cu:16), STATIC mode
  Scene.trace(rays)               — traverseIterative (BVH.cuh:282) for a batch of rays
  Device.buildBVH(...)            — the device-pointer build on caller-owned buffers
  filter_bilateral / filter_temporal — gaussianSeparate (Render.cu:356-398) / addPrevious
                                    (Render.cu:400-420) on device tensors

Everything goes through the C ABI; there is no Python or CPU compute path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._lib import check, lib


def _vp(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    if hasattr(a, "data_ptr"):   # torch tensor
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(a)


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().cpt_context_create(device, C.byref(h)), "cpt_context_create")
        self.h = h
        self.device = device

    def set_render_block(self, bx: int, by: int) -> None:
        check(lib().cpt_context_set_render_block(self.h, bx, by), "cpt_context_set_render_block")

    def set_bvh_width(self, width: int) -> None:
        check(lib().cpt_context_set_bvh_width(self.h, width), "cpt_context_set_bvh_width")

    def set_wavefront(self, slots: int, block_trace: int = 128, block_shade: int = 128, use_graph: int = 1) -> None:
        check(lib().cpt_context_set_wavefront(self.h, slots, block_trace, block_shade, use_graph),
              "cpt_context_set_wavefront")

    def set_bvh_compression(self, on: bool) -> None:
        """32-byte quantised BVH2 nodes for later builds (cpt_context_set_bvh_compression)."""
        check(lib().cpt_context_set_bvh_compression(self.h, 1 if on else 0), "cpt_context_set_bvh_compression")

    def set_material_sort(self, on: bool) -> None:
        """Wavefront shade queue binned by material (cpt_context_set_material_sort)."""
        check(lib().cpt_context_set_material_sort(self.h, 1 if on else 0), "cpt_context_set_material_sort")

    def set_loop_limits(self, max_trips: int = 1 << 16, max_replays: int = 1 << 20) -> None:
        """Device loop bounds (cpt_context_set_loop_limits); the defaults are the maxima."""
        check(lib().cpt_context_set_loop_limits(self.h, max_trips, max_replays), "cpt_context_set_loop_limits")

    def set_short_stack(self, entries: int) -> None:
        check(lib().cpt_context_set_short_stack(self.h, entries), "cpt_context_set_short_stack")

    def close(self):
        if self.h:
            lib().cpt_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class IniParser:
    """Parses a scene file with the library's native parser (no GPU needed)."""

    def __init__(self):
        self.h = None
        self.desc = None

    def Parse(self, filename: str) -> None:
        h = C.c_void_p()
        check(lib().cpt_ini_load(filename.encode(), C.byref(h)), "cpt_ini_load")
        self.h = h
        d = abi.cpt_scene_desc()
        check(lib().cpt_ini_describe(h, C.byref(d)), "cpt_ini_describe")
        self.desc = d

    def to_scene_desc(self) -> abi.SceneDesc:
        """Copy of the assembled scene as an abi.SceneDesc (owning numpy arrays)."""
        d = self.desc
        sd = abi.SceneDesc()
        for i in range(d.num_lights):
            L = d.lights[i]
            sd.lights.append(dict(center=tuple(L.center), normal=tuple(L.normal), width=L.width, height=L.height,
                                  color=tuple(L.color), visible=L.visible))
        for i in range(d.num_materials):
            m = d.materials[i]
            sd.materials.append(dict(color=tuple(m.color), alpha_x=m.alpha_x, alpha_y=m.alpha_y, type=m.type, eta=m.eta,
                                     sigma_t=m.sigma_t, albedo=m.albedo, texture=m.texture))
        for i in range(d.num_spheres):
            S = d.spheres[i]
            sd.spheres.append(dict(center=tuple(S.center), radius=S.radius, material=S.material))
        T = d.num_triangles
        if T:
            sd.tri_vertices = np.ctypeslib.as_array(d.tri_vertices_f64, shape=(T * 9,)).reshape(T, 9).copy()
            sd.tri_material = np.ctypeslib.as_array(d.tri_material, shape=(T,)).copy()
            if d.tri_uvs:
                sd.tri_uvs = np.ctypeslib.as_array(d.tri_uvs, shape=(T * 6,)).reshape(T, 6).copy()
            if d.tri_normals:
                sd.tri_normals = np.ctypeslib.as_array(d.tri_normals, shape=(T * 9,)).reshape(T, 9).copy()

        def image(im):
            return np.ctypeslib.as_array(im.rgb, shape=(im.height * im.width * 3,)).reshape(im.height, im.width, 3).copy()
        sd.textures = [image(d.textures[i]) for i in range(d.num_textures)]
        sd.sky = image(d.sky) if d.sky.rgb else None
        sd.bounds_min = tuple(d.bounds_min)
        sd.bounds_max = tuple(d.bounds_max)
        c = d.camera
        sd.camera = abi.Camera(c.width, c.aspect_ratio, tuple(c.look_from), tuple(c.look_at), c.vfov_deg,
                               tuple(c.background))
        return sd

    def __del__(self):
        if self.h:
            try:
                lib().cpt_ini_free(self.h)
            except Exception:
                pass
            self.h = None


class Scene:
    """A scene resident on the GPU with its LBVH."""

    def __init__(self, ctx: Context, desc: abi.SceneDesc | None = None, ini_path: str | None = None):
        self.ctx = ctx
        h = C.c_void_p()
        if ini_path is not None:
            check(lib().cpt_scene_load_ini(ctx.h, ini_path.encode(), C.byref(h)), "cpt_scene_load_ini")
        else:
            cd, keep = desc.to_c()
            check(lib().cpt_scene_create(ctx.h, C.byref(cd), C.byref(h)), "cpt_scene_create")
        self.h = h
        nl, ns, nt = C.c_uint32(), C.c_uint32(), C.c_uint32()
        cam = abi.cpt_camera()
        check(lib().cpt_scene_info(h, C.byref(nl), C.byref(ns), C.byref(nt), C.byref(cam)), "cpt_scene_info")
        self.num_lights, self.num_spheres, self.num_triangles = nl.value, ns.value, nt.value
        self.num_prims = self.num_lights + self.num_spheres + self.num_triangles
        self.width, self.height = cam.width, cam.height
        self.stats = None

    # Scene::init — upload happened in __init__; build the LBVH.
    def init(self, stream=None) -> "Scene":
        self.buildBVH(stream)
        return self

    def buildBVH(self, stream=None) -> abi.cpt_bvh_stats:
        st = abi.cpt_bvh_stats()
        check(lib().cpt_lbvh_build(self.h, _vp(stream), C.byref(st)), "cpt_lbvh_build")
        self.stats = st
        return st

    def refit(self, stream=None) -> abi.cpt_bvh_stats:
        st = abi.cpt_bvh_stats()
        check(lib().cpt_lbvh_refit(self.h, _vp(stream), C.byref(st)), "cpt_lbvh_refit")
        return st

    def Update(self, tri_vertices: np.ndarray, first: int = 0, rebuild: bool = True, stream=None):
        """New FP32 vertices for triangles [first, first+len), then a full rebuild (the
        reference rebuilds every frame) or a refit when rebuild is False."""
        tv = np.ascontiguousarray(tri_vertices, np.float32).reshape(-1, 9)
        check(lib().cpt_scene_update_triangles(self.h, _vp(tv), first, tv.shape[0], _vp(stream)),
              "cpt_scene_update_triangles")
        return self.buildBVH(stream) if rebuild else self.refit(stream)

    def export_lbvh(self) -> dict:
        n = self.num_prims
        ni = max(n - 1, 0)
        out = dict(keys=np.zeros(n, np.uint64), order=np.zeros(n, np.uint32), child_a=np.zeros(ni, np.int32),
                   child_b=np.zeros(ni, np.int32), node_boxes=np.zeros((ni, 6), np.float32),
                   leaf_boxes=np.zeros((n, 6), np.float32))
        check(lib().cpt_lbvh_export(self.h, *(_vp(out[k]) for k in ("keys", "order", "child_a", "child_b",
                                                                     "node_boxes", "leaf_boxes"))),
              "cpt_lbvh_export")
        return out

    def trace(self, rays, hits=None, stream=None):
        """Closest hits.  numpy structured arrays (abi.RAY_DTYPE) are traced through host
        buffers; torch CUDA tensors of shape (n, 8) float32 are traced in place on the device
        (hits: (n, 4) tensor, viewed as t, prim, u, v)."""
        if isinstance(rays, np.ndarray):
            rays = np.ascontiguousarray(rays)
            out = np.zeros(rays.shape[0], abi.HIT_DTYPE)
            check(lib().cpt_trace_closest(self.h, _vp(rays), rays.shape[0], _vp(out), 0, _vp(stream)),
                  "cpt_trace_closest")
            return out
        n = rays.shape[0]
        check(lib().cpt_trace_closest(self.h, _vp(rays), n, _vp(hits), 1, _vp(stream)), "cpt_trace_closest")
        return hits

    def render(self, spp: int = 1, estimator: int = abi.ESTIMATOR_REFERENCE, integrator: int = abi.INTEGRATOR_MEGAKERNEL,
               max_depth: int = 0, rr_depth: int = 0, rr_prob: float = 0.7, seed: int = 0, rows=(0, 0),
               rgb=None, rgba8=None, gbuffer=None, flags: int = 0, stream=None, want_rgba8: bool = True):
        """Render the camera view.  With no output buffers, host numpy arrays are returned;
        torch CUDA tensors may be passed as rgb (H, W, 3) / rgba8 (H, W, 4) / gbuffer (H, W, 8)."""
        params = abi.render_params(spp, estimator, integrator, max_depth, rr_depth, rr_prob, seed, rows[0], rows[1],
                                   flags)
        on_device = rgb is not None and not isinstance(rgb, np.ndarray)
        if rgb is None:
            rgb = np.zeros((self.height, self.width, 3), np.float32)
            if want_rgba8:
                rgba8 = np.zeros((self.height, self.width, 4), np.uint8)
        out = abi.cpt_render_output(_vp(rgb).value if rgb is not None else None,
                                    _vp(rgba8).value if rgba8 is not None else None,
                                    _vp(gbuffer).value if gbuffer is not None else None, 1 if on_device else 0, 0)
        st = abi.cpt_render_stats()
        check(lib().cpt_render(self.h, C.byref(params), C.byref(out), _vp(stream), C.byref(st)), "cpt_render")
        return dict(rgb=rgb, rgba8=rgba8, gbuffer=gbuffer, rays=int(st.rays), paths=int(st.paths), ms=float(st.ms))

    def pick(self, x: int, y: int) -> int:
        """getObject (Render.cu:485-496): primitive under pixel (x, y), -1 on a miss or a light."""
        out = C.c_int32()
        check(lib().cpt_pick(self.h, int(x), int(y), C.byref(out)), "cpt_pick")
        return out.value

    def set_material(self, first: int, end: int, alpha_x: float, alpha_y: float, glass: bool) -> None:
        """changeMaterial (Render.cu:498-522) over primitives [first, end)."""
        check(lib().cpt_scene_set_material(self.h, int(first), int(end), float(alpha_x), float(alpha_y),
                                           1 if glass else 0), "cpt_scene_set_material")

    def close(self):
        if self.h:
            lib().cpt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Device:
    """Device::buildBVH on caller-owned device buffers (torch CUDA tensors)."""

    @staticmethod
    def scratch_bytes(n: int) -> int:
        return int(lib().cpt_lbvh_scratch_bytes(n))

    @staticmethod
    def buildBVH(extra_centroids, extra_boxes, tri_vertices, scene_min, scene_max, out: dict, scratch, stream=None):
        """All arrays are torch CUDA tensors; `out` holds keys (N, int64), order (N, int32),
        children (N-1, 2), node_range (N-1, 2), node_boxes (N-1, 8), leaf_boxes (N, 8)."""
        ne = 0 if extra_centroids is None else int(extra_centroids.shape[0])
        nt = 0 if tri_vertices is None else int(tri_vertices.shape[0])
        smin = (C.c_double * 3)(*scene_min)
        smax = (C.c_double * 3)(*scene_max)
        check(lib().cpt_lbvh_build_device(ne, _vp(extra_centroids), _vp(extra_boxes), nt, _vp(tri_vertices), smin, smax,
                                          _vp(out.get("keys")), _vp(out["order"]), _vp(out.get("children")),
                                          _vp(out.get("node_range")), _vp(out.get("node_boxes")),
                                          _vp(out["leaf_boxes"]), _vp(scratch), scratch.numel() * scratch.element_size(),
                                          _vp(stream)),
              "cpt_lbvh_build_device")


def _cam(c):
    return c.to_c() if hasattr(c, "to_c") else c


def filter_bilateral(ctx: Context, rgb, gbuf, out=None, params: abi.cpt_filter_params | None = None, stream=None):
    """Joint-bilateral filter of a device image [H, W, 3] float32 with the renderer's G-buffer
    [H, W, 8] float32; returns `out` (allocated like rgb when None)."""
    import torch
    if out is None:
        out = torch.empty_like(rgb)
    H, W = int(rgb.shape[0]), int(rgb.shape[1])
    check(lib().cpt_filter_bilateral(ctx.h, _vp(rgb), _vp(gbuf), _vp(out), W, H,
                                     C.byref(params) if params is not None else None, _vp(stream)),
          "cpt_filter_bilateral")
    return out


def filter_temporal(ctx: Context, rgb, prev, gbuf, camera, prev_camera, alpha: float = 0.1, stream=None):
    """In place: rgb = alpha * rgb + (1 - alpha) * prev at the reprojected pixel (device tensors)."""
    c, pc = _cam(camera), _cam(prev_camera)
    check(lib().cpt_filter_temporal(ctx.h, _vp(rgb), _vp(prev), _vp(gbuf), C.byref(c), C.byref(pc), float(alpha),
                                    _vp(stream)), "cpt_filter_temporal")
    return rgb


def render_batch(ctx: Context, jobs: list, stream=None) -> dict:
    """Renders several jobs in one wavefront (cpt_render_batch).  Each job is a dict with "scene"
    (a built Scene of ctx), the render parameters of Scene.render (spp, max_depth, rr_depth,
    rr_prob, seed, rows, flags; the config estimator) and optionally "rgb" / "rgba8" / "gbuffer"
    outputs (torch CUDA tensors, or omitted for host numpy arrays, as in Scene.render).  Returns
    the batch's stats and the jobs' outputs."""
    arr = (abi.cpt_render_job * len(jobs))()
    outs = []
    for i, j in enumerate(jobs):
        sc = j["scene"]
        rows = j.get("rows", (0, 0))
        params = abi.render_params(j.get("spp", 1), abi.ESTIMATOR_CONFIG, abi.INTEGRATOR_WAVEFRONT,
                                   j.get("max_depth", 0), j.get("rr_depth", 0), j.get("rr_prob", 0.8),
                                   j.get("seed", 0), rows[0], rows[1], j.get("flags", 0))
        rgb, rgba8, gbuf = j.get("rgb"), j.get("rgba8"), j.get("gbuffer")
        on_device = rgb is not None and not isinstance(rgb, np.ndarray)
        if rgb is None:
            rgb = np.zeros((sc.height, sc.width, 3), np.float32)
            rgba8 = np.zeros((sc.height, sc.width, 4), np.uint8) if j.get("want_rgba8", True) else None
        out = abi.cpt_render_output(_vp(rgb).value, _vp(rgba8).value if rgba8 is not None else None,
                                    _vp(gbuf).value if gbuf is not None else None, 1 if on_device else 0, 0)
        arr[i] = abi.cpt_render_job(sc.h.value if hasattr(sc.h, "value") else sc.h, params, out)
        outs.append(dict(rgb=rgb, rgba8=rgba8, gbuffer=gbuf))
    st = abi.cpt_render_stats()
    check(lib().cpt_render_batch(ctx.h, arr, len(jobs), _vp(stream), C.byref(st)), "cpt_render_batch")
    return dict(jobs=outs, rays=int(st.rays), paths=int(st.paths), ms=float(st.ms))
