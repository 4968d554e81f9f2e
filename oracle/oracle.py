"""TEST INFRASTRUCTURE ONLY — ctypes wrappers of the FP64 CPU oracle (oracle/_build/
libcpt_oracle.so, a restatement of the reference's path) and, where it was built, of the
reference's own code (oracle/_ref/libcpt_ref.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module;
the shipped library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from cudapathtracing_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libcpt_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libcpt_ref.so")

_oracle = None
_ref = None


def build(ref: bool = True) -> None:
    """Builds the oracle (and the reference harness when the reference is mounted)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all" if ref else "oracle"])


def reference_dir() -> str | None:
    """The reference's source folder as oracle/Makefile names it, or None where it is absent."""
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    d = r.stdout.strip()
    return d if r.returncode == 0 and d and os.path.isdir(d) else None


def _sig(lib):
    P = C.c_void_p
    lib.orc_scene_create.restype = P
    lib.orc_scene_create.argtypes = [C.POINTER(abi.cpt_scene_desc)]
    lib.orc_scene_destroy.argtypes = [P]
    lib.orc_scene_size.restype = C.c_int
    lib.orc_scene_size.argtypes = [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.orc_lbvh_export.restype = C.c_int
    lib.orc_lbvh_export.argtypes = [P] * 8
    lib.orc_trace.argtypes = [P, P, C.c_int64, P, P, P, P, C.c_int]
    lib.orc_prim_t.argtypes = [P, P, C.c_int64, P, P]
    lib.orc_trace_counts.argtypes = [P, P, C.c_int64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int]
    lib.orc_render.restype = C.c_uint64
    lib.orc_render.argtypes = [P, C.POINTER(abi.cpt_render_params), P, P, P, C.c_int]
    lib.orc_render_visit_counts.argtypes = [P, C.POINTER(abi.cpt_render_params), C.c_int, P]
    lib.orc_pick.restype = C.c_int
    lib.orc_pick.argtypes = [P, C.c_int, C.c_int]
    lib.orc_set_material.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        _oracle = C.CDLL(ORACLE_SO)
        _sig(_oracle)
    return _oracle


def ref_lib():
    """The reference's own code, or None where it was not built (e.g. on the GPU machine)."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        lib = C.CDLL(REF_SO)
        P = C.c_void_p
        lib.ref_scene_create.restype = P
        lib.ref_scene_create.argtypes = [C.POINTER(abi.cpt_scene_desc)]
        lib.ref_scene_create_ini.restype = P
        lib.ref_scene_create_ini.argtypes = [C.c_char_p]
        lib.ref_scene_destroy.argtypes = [P]
        lib.ref_scene_size.restype = C.c_int
        lib.ref_scene_size.argtypes = [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.ref_lbvh_export.argtypes = [P] * 8
        lib.ref_trace.argtypes = [P, P, C.c_int64, P, P]
        lib.ref_render.argtypes = [P, C.c_int, C.c_uint64, C.c_int, C.c_int, P, P, C.c_int]
        lib.ref_ini_dump.restype = C.c_int
        lib.ref_ini_dump.argtypes = [C.c_char_p, P, C.c_int]
        if hasattr(lib, "ref_pick"):
            lib.ref_pick.restype = C.c_int
            lib.ref_pick.argtypes = [P, C.c_int, C.c_int]
            lib.ref_change_material.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        if hasattr(lib, "ref_gaussian_separate"):
            D = C.c_double
            lib.ref_gaussian_separate.argtypes = [P, P, P, D, D, D, D, C.c_int, C.c_int, C.c_int]
            lib.ref_add_previous.argtypes = [P, P, P, C.POINTER(abi.cpt_camera), P, P, C.c_int]
        _ref = lib
    return _ref


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class _SceneBase:
    def _size(self):
        w, h = C.c_int(), C.c_int()
        n = self._lib_size(self.h, C.byref(w), C.byref(h))
        return n, w.value, h.value

    def lbvh(self) -> dict:
        n = self.n
        out = dict(keys=np.zeros(n, np.uint64), order=np.zeros(n, np.uint32),
                   child_a=np.zeros(max(n - 1, 0), np.int32), child_b=np.zeros(max(n - 1, 0), np.int32),
                   node_boxes=np.zeros((max(n - 1, 0), 6)), leaf_boxes=np.zeros((n, 6)), centroids=np.zeros((n, 3)))
        self._lib_export(self.h, *(_p(out[k]) for k in ("keys", "order", "child_a", "child_b", "node_boxes",
                                                         "leaf_boxes", "centroids")))
        return out


class OracleScene(_SceneBase):
    """FP64 restated oracle over a SceneDesc."""

    def __init__(self, desc: abi.SceneDesc):
        lib = oracle_lib()
        self.lib = lib
        cd, self._keep = desc.to_c()
        self.h = lib.orc_scene_create(C.byref(cd))
        if not self.h:
            raise ValueError("oracle rejected the scene description")
        self._lib_size = lib.orc_scene_size
        self._lib_export = lib.orc_lbvh_export
        self.n, self.width, self.height = self._size()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_scene_destroy(self.h)
            self.h = None

    def trace(self, rays_f64: np.ndarray, threads: int = 0):
        rays_f64 = np.ascontiguousarray(rays_f64, np.float64)
        n = rays_f64.shape[0]
        ids = np.empty(n, np.int32)
        t, u, v = np.empty(n), np.empty(n), np.empty(n)
        self.lib.orc_trace(self.h, _p(rays_f64), n, _p(ids), _p(t), _p(u), _p(v), threads)
        return ids, t, u, v

    def prim_t(self, rays_f64: np.ndarray, prims: np.ndarray) -> np.ndarray:
        rays_f64 = np.ascontiguousarray(rays_f64, np.float64)
        prims = np.ascontiguousarray(prims, np.int32)
        out = np.empty(rays_f64.shape[0])
        self.lib.orc_prim_t(self.h, _p(rays_f64), rays_f64.shape[0], _p(prims), _p(out))
        return out

    def trace_counts(self, rays_f64: np.ndarray, threads: int = 0):
        rays_f64 = np.ascontiguousarray(rays_f64, np.float64)
        vi, vl = C.c_uint64(), C.c_uint64()
        self.lib.orc_trace_counts(self.h, _p(rays_f64), rays_f64.shape[0], C.byref(vi), C.byref(vl), threads)
        return vi.value, vl.value

    def render_visit_counts(self, params: abi.cpt_render_params, threads: int = 0):
        """(queries, internal-node visits, primitive tests) of the ordered pruned traversal
        over the closest-hit queries a render of params makes."""
        out = np.zeros(3, np.uint64)
        self.lib.orc_render_visit_counts(self.h, C.byref(params), threads, _p(out))
        return tuple(int(x) for x in out)

    def pick(self, x: int, y: int) -> int:
        """getObject (Render.cu:485-496) at pixel (x, y)."""
        return int(self.lib.orc_pick(self.h, int(x), int(y)))

    def set_material(self, first: int, end: int, alpha_x: float, alpha_y: float, glass: bool) -> None:
        """changeMaterial (Render.cu:498-522) over primitives [first, end)."""
        self.lib.orc_set_material(self.h, int(first), int(end), float(alpha_x), float(alpha_y), 1 if glass else 0)

    def render(self, params: abi.cpt_render_params, threads: int = 0, gbuffer: bool = False):
        rgb = np.zeros((self.height, self.width, 3))
        rgba = np.zeros((self.height, self.width, 4), np.uint8)
        gb = np.zeros((self.height, self.width, 8)) if gbuffer else None
        rays = self.lib.orc_render(self.h, C.byref(params), _p(rgb), _p(rgba), _p(gb), threads)
        return dict(rgb=rgb, rgba8=rgba, gbuffer=gb, rays=int(rays))


class RefScene(_SceneBase):
    """The reference's own code over a SceneDesc (or an INI file)."""

    def __init__(self, desc: abi.SceneDesc | None = None, ini_path: str | None = None):
        lib = ref_lib()
        if lib is None:
            raise RuntimeError("oracle/_ref was not built (the reference is not mounted here)")
        self.lib = lib
        if ini_path is not None:
            self.h = lib.ref_scene_create_ini(ini_path.encode())
        else:
            cd, self._keep = desc.to_c()
            self.h = lib.ref_scene_create(C.byref(cd))
        if not self.h:
            raise ValueError("reference harness rejected the scene")
        self._lib_size = lib.ref_scene_size
        self._lib_export = lib.ref_lbvh_export
        self.n, self.width, self.height = self._size()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_scene_destroy(self.h)
            self.h = None

    def trace(self, rays_f64: np.ndarray):
        rays_f64 = np.ascontiguousarray(rays_f64, np.float64)
        n = rays_f64.shape[0]
        ids = np.empty(n, np.int32)
        t = np.empty(n)
        self.lib.ref_trace(self.h, _p(rays_f64), n, _p(ids), _p(t))
        return ids, t

    def pick(self, x: int, y: int) -> int:
        return int(self.lib.ref_pick(self.h, int(x), int(y)))

    def set_material(self, first: int, end: int, alpha_x: float, alpha_y: float, glass: bool) -> None:
        self.lib.ref_change_material(self.h, int(first), int(end), float(alpha_x), float(alpha_y), 1 if glass else 0)

    def render(self, spp: int, seed: int = 0, row_begin: int = 0, row_end: int = 0, threads: int = 0):
        rgb = np.zeros((self.height, self.width, 3))
        rgba = np.zeros((self.height, self.width, 4), np.uint8)
        self.lib.ref_render(self.h, spp, seed, row_begin, row_end, _p(rgb), _p(rgba), threads)
        return dict(rgb=rgb, rgba8=rgba)


def ref_ini_dump(path: str) -> np.ndarray:
    lib = ref_lib()
    buf = np.zeros(65536)
    n = lib.ref_ini_dump(path.encode(), _p(buf), buf.size)
    return buf[:n].copy()


def ref_bilateral(rgb, gbuf4, sigma_g=8.0, sigma_r=5.0, sigma_n=0.1, sigma_d=0.2):
    """The reference's gaussianSeparate run twice as in main.cu:99-103 (horizontal pass, copyPic,
    vertical pass), on FP64 copies; radius is the compiled KERNEL_RADIUS (16)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("oracle/_ref was not built (the reference is not mounted here)")
    H, W, _ = rgb.shape
    pic = np.ascontiguousarray(rgb, dtype=np.float64).copy()
    before = pic.copy()
    g = np.ascontiguousarray(gbuf4, dtype=np.float64)
    L.ref_gaussian_separate(_p(pic), _p(before), _p(g), sigma_g, sigma_r, sigma_n, sigma_d, W, H, 1)
    before = pic.copy()
    L.ref_gaussian_separate(_p(pic), _p(before), _p(g), sigma_g, sigma_r, sigma_n, sigma_d, W, H, 0)
    return pic


def ref_temporal(rgb, prev, gpos, camera, pre_from, pre_at, moving):
    """The reference's addPrevious over the image (alpha 0.1, or 0.4 when moving)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("oracle/_ref was not built (the reference is not mounted here)")
    pic = np.ascontiguousarray(rgb, dtype=np.float64).copy()
    pv = np.ascontiguousarray(prev, dtype=np.float64)
    gp = np.ascontiguousarray(gpos, dtype=np.float64)
    pf = np.asarray(pre_from, dtype=np.float64)
    pa = np.asarray(pre_at, dtype=np.float64)
    cam = camera.to_c() if hasattr(camera, "to_c") else camera
    L.ref_add_previous(_p(pic), _p(pv), _p(gp), C.byref(cam), _p(pf), _p(pa), int(moving))
    return pic
