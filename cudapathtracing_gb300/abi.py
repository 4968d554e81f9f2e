"""ctypes mirror of include/cpt.h (data layouts only) and a scene-description builder.

The structures here match the C declarations field for field; `SceneDesc` owns the numpy
arrays a `cpt_scene_desc` points into, so the pointers stay valid while it is alive.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

# cpt_status
CPT_OK = 0
STATUS_NAMES = {
    0: "CPT_OK",
    1: "CPT_ERR_INVALID_ARGUMENT",
    2: "CPT_ERR_CUDA",
    3: "CPT_ERR_OUT_OF_MEMORY",
    4: "CPT_ERR_TIMEOUT",
    5: "CPT_ERR_STACK_OVERFLOW",
    6: "CPT_ERR_PARSE",
    7: "CPT_ERR_NOT_BUILT",
    8: "CPT_ERR_UNSUPPORTED",
    9: "CPT_ERR_IO",
}

# cpt_material_type — values 0..5 are the reference's MaterialType (rtmath.cuh:15)
M_NONE, M_LIGHT, M_OPAQUE, M_SPECULAR_DIELECTRIC, M_ROUGH_DIELECTRIC, M_VOLUME, M_LAMBERTIAN = range(7)

ESTIMATOR_REFERENCE = 0
ESTIMATOR_CONFIG = 1
INTEGRATOR_MEGAKERNEL = 0
INTEGRATOR_WAVEFRONT = 1
RENDER_ACCUMULATE = 1


class cpt_material(C.Structure):
    _fields_ = [
        ("color", C.c_double * 3),
        ("alpha_x", C.c_double),
        ("alpha_y", C.c_double),
        ("type", C.c_int32),
        ("texture", C.c_int32),
        ("eta", C.c_double),
        ("sigma_t", C.c_double),
        ("albedo", C.c_double),
    ]


class cpt_light(C.Structure):
    _fields_ = [
        ("center", C.c_double * 3),
        ("normal", C.c_double * 3),
        ("width", C.c_double),
        ("height", C.c_double),
        ("color", C.c_double * 3),
        ("visible", C.c_int32),
        ("reserved", C.c_int32),
    ]


class cpt_sphere(C.Structure):
    _fields_ = [
        ("center", C.c_double * 3),
        ("radius", C.c_double),
        ("material", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class cpt_filter_params(C.Structure):
    _fields_ = [("sigma_g", C.c_float), ("sigma_r", C.c_float), ("sigma_n", C.c_float), ("sigma_d", C.c_float),
                ("radius", C.c_int32)]


def filter_params(sigma_g=8.0, sigma_r=5.0, sigma_n=0.1, sigma_d=0.2, radius=16) -> cpt_filter_params:
    """Defaults of the reference's real-time filter (Window.cu:11-14, Render.cuh:8)."""
    return cpt_filter_params(sigma_g, sigma_r, sigma_n, sigma_d, radius)


class cpt_camera(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("aspect_ratio", C.c_double),
        ("look_from", C.c_double * 3),
        ("look_at", C.c_double * 3),
        ("vfov_deg", C.c_double),
        ("background", C.c_double * 3),
    ]


class cpt_image(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", C.POINTER(C.c_uint8))]


class cpt_scene_desc(C.Structure):
    _fields_ = [
        ("num_lights", C.c_uint32),
        ("lights", C.POINTER(cpt_light)),
        ("num_spheres", C.c_uint32),
        ("spheres", C.POINTER(cpt_sphere)),
        ("num_triangles", C.c_uint32),
        ("tri_vertices", C.POINTER(C.c_float)),
        ("tri_vertices_f64", C.POINTER(C.c_double)),
        ("tri_normals", C.POINTER(C.c_float)),
        ("tri_material", C.POINTER(C.c_uint32)),
        ("num_materials", C.c_uint32),
        ("materials", C.POINTER(cpt_material)),
        ("bounds_min", C.c_double * 3),
        ("bounds_max", C.c_double * 3),
        ("camera", cpt_camera),
        ("tri_uvs", C.POINTER(C.c_float)),
        ("num_textures", C.c_uint32),
        ("textures", C.POINTER(cpt_image)),
        ("sky", cpt_image),
    ]


class cpt_ray(C.Structure):
    _fields_ = [
        ("origin", C.c_float * 3),
        ("tmin", C.c_float),
        ("direction", C.c_float * 3),
        ("tmax", C.c_float),
    ]


class cpt_hit(C.Structure):
    _fields_ = [("t", C.c_float), ("prim", C.c_int32), ("u", C.c_float), ("v", C.c_float)]


class cpt_bvh_stats(C.Structure):
    _fields_ = [
        ("num_prims", C.c_uint32),
        ("max_depth", C.c_uint32),
        ("num_wide_nodes", C.c_uint32),
        ("reserved", C.c_uint32),
        ("ms_prep", C.c_float),
        ("ms_sort", C.c_float),
        ("ms_emit", C.c_float),
        ("ms_refit", C.c_float),
        ("ms_collapse", C.c_float),
        ("ms_total", C.c_float),
    ]


class cpt_render_params(C.Structure):
    _fields_ = [
        ("spp", C.c_int32),
        ("estimator", C.c_int32),
        ("integrator", C.c_int32),
        ("max_depth", C.c_int32),
        ("rr_depth", C.c_int32),
        ("rr_prob", C.c_float),
        ("seed", C.c_uint64),
        ("row_begin", C.c_int32),
        ("row_end", C.c_int32),
        ("flags", C.c_int32),
        ("reserved", C.c_int32),
    ]


class cpt_render_output(C.Structure):
    _fields_ = [
        ("rgb", C.c_void_p),
        ("rgba8", C.c_void_p),
        ("gbuffer", C.c_void_p),
        ("on_device", C.c_int32),
        ("reserved", C.c_int32),
    ]


class cpt_render_job(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("params", cpt_render_params), ("output", cpt_render_output)]


class cpt_render_stats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("paths", C.c_uint64), ("ms", C.c_double)]


RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("tmin", "<f4"), ("direction", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<i4"), ("u", "<f4"), ("v", "<f4")])
assert RAY_DTYPE.itemsize == C.sizeof(cpt_ray) == 32
assert HIT_DTYPE.itemsize == C.sizeof(cpt_hit) == 16


def render_params(spp=1, estimator=ESTIMATOR_REFERENCE, integrator=INTEGRATOR_MEGAKERNEL, max_depth=0,
                  rr_depth=0, rr_prob=0.7, seed=0, row_begin=0, row_end=0, flags=0) -> cpt_render_params:
    return cpt_render_params(spp, estimator, integrator, max_depth, rr_depth, rr_prob, seed, row_begin, row_end,
                             flags, 0)


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


@dataclass
class Camera:
    """Pinhole camera (Camera.cu:5-40); height follows the reference rule."""
    width: int = 800
    aspect_ratio: float = 16.0 / 9.0
    look_from: tuple = (0.0, 0.0, 1.0)
    look_at: tuple = (0.0, 0.0, 0.0)
    vfov_deg: float = 90.0
    background: tuple = (0.0, 0.0, 0.0)

    @property
    def height(self) -> int:
        h = self.width / self.aspect_ratio
        return 1 if h < 1 else int(h)

    def to_c(self) -> cpt_camera:
        return cpt_camera(int(self.width), int(self.height), float(self.aspect_ratio), (C.c_double * 3)(*self.look_from),
                          (C.c_double * 3)(*self.look_at), float(self.vfov_deg), (C.c_double * 3)(*self.background))


@dataclass
class SceneDesc:
    """Host-side scene in the C-ABI's layout (primitive order: lights, spheres, triangles)."""
    lights: list = field(default_factory=list)        # dicts: center, normal, width, height, color, visible
    spheres: list = field(default_factory=list)       # dicts: center, radius, material
    materials: list = field(default_factory=list)     # dicts: color, alpha_x, alpha_y, type, eta, sigma_t, albedo
    tri_vertices: np.ndarray | None = None            # (T, 9) float32 or float64
    tri_normals: np.ndarray | None = None             # (T, 9) float32
    tri_material: np.ndarray | None = None            # (T,) uint32
    tri_uvs: np.ndarray | None = None                 # (T, 6) float32: uv0, uv1, uv2
    textures: list = field(default_factory=list)      # (h, w, 3) uint8 images; material texture k -> [k-1]
    sky: np.ndarray | None = None                     # (h, w, 3) uint8 equirectangular sky image
    bounds_min: tuple = (999999.0,) * 3
    bounds_max: tuple = (-999999.0,) * 3
    camera: Camera = field(default_factory=Camera)

    @property
    def num_triangles(self) -> int:
        return 0 if self.tri_vertices is None else int(self.tri_vertices.shape[0])

    @property
    def num_prims(self) -> int:
        return len(self.lights) + len(self.spheres) + self.num_triangles

    def add_material(self, color, alpha_x=0.5, alpha_y=0.5, type=M_OPAQUE, eta=1.51, sigma_t=0.0, albedo=0.0,
                     texture=0) -> int:
        self.materials.append(dict(color=tuple(color), alpha_x=alpha_x, alpha_y=alpha_y, type=type, eta=eta,
                                   sigma_t=sigma_t, albedo=albedo, texture=texture))
        return len(self.materials) - 1

    def add_texture(self, rgb: np.ndarray) -> int:
        """Registers an (h, w, 3) uint8 image; returns the material texture number (1-based)."""
        rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
        assert rgb.ndim == 3 and rgb.shape[2] == 3
        self.textures.append(rgb)
        return len(self.textures)

    def to_c(self):
        """Returns (cpt_scene_desc, keepalive) — keep `keepalive` referenced during the call."""
        keep = []
        d = cpt_scene_desc()
        if self.lights:
            arr = (cpt_light * len(self.lights))()
            for i, L in enumerate(self.lights):
                arr[i] = cpt_light((C.c_double * 3)(*L["center"]), (C.c_double * 3)(*L["normal"]), L["width"],
                                   L["height"], (C.c_double * 3)(*L["color"]), int(L.get("visible", 1)), 0)
            keep.append(arr)
            d.lights = C.cast(arr, C.POINTER(cpt_light))
        d.num_lights = len(self.lights)
        if self.spheres:
            arr = (cpt_sphere * len(self.spheres))()
            for i, S in enumerate(self.spheres):
                arr[i] = cpt_sphere((C.c_double * 3)(*S["center"]), S["radius"], S["material"], 0)
            keep.append(arr)
            d.spheres = C.cast(arr, C.POINTER(cpt_sphere))
        d.num_spheres = len(self.spheres)
        mats = self.materials or [dict(color=(1.0, 1.0, 1.0), alpha_x=0.5, alpha_y=0.5, type=M_OPAQUE, eta=1.51,
                                       sigma_t=0.0, albedo=0.0)]
        marr = (cpt_material * len(mats))()
        for i, m in enumerate(mats):
            marr[i] = cpt_material((C.c_double * 3)(*m["color"]), m["alpha_x"], m["alpha_y"], int(m["type"]),
                                   int(m.get("texture", 0)), m.get("eta", 1.51), m.get("sigma_t", 0.0),
                                   m.get("albedo", 0.0))
        keep.append(marr)
        d.materials = C.cast(marr, C.POINTER(cpt_material))
        d.num_materials = len(mats)
        T = self.num_triangles
        d.num_triangles = T
        if T:
            tv = np.ascontiguousarray(self.tri_vertices)
            keep.append(tv)
            if tv.dtype == np.float64:
                d.tri_vertices_f64 = _ptr(tv, C.c_double)
            else:
                tv = np.ascontiguousarray(tv, dtype=np.float32)
                keep.append(tv)
                d.tri_vertices = _ptr(tv, C.c_float)
            if self.tri_normals is not None:
                tn = np.ascontiguousarray(self.tri_normals, dtype=np.float32)
                keep.append(tn)
                d.tri_normals = _ptr(tn, C.c_float)
            tm = (np.zeros(T, np.uint32) if self.tri_material is None
                  else np.ascontiguousarray(self.tri_material, dtype=np.uint32))
            keep.append(tm)
            d.tri_material = _ptr(tm, C.c_uint32)
            if self.tri_uvs is not None:
                tu = np.ascontiguousarray(self.tri_uvs, dtype=np.float32).reshape(T, 6)
                keep.append(tu)
                d.tri_uvs = _ptr(tu, C.c_float)

        def image(a):
            a = np.ascontiguousarray(a, dtype=np.uint8)
            keep.append(a)
            return cpt_image(int(a.shape[1]), int(a.shape[0]), _ptr(a, C.c_uint8))
        if self.textures:
            tarr = (cpt_image * len(self.textures))(*[image(t) for t in self.textures])
            keep.append(tarr)
            d.textures = C.cast(tarr, C.POINTER(cpt_image))
        d.num_textures = len(self.textures)
        if self.sky is not None:
            d.sky = image(self.sky)
        d.bounds_min = (C.c_double * 3)(*self.bounds_min)
        d.bounds_max = (C.c_double * 3)(*self.bounds_max)
        d.camera = self.camera.to_c()
        return d, keep
