"""Seeded procedural scenes and ray sets.

The reference's scene files point at OBJ meshes and textures that are not available, so
the workloads are generated here from PCG32 streams (the same generator the renderer
uses).  Everything is deterministic for a given seed and produced with numpy.

  cornell_box()      — 512x512 Cornell box: 5 wall quads, 2 boxes rotated +-18 deg about y,
                       a 0.5x0.5 emissive ceiling light with radiance 15 (34 triangles + 1 light)
  icosphere_scene()  — icosphere subdivided 8 times (1,310,720 triangles) displaced radially by
                       seeded 3-octave value noise with amplitude 0.1
  uniform_rays()     — origins uniform in [-2,2]^3, directions uniform on the sphere
  spheres_scene()    — 1920x1080: 200 displaced level-5 icospheres on a ground plane, materials
                       Lambertian / GGX / dielectric by index mod 3, a homogeneous volume box,
                       two area lights
"""
from __future__ import annotations

import math

import numpy as np

from .abi import (M_LAMBERTIAN, M_LIGHT, M_OPAQUE, M_SPECULAR_DIELECTRIC, M_VOLUME, RAY_DTYPE, Camera,
                  SceneDesc)

_MULT = np.uint64(6364136223846793005)


class PCG32Streams:
    """Vectorised PCG32 (O'Neill 2014): one independent stream per element."""

    def __init__(self, seed: int, streams):
        streams = np.asarray(streams, dtype=np.uint64)
        with np.errstate(over="ignore"):
            self.inc = (streams << np.uint64(1)) | np.uint64(1)
            self.state = np.zeros_like(streams)
            self.next()
            self.state = self.state + np.uint64(seed)
            self.next()

    def next(self) -> np.ndarray:
        old = self.state
        with np.errstate(over="ignore"):
            self.state = old * _MULT + self.inc
        xs = (((old >> np.uint64(18)) ^ old) >> np.uint64(27)).astype(np.uint32)
        rot = (old >> np.uint64(59)).astype(np.uint32)
        return ((xs >> rot) | (xs << ((np.uint32(32) - rot) & np.uint32(31)))).astype(np.uint32)

    def uniform(self) -> np.ndarray:
        """(x + 1) * 2^-32 in (0, 1], as double."""
        return (self.next().astype(np.float64) + 1.0) * (1.0 / 4294967296.0)

    def advance(self, delta: int) -> "PCG32Streams":
        """Moves every stream `delta` draws ahead in O(log delta) (LCG jump-ahead, Brown 1994)."""
        cm, cp = _MULT, self.inc.copy()
        am, ap = np.uint64(1), np.zeros_like(self.state)
        delta = int(delta)
        with np.errstate(over="ignore"):
            while delta:
                if delta & 1:
                    am = am * cm
                    ap = ap * cm + cp
                cp = (cm + np.uint64(1)) * cp
                cm = cm * cm
                delta >>= 1
            self.state = am * self.state + ap
        return self


def pcg32_sequence(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n consecutive uniforms of one stream."""
    g = PCG32Streams(seed, np.array([stream], dtype=np.uint64))
    return np.array([g.uniform()[0] for _ in range(n)])


# ------------------------------------------------------------------ value noise
class ValueNoise:
    """3-octave value noise: a 64^3 lattice whose value at linear index i = (z*64 + y)*64 + x
    is 2u - 1 with u the first draw of PCG32(seed, stream i); smoothstep-weighted trilinear
    interpolation; octave frequencies 1, 2, 4 with amplitudes 1, 1/2, 1/4, normalised to
    [-1, 1].  The lattice spacing at frequency 1 is 0.25 and it wraps every 16 units."""

    G = 64

    def __init__(self, seed: int = 0):
        n = self.G ** 3
        vals = PCG32Streams(seed, np.arange(n, dtype=np.uint64)).uniform()
        self.lattice = (vals * 2.0 - 1.0).reshape(self.G, self.G, self.G)  # [z][y][x]

    def _octave(self, p: np.ndarray) -> np.ndarray:
        q = p * 4.0
        i0 = np.floor(q)
        f = q - i0
        w = f * f * (3.0 - 2.0 * f)
        i0 = i0.astype(np.int64) % self.G
        i1 = (i0 + 1) % self.G
        L = self.lattice
        x0, y0, z0 = i0[:, 0], i0[:, 1], i0[:, 2]
        x1, y1, z1 = i1[:, 0], i1[:, 1], i1[:, 2]
        wx, wy, wz = w[:, 0], w[:, 1], w[:, 2]
        c00 = L[z0, y0, x0] * (1 - wx) + L[z0, y0, x1] * wx
        c10 = L[z0, y1, x0] * (1 - wx) + L[z0, y1, x1] * wx
        c01 = L[z1, y0, x0] * (1 - wx) + L[z1, y0, x1] * wx
        c11 = L[z1, y1, x0] * (1 - wx) + L[z1, y1, x1] * wx
        c0 = c00 * (1 - wy) + c10 * wy
        c1 = c01 * (1 - wy) + c11 * wy
        return c0 * (1 - wz) + c1 * wz

    def __call__(self, p: np.ndarray) -> np.ndarray:
        p = np.asarray(p, np.float64)
        total = 0.0
        acc = np.zeros(p.shape[0])
        for freq, amp in ((1.0, 1.0), (2.0, 0.5), (4.0, 0.25)):
            acc += amp * self._octave(p * freq)
            total += amp
        return acc / total


_NOISE_CACHE: dict = {}


def value_noise(seed: int = 0) -> ValueNoise:
    if seed not in _NOISE_CACHE:
        _NOISE_CACHE[seed] = ValueNoise(seed)
    return _NOISE_CACHE[seed]


# ------------------------------------------------------------------ icosphere
def icosphere(level: int):
    """Unit icosphere: vertices (V,3) float64 and faces (F,3) int64, F = 20 * 4^level."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = v.shape[0]
        v = np.concatenate([v, mid], axis=0)
        nf = f.shape[0]
        a = base + inv[:nf]
        b = base + inv[nf:2 * nf]
        c = base + inv[2 * nf:]
        f = np.concatenate([np.stack([f[:, 0], a, c], 1), np.stack([f[:, 1], b, a], 1),
                            np.stack([f[:, 2], c, b], 1), np.stack([a, b, c], 1)], axis=0)
    return v, f


_ICO_CACHE: dict = {}


def _ico(level: int):
    if level not in _ICO_CACHE:
        _ICO_CACHE[level] = icosphere(level)
    return _ICO_CACHE[level]


def displaced_icosphere(level: int, amplitude: float = 0.1, noise_seed: int = 0, offset=(0.0, 0.0, 0.0)):
    """Unit icosphere with vertices scaled by 1 + amplitude * n(p + offset); returns (T, 9) float64."""
    v, f = _ico(level)
    n = value_noise(noise_seed)(v + np.asarray(offset, np.float64))
    vd = v * (1.0 + amplitude * n)[:, None]
    return vd[f].reshape(-1, 9)


def icosphere_scene(level: int = 8, amplitude: float = 0.1, noise_seed: int = 0) -> SceneDesc:
    """Microbench scene: one displaced icosphere, FP32 vertices, Lambertian grey.
    Scene bounds are the vertex bounds (the mesh rule of ObjLoader.cuh:107-112)."""
    tri = displaced_icosphere(level, amplitude, noise_seed).astype(np.float32)
    d = SceneDesc()
    d.add_material((0.7, 0.7, 0.7), 0.5, 0.5, M_LAMBERTIAN)
    d.tri_vertices = tri
    d.tri_material = np.zeros(tri.shape[0], np.uint32)
    pts = tri.reshape(-1, 3).astype(np.float64)
    d.bounds_min = tuple(pts.min(0))
    d.bounds_max = tuple(pts.max(0))
    d.camera = Camera(512, 1.0, (0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 45.0, (0.5, 0.6, 0.8))
    return d


def uniform_rays(n: int, seed: int = 1, box: float = 2.0, tmin: float = 0.001, tmax: float = 999999.0,
                 first: int = 0) -> np.ndarray:
    """Rays i in [first, first+n): PCG32(seed, stream i) draws ox, oy, oz, u1, u2; origin uniform in
    [-box, box]^3, direction z = 1 - 2 u1, phi = 2 pi u2 (uniform on the sphere)."""
    out = np.empty(n, RAY_DTYPE)
    chunk = 1 << 20
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        g = PCG32Streams(seed, np.arange(first + s, first + s + m, dtype=np.uint64))
        ox, oy, oz, u1, u2 = (g.uniform() for _ in range(5))
        org = np.stack([ox, oy, oz], 1) * (2.0 * box) - box
        z = 1.0 - 2.0 * u1
        r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
        phi = 2.0 * math.pi * u2
        d = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
        out["origin"][s:s + m] = org
        out["direction"][s:s + m] = d
        out["tmin"][s:s + m] = tmin
        out["tmax"][s:s + m] = tmax
    return out


def rays_as_f64(rays: np.ndarray) -> np.ndarray:
    """(n, 8) doubles (origin, tmin, direction, tmax) from the FP32 ray records (exact)."""
    out = np.empty((rays.shape[0], 8), np.float64)
    out[:, 0:3] = rays["origin"]
    out[:, 3] = rays["tmin"]
    out[:, 4:7] = rays["direction"]
    out[:, 7] = rays["tmax"]
    return out


# ------------------------------------------------------------------ Cornell box
def _quad(lt, rt, lb, rb):
    """Two triangles (lt, lb, rt), (rt, lb, rb) — the reference's floor split (Device.cuh:42-43)."""
    return [np.concatenate([lt, lb, rt]), np.concatenate([rt, lb, rb])]


def _box_quads(center, size, angle_deg):
    """Six faces of an axis-aligned box rotated about y, as (lt, rt, lb, rb) quads."""
    cx, cy, cz = center
    sx, sy, sz = (s / 2.0 for s in size)
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)

    def P(x, y, z):
        return np.array([cx + ca * x + sa * z, cy + y, cz - sa * x + ca * z])

    c = {(i, j, k): P(i * sx, j * sy, k * sz) for i in (-1, 1) for j in (-1, 1) for k in (-1, 1)}
    faces = [
        (c[(-1, 1, 1)], c[(1, 1, 1)], c[(-1, -1, 1)], c[(1, -1, 1)]),      # front  (+z)
        (c[(1, 1, -1)], c[(-1, 1, -1)], c[(1, -1, -1)], c[(-1, -1, -1)]),  # back   (-z)
        (c[(-1, 1, -1)], c[(-1, 1, 1)], c[(-1, -1, -1)], c[(-1, -1, 1)]),  # left   (-x)
        (c[(1, 1, 1)], c[(1, 1, -1)], c[(1, -1, 1)], c[(1, -1, -1)]),      # right  (+x)
        (c[(-1, 1, -1)], c[(1, 1, -1)], c[(-1, 1, 1)], c[(1, 1, 1)]),      # top    (+y)
        (c[(-1, -1, 1)], c[(1, -1, 1)], c[(-1, -1, -1)], c[(1, -1, -1)]),  # bottom (-y)
    ]
    return faces


def cornell_box(width: int = 512, lambertian: bool = True, seed: int = 0) -> SceneDesc:
    """Cornell box in [-1,1]^3 (open towards +z), camera on the +z axis.  Albedos of the 7
    objects (5 walls, 2 boxes) are PCG32(seed, stream 0) uniforms mapped to [0.1, 0.8], three
    per object in order.  Materials are Lambertian (the reference falls back to Opaque with
    its default roughness 0.5)."""
    g = PCG32Streams(seed, np.array([0], dtype=np.uint64))
    albedo = [tuple(0.1 + 0.7 * g.uniform()[0] for _ in range(3)) for _ in range(7)]
    mtype = M_LAMBERTIAN if lambertian else M_OPAQUE
    d = SceneDesc()
    mats = [d.add_material(a, 0.5, 0.5, mtype) for a in albedo]
    P = lambda x, y, z: np.array([x, y, z], np.float64)  # noqa: E731
    walls = [
        (P(-1, -1, -1), P(1, -1, -1), P(-1, -1, 1), P(1, -1, 1)),   # floor
        (P(-1, 1, 1), P(1, 1, 1), P(-1, 1, -1), P(1, 1, -1)),       # ceiling
        (P(-1, 1, -1), P(1, 1, -1), P(-1, -1, -1), P(1, -1, -1)),   # back
        (P(-1, 1, 1), P(-1, 1, -1), P(-1, -1, 1), P(-1, -1, -1)),   # left
        (P(1, 1, -1), P(1, 1, 1), P(1, -1, -1), P(1, -1, 1)),       # right
    ]
    tris, tmat = [], []
    for w, q in enumerate(walls):
        for t in _quad(*q):
            tris.append(t)
            tmat.append(mats[w])
    for b, (center, size, ang) in enumerate([((0.35, -0.7, 0.3), (0.6, 0.6, 0.6), -18.0),
                                             ((-0.35, -0.4, -0.3), (0.6, 1.2, 0.6), 18.0)]):
        for q in _box_quads(center, size, ang):
            for t in _quad(*q):
                tris.append(t)
                tmat.append(mats[5 + b])
    d.tri_vertices = np.array(tris, np.float64).astype(np.float32)
    d.tri_material = np.array(tmat, np.uint32)
    d.lights.append(dict(center=(0.0, 0.999, 0.0), normal=(0.0, -1.0, 0.0), width=0.5, height=0.5,
                         color=(15.0, 15.0, 15.0), visible=1))
    # No [Mesh] objects: the reference falls back to [-20, 20]^3 scene bounds (Device.cuh:177-181).
    d.camera = Camera(width, 1.0, (0.0, 0.0, 3.9), (0.0, 0.0, 0.0), 38.0, (0.0, 0.0, 0.0))
    return d


# ------------------------------------------------------------------ 200 spheres at 1080p
def spheres_scene(num_spheres: int = 200, level: int = 5, width: int = 1920, seed: int = 2,
                  amplitude: float = 0.1) -> SceneDesc:
    """Wavefront workload.  Sphere k draws, from PCG32(seed, stream k): x, z in [-10, 10],
    radius in [0.3, 1.0], a noise offset in [0, 16)^3 and a roughness U[0.05, 0.8]; it rests
    on the ground (y = radius).  Materials by k mod 3: Lambertian / GGX (alpha = roughness) /
    dielectric (IOR 1.5).  Ground: two triangles over [-30, 30]^2 at y = 0.  A 3x3x3 volume box
    (12 triangles, sigma_t 0.5, albedo 0.8) at (0, 1.5, 3).  Two 4x4 lights at height 12."""
    d = SceneDesc()
    ground = d.add_material((0.6, 0.6, 0.6), 0.5, 0.5, M_LAMBERTIAN)
    tris = [np.concatenate([[-30, 0, -30], [-30, 0, 30], [30, 0, -30]]),
            np.concatenate([[30, 0, -30], [-30, 0, 30], [30, 0, 30]])]
    tmat = [ground, ground]
    parts = [np.array(tris, np.float64)]
    mats = list(tmat)
    g = PCG32Streams(seed, np.arange(num_spheres, dtype=np.uint64))
    x = g.uniform() * 20.0 - 10.0
    z = g.uniform() * 20.0 - 10.0
    rad = 0.3 + 0.7 * g.uniform()
    off = np.stack([g.uniform() * 16.0, g.uniform() * 16.0, g.uniform() * 16.0], 1)
    rough = 0.05 + 0.75 * g.uniform()
    cr, cg, cb = g.uniform(), g.uniform(), g.uniform()
    for k in range(num_spheres):
        kind = k % 3
        col = (0.2 + 0.7 * cr[k], 0.2 + 0.7 * cg[k], 0.2 + 0.7 * cb[k])
        if kind == 0:
            m = d.add_material(col, 0.5, 0.5, M_LAMBERTIAN)
        elif kind == 1:
            m = d.add_material(col, float(rough[k]), float(rough[k]), M_OPAQUE)
        else:
            m = d.add_material((1.0, 1.0, 1.0), 0.5, 0.5, M_SPECULAR_DIELECTRIC, eta=1.5)
        t = displaced_icosphere(level, amplitude, 0, off[k]) * rad[k]
        t = t.reshape(-1, 3, 3) + np.array([x[k], rad[k], z[k]])
        parts.append(t.reshape(-1, 9))
        mats.extend([m] * t.shape[0])
    vol = d.add_material((1.0, 1.0, 1.0), 0.5, 0.5, M_VOLUME, sigma_t=0.5, albedo=0.8)
    for q in _box_quads((0.0, 1.5, 3.0), (3.0, 3.0, 3.0), 0.0):
        for t in _quad(*q):
            parts.append(np.asarray(t, np.float64)[None, :])
            mats.append(vol)
    d.tri_vertices = np.concatenate(parts, 0).astype(np.float32)
    d.tri_material = np.array(mats, np.uint32)
    for c in ((-5.0, 12.0, 0.0), (5.0, 12.0, 5.0)):
        d.lights.append(dict(center=c, normal=(0.0, -1.0, 0.0), width=4.0, height=4.0, color=(12.0, 12.0, 12.0),
                             visible=1))
    pts = d.tri_vertices.reshape(-1, 3).astype(np.float64)
    d.bounds_min = tuple(pts.min(0))
    d.bounds_max = tuple(pts.max(0))
    d.camera = Camera(width, 16.0 / 9.0, (0.0, 7.0, 24.0), (0.0, 1.0, 0.0), 40.0, (0.05, 0.06, 0.08))
    return d


def random_scene(seed: int, width: int = 256, aspect: float = 1.0, max_level: int = 6,
                 max_objects: int = 6) -> SceneDesc:
    """A seeded scene of the icosphere-microbench type (denoiser training data and serving jobs).

    All draws come in order from one PCG32 stream (seed, stream 0): the number of displaced
    icospheres in [1, max_objects]; per sphere a subdivision level in [4, max_level], radius
    [0.4, 1.4], position x, z in [-4, 4] resting on the ground, a noise offset, a colour, and a
    material (Lambertian / GGX with roughness U[0.05, 0.8] / dielectric IOR 1.5, equal odds);
    with odds 0.3 a homogeneous volume box (sigma_t U[0.3, 1.0], albedo 0.8; side 2, its bottom
    0.01 above the ground); one or two area
    lights 8-12 units up (side 2-4, radiance 8-20); a camera orbiting at distance 8-12, height
    1.5-6, looking at (0, 0.8, 0) with a 35-50 degree field of view.  Ground: [-30, 30]^2 at y = 0."""
    g = PCG32Streams(seed, np.array([0], dtype=np.uint64))
    u = lambda: float(g.uniform()[0])
    d = SceneDesc()
    ground = d.add_material((0.3 + 0.5 * u(), 0.3 + 0.5 * u(), 0.3 + 0.5 * u()), 0.5, 0.5, M_LAMBERTIAN)
    parts = [np.array([[-30, 0, -30, -30, 0, 30, 30, 0, -30], [30, 0, -30, -30, 0, 30, 30, 0, 30]], np.float64)]
    mats = [ground, ground]
    n_obj = 1 + min(int(u() * max_objects), max_objects - 1)
    for k in range(n_obj):
        level = 4 + min(int(u() * (max_level - 3)), max_level - 4)
        rad = 0.4 + u()
        x, z = u() * 8.0 - 4.0, u() * 8.0 - 4.0
        off = (u() * 16.0, u() * 16.0, u() * 16.0)
        col = (0.15 + 0.8 * u(), 0.15 + 0.8 * u(), 0.15 + 0.8 * u())
        kind = min(int(u() * 3), 2)
        rough = 0.05 + 0.75 * u()
        if kind == 0:
            m = d.add_material(col, 0.5, 0.5, M_LAMBERTIAN)
        elif kind == 1:
            m = d.add_material(col, rough, rough, M_OPAQUE)
        else:
            m = d.add_material((1.0, 1.0, 1.0), 0.5, 0.5, M_SPECULAR_DIELECTRIC, eta=1.5)
        t = displaced_icosphere(level, 0.1, 0, off) * rad
        t = t.reshape(-1, 3, 3) + np.array([x, rad, z])
        parts.append(t.reshape(-1, 9))
        mats.extend([m] * t.shape[0])
    if u() < 0.3:
        vol = d.add_material((1.0, 1.0, 1.0), 0.5, 0.5, M_VOLUME, sigma_t=0.3 + 0.7 * u(), albedo=0.8)
        # 0.01 above the ground: a bottom face coplanar with the ground would make every ground hit
        # inside the box's footprint a tie between two triangles at the same distance
        c = (u() * 6.0 - 3.0, 1.01, u() * 6.0 - 3.0)
        for q in _box_quads(c, (2.0, 2.0, 2.0), 360.0 * u()):
            for t in _quad(*q):
                parts.append(np.asarray(t, np.float64)[None, :])
                mats.append(vol)
    d.tri_vertices = np.concatenate(parts, 0).astype(np.float32)
    d.tri_material = np.array(mats, np.uint32)
    for _ in range(1 + int(u() < 0.5)):
        side = 2.0 + 2.0 * u()
        c = (u() * 10.0 - 5.0, 8.0 + 4.0 * u(), u() * 10.0 - 5.0)
        e = 8.0 + 12.0 * u()
        d.lights.append(dict(center=c, normal=(0.0, -1.0, 0.0), width=side, height=side, color=(e, e, e),
                             visible=1))
    ang = 2.0 * math.pi * u()
    dist = 8.0 + 4.0 * u()
    h = 1.5 + 4.5 * u()
    fov = 35.0 + 15.0 * u()
    pts = d.tri_vertices.reshape(-1, 3).astype(np.float64)
    d.bounds_min = tuple(pts.min(0))
    d.bounds_max = tuple(pts.max(0))
    d.camera = Camera(width, aspect, (dist * math.sin(ang), h, dist * math.cos(ang)), (0.0, 0.8, 0.0), fov,
                      (0.04 + 0.06 * u(), 0.05 + 0.06 * u(), 0.08 + 0.06 * u()))
    return d
