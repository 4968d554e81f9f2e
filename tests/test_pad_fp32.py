"""FP32 forms of FP64 operations in the LBVH kernels, restated in numpy float32.

The box padding of the prep kernel (csrc/lbvh.cu pad_fp32, AABB::pad AABB.cuh:30-40), bit for bit against
the FP64 sequence RD32(RN64(x - 1e-4)) / RU32(RN64(x + 1e-4)) on sweeps of float32 bit patterns.
Values the FP32 form cannot certify take the FP64 sequence in the kernel; they are counted here and
must not occur for coordinates of magnitude 0.01 .. 4000.  The kernel itself is checked by the
bit-exact leaf boxes of the LBVH parity tests."""
from __future__ import annotations

import numpy as np

PAD_HI = np.float32(float.fromhex("0x1.a36e2ep-14"))
PAD_LO = np.float32(float.fromhex("0x1.638866p-39"))


def _ref(x: np.ndarray, up: bool) -> np.ndarray:
    d = x.astype(np.float64) + (1e-4 if up else -1e-4)
    f = d.astype(np.float32)
    if up:
        f = np.where(f.astype(np.float64) < d, np.nextafter(f, np.float32(np.inf)), f)
    else:
        f = np.where(f.astype(np.float64) > d, np.nextafter(f, np.float32(-np.inf)), f)
    return f


def _fast(x: np.ndarray, up: bool):
    with np.errstate(over="ignore", invalid="ignore"):
        h = PAD_HI if up else -PAD_HI
        s = x + h
        bb = s - x
        e = (x - (s - bb)) + (h - bb)
        r = e + PAD_LO if up else e - PAD_LO
        a = np.abs(s)
        tol = np.float32(2.0 ** -50) * a + np.float32(2.0 ** -23) * np.abs(r) + np.float32(2.0 ** -62)
        certain = (a >= np.float32(2.0 ** -10)) & (a < np.float32(2.0 ** 100)) & (np.abs(r) > tol)
        sb = s.view(np.uint32)
        neg = (sb >> 31) != 0
        away = (r > 0) if up else (r < 0)
        step = np.where(neg != up, np.uint32(1), np.uint32(0xFFFFFFFF))   # +1 or -1 on the bits
        out = np.where(away, (sb + step).view(np.float32), s)
    return out, certain


def _check(x: np.ndarray):
    fallbacks = 0
    for up in (False, True):
        got, certain = _fast(x, up)
        ref = _ref(x, up)
        ok = got.view(np.uint32) == ref.view(np.uint32)
        assert ok[certain].all(), x[certain & ~ok][:5]
        fallbacks += int((~certain).sum())
    return fallbacks


def test_pad_fp32_bit_patterns():
    bits = np.arange(0, 2 ** 32, 4099, dtype=np.uint64).astype(np.uint32)
    x = bits.view(np.float32)
    _check(x[np.isfinite(x)])


def test_pad_fp32_near_powers_of_two_and_the_pad():
    parts = []
    for k in range(-20, 20):
        for sgn in (-1.0, 1.0):
            b = np.float32(sgn * 2.0 ** k).view(np.uint32).astype(np.int64)
            parts.append((b + np.arange(-3000, 3001)).astype(np.uint32))
    for sgn in (-1.0, 1.0):
        b = np.float32(sgn * 1e-4).view(np.uint32).astype(np.int64)
        parts.append((b + np.arange(-100000, 100001)).astype(np.uint32))
    x = np.concatenate(parts).view(np.float32)
    _check(x[np.isfinite(x)])


def test_pad_fp32_scene_coordinates_never_fall_back():
    rng = np.random.default_rng(5)
    mag = 10.0 ** rng.uniform(-2, np.log10(4000), 2_000_000)
    x = (mag * rng.choice([-1.0, 1.0], mag.size)).astype(np.float32)
    assert _check(x) == 0


def test_edge_fp32_matches_fp64_difference():
    """Triangle edges of the leaf records (csrc/lbvh.cu edge32): one FP32 subtraction where the FP64
    difference is exact (both normal, exponents within 28, or either zero), which must equal the FP64
    difference rounded once."""
    rng = np.random.default_rng(9)
    n = 2_000_000
    a = (rng.standard_normal(n) * 10.0 ** rng.uniform(-12, 12, n)).astype(np.float32)
    b = (rng.standard_normal(n) * 10.0 ** rng.uniform(-12, 12, n)).astype(np.float32)
    a[::7] = 0.0
    b[::11] = -0.0
    ea = (a.view(np.uint32) >> 23) & 0xFF
    eb = (b.view(np.uint32) >> 23) & 0xFF
    normal = (ea != 0) & (ea != 255) & (eb != 0) & (eb != 255)
    zero = ((a.view(np.uint32) << 1) == 0) | ((b.view(np.uint32) << 1) == 0)
    fast = (normal & (np.abs(ea.astype(int) - eb.astype(int)) <= 28)) | zero
    with np.errstate(over="ignore"):
        got = b - a
        ref = (b.astype(np.float64) - a.astype(np.float64)).astype(np.float32)
    assert fast.mean() > 0.3
    assert (got.view(np.uint32)[fast] == ref.view(np.uint32)[fast]).all()


THIRD_HI = np.float32(float.fromhex("0x1.555556p-2"))
THIRD_LO = np.float32(float.fromhex("-0x1.555556p-27"))


def _morton_ref(a, b, c, mn, mx):
    """The reference's FP64 sequence (BVH.cuh:23-33 on the centroid, Hittable.cuh:459-461)."""
    s = (a.astype(np.float64) + b) + c
    cen = s / 3.0
    with np.errstate(invalid="ignore"):
        x = (cen - mn) / (mx - mn) * 1024.0
    x = np.where(x > 0.0, x, 0.0)
    x = np.where(x < 1023.0, x, 1023.0)
    return x.astype(np.int64)


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _two_prod(a, b):
    p = a * b
    return p, (a.astype(np.float64) * b.astype(np.float64) - p.astype(np.float64)).astype(np.float32)


def _morton_ff(a, b, c, mn, mx):
    """csrc/lbvh.cu morton_tri_axis_ff restated: the cell, or -1 where it defers to FP64."""
    f32 = np.float32
    k64 = 1024.0 / (mx - mn)
    mn32, k32 = f32(mn), f32(k64)
    mn_lo, k_lo = f32(mn - float(mn32)), f32(k64 - float(k32))
    s1, e1 = _two_sum(a, b)
    s2, e2 = _two_sum(s1, c)
    slo = e1 + e2
    y, ye = _two_prod(s2, np.full_like(s2, THIRD_HI))
    ye = ye + (s2 * THIRD_LO + slo * THIRD_HI)
    z, ze = _two_sum(y, np.full_like(y, -mn32))
    ze = ze + (ye - mn_lo)
    x, xe = _two_prod(z, np.full_like(z, k32))
    xe = xe + (z * k_lo + ze * k32)
    mag = np.abs(a) + np.abs(b) + np.abs(c) + np.abs(mn32)
    tol = f32(2.0 ** -40) * (k32 * mag + f32(2) * np.abs(x))
    xs = x + xe
    f = np.floor(np.clip(x, 0, 1024)).astype(np.float32)
    below = (x - f) + xe
    above = ((f + f32(1)) - x) - xe
    fi = f.astype(np.int64)
    out = np.where((below > tol) & (above > tol), np.minimum(fi, 1023), -1)
    out = np.where((below < -tol) & (fi >= 1), np.minimum(fi - 1, 1023), out)
    out = np.where(above < -tol, np.minimum(fi + 1, 1023), out)
    out = np.where(xs > f32(1023) + tol, 1023, out)
    out = np.where(xs < f32(1) - tol, 0, out)
    return out


def test_morton_float_float_step_matches_fp64():
    """The Morton cell's second step (csrc/lbvh.cu morton_tri_axis_ff, pairs of FP32 numbers) against
    the reference's FP64 sequence, on triangles whose centroid coordinate lies within about 1e-6
    cell of a cell boundary (where the FP32 first step defers) and on random ones: every decided cell
    equal; deferred to FP64 only within 1e-8 cell of a boundary, and for fewer than one in a million
    random coordinates."""
    rng = np.random.default_rng(11)
    n = 1_000_000
    mn, mx = -2.1, 2.3
    k = 1024.0 / (mx - mn)
    target = rng.integers(1, 1023, n) + rng.uniform(-1e-6, 1e-6, n)
    cen = mn + target / k
    a = (cen + rng.uniform(-0.05, 0.05, n)).astype(np.float32)
    b = (cen + rng.uniform(-0.05, 0.05, n)).astype(np.float32)
    c = (3.0 * cen - a.astype(np.float64) - b.astype(np.float64)).astype(np.float32)
    for near, (A, B, Cc) in ((True, (a, b, c)), (False, tuple(rng.uniform(mn, mx, (3, n)).astype(np.float32)))):
        got = _morton_ff(A, B, Cc, mn, mx)
        ref = _morton_ref(A, B, Cc, mn, mx)
        decided = got >= 0
        assert (got[decided] == ref[decided]).all()
        if near:
            # deferred only where the exact coordinate is within 1e-8 cell of a boundary (here about
            # a fifth of the cases land exactly on one: the sum's grid meets the integers)
            x = ((A.astype(np.float64) + B + Cc) / 3.0 - mn) * k
            assert (np.abs(x[~decided] - np.round(x[~decided])) < 1e-8).all()
        else:
            assert (~decided).mean() < 1e-6, (~decided).mean()
