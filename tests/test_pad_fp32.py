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
