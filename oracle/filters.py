"""TEST INFRASTRUCTURE ONLY — FP64 numpy restatement of the reference's real-time filters.

Used by tests/ as the checker of cpt_filter_bilateral / cpt_filter_temporal; never by the
library.  Pinned in tests/test_filters.py against the reference's own kernels run as host loops
(oracle/_ref, ref_gaussian_separate / ref_add_previous) where the reference is mounted.

Images are numpy arrays [H, W, 3] with row 0 the bottom row (pixel offset j * W + i), as the
renderer writes them; gbuf4 is [H, W, 4] = (normal xyz, depth), depth 999999 on a miss.
"""
from __future__ import annotations

import math

import numpy as np

INF = 999999.0   # rtmath.cuh:8


def bilateral_pass(src, gbuf4, sigma_g, sigma_r, sigma_n, sigma_d, radius, horizontal):
    """gaussianSeparate (Render.cu:356-398) over a whole image: the centre value is pic[offset],
    which in the REAL_TIME loop holds the same values as the pass input."""
    H, W, _ = src.shape
    acc = np.zeros_like(src, dtype=np.float64)
    wsum = np.zeros((H, W), dtype=np.float64)
    n0, d0 = gbuf4[..., :3], gbuf4[..., 3]
    for i in range(-radius, radius + 1):
        if horizontal:
            idx = np.clip(np.arange(W) + i, 0, W - 1)
            p, gp = src[:, idx], gbuf4[:, idx]
        else:
            idx = np.clip(np.arange(H) + i, 0, H - 1)
            p, gp = src[idx], gbuf4[idx]
        gw = -(i * i) / (2.0 * sigma_g * sigma_g)
        bw = -np.sum((p - src) ** 2, axis=-1) / (2.0 * sigma_r * sigma_r)
        nw = -np.sum((n0 - gp[..., :3]) ** 2, axis=-1) / (2.0 * sigma_n * sigma_n)
        dd = d0 - gp[..., 3]
        dw = -dd * dd / (2.0 * sigma_d * sigma_d)
        w = np.exp(gw + bw + nw + dw)
        wsum += w
        acc += p * w[..., None]
    return acc / wsum[..., None]


def bilateral(rgb, gbuf4, sigma_g=8.0, sigma_r=5.0, sigma_n=0.1, sigma_d=0.2, radius=16):
    """Horizontal then vertical pass (main.cu:99-103; defaults Window.cu:11-14, Render.cuh:8)."""
    src = np.asarray(rgb, dtype=np.float64)
    g = np.asarray(gbuf4, dtype=np.float64)
    tmp = bilateral_pass(src, g, sigma_g, sigma_r, sigma_n, sigma_d, radius, True)
    return bilateral_pass(tmp, g, sigma_g, sigma_r, sigma_n, sigma_d, radius, False)


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def camera_height(width, aspect):
    h = width / aspect   # Camera.cu:8-9
    return 1 if h < 1 else int(h)


def camera_rays(width, aspect, look_from, look_at, vfov_deg):
    """Pixel-centre ray directions [H, W, 3] of the camera (Camera.cu:5-40), row 0 at the bottom."""
    H = camera_height(width, aspect)
    frm, at = np.asarray(look_from, float), np.asarray(look_at, float)
    focal = np.linalg.norm(frm - at)
    h = math.tan(math.radians(vfov_deg) / 2.0)
    vh = 2.0 * h * focal
    vw = width / H * vh
    w = _unit(frm - at)
    u = _unit(np.cross([0.0, 1.0, 0.0], w))
    v = np.cross(w, u)
    hor, ver = u * vw, v * vh
    dh, dv = hor / width, ver / H
    pc = frm - hor / 2 - ver / 2 - w * focal + dh / 2 + dv / 2
    jj, ii = np.meshgrid(np.arange(H), np.arange(width), indexing="ij")
    p = pc + ii[..., None] * dh + jj[..., None] * dv
    return p - frm


def positions_from_depth(gbuf4, width, aspect, look_from, look_at, vfov_deg):
    """The library's hit-position rebuild: look_from + depth * unit(pixel-centre direction);
    (INF, INF, INF) where the depth is a miss."""
    d = gbuf4[..., 3].astype(np.float64)
    pos = np.asarray(look_from, float) + d[..., None] * _unit(camera_rays(width, aspect, look_from, look_at, vfov_deg))
    pos[d >= INF] = INF
    return pos


def reproject(pos, width, height, pre_from, pre_at, vfov_deg):
    """Camera::getPrePositionInImg (Camera.cuh:103-132) for every pixel: (i, j) or (-1, -1)."""
    pre_from, pre_at = np.asarray(pre_from, float), np.asarray(pre_at, float)
    d = _unit(pos - pre_from)
    fwd = _unit(pre_at - pre_from)
    right = _unit(np.cross(fwd, [0.0, 1.0, 0.0]))
    up = np.cross(right, fwd)
    focal = np.linalg.norm(pre_from - pre_at)
    h = math.tan(math.radians(vfov_deg) / 2.0)
    vh = 2.0 * h * focal
    vw = width / height * vh
    px, py, pz = d @ right, d @ up, d @ fwd
    with np.errstate(divide="ignore", invalid="ignore"):
        x = 0.5 + (px / pz) * (focal / vw)
        y = 0.5 + (py / pz) * (focal / vh)
    ok = (x >= 0) & (y >= 0) & (x <= 1) & (y <= 1) & ~(pos[..., 0] + pos[..., 1] > INF)
    xi = np.clip(np.nan_to_num(np.floor(x * width), nan=-1.0, posinf=-1.0, neginf=-1.0), -1, width - 1)
    yi = np.clip(np.nan_to_num(np.floor(y * height), nan=-1.0, posinf=-1.0, neginf=-1.0), -1, height - 1)
    i = np.where(ok, xi.astype(np.int64), -1)
    j = np.where(ok, yi.astype(np.int64), -1)
    return i, j, ok


def temporal(rgb, prev, pos, width, pre_from, pre_at, vfov_deg, alpha):
    """addPrevious (Render.cu:400-420): alpha * pic + (1 - alpha) * previous at the reprojected
    pixel (the pixel itself when the reprojection is invalid).  The index is clamped to the
    image (the reference can reach W or H at x = 1 or y = 1)."""
    H = rgb.shape[0]
    i, j, ok = reproject(pos, width, H, pre_from, pre_at, vfov_deg)
    jj, ii = np.meshgrid(np.arange(H), np.arange(width), indexing="ij")
    si, sj = np.where(ok, i, ii), np.where(ok, j, jj)
    return rgb * alpha + prev[sj, si] * (1.0 - alpha)
