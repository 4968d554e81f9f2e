"""Image files for the headless renderer: 8-bit PPM with the reference's display transform and
32-bit PFM.  Images are [H, W, 3] float arrays with row 0 at the bottom, as rendered."""
from __future__ import annotations

import numpy as np


def to_rgb8(rgb: np.ndarray) -> np.ndarray:
    """pic2RGBW (Render.cu:462-481): sqrt gamma, clamp to [0, 1], times 254.99, truncated."""
    c = np.clip(np.sqrt(np.maximum(rgb.astype(np.float64), 0.0)), 0.0, 1.0)
    return (254.99 * c).astype(np.uint8)


def write_ppm(path: str, rgb: np.ndarray) -> None:
    """Binary PPM (P6), top row first."""
    img = to_rgb8(rgb)[::-1]
    H, W, _ = img.shape
    with open(path, "wb") as f:
        f.write(f"P6\n{W} {H}\n255\n".encode())
        f.write(np.ascontiguousarray(img).tobytes())


def read_ppm(path: str) -> np.ndarray:
    """[H, W, 3] uint8 with row 0 at the bottom (inverse of write_ppm's row order)."""
    data = open(path, "rb").read()
    parts, pos = [], 0
    while len(parts) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        parts.append(data[pos:end])
        pos = end
    pos += 1
    W, H = int(parts[1]), int(parts[2])
    return np.frombuffer(data[pos:pos + W * H * 3], np.uint8).reshape(H, W, 3)[::-1]


def write_pfm(path: str, rgb: np.ndarray) -> None:
    """Little-endian PFM; PFM stores the bottom row first, as rendered."""
    img = np.ascontiguousarray(rgb, dtype="<f4")
    H, W, _ = img.shape
    with open(path, "wb") as f:
        f.write(f"PF\n{W} {H}\n-1.0\n".encode())
        f.write(img.tobytes())


def read_pfm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        assert f.readline().strip() == b"PF"
        W, H = (int(v) for v in f.readline().split())
        scale = float(f.readline())
        dt = "<f4" if scale < 0 else ">f4"
        return np.frombuffer(f.read(W * H * 12), dt).reshape(H, W, 3).astype(np.float32)
