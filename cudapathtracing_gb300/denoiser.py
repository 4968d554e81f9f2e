"""Kernel-predicting denoiser (cpt_denoiser_* in include/cpt.h) — host wrapper.

The network, its training step and inference run in libcpt.so (csrc/kpcn.cu); this module holds
device tensors and parameters, and saves/loads weights.  Images are device torch tensors:
rgb / target [n, h, w, 3] float32, gbuf [n, h, w, 8] float32 (the renderer's G-buffer).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib

# (cin, cout, relu) of the 19 convolutions, in parameter order (mirrors csrc/kpcn.cu)
SPECS = [
    (32, 32, True), (32, 32, True), (32, 64, True), (64, 64, True), (64, 96, True), (96, 96, True),
    (96, 128, True), (128, 128, True), (128, 160, True), (160, 160, True),
    (288, 128, True), (128, 128, True), (224, 96, True), (96, 96, True), (160, 64, True), (64, 64, True),
    (96, 32, True), (32, 32, True), (32, 32, False),
]
NAMES = ["c0a", "c0b", "c1a", "c1b", "c2a", "c2b", "c3a", "c3b", "c4a", "c4b",
         "d3a", "d3b", "d2a", "d2b", "d1a", "d1b", "d0a", "d0b", "out"]
FORMAT = "cpt-kpcn-v1"


def layer_slices():
    """[(name, weight slice, bias slice, (9, cin, cout))] into the flat parameter array."""
    out, off = [], 0
    for name, (ci, co, _) in zip(NAMES, SPECS):
        n = 9 * ci * co
        out.append((name, slice(off, off + n), slice(off + n, off + n + co), (9, ci, co)))
        off += n + co
    return out


def num_params() -> int:
    return sum(9 * ci * co + co for ci, co, _ in SPECS)


def _vp(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class Denoiser:
    def __init__(self, device: int = 0, seed: int = 0):
        h = C.c_void_p()
        check(lib().cpt_denoiser_create(device, seed, C.byref(h)), "cpt_denoiser_create")
        self.h = h
        self.device = device
        self.n = int(lib().cpt_denoiser_num_params(h))
        assert self.n == num_params()

    @property
    def params(self) -> np.ndarray:
        a = np.empty(self.n, dtype=np.float32)
        check(lib().cpt_denoiser_get_params(self.h, a.ctypes.data_as(C.c_void_p)), "cpt_denoiser_get_params")
        return a

    @params.setter
    def params(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.size != self.n:
            raise ValueError(f"expected {self.n} parameters, got {a.size}")
        check(lib().cpt_denoiser_set_params(self.h, a.ctypes.data_as(C.c_void_p)), "cpt_denoiser_set_params")

    def grads(self) -> np.ndarray:
        a = np.empty(self.n, dtype=np.float32)
        check(lib().cpt_denoiser_get_grads(self.h, a.ctypes.data_as(C.c_void_p)), "cpt_denoiser_get_grads")
        return a

    def set_backend(self, backend: int) -> None:
        """2: TMA-fed warp-specialised tcgen05 convolutions (default), 1: tcgen05 convolutions with
        cp.async copies, 0: mma.sync convolutions (cpt_denoiser_set_backend)."""
        check(lib().cpt_denoiser_set_backend(self.h, backend), "cpt_denoiser_set_backend")

    def check(self) -> None:
        """Raises if a tensor-core barrier wait timed out since the last check."""
        check(lib().cpt_denoiser_check(self.h), "cpt_denoiser_check")

    def export(self, name: str) -> np.ndarray:
        """An internal tensor of the last pass, flattened (see cpt_denoiser_export)."""
        cnt = C.c_uint64()
        check(lib().cpt_denoiser_export(self.h, name.encode(), None, 0, C.byref(cnt)), "cpt_denoiser_export")
        a = np.empty(cnt.value, dtype=np.float32)
        check(lib().cpt_denoiser_export(self.h, name.encode(), a.ctypes.data_as(C.c_void_p), cnt.value, C.byref(cnt)),
              "cpt_denoiser_export")
        return a

    def train_step(self, rgb, gbuf, target, lr: float = 1e-3, update: bool = True, stream=None) -> float:
        n, h, w = int(rgb.shape[0]), int(rgb.shape[1]), int(rgb.shape[2])
        loss = C.c_float()
        check(lib().cpt_denoiser_train_step(self.h, n, h, w, _vp(rgb), _vp(gbuf), _vp(target), float(lr),
                                            1 if update else 0, C.byref(loss), stream), "cpt_denoiser_train_step")
        return float(loss.value)

    def denoise(self, rgb, gbuf, out=None, stream=None):
        import torch
        if rgb.dim() == 3:
            rgb, gbuf = rgb[None], gbuf[None]
            if out is not None:
                out = out[None]
        if out is None:
            out = torch.empty_like(rgb)
        n, h, w = int(rgb.shape[0]), int(rgb.shape[1]), int(rgb.shape[2])
        check(lib().cpt_denoise(self.h, n, h, w, _vp(rgb.contiguous()), _vp(gbuf.contiguous()), _vp(out), stream),
              "cpt_denoise")
        return out

    def save(self, path: str) -> None:
        np.savez(path, format=FORMAT, params=self.params)

    def load(self, path: str) -> None:
        z = np.load(path)
        if str(z["format"]) != FORMAT:
            raise ValueError(f"{path}: not a {FORMAT} file")
        self.params = z["params"]

    def close(self):
        if self.h:
            lib().cpt_denoiser_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def main():
    """Times inference on one image and a training step on a batch of crops (random inputs):
    python -m cudapathtracing_gb300.denoiser --size 1920x1080 --batch 8 --crop 256"""
    import argparse
    import time
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", default="1920x1080")
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--crop", type=int, default=256)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--backend", type=int, default=None, help="0: mma.sync, 1: tcgen05, 2: tcgen05 warp-specialised (default: the library's)")
    a = ap.parse_args()
    W, H = (int(x) for x in a.size.split("x"))
    net = Denoiser(seed=0)
    if a.backend is not None:
        net.set_backend(a.backend)
    rgb = torch.rand(1, H, W, 3, device="cuda")
    gb = torch.rand(1, H, W, 8, device="cuda")
    out = torch.empty_like(rgb)
    for _ in range(3):
        net.denoise(rgb, gb, out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        net.denoise(rgb, gb, out)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.reps
    Hp, Wp = (H + 15) // 16 * 16, (W + 15) // 16 * 16
    lv = [0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 3, 3, 2, 2, 1, 1, 0, 0, 0]
    flops = 2 * Hp * Wp * 9 * sum(ci * co / 4 ** l for (ci, co, _), l in zip(SPECS, lv))
    print(f"inference {W}x{H}: {ms:.3f} ms, convolutions {flops / 1e12:.3f} TFLOP -> {flops / ms / 1e9:.1f} TFLOP/s")
    c = a.crop
    r = torch.rand(a.batch, c, c, 3, device="cuda")
    g = torch.rand(a.batch, c, c, 8, device="cuda")
    t = torch.rand(a.batch, c, c, 3, device="cuda")
    for _ in range(3):
        net.train_step(r, g, t, lr=1e-5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.reps):
        net.train_step(r, g, t, lr=1e-5)
    torch.cuda.synchronize()
    print(f"train step {a.batch}x{c}x{c}: {(time.perf_counter() - t0) / a.reps * 1e3:.3f} ms")


if __name__ == "__main__":
    main()
