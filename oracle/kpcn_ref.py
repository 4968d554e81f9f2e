"""TEST INFRASTRUCTURE ONLY — FP64 numpy restatement of the kernel-predicting denoiser
(csrc/kpcn.cu): features, U-Net forward, kernel apply, loss, and the full backward pass.

It is the checker of the library's BF16 tensor-core training kernels: values are rounded to
BF16 exactly where the CUDA path stores BF16 (features, weights, activations after bias and
ReLU, pooled activations, and every convolution's output gradient dZ); everything else is FP64.
Parameters use the library's flat layout (per convolution W[9][cin][cout] then b[cout]).
"""
from __future__ import annotations

import numpy as np

INF = 999999.0
KS = 5
LOSS_EPS = 1e-3   # loss: L1 of sqrt(x + LOSS_EPS)
SPECS = [
    (32, 32, True), (32, 32, True), (32, 64, True), (64, 64, True), (64, 96, True), (96, 96, True),
    (96, 128, True), (128, 128, True), (128, 160, True), (160, 160, True),
    (288, 128, True), (128, 128, True), (224, 96, True), (96, 96, True), (160, 64, True), (64, 64, True),
    (96, 32, True), (32, 32, True), (32, 32, False),
]


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    ws, bs, off = [], [], 0
    for ci, co, _ in SPECS:
        n = 9 * ci * co
        ws.append(np.asarray(params[off:off + n], np.float64).reshape(9, ci, co))
        bs.append(np.asarray(params[off + n:off + n + co], np.float64))
        off += n + co
    return ws, bs


def exact(x):
    return np.asarray(x, dtype=np.float64)


def features(rgb, gbuf, H, W, rnd=bf16):
    """rgb [N, Hr, Wr, 3], gbuf [N, Hr, Wr, 8] -> X0 [N, H, W, 32] (rounded by rnd), rad [N, H, W, 3]."""
    N, Hr, Wr, _ = rgb.shape
    rgb = rgb.astype(np.float64)
    X = np.zeros((N, H, W, 32))
    rad = np.zeros((N, H, W, 3))
    r = np.maximum(rgb, 0.0)
    rad[:, :Hr, :Wr] = r
    X[:, :Hr, :Wr, 0:3] = np.log1p(r)
    X[:, :Hr, :Wr, 3:6] = gbuf[..., 4:7]
    n = gbuf[..., 0:3].astype(np.float64)
    l1 = np.abs(n).sum(-1)
    nz = np.where(l1 > 0, 1.0, 0.0)
    safe = np.where(l1 > 0, l1, 1.0)
    nx, ny = n[..., 0] / safe, n[..., 1] / safe
    flip = (n[..., 2] < 0) & (l1 > 0)
    sx = np.where(nx >= 0, 1.0, -1.0)
    sy = np.where(ny >= 0, 1.0, -1.0)
    ox, oy = (1 - np.abs(ny)) * sx, (1 - np.abs(nx)) * sy
    X[:, :Hr, :Wr, 6] = np.where(flip, ox, nx) * nz + 0.0
    X[:, :Hr, :Wr, 7] = np.where(flip, oy, ny) * nz + 0.0
    d = gbuf[..., 3].astype(np.float64)
    X[:, :Hr, :Wr, 8] = np.where(d >= INF, 1.0, d / (1.0 + d))
    lum = np.log1p(np.maximum(0.0, 0.2126 * rgb[..., 0] + 0.7152 * rgb[..., 1] + 0.0722 * rgb[..., 2]))
    nb = []
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            yy = np.clip(np.arange(Hr) + dy, 0, Hr - 1)
            xx = np.clip(np.arange(Wr) + dx, 0, Wr - 1)
            nb.append(lum[:, yy][:, :, xx])
    nb = np.stack(nb)
    X[:, :Hr, :Wr, 9] = ((nb - nb.mean(0)) ** 2).mean(0)
    X[:, :Hr, :Wr, 10] = np.log1p(np.sqrt(np.maximum(gbuf[..., 7].astype(np.float64), 0.0)))
    return rnd(X), rad


def shift(x, dy, dx):
    """out[n, y, x] = x[n, y + dy, x + dx], zero outside."""
    out = np.zeros_like(x)
    H, W = x.shape[1], x.shape[2]
    ys, ye = max(0, -dy), H - max(0, dy)
    xs, xe = max(0, -dx), W - max(0, dx)
    if ys < ye and xs < xe:
        out[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


TAPS = [(t // 3 - 1, t % 3 - 1) for t in range(9)]


def conv(x, w, b):
    z = np.zeros(x.shape[:3] + (w.shape[2],))
    for t, (dy, dx) in enumerate(TAPS):
        z += shift(x, dy, dx) @ w[t]
    return z + b


def conv_dgrad(dz, w):
    dx = np.zeros(dz.shape[:3] + (w.shape[1],))
    for t, (dy, dx_) in enumerate(TAPS):
        dx += shift(dz @ w[t].T, -dy, -dx_)
    return dx


def conv_wgrad(x, dz):
    ci, co = x.shape[3], dz.shape[3]
    g = np.zeros((9, ci, co))
    dzf = dz.reshape(-1, co)
    for t, (dy, dx) in enumerate(TAPS):
        g[t] = shift(x, dy, dx).reshape(-1, ci).T @ dzf
    return g, dzf.sum(0)


def pool(x):
    return 0.25 * (x[:, 0::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 0::2] + x[:, 1::2, 1::2])


def pool_back(g):
    return 0.25 * np.repeat(np.repeat(g, 2, axis=1), 2, axis=2)


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_back(g):
    return g[:, 0::2, 0::2] + g[:, 0::2, 1::2] + g[:, 1::2, 0::2] + g[:, 1::2, 1::2]


def kernel_offsets(H, W, Hr, Wr):
    """For every padded pixel and filter tap k, the flat source pixel (clamped to the real image)."""
    y, x = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    yc, xc = np.minimum(y, Hr - 1), np.minimum(x, Wr - 1)
    idx = np.zeros((H, W, KS * KS), np.int64)
    for k in range(KS * KS):
        yy = np.clip(yc + k // KS - KS // 2, 0, Hr - 1)
        xx = np.clip(xc + k % KS - KS // 2, 0, Wr - 1)
        idx[..., k] = yy * W + xx
    return idx


class Net:
    """Forward + backward of the whole network for one batch.  rounded=False gives the exact
    FP64 network (used to check the backward pass by finite differences)."""

    def __init__(self, params, rounded=True):
        ws, self.b = unpack(params)
        self.r = bf16 if rounded else exact
        self.w = [self.r(w) for w in ws]

    def forward(self, rgb, gbuf):
        N, Hr, Wr, _ = rgb.shape
        H, W = (Hr + 15) // 16 * 16, (Wr + 15) // 16 * 16
        self.dims = (N, H, W, Hr, Wr)
        R = self.r
        X0, rad = features(rgb, gbuf, H, W, R)
        w, b = self.w, self.b
        a = {}
        a["X0"] = X0
        cv = lambda i, x: R(np.maximum(conv(x, w[i], b[i]), 0.0))
        a["A0a"] = cv(0, X0); a["A0b"] = cv(1, a["A0a"]); a["p1"] = R(pool(a["A0b"]))
        a["A1a"] = cv(2, a["p1"]); a["A1b"] = cv(3, a["A1a"]); a["p2"] = R(pool(a["A1b"]))
        a["A2a"] = cv(4, a["p2"]); a["A2b"] = cv(5, a["A2a"]); a["p3"] = R(pool(a["A2b"]))
        a["A3a"] = cv(6, a["p3"]); a["A3b"] = cv(7, a["A3a"]); a["p4"] = R(pool(a["A3b"]))
        a["A4a"] = cv(8, a["p4"]); a["A4b"] = cv(9, a["A4a"])
        a["cat3"] = np.concatenate([up(a["A4b"]), a["A3b"]], -1)
        a["D3a"] = cv(10, a["cat3"]); a["D3b"] = cv(11, a["D3a"])
        a["cat2"] = np.concatenate([up(a["D3b"]), a["A2b"]], -1)
        a["D2a"] = cv(12, a["cat2"]); a["D2b"] = cv(13, a["D2a"])
        a["cat1"] = np.concatenate([up(a["D2b"]), a["A1b"]], -1)
        a["D1a"] = cv(14, a["cat1"]); a["D1b"] = cv(15, a["D1a"])
        a["cat0"] = np.concatenate([up(a["D1b"]), a["A0b"]], -1)
        a["D0a"] = cv(16, a["cat0"]); a["D0b"] = cv(17, a["D0a"])
        logits = conv(a["D0b"], w[18], b[18])[..., :KS * KS]
        e = np.exp(logits - logits.max(-1, keepdims=True))
        wts = e / e.sum(-1, keepdims=True)
        idx = kernel_offsets(H, W, Hr, Wr)
        radf = rad.reshape(N, H * W, 3)
        nb = radf[:, idx]                                   # [N, H, W, 25, 3]
        out = (wts[..., None] * nb).sum(-2)
        self.a, self.wts, self.nb, self.out = a, wts, nb, out
        return out[:, :Hr, :Wr]

    def use_activations(self, ex, rgb, gbuf):
        """Replaces the forward activations by another implementation's (ex: name -> flat array,
        as cpt_denoiser_export names them), so that backward() checks that implementation's
        backward pass on its own forward values (identical ReLU masks) instead of re-deriving
        them: in a deep BF16 network the two forward passes drift apart by rounding, and a
        pre-activation within a rounding step of zero can take the other side of the ReLU."""
        N, Hr, Wr, _ = rgb.shape
        H, W = (Hr + 15) // 16 * 16, (Wr + 15) // 16 * 16
        self.dims = (N, H, W, Hr, Wr)
        chans = {"X0": 32, "A0a": 32, "cat0": 96, "p1": 32, "A1a": 64, "cat1": 160, "p2": 64, "A2a": 96,
                 "cat2": 224, "p3": 96, "A3a": 128, "cat3": 288, "p4": 128, "A4a": 160, "A4b": 160, "D3a": 128,
                 "D3b": 128, "D2a": 96, "D2b": 96, "D1a": 64, "D1b": 64, "D0a": 32, "D0b": 32, "logits": 32}
        level = {"X0": 0, "A0a": 0, "cat0": 0, "p1": 1, "A1a": 1, "cat1": 1, "p2": 2, "A2a": 2, "cat2": 2, "p3": 3,
                 "A3a": 3, "cat3": 3, "p4": 4, "A4a": 4, "A4b": 4, "D3a": 3, "D3b": 3, "D2a": 2, "D2b": 2, "D1a": 1,
                 "D1b": 1, "D0a": 0, "D0b": 0, "logits": 0}
        a = {k: np.asarray(ex[k], np.float64).reshape(N, H >> level[k], W >> level[k], c) for k, c in chans.items()}
        a["A0b"], a["A1b"] = a["cat0"][..., 64:], a["cat1"][..., 96:]
        a["A2b"], a["A3b"] = a["cat2"][..., 128:], a["cat3"][..., 160:]
        self.a = a
        _, rad = features(rgb, gbuf, H, W, self.r)
        logits = a["logits"][..., :KS * KS]
        e = np.exp(logits - logits.max(-1, keepdims=True))
        self.wts = e / e.sum(-1, keepdims=True)
        self.nb = rad.reshape(N, H * W, 3)[:, kernel_offsets(H, W, Hr, Wr)]
        self.out = (self.wts[..., None] * self.nb).sum(-2)

    def layer_outputs(self):
        """Each convolution recomputed from this Net's stored inputs: {output name: (value, layer)}."""
        a, w, b, R = self.a, self.w, self.b, self.r
        cv = lambda i, x: R(np.maximum(conv(x, w[i], b[i]), 0.0))
        pairs = [("A0a", 0, "X0"), ("A0b", 1, "A0a"), ("A1a", 2, "p1"), ("A1b", 3, "A1a"), ("A2a", 4, "p2"),
                 ("A2b", 5, "A2a"), ("A3a", 6, "p3"), ("A3b", 7, "A3a"), ("A4a", 8, "p4"), ("A4b", 9, "A4a"),
                 ("D3a", 10, "cat3"), ("D3b", 11, "D3a"), ("D2a", 12, "cat2"), ("D2b", 13, "D2a"),
                 ("D1a", 14, "cat1"), ("D1b", 15, "D1a"), ("D0a", 16, "cat0"), ("D0b", 17, "D0a")]
        out = {name: (cv(i, a[src]), i) for name, i, src in pairs}
        out["logits"] = (conv(a["D0b"], w[18], b[18]), 18)
        out["p1"] = (R(pool(a["A0b"])), -1)
        out["p2"] = (R(pool(a["A1b"])), -1)
        out["p3"] = (R(pool(a["A2b"])), -1)
        out["p4"] = (R(pool(a["A3b"])), -1)
        return out

    def loss(self, target):
        N, H, W, Hr, Wr = self.dims
        o = self.out[:, :Hr, :Wr]
        lo = np.sqrt(np.maximum(o, 0.0) + LOSS_EPS)
        d = lo - np.sqrt(np.maximum(target, 0.0) + LOSS_EPS)
        scale = 1.0 / (N * Hr * Wr * 3)
        dout = np.zeros_like(self.out)
        dout[:, :Hr, :Wr] = np.where(o > 0, scale * np.sign(d) * 0.5 / lo, 0.0)
        self.dout = dout
        return np.abs(d).sum() * scale

    def backward(self):
        a, w = self.a, self.w
        gw = [None] * 19
        gb = [None] * 19
        dwk = (self.dout[..., None, :] * self.nb).sum(-1)   # [N, H, W, 25]
        dl = self.wts * (dwk - (self.wts * dwk).sum(-1, keepdims=True))
        dz = np.zeros(dl.shape[:3] + (32,))
        dz[..., :KS * KS] = dl
        R = self.r
        dz = R(dz)

        def layer(i, x, dz, need_dx=True):
            gw[i], gb[i] = conv_wgrad(x, dz)
            return conv_dgrad(dz, w[i]) if need_dx else None

        rb = lambda g, act: R(g * (act > 0))
        G = self.g = {}   # activation gradients, named as the library's cpt_denoiser_export
        g = G["G_D0b"] = layer(18, a["D0b"], dz)
        g = G["G_D0a"] = layer(17, a["D0a"], rb(g, a["D0b"]))
        gcat0 = layer(16, a["cat0"], rb(g, a["D0a"]))
        g = G["G_D1b"] = up_back(gcat0[..., :64])
        g = layer(15, a["D1a"], rb(g, a["D1b"]))
        gcat1 = layer(14, a["cat1"], rb(g, a["D1a"]))
        g = G["G_D2b"] = up_back(gcat1[..., :96])
        g = layer(13, a["D2a"], rb(g, a["D2b"]))
        gcat2 = layer(12, a["cat2"], rb(g, a["D2a"]))
        g = G["G_D3b"] = up_back(gcat2[..., :128])
        g = layer(11, a["D3a"], rb(g, a["D3b"]))
        gcat3 = layer(10, a["cat3"], rb(g, a["D3a"]))
        g = G["G_A4b"] = up_back(gcat3[..., :160])
        g = layer(9, a["A4a"], rb(g, a["A4b"]))
        g = G["G_p4"] = layer(8, a["p4"], rb(g, a["A4a"]))
        g = gcat3[..., 160:] + pool_back(g)
        G["G_cat3"] = np.concatenate([gcat3[..., :160], g], -1)
        g = layer(7, a["A3a"], rb(g, a["A3b"]))
        g = G["G_p3"] = layer(6, a["p3"], rb(g, a["A3a"]))
        g = gcat2[..., 128:] + pool_back(g)
        G["G_cat2"] = np.concatenate([gcat2[..., :128], g], -1)
        g = layer(5, a["A2a"], rb(g, a["A2b"]))
        g = G["G_p2"] = layer(4, a["p2"], rb(g, a["A2a"]))
        g = gcat1[..., 96:] + pool_back(g)
        G["G_cat1"] = np.concatenate([gcat1[..., :96], g], -1)
        g = layer(3, a["A1a"], rb(g, a["A1b"]))
        g = G["G_p1"] = layer(2, a["p1"], rb(g, a["A1a"]))
        g = gcat0[..., 64:] + pool_back(g)
        G["G_cat0"] = np.concatenate([gcat0[..., :64], g], -1)
        g = G["G_A0a"] = layer(1, a["A0a"], rb(g, a["A0b"]))
        layer(0, a["X0"], rb(g, a["A0a"]), need_dx=False)
        flat = []
        for i in range(19):
            flat.append(gw[i].reshape(-1))
            flat.append(gb[i])
        return np.concatenate(flat)
