"""CPU reference of the learned p' initial-guess network (TEST INFRASTRUCTURE ONLY).

This is the checker of the GPU network kernels in gfm_gb300/csrc/lp.cu: the
same layers, parameter layout and storage precision, in numpy FP64.  With
`bf16=True` every tensor the GPU stores in BF16 (weights, activations, the
activation gradients) is rounded to BF16 at the same points, so the GPU and
this reference differ only by FP32 versus FP64 accumulation.  Only tests/
use it.

Layout: tensors (nz, ny, nx, C); parameters per layer W[27][cout][cin] then
b[cout], tap t = (dz+1)*9 + (dy+1)*3 + (dx+1).
"""
from __future__ import annotations

import numpy as np

LAYERS = [(16, 16), (16, 16), (16, 32), (32, 32), (48, 16), (16, 16)]
FEAT_CHANNELS = 2


def num_params() -> int:
    return sum(27 * ci * co + co for ci, co in LAYERS)


def unpack(p: np.ndarray) -> list:
    out, off = [], 0
    for ci, co in LAYERS:
        w = p[off:off + 27 * ci * co].reshape(27, co, ci)
        off += 27 * ci * co
        b = p[off:off + co]
        off += co
        out.append((w, b))
    return out


def pack(grads: list) -> np.ndarray:
    return np.concatenate([np.concatenate([w.reshape(-1), b.reshape(-1)]) for w, b in grads])


def to_bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    u = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def _taps():
    for t in range(27):
        yield t, t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1


def _shift(x: np.ndarray, dx: int, dy: int, dz: int) -> np.ndarray:
    """y[z,y,x] = x[z+dz, y+dy, x+dx], zero outside."""
    nz, ny, nx = x.shape[:3]
    y = np.zeros_like(x)
    zs, ys, xs = slice(max(0, -dz), nz - max(0, dz)), slice(max(0, -dy), ny - max(0, dy)), slice(max(0, -dx), nx - max(0, dx))
    zt, yt, xt = slice(max(0, dz), nz + min(0, dz)), slice(max(0, dy), ny + min(0, dy)), slice(max(0, dx), nx + min(0, dx))
    y[zs, ys, xs] = x[zt, yt, xt]
    return y


def conv(x: np.ndarray, w: np.ndarray, b=None) -> np.ndarray:
    """out[v][co] = b[co] + sum_t sum_ci x[v + d_t][ci] * w[t][co][ci]"""
    out = np.zeros(x.shape[:3] + (w.shape[1],))
    for t, dx, dy, dz in _taps():
        out += np.einsum("zyxc,oc->zyxo", _shift(x, dx, dy, dz), w[t])
    if b is not None:
        out += b
    return out


def conv_wgrad(dy: np.ndarray, x: np.ndarray, cin: int, cout: int) -> np.ndarray:
    dw = np.zeros((27, cout, cin))
    for t, dx, dyy, dz in _taps():
        dw[t] = np.einsum("zyxo,zyxc->oc", dy, _shift(x, dx, dyy, dz))
    return dw


def conv_dgrad(dy: np.ndarray, w: np.ndarray) -> np.ndarray:
    """d x[u][ci] = sum_t sum_co dy[u - d_t][co] * w[t][co][ci]"""
    out = np.zeros(dy.shape[:3] + (w.shape[2],))
    for t, dx, dyy, dz in _taps():
        out += np.einsum("zyxo,oc->zyxc", _shift(dy, -dx, -dyy, -dz), w[t])
    return out


def pool(x):
    nz, ny, nx, c = x.shape
    return x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).mean(axis=(1, 3, 5))


def up(x):
    return x.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)


def up_bwd(d):
    nz, ny, nx, c = d.shape
    return d.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).sum(axis=(1, 3, 5))


def forward(p: np.ndarray, x: np.ndarray, bf16: bool = True) -> dict:
    q = to_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    f32 = (lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)) if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    L = [(q(w), f32(b)) for w, b in unpack(p)]
    s = {"x": q(x)}
    s["a1"] = q(np.maximum(conv(s["x"], *L[0]), 0))
    s["e0"] = q(np.maximum(conv(s["a1"], *L[1]), 0))
    s["p0"] = q(pool(s["e0"]))
    s["a2"] = q(np.maximum(conv(s["p0"], *L[2]), 0))
    s["e1"] = q(np.maximum(conv(s["a2"], *L[3]), 0))
    s["cat"] = np.concatenate([s["e0"], up(s["e1"])], axis=3)
    s["a3"] = q(np.maximum(conv(s["cat"], *L[4]), 0))
    s["out"] = f32(conv(s["a3"], *L[5]))
    s["layers"] = L
    return s


def loss_and_grads(p: np.ndarray, x: np.ndarray, target: np.ndarray, bf16: bool = True):
    """Mean squared error over open voxels (channel 1 of x) and its gradient."""
    q = to_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    s = forward(p, x, bf16)
    L = s["layers"]
    open_ = s["x"][..., 1] > 0.5
    n = max(int(open_.sum()), 1)
    e = np.where(open_, s["out"][..., 0] - target, 0.0)
    loss = float((e * e).sum() / n)
    dout = np.zeros_like(s["out"])
    dout[..., 0] = 2.0 * e / n
    dout = q(dout)
    g = [None] * 6
    # c6
    g[5] = (conv_wgrad(dout, s["a3"], 16, 16), dout.sum(axis=(0, 1, 2)))
    da3 = q(conv_dgrad(dout, L[5][0])) * (s["a3"] > 0)
    # c5
    g[4] = (conv_wgrad(da3, s["cat"], 48, 16), da3.sum(axis=(0, 1, 2)))
    dcat = q(conv_dgrad(da3, L[4][0]))
    # up
    de1 = q(up_bwd(dcat[..., 16:])) * (s["e1"] > 0)
    # c4
    g[3] = (conv_wgrad(de1, s["a2"], 32, 32), de1.sum(axis=(0, 1, 2)))
    da2 = q(conv_dgrad(de1, L[3][0])) * (s["a2"] > 0)
    # c3
    g[2] = (conv_wgrad(da2, s["p0"], 16, 32), da2.sum(axis=(0, 1, 2)))
    dp0 = q(conv_dgrad(da2, L[2][0]))
    # pool + skip
    de0 = q(dcat[..., :16] + up(dp0) / 8.0) * (s["e0"] > 0)
    # c2
    g[1] = (conv_wgrad(de0, s["a1"], 16, 16), de0.sum(axis=(0, 1, 2)))
    da1 = q(conv_dgrad(de0, L[1][0])) * (s["a1"] > 0)
    # c1
    g[0] = (conv_wgrad(da1, s["x"], 16, 16), da1.sum(axis=(0, 1, 2)))
    return loss, pack(g), s


def init_params(seed: int = 1) -> np.ndarray:
    """Small random parameters with the GPU's zero pattern (unused input channels
    of c1, unused output channels of c6)."""
    rng = np.random.default_rng(seed)
    parts = []
    for l, (ci, co) in enumerate(LAYERS):
        a = np.sqrt(6.0 / (27 * ci))
        w = rng.uniform(-a, a, (27, co, ci))
        if l == 0:
            w[:, :, FEAT_CHANNELS:] = 0
        if l == len(LAYERS) - 1:
            w[:, 1:, :] = 0
        b = rng.uniform(-0.05, 0.05, co)
        if l == len(LAYERS) - 1:
            b[1:] = 0
        parts += [w.reshape(-1), b]
    return np.concatenate(parts).astype(np.float32)
