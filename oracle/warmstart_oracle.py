"""CPU oracle of the warm-start network (test infrastructure only).

The product runs the network in the library's CUDA kernels; this numpy
restatement is the checker the GPU tests compare against: the feature
assembly, the 3x3 convolution forward pass, its input gradient and weight
gradient, GELU, and the residual loss through the 5-point operator with its
gradient.  The network has no counterpart in the reference, so there is no
reference line to cite; the operator is the tealeaf-mode `smvp` of
src/kernels.jl:178-184 with Kx/Ky of src/solvers/CG.jl:57-72 (conductivity =
density) and the reflective (zero-flux) domain boundary.

Two precisions: `rounded=True` rounds to BF16 at exactly the points where the
kernels store BF16 (features, activations, pre-activations, gradients) and
sums in float64; `rounded=False` is plain float64, used to check the backward
pass against finite differences.

Arrays: images are NHWC, a deck's fields are [ny, nx] (x contiguous), weights
W[cout][9][cin] with tap = 3*dy + dx, biases b[cout].
"""
from __future__ import annotations

import numpy as np

LAYERS = [(16, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 16)]
NPARAMS = sum(co * 9 * ci + co for ci, co in LAYERS)
GELU_C = 0.7978845608028654


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray):
    """Flat parameter vector -> [(W[cout, 9, cin], b[cout]), ...]."""
    out, off = [], 0
    for ci, co in LAYERS:
        w = params[off:off + co * 9 * ci].reshape(co, 9, ci)
        off += co * 9 * ci
        b = params[off:off + co]
        off += co
        out.append((np.asarray(w, dtype=np.float64), np.asarray(b, dtype=np.float64)))
    return out


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GELU_C * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(GELU_C * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * 0.044715 * z * z)


def conv(x, w):
    """y[n, h, w, co] = sum_{dy, dx, ci} W[co, 3dy+dx, ci] x[n, h+dy-1, w+dx-1, ci] (zero padding)."""
    n, hh, ww, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((n, hh, ww, w.shape[0]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        y += xp[:, dy:dy + hh, dx:dx + ww, :] @ w[:, tap, :].T
    return y


def conv_input_grad(dz, w):
    """dx[n, h, w, ci] = sum_{tap, co} dz[n, h-dy+1, w-dx+1, co] W[co, tap, ci]."""
    n, hh, ww, _ = dz.shape
    zp = np.pad(dz, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dx_ = np.zeros((n, hh, ww, w.shape[2]))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        dx_ += zp[:, 2 - dy:2 - dy + hh, 2 - dx:2 - dx + ww, :] @ w[:, tap, :]
    return dx_


def conv_weight_grad(x, dz):
    """(dW[co, tap, ci], db[co]) of y = conv(x, W) + b for the output gradient dz."""
    n, hh, ww, ci = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((dz.shape[3], 9, ci))
    for tap in range(9):
        dy, dx = divmod(tap, 3)
        dw[:, tap, :] = np.einsum("nhwc,nhwd->cd", dz, xp[:, dy:dy + hh, dx:dx + ww, :])
    return dw, dz.sum(axis=(0, 1, 2))


class Crop:
    """A crop of a deck (fields [ny, nx]): origin (ox, oy), size h x w."""

    def __init__(self, u, uprev, rho, ox, oy, h, w, rx, ry):
        self.u, self.uprev, self.rho = u, uprev, rho
        self.ox, self.oy, self.h, self.w, self.rx, self.ry = ox, oy, h, w, rx, ry
        ny, nx = u.shape
        self.nx, self.ny = nx, ny
        self.inv_su = 1.0 / np.sqrt(np.mean(u * u))
        self.inv_sd = 1.0 / np.sqrt(np.mean((u - uprev) ** 2))

    def window(self, a, pad=0):
        return a[self.oy - pad:self.oy + self.h + pad, self.ox - pad:self.ox + self.w + pad]


def features(crops, rounded=True):
    """feat[B, h, w, 16]: u / rms(u), log(rx / rho) / 4, (u - uprev) / rms(u - uprev), zeros."""
    out = []
    for c in crops:
        u, up, rho = c.window(c.u), c.window(c.uprev), c.window(c.rho)
        f = np.zeros(u.shape + (16,))
        if rounded:
            f[..., 0] = bf16(np.float32(u * c.inv_su))
            f[..., 1] = bf16(np.float32(0.25) * np.float32(np.log(c.rx / rho)))
            f[..., 2] = bf16(np.float32((u - up) * c.inv_sd))
        else:
            f[..., 0] = u * c.inv_su
            f[..., 1] = 0.25 * np.log(c.rx / rho)
            f[..., 2] = (u - up) * c.inv_sd
        out.append(f)
    return np.stack(out)


def forward(params, feat, rounded=True):
    """Returns g[B, h, w] (channel 0 of the last layer) and the saved (x, z) per layer."""
    r = bf16 if rounded else (lambda v: v)
    layers = unpack(params)
    x = feat
    saved = []
    for k, (w, b) in enumerate(layers):
        wv = r(w)
        z = conv(x, wv) + b
        saved.append((x, r(z)))
        if k < len(layers) - 1:
            x = r(gelu(z))
        else:
            g = z[..., 0].astype(np.float32).astype(np.float64) if rounded else z[..., 0]
    return g, saved


def _faces(c):
    """Face coefficients around each crop cell (West, East, South, North), zero across the domain edge."""
    rho = c.rho
    ny, nx = rho.shape
    kxf = np.zeros((ny, nx + 1))   # face between x-1 and x
    kyf = np.zeros((ny + 1, nx))
    kxf[:, 1:nx] = c.rx * (rho[:, :-1] + rho[:, 1:]) / (2.0 * rho[:, :-1] * rho[:, 1:])
    kyf[1:ny, :] = c.ry * (rho[:-1, :] + rho[1:, :]) / (2.0 * rho[:-1, :] * rho[1:, :])
    ys, xs = slice(c.oy, c.oy + c.h), slice(c.ox, c.ox + c.w)
    kw = kxf[ys, c.ox:c.ox + c.w]
    ke = kxf[ys, c.ox + 1:c.ox + c.w + 1]
    ks = kyf[c.oy:c.oy + c.h, xs]
    kn = kyf[c.oy + 1:c.oy + c.h + 1, xs]
    return kw, ke, ks, kn


def _apply_a(v, k):
    """A v on the crop for v given on the crop with a 1-cell zero border in `v` (shape (h+2, w+2))."""
    kw, ke, ks, kn = k
    c = v[1:-1, 1:-1]
    return (c + kw * (c - v[1:-1, :-2]) + ke * (c - v[1:-1, 2:]) + ks * (c - v[:-2, 1:-1])
            + kn * (c - v[2:, 1:-1]))


def loss(crops, g, margin, objective=0):
    """(L, per-crop (term, plain), dL/dg[B, h, w]) of the residual loss (float64):
    objective 0 averages the terms, 1 averages log(term / plain)."""
    B = len(crops)
    terms, dg = [], np.zeros(g.shape)
    for b, c in enumerate(crops):
        h, w = c.h, c.w
        d = c.window(c.u) - c.window(c.uprev)
        x = (1.0 + g[b]) * d
        k = _faces(c)
        xp = np.pad(x, 1)
        r = d - _apply_a(xp, k)
        mask = np.zeros((h, w), dtype=bool)
        mask[margin:h - margin, margin:w - margin] = True
        ncell = mask.sum()
        s2 = c.inv_sd ** 2
        term = np.sum((r[mask] ** 2)) * s2 / ncell
        terms.append((term, np.sum(d[mask] ** 2) * s2 / ncell))
        rt = np.where(mask, r, 0.0)
        ar = _apply_a(np.pad(rt, 1), k)
        band = np.zeros((h, w), dtype=bool)
        band[margin - 1:h - margin + 1, margin - 1:w - margin + 1] = True
        scale = -2.0 * s2 / (ncell * B)
        if objective == 1:
            scale = scale / term if term > 0 else 0.0
        dg[b] = np.where(band, ar * d * scale, 0.0)
    if objective == 1:
        return float(np.mean([np.log(t / p) for t, p in terms])), terms, dg
    return float(np.mean([t[0] for t in terms])), terms, dg


def backward(params, saved, dg, rounded=True):
    """Flat gradient of the loss for the output gradient dg[B, h, w] (channel 0)."""
    r = bf16 if rounded else (lambda v: v)
    layers = unpack(params)
    dz = np.zeros(dg.shape + (LAYERS[-1][1],))
    dz[..., 0] = r(np.float32(dg)) if rounded else dg
    grads = [None] * len(layers)
    for k in range(len(layers) - 1, -1, -1):
        x, _ = saved[k]
        dw, db = conv_weight_grad(x, dz)
        grads[k] = (dw, db)
        if k > 0:
            w = r(layers[k][0])
            dx = conv_input_grad(dz, w)
            zprev = saved[k - 1][1]
            dz = r(dx * gelu_grad(zprev))
    return np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])


def init_params(seed: int = 0, out_scale: float = 1e-3) -> np.ndarray:
    """He-normal weights on the used channels, zero biases; the last layer's
    channel 0 starts small (g ~ 0: the prediction starts as u^n + (u^n - u^{n-1}))."""
    rng = np.random.default_rng(seed)
    parts = []
    for k, (ci, co) in enumerate(LAYERS):
        used_in = 3 if k == 0 else ci
        w = np.zeros((co, 9, ci))
        if k == len(LAYERS) - 1:
            w[0, :, :used_in] = rng.standard_normal((9, used_in)) * out_scale
        else:
            w[:, :, :used_in] = rng.standard_normal((co, 9, used_in)) * np.sqrt(2.0 / (9 * used_in))
        parts += [w.ravel(), np.zeros(co)]
    return np.concatenate(parts).astype(np.float32)
