"""CPU oracle of the learned-guess U-Net (TEST INFRASTRUCTURE ONLY).

The reference solver has no learned component, so there is no reference
code to follow here: this is an independent numpy statement of the network
the library trains (ekman_bl_gb300/csrc/ek_unet.cu), used to check the GPU
forward pass and parameter gradients.  With bf16_round=True it rounds at
the points where the GPU stores or stages BF16 values:

  - every GEMM operand: activations (already BF16), weights, and the FP32
    gradient dZ when it feeds the input- and weight-gradient products;
  - the outputs of the ReLU convolutions and of the average pooling;
then accumulates in float64 (the GPU accumulates in FP32, in a different
order) and stores gradients in float32.  With bf16_round=False it runs in
plain float64, which is what the finite-difference test of the backward
pass uses.

Layout: images NHWC, weights W[cout][9][cin] with tap = 3*(dy+1) + (dx+1),
parameters flat, layer after layer, W then b.
"""
from __future__ import annotations

import numpy as np

LEVELS = 4


def bf16(a: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16) & 0xFFFFFFFF
    out = r.astype(np.uint32).view(np.float32).copy()
    nan = np.isnan(a)
    out[nan] = np.nan
    return out


def layer_specs(cin: int, C: int):
    """(cin, cout, c1, c2, relu) of the 15 convolutions in parameter order."""
    s = [(cin, C, cin, 0)] + [(C, C, C, 0)] * 7
    for _ in range(3):
        s += [(2 * C, C, C, C), (C, C, C, 0)]
    s += [(C, 1, C, 0)]
    return [(a, b, c, d, i < len(s) - 1) for i, (a, b, c, d) in enumerate(s)]


def split_params(params: np.ndarray, cin: int, C: int):
    out, off = [], 0
    for ci, co, *_ in layer_specs(cin, C):
        w = params[off:off + co * 9 * ci].reshape(co, 9, ci)
        off += co * 9 * ci
        b = params[off:off + co]
        off += co
        out.append((w, b))
    assert off == params.size
    return out


def init_params(cin: int, C: int, seed: int) -> np.ndarray:
    """He-normal weights, zero biases (float32)."""
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co, *_ in layer_specs(cin, C):
        parts.append((rng.standard_normal(co * 9 * ci) * np.sqrt(2.0 / (9 * ci))).astype(np.float32))
        parts.append(np.zeros(co, np.float32))
    return np.concatenate(parts)


TAPS = [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def _shift(x, dy, dx):
    """x[:, y+dy, x+dx, :] with zeros outside."""
    n, H, W, c = x.shape
    p = np.zeros((n, H + 2, W + 2, c), x.dtype)
    p[:, 1:H + 1, 1:W + 1] = x
    return p[:, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W]


class Net:
    def __init__(self, params, cin: int, C: int, bf16_round: bool = True):
        self.cin, self.C, self.rb = cin, C, bf16_round
        self.specs = layer_specs(cin, C)
        self.layers = split_params(np.asarray(params, np.float32 if bf16_round else np.float64), cin, C)

    def _r(self, a):
        return bf16(a) if self.rb else np.asarray(a, np.float64)

    def _store(self, a):
        return np.asarray(a, np.float32) if self.rb else a

    def conv(self, l, x):
        w, b = self.layers[l]
        wr = self._r(w).astype(np.float64)
        n, H, W, _ = x.shape
        acc = np.zeros((n, H, W, w.shape[0]))
        for t, (dy, dx) in enumerate(TAPS):
            acc += _shift(x.astype(np.float64), dy, dx) @ wr[:, t, :].T
        v = acc.astype(np.float32) + b.astype(np.float32) if self.rb else acc + b
        if self.specs[l][4]:
            v = np.maximum(v, 0)
            return bf16(v) if self.rb else v
        return v

    def pool(self, s):
        if self.rb:
            v = ((s[:, 0::2, 0::2] + s[:, 0::2, 1::2]) + s[:, 1::2, 0::2]) + s[:, 1::2, 1::2]
            return bf16(np.float32(0.25) * v.astype(np.float32))
        return 0.25 * (s[:, 0::2, 0::2] + s[:, 0::2, 1::2] + s[:, 1::2, 0::2] + s[:, 1::2, 1::2])

    @staticmethod
    def up(d):
        return d.repeat(2, axis=1).repeat(2, axis=2)

    def forward(self, x):
        """x: (n, H, W, cin); returns the output (n, H, W) and the activations."""
        a = {}
        a["x"] = self._r(x) if self.rb else np.asarray(x, np.float64)
        a["t0"] = self.conv(0, a["x"])
        a["s0"] = self.conv(1, a["t0"])
        for l in range(1, LEVELS):
            a[f"p{l}"] = self.pool(a[f"s{l - 1}"])
            a[f"t{l}"] = self.conv(2 * l, a[f"p{l}"])
            a[f"s{l}"] = self.conv(2 * l + 1, a[f"t{l}"])
        below = a[f"s{LEVELS - 1}"]
        for l in range(LEVELS - 2, -1, -1):
            li = 8 + 2 * (LEVELS - 2 - l)
            a[f"u{l}"] = self.up(below)
            a[f"v{l}"] = self.conv(li, np.concatenate([a[f"u{l}"], a[f"s{l}"]], axis=-1))
            a[f"d{l}"] = self.conv(li + 1, a[f"v{l}"])
            below = a[f"d{l}"]
        y = self.conv(14, a["d0"])[..., 0]
        return y, a

    def _back(self, l, x, dz, grads, need_dx=True):
        """dW, db of layer l into grads; returns dX (float64 before storage)."""
        w, _ = self.layers[l]
        wr = self._r(w).astype(np.float64)
        dzr = self._r(dz).astype(np.float64)
        xr = np.asarray(x, np.float64)
        cout, _, cin = w.shape
        gw = np.zeros((cout, 9, cin))
        for t, (dy, dx) in enumerate(TAPS):
            gw[:, t, :] = dzr.reshape(-1, cout).T @ _shift(xr, dy, dx).reshape(-1, cin)
        grads[l] = (gw, np.asarray(dz, np.float64).sum(axis=(0, 1, 2)))
        if not need_dx:
            return None
        dx_ = np.zeros(x.shape)
        for t, (dy, dx) in enumerate(TAPS):
            dx_ += _shift(dzr, -dy, -dx) @ wr[:, t, :]
        return dx_

    def _mask(self, g, act):
        g = np.where(np.asarray(act) > 0, g, 0.0)
        return self._store(g)

    def loss_and_grads(self, x, t, hv, wv):
        """Mean-square error over the top-left hv x wv pixels, the output and
        the flat parameter gradient."""
        y, a = self.forward(x)
        n, H, W = y.shape
        valid = np.zeros((H, W), bool)
        valid[:hv, :wv] = True
        if self.rb:
            d = (np.asarray(y, np.float32) - np.asarray(t, np.float32)) * valid
            loss = float((d.astype(np.float64) ** 2).sum() / (n * hv * wv))
            gy = (np.float32(2.0 / (n * hv * wv)) * d).astype(np.float32)
        else:
            d = (y - t) * valid
            loss = float((d ** 2).sum() / (n * hv * wv))
            gy = 2.0 * d / (n * hv * wv)
        grads = [None] * 15
        g = self._back(14, a["d0"], gy[..., None], grads)
        gd = self._mask(g, a["d0"])
        gs = {}
        C = self.C
        for l in range(0, LEVELS - 1):
            li = 8 + 2 * (LEVELS - 2 - l)
            gv = self._mask(self._back(li + 1, a[f"v{l}"], gd, grads), a[f"v{l}"])
            g = self._back(li, np.concatenate([a[f"u{l}"], a[f"s{l}"]], axis=-1), gv, grads)
            gu = self._store(g[..., :C])
            gs[l] = self._mask(g[..., C:], a[f"s{l}"])
            below = a[f"d{l + 1}"] if l + 1 <= LEVELS - 2 else a[f"s{LEVELS - 1}"]
            su = ((gu[:, 0::2, 0::2] + gu[:, 0::2, 1::2]) + gu[:, 1::2, 0::2]) + gu[:, 1::2, 1::2]
            gnext = self._mask(su, below)
            if l + 1 <= LEVELS - 2:
                gd = gnext
            else:
                gs[LEVELS - 1] = gnext
        for l in range(LEVELS - 1, 0, -1):
            gt = self._mask(self._back(2 * l + 1, a[f"t{l}"], gs[l], grads), a[f"t{l}"])
            gp = self._store(self._back(2 * l, a[f"p{l}"], gt, grads))
            q = (np.float32(0.25) * gp) if self.rb else 0.25 * gp
            q = self._mask(self.up(q), a[f"s{l - 1}"])
            gs[l - 1] = self._store(gs[l - 1] + q)
        gt = self._mask(self._back(1, a["t0"], gs[0], grads), a["t0"])
        self._back(0, a["x"], gt, grads, need_dx=False)
        flat = np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])
        return loss, y, flat
