"""FP64 CPU oracle of the learned surrogate network: forward pass, loss and
every parameter gradient, in numpy.

Test infrastructure only (the GPU tests compare the tensor-core network with
it; nothing in the product path imports it). The surrogate has no
counterpart in the reference; this restates the network the library builds
(include/fastscape_surrogate.h): a 4-level encoder-decoder of 3x3
convolutions with ReLU (channels c, 2c, 4c, 8c), 2x2 average pooling,
nearest upsampling concatenated with the encoder output of the same level,
and a 1x1 head, trained on

    L = (1/n) sum_s w_s * mean_interior (z_s - y_s)^2,
    w_s = (u_s / max(hmax_next_s, u_s))^2, y = (h_next - h) / u, u = jump*U*dt.

With bf16=True every tensor the device stores as BF16 (input planes, layer
outputs, pooled and concatenated tensors, and their gradients) is rounded to
BF16 at the same place, and the BF16 copies of the weights are used in the
convolutions, so the remaining differences are FP32 versus FP64 accumulation.
With bf16=False it is the exact FP64 function (for finite differences).
"""
from __future__ import annotations

import math

import numpy as np

from oracle import conv_oracle as co

INPUT_CHANNELS = 16
LOG10_U_MID = -3.1505
LOG10_U_HALF = 0.8495


def layer_shapes(c: int):
    """(cin, cout) of the 14 convolutions in forward order."""
    return [(INPUT_CHANNELS, c), (c, c), (c, 2 * c), (2 * c, 2 * c), (2 * c, 4 * c),
            (4 * c, 4 * c), (4 * c, 8 * c), (8 * c, 8 * c), (12 * c, 4 * c), (4 * c, 4 * c),
            (6 * c, 2 * c), (2 * c, 2 * c), (3 * c, c), (c, c)]


def param_layout(c: int):
    """[(w_off, b_off, cin, cout)] per layer, head offset, total count."""
    out, off = [], 0
    for cin, cout in layer_shapes(c):
        w = off
        off += cout * 9 * cin
        out.append((w, off, cin, cout))
        off += cout
    return out, off, off + c + 1


def make_meta(keq, meq, ueq, hmax, hmax_next, jump=50, dt=1000.0):
    """The per-sample constants, as FP32 values like the library's."""
    f = np.float32
    u = jump * ueq * dt
    s = max(hmax, u)
    r = max(hmax_next, u)
    return {"s": f(s), "u": f(u), "log_su": f(math.log(s / u) / 4.0),
            "k_n": f((math.log10(keq) + 5.5) / 0.5), "m_n": f((meq - 0.45) / 0.15),
            "u_n": f((math.log10(ueq) - LOG10_U_MID) / LOG10_U_HALF),
            "weight": f((u / r) * (u / r)), "inv_s": f(1) / f(s), "inv_u": f(1) / f(u)}


def ring_mask(W: int, H: int) -> np.ndarray:
    yy, xx = np.mgrid[0:H, 0:W]
    return (xx < 2) | (yy < 2) | (xx >= W - 2) | (yy >= H - 2)


def input_planes(h: np.ndarray, meta: dict, W: int, H: int, counts=None) -> np.ndarray:
    """The 16 input planes of one field (before BF16 rounding), in FP32 like
    the library: h*(1/s), log(s/u)/4, K, m, U, ring mask, log2(drainage
    count)/16, and on cells with a full neighbourhood the drop to the D8
    receiver, the central differences along x and y (times 1/2) and h minus
    0.125 times the sum of its 8 neighbours, each times 1/u."""
    f32 = np.float32
    hh = np.asarray(h, np.float64).reshape(H, W).astype(f32)
    x = np.zeros((H, W, INPUT_CHANNELS), np.float64)
    x[..., 0] = hh * meta["inv_s"]
    x[..., 1] = meta["log_su"]
    x[..., 2] = meta["k_n"]
    x[..., 3] = meta["m_n"]
    x[..., 4] = meta["u_n"]
    x[..., 5] = ring_mask(W, H).astype(np.float64)
    if counts is not None:
        c = np.maximum(np.asarray(counts, np.float64).reshape(H, W), 1.0).astype(f32)
        x[..., 6] = np.log2(c) * f32(0.0625)
    iu = meta["inv_u"]
    c0 = hh[1:H - 1, 1:W - 1]
    # neighbours in the reference's order W, NW, N, NE, E, SE, S, SW
    sh = [(0, -1), (-1, -1), (-1, 0), (-1, 1), (0, 1), (1, 1), (1, 0), (1, -1)]
    nb = [hh[1 + dy:H - 1 + dy, 1 + dx:W - 1 + dx] for dy, dx in sh]
    best = np.zeros_like(c0)
    drop = np.zeros_like(c0)
    total = np.zeros_like(c0)
    for k in range(8):
        d = c0 - nb[k]
        slope = d / f32(1.41421356) if k & 1 else d
        better = slope > best
        best = np.where(better, slope, best)
        drop = np.where(better, d, drop)
        total = total + nb[k]
    x[1:H - 1, 1:W - 1, 7] = drop * iu
    x[1:H - 1, 1:W - 1, 8] = (nb[4] - nb[0]) * f32(0.5) * iu
    x[1:H - 1, 1:W - 1, 9] = (nb[6] - nb[2]) * f32(0.5) * iu
    x[1:H - 1, 1:W - 1, 10] = (c0 - f32(0.125) * total) * iu
    return x


class Net:
    def __init__(self, c: int, W: int, H: int, bf16: bool = True):
        self.c, self.W, self.H, self.bf16 = c, W, H, bf16
        self.layout, self.head, self.count = param_layout(c)

    def q(self, a):
        return co.bf16_value(co.bf16_bits(a)) if self.bf16 else np.asarray(a, np.float64)

    def weights(self, p, l):
        w_off, b_off, cin, cout = self.layout[l]
        w = np.asarray(p[w_off:w_off + cout * 9 * cin], np.float64).reshape(cout, 9, cin)
        b = np.asarray(p[b_off:b_off + cout], np.float64)
        return self.q(w), b

    def conv(self, p, l, x):
        w, b = self.weights(p, l)
        return self.q(co.conv_forward(x, w, b, relu=True))

    @staticmethod
    def pool(x):
        return 0.25 * (x[:, 0::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 0::2] + x[:, 1::2, 1::2])

    @staticmethod
    def up(x):
        return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)

    def forward(self, p, x0):
        """x0 [n,H,W,16] -> activations dict."""
        q = self.q
        a = {"in0": q(x0)}
        a["e0a"] = self.conv(p, 0, a["in0"])
        a["s0"] = self.conv(p, 1, a["e0a"])
        a["p0"] = q(self.pool(a["s0"]))
        a["e1a"] = self.conv(p, 2, a["p0"])
        a["s1"] = self.conv(p, 3, a["e1a"])
        a["p1"] = q(self.pool(a["s1"]))
        a["e2a"] = self.conv(p, 4, a["p1"])
        a["s2"] = self.conv(p, 5, a["e2a"])
        a["p2"] = q(self.pool(a["s2"]))
        a["b1"] = self.conv(p, 6, a["p2"])
        a["b2"] = self.conv(p, 7, a["b1"])
        a["cat2"] = np.concatenate([self.up(a["b2"]), a["s2"]], axis=3)
        a["d2a"] = self.conv(p, 8, a["cat2"])
        a["d2b"] = self.conv(p, 9, a["d2a"])
        a["cat1"] = np.concatenate([self.up(a["d2b"]), a["s1"]], axis=3)
        a["d1a"] = self.conv(p, 10, a["cat1"])
        a["d1b"] = self.conv(p, 11, a["d1a"])
        a["cat0"] = np.concatenate([self.up(a["d1b"]), a["s0"]], axis=3)
        a["d0a"] = self.conv(p, 12, a["cat0"])
        a["d0b"] = self.conv(p, 13, a["d0a"])
        hw = np.asarray(p[self.head:self.head + self.c + 1], np.float64)
        a["z"] = np.einsum("nhwc,c->nhw", a["d0b"], hw[:-1]) + hw[-1]
        return a

    def loss_grad(self, p, x0, y, weights):
        """Loss and the gradient of every parameter (float64 vector)."""
        q = self.q
        n = x0.shape[0]
        W, H, c = self.W, self.H, self.c
        a = self.forward(p, x0)
        interior = ~ring_mask(W, H)
        inv = 1.0 / ((W - 4) * (H - 4) * n)
        err = (a["z"] - y) * interior
        wgt = np.asarray(weights, np.float64)[:, None, None]
        loss = float(np.sum(wgt * err * err) * inv)
        dz = 2.0 * wgt * err * inv
        if self.bf16:
            dz = dz.astype(np.float32).astype(np.float64)
        g = np.zeros(self.count, np.float64)
        hw = np.asarray(p[self.head:self.head + c + 1], np.float64)
        g[self.head:self.head + c] = np.einsum("nhw,nhwc->c", dz, a["d0b"])
        g[self.head + c] = dz.sum()
        gy = q(dz[..., None] * hw[None, None, None, :-1] * (a["d0b"] > 0))

        def layer(l, x, gy, mask):
            w_off, b_off, cin, cout = self.layout[l]
            g[w_off:w_off + cout * 9 * cin] = co.conv_weight_grad(x, gy, 9).reshape(-1)
            g[b_off:b_off + cout] = gy.sum(axis=(0, 1, 2))
            if mask is None and l == 0:
                return None
            w, _ = self.weights(p, l)
            gx = co.conv_data_grad(gy, w, mask=mask)
            return q(gx)

        def sumpool(gcat, cd):
            t = gcat[..., :cd]
            return q(t[:, 0::2, 0::2] + t[:, 0::2, 1::2] + t[:, 1::2, 0::2] + t[:, 1::2, 1::2])

        def skipgrad(gcat, cd, s, gp):
            return q(gcat[..., cd:] + np.where(s > 0, 0.25 * self.up(gp), 0.0))

        g_d0a = layer(13, a["d0a"], gy, a["d0a"])
        g_cat0 = layer(12, a["cat0"], g_d0a, a["cat0"])
        g_d1b = sumpool(g_cat0, 2 * c)
        g_d1a = layer(11, a["d1a"], g_d1b, a["d1a"])
        g_cat1 = layer(10, a["cat1"], g_d1a, a["cat1"])
        g_d2b = sumpool(g_cat1, 4 * c)
        g_d2a = layer(9, a["d2a"], g_d2b, a["d2a"])
        g_cat2 = layer(8, a["cat2"], g_d2a, a["cat2"])
        g_b2 = sumpool(g_cat2, 8 * c)
        g_b1 = layer(7, a["b1"], g_b2, a["b1"])
        g_p2 = layer(6, a["p2"], g_b1, None)
        g_s2 = skipgrad(g_cat2, 8 * c, a["s2"], g_p2)
        g_e2a = layer(5, a["e2a"], g_s2, a["e2a"])
        g_p1 = layer(4, a["p1"], g_e2a, None)
        g_s1 = skipgrad(g_cat1, 4 * c, a["s1"], g_p1)
        g_e1a = layer(3, a["e1a"], g_s1, a["e1a"])
        g_p0 = layer(2, a["p0"], g_e1a, None)
        g_s0 = skipgrad(g_cat0, 2 * c, a["s0"], g_p0)
        g_e0a = layer(1, a["e0a"], g_s0, a["e0a"])
        layer(0, a["in0"], g_e0a, None)
        return loss, g, a


def init_params(c: int, seed: int = 0) -> np.ndarray:
    """He-normal weights and small biases (for CPU checks)."""
    rng = np.random.default_rng(seed)
    layout, head, count = param_layout(c)
    p = np.zeros(count)
    for (w, b, cin, cout) in layout:
        p[w:w + cout * 9 * cin] = rng.normal(0, math.sqrt(2.0 / (9 * cin)), cout * 9 * cin)
        p[b:b + cout] = rng.normal(0, 0.05, cout)
    p[head:head + c] = rng.normal(0, 0.3, c)
    p[head + c] = 0.1
    return p
