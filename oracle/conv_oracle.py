"""FP64 CPU oracle for the learned surrogate's convolutions and optimiser.

Test infrastructure only: the GPU tests compare the tensor-core kernels (and
the network built on them) with these restatements; nothing in the product
path imports this module. The surrogate has no counterpart in the reference
(it is the learned pattern the task adds beside the plain FastScape step of
fastscape_RB.cpp:366-373), so these are the textbook definitions:

* 3x3 convolution with zero padding (cross-correlation, as in every deep
  learning framework): y[b,y,x,co] = sum_{dy,dx,ci} x[b,y+dy-1,x+dx-1,ci] *
  w[co,3dy+dx,ci]; a 1x1 convolution is the same with one tap;
* its data gradient (the transposed convolution) and weight gradient;
* Adam (Kingma & Ba 2015) with bias correction.

Tensors are NHWC; BF16 values travel as uint16 bit patterns and are widened
exactly to float64 before any arithmetic.
"""
from __future__ import annotations

import numpy as np


def bf16_bits(a) -> np.ndarray:
    """float -> BF16 bit patterns, round to nearest even (NaN kept NaN)."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    nan = np.isnan(f)
    if nan.any():
        r[nan] = 0x7FC0
    return r


def bf16_value(bits) -> np.ndarray:
    """BF16 bit patterns -> float64 (exact)."""
    b = np.ascontiguousarray(bits, dtype=np.uint16).astype(np.uint32) << 16
    return b.view(np.float32).astype(np.float64)


def _taps(taps: int):
    return [(0, 0)] if taps == 1 else [(dy - 1, dx - 1) for dy in range(3) for dx in range(3)]


def _shift(x: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """s[b,y,x,:] = x[b,y+dy,x+dx,:], zero outside the image."""
    B, H, W, C = x.shape
    s = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    s[:, ys:ye, xs:xe, :] = x[:, ys + dy:ye + dy, xs + dx:xe + dx, :]
    return s


def conv_forward(x: np.ndarray, w: np.ndarray, bias=None, relu=False) -> np.ndarray:
    """x [B,H,W,cin], w [cout,taps,cin] -> [B,H,W,cout] (float64)."""
    cout, taps, cin = w.shape
    y = np.zeros(x.shape[:3] + (cout,), np.float64)
    for t, (dy, dx) in enumerate(_taps(taps)):
        y += np.einsum("bhwc,oc->bhwo", _shift(x, dy, dx), w[:, t, :], optimize=True)
    if bias is not None:
        y += np.asarray(bias, np.float64)
    if relu:
        y = np.maximum(y, 0.0)
    return y


def conv_data_grad(dy: np.ndarray, w: np.ndarray, mask=None) -> np.ndarray:
    """dL/dx of conv_forward (no activation) given dL/dy [B,H,W,cout];
    zeroed where mask <= 0 when a mask is given."""
    cout, taps, cin = w.shape
    dx = np.zeros(dy.shape[:3] + (cin,), np.float64)
    for t, (oy, ox) in enumerate(_taps(taps)):
        # y[p] uses x[p + off]; so x[q] receives dy[q - off]
        dx += np.einsum("bhwo,oc->bhwc", _shift(dy, -oy, -ox), w[:, t, :], optimize=True)
    if mask is not None:
        dx = np.where(np.asarray(mask) > 0, dx, 0.0)
    return dx


def conv_weight_grad(x: np.ndarray, dy: np.ndarray, taps: int) -> np.ndarray:
    """dL/dw [cout,taps,cin] of conv_forward given dL/dy."""
    cout, cin = dy.shape[3], x.shape[3]
    dw = np.zeros((cout, taps, cin), np.float64)
    for t, (oy, ox) in enumerate(_taps(taps)):
        dw[:, t, :] = np.einsum("bhwo,bhwc->oc", dy, _shift(x, oy, ox), optimize=True)
    return dw


def adam_step(p, g, m, v, t: int, lr: float, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
