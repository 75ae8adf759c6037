"""CPU checks of the surrogate's FP64 convolution oracle (oracle/conv_oracle.py):
BF16 conversion against torch, the forward convolution against a literal loop
over pixels, taps and channels, and the two gradients through the adjoint
identities <conv(x,w), g> = <x, dgrad(g,w)> = <w, wgrad(x,g)>, plus a finite
difference of Adam's first step. No GPU."""
import numpy as np
import pytest

from oracle import conv_oracle as co


def test_bf16_round_trip_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    a = np.concatenate([rng.normal(0, 1, 10000), rng.normal(0, 1e-30, 100),
                        [0.0, -0.0, 1.0, 3.0, 1e38]]).astype(np.float32)
    ref = torch.from_numpy(a).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(co.bf16_bits(a), ref)
    back = torch.from_numpy(ref.view(np.int16)).view(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(co.bf16_value(ref), back)


@pytest.mark.parametrize("taps", [1, 9])
def test_forward_equals_literal_loops(taps):
    rng = np.random.default_rng(taps)
    B, H, W, cin, cout = 2, 5, 6, 3, 4
    x = rng.normal(size=(B, H, W, cin))
    w = rng.normal(size=(cout, taps, cin))
    bias = rng.normal(size=cout)
    y = co.conv_forward(x, w, bias)
    ref = np.zeros_like(y)
    offs = [(0, 0)] if taps == 1 else [(dy - 1, dx - 1) for dy in range(3) for dx in range(3)]
    for b in range(B):
        for yy in range(H):
            for xx in range(W):
                for o in range(cout):
                    acc = bias[o]
                    for t, (dy, dx) in enumerate(offs):
                        sy, sx = yy + dy, xx + dx
                        if 0 <= sy < H and 0 <= sx < W:
                            acc += float(np.dot(x[b, sy, sx], w[o, t]))
                    ref[b, yy, xx, o] = acc
    assert np.allclose(y, ref, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("taps", [1, 9])
def test_gradients_are_adjoint(taps):
    rng = np.random.default_rng(10 + taps)
    B, H, W, cin, cout = 2, 7, 9, 5, 6
    x = rng.normal(size=(B, H, W, cin))
    w = rng.normal(size=(cout, taps, cin))
    g = rng.normal(size=(B, H, W, cout))
    lhs = np.sum(co.conv_forward(x, w) * g)
    assert np.isclose(lhs, np.sum(x * co.conv_data_grad(g, w)), rtol=1e-12)
    assert np.isclose(lhs, np.sum(w * co.conv_weight_grad(x, g, taps)), rtol=1e-12)


def test_adam_first_step_moves_by_lr_times_sign():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -4.0, 1e-3])
    p1, m, v = co.adam_step(p, g, np.zeros(3), np.zeros(3), 1, lr=1e-2)
    assert np.allclose(p1, p - 1e-2 * np.sign(g), rtol=0, atol=1e-7)
