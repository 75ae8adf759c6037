"""The surrogate's tensor-core convolutions (tcgen05 + TMA + TMEM) against
the FP64 CPU oracle, called through the C ABI (fs_test_sg_conv).

Inputs are BF16; the kernels accumulate in FP32. Tolerances: forward and
data-gradient outputs are rounded to BF16 (relative 2^-8 of the value) on
top of FP32 accumulation (at most ~1e-6 of the sum of |terms|); the weight
gradient stays FP32, compared at 2e-5 of the sum of |terms| per entry.
Shapes cover every channel-block width (16, 32, 64), N tiles above 256, the
narrow-image pixel tile (W < 128), rows of 256 and 512 pixels (two planar
CTAs per SM where their weights leave room, else -- forward, at least 64
input channels -- the output channels on M and 256 pixels on N), 1x1 and
3x3 taps, zero padding at every border, bias, ReLU and the data gradient's
mask."""
import numpy as np
import pytest

from oracle import conv_oracle as co

pytestmark = pytest.mark.gpu


def _bits(rng, shape, scale=1.0):
    return co.bf16_bits(rng.normal(0, scale, shape))


def _close(got, ref, terms, rel_value, rel_terms):
    err = np.abs(got - ref)
    tol = rel_value * np.abs(ref) + rel_terms * terms + 1e-30
    bad = err > tol
    assert not bad.any(), (f"{bad.sum()} of {bad.size} entries off; worst "
                           f"{np.max(err / tol):.3g} x tolerance")


SHAPES = [
    # B, H, W, cin, cout, taps
    (1, 2, 128, 16, 32, 9),
    (2, 4, 128, 32, 32, 9),
    (1, 8, 64, 64, 64, 9),
    (2, 2, 256, 96, 32, 9),
    (1, 3, 512, 32, 32, 9),
    (1, 2, 256, 16, 48, 9),
    (1, 2, 256, 64, 128, 9),
    (1, 4, 128, 128, 256, 9),
    (1, 2, 128, 64, 384, 9),
    (2, 16, 32, 32, 16, 1),
    (1, 2, 128, 256, 128, 1),
]


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_forward(pkg, shape):
    B, H, W, cin, cout, taps = shape
    rng = np.random.default_rng(sum(shape))
    x = _bits(rng, (B, H, W, cin))
    w = _bits(rng, (cout, taps, cin), 1 / np.sqrt(taps * cin))
    bias = rng.normal(0, 0.1, cout).astype(np.float32)
    for relu in (False, True):
        got = co.bf16_value(pkg.sg_conv(0, x, w, taps, bias=bias, relu=relu))
        xv, wv = co.bf16_value(x), co.bf16_value(w)
        ref = co.conv_forward(xv, wv, bias.astype(np.float64), relu=relu)
        terms = co.conv_forward(np.abs(xv), np.abs(wv)) + np.abs(bias)
        _close(got, ref, terms, 2 ** -8, 2e-6)


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_forward_into_wider_and_upsampled_outputs(pkg, shape):
    # The network writes its skip tensors into the concatenations they join
    # (planes inside a wider tensor) and its decoder outputs upsampled 2x
    # into them: same values as the plain forward, bit for bit, and nothing
    # written outside the output's planes (the library checks the sentinels).
    B, H, W, cin, cout, taps = shape
    rng = np.random.default_rng(sum(shape) + 1)
    x = _bits(rng, (B, H, W, cin))
    w = _bits(rng, (cout, taps, cin), 1 / np.sqrt(taps * cin))
    bias = rng.normal(0, 0.1, cout).astype(np.float32)
    plain = pkg.sg_conv(0, x, w, taps, bias=bias, relu=True)
    assert np.array_equal(pkg.sg_conv(3, x, w, taps, bias=bias, relu=True), plain)
    up = pkg.sg_conv(4, x, w, taps, bias=bias, relu=True)
    assert np.array_equal(up, np.repeat(np.repeat(plain, 2, axis=1), 2, axis=2))


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_data_gradient(pkg, shape):
    B, H, W, cin, cout, taps = shape
    rng = np.random.default_rng(7 + sum(shape))
    dy = _bits(rng, (B, H, W, cout))
    w = _bits(rng, (cout, taps, cin), 1 / np.sqrt(taps * cout))
    mask = _bits(rng, (B, H, W, cin))   # about half the entries <= 0
    dyv, wv = co.bf16_value(dy), co.bf16_value(w)
    terms = co.conv_data_grad(np.abs(dyv), np.abs(wv))
    got = co.bf16_value(pkg.sg_conv(1, dy, w, taps))
    _close(got, co.conv_data_grad(dyv, wv), terms, 2 ** -8, 2e-6)
    got = co.bf16_value(pkg.sg_conv(1, dy, w, taps, mask_bits=mask))
    ref = co.conv_data_grad(dyv, wv, mask=co.bf16_value(mask))
    _close(got, ref, terms, 2 ** -8, 2e-6)


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_weight_gradient(pkg, shape):
    B, H, W, cin, cout, taps = shape
    if cout > 256:
        pytest.skip("weight gradient takes at most 256 output channels (one accumulator)")
    rng = np.random.default_rng(13 + sum(shape))
    x = _bits(rng, (B, H, W, cin))
    dy = _bits(rng, (B, H, W, cout))
    got = pkg.sg_conv(2, x, dy, taps).astype(np.float64)
    xv, dyv = co.bf16_value(x), co.bf16_value(dy)
    ref = co.conv_weight_grad(xv, dyv, taps)
    terms = co.conv_weight_grad(np.abs(xv), np.abs(dyv), taps)
    _close(got, ref, terms, 0.0, 2e-5)


def test_large_pixel_count_weight_gradient(pkg):
    """Many pixel steps split across CTAs (512^2 image, batch 2)."""
    rng = np.random.default_rng(99)
    x = _bits(rng, (2, 512, 512, 32))
    dy = _bits(rng, (2, 512, 512, 32), 0.1)
    got = pkg.sg_conv(2, x, dy, 9).astype(np.float64)
    xv, dyv = co.bf16_value(x), co.bf16_value(dy)
    ref = co.conv_weight_grad(xv, dyv, 9)
    terms = co.conv_weight_grad(np.abs(xv), np.abs(dyv), 9)
    _close(got, ref, terms, 0.0, 2e-5)
