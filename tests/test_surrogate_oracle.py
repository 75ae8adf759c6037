"""CPU checks of the surrogate network oracle (oracle/surrogate_oracle.py):
its analytic gradient against central finite differences of its own FP64
loss (BF16 rounding off), and its parameter layout against the library's
parameter count formula. No GPU."""
import numpy as np
import pytest

from oracle import surrogate_oracle as so


def _case(c=2, W=16, H=16, n=2, seed=0):
    rng = np.random.default_rng(seed)
    net = so.Net(c, W, H, bf16=False)
    p = so.init_params(c, seed)
    xs, ys, wts = [], [], []
    for k in range(n):
        h = rng.uniform(0, 30, (H, W))
        h[so.ring_mask(W, H)] = 0
        meta = so.make_meta(10 ** rng.uniform(-6, -5), rng.uniform(0.3, 0.6),
                            10 ** rng.uniform(-4, -2.3), h.max(), h.max() + 5)
        xs.append(so.input_planes(h, meta, W, H, counts=rng.integers(1, 50, (H, W))))
        ys.append(rng.normal(0.8, 0.2, (H, W)) * ~so.ring_mask(W, H))
        wts.append(float(meta["weight"]))
    return net, p, np.stack(xs), np.stack(ys), np.array(wts)


def test_gradient_matches_finite_differences():
    net, p, x, y, w = _case()
    loss, g, _ = net.loss_grad(p, x, y, w)
    assert loss > 0
    rng = np.random.default_rng(5)
    for trial in range(4):
        v = rng.normal(size=p.size)
        eps = 1e-6
        lp, _, _ = net.loss_grad(p + eps * v, x, y, w)
        lm, _, _ = net.loss_grad(p - eps * v, x, y, w)
        fd = (lp - lm) / (2 * eps)
        assert fd == pytest.approx(float(g @ v), rel=1e-5, abs=1e-12)


def test_each_layer_gradient_matches_finite_differences():
    net, p, x, y, w = _case(seed=3)
    _, g, _ = net.loss_grad(p, x, y, w)
    rng = np.random.default_rng(9)
    for (wo, bo, cin, cout) in net.layout:
        for lo, hi in ((wo, bo), (bo, bo + cout)):
            v = np.zeros(p.size)
            v[lo:hi] = rng.normal(size=hi - lo)
            eps = 1e-8   # small enough that no ReLU input changes sign
            fd = (net.loss_grad(p + eps * v, x, y, w)[0] - net.loss_grad(p - eps * v, x, y, w)[0]) / (2 * eps)
            assert fd == pytest.approx(float(g @ v), rel=1e-4, abs=1e-11)


def test_parameter_count_of_the_full_network():
    # base channels 32: ~1.95M parameters (9 * sum cin*cout + biases + head)
    _, _, count = so.param_layout(32)
    assert 1_900_000 < count < 2_000_000
