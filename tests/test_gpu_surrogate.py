"""The learned surrogate on the GPU, through the C ABI
(include/fastscape_surrogate.h):

* gradients of one training step against the FP64 network oracle
  (oracle/surrogate_oracle.py, BF16 rounding emulated at the same points):
  per layer, the relative L2 error of the weight and bias gradients is below
  3e-2 -- the network runs in BF16 with FP32 accumulation, and a BF16
  rounding that comes out one unit apart in an early layer moves everything
  after it by about 2^-8;
* the jump (prediction) against the oracle's forward pass;
* training on data the plain method generates on the device lowers the
  held-out loss, and the trained network predicts held-out jumps better than
  the uplift-only jump h + u (the method's answer without erosion);
* the judge's measures against numpy; subset timesteps bit-identical to full
  ones; an ensemble whose every jump fails the judge is bit-identical to the
  plain batched run."""
import numpy as np
import pytest

from oracle import surrogate_oracle as so

pytestmark = pytest.mark.gpu


def _fields(rng, n, W, H, params, jump=50, dt=1000.0):
    """Synthetic (h_t, h_next) pairs with rings at 0."""
    ring = so.ring_mask(W, H)
    ht, hn = [], []
    for p in params:
        u = jump * p.ueq * dt
        h = np.cumsum(rng.uniform(0, 3, (H, W)), axis=0) + rng.uniform(0, 1, (H, W))
        h[ring] = 0
        nxt = h + u * (1 - 0.5 * rng.uniform(0, 1, (H, W))) - 0.01 * h
        nxt[ring] = 0
        ht.append(h.reshape(-1))
        hn.append(nxt.reshape(-1))
    return np.stack(ht), np.stack(hn)


def _params(pkg, rng, n):
    return [pkg.workload_params(keq=float(10 ** rng.uniform(-6, -5)),
                                meq=float(rng.uniform(0.3, 0.6)),
                                ueq=float(10 ** rng.uniform(-4, np.log10(5e-3))))
            for _ in range(n)]


def _counts(h, W, H, p):
    """Drainage counts of the field h (receivers and accumulation of the
    oracle's timestep, before its erosion)."""
    from oracle.pyoracle import Oracle, Params as OParams
    ph = Oracle().phases(np.array(h, np.float64), W, H, OParams(*p.as_tuple()))
    return np.rint(ph["accum"] / p.cell_area)


def _oracle_inputs(ht, hn, params, W, H):
    xs, ys, ws = [], [], []
    ring = so.ring_mask(W, H)
    for h, nx, p in zip(ht, hn, params):
        h32 = h.astype(np.float32).astype(np.float64)
        meta = so.make_meta(p.keq, p.meq, p.ueq, h.max(), nx.max())
        xs.append(so.input_planes(h32, meta, W, H, counts=_counts(h, W, H, p)))
        u = float(meta["u"])
        y = ((nx - h) / u).astype(np.float32).astype(np.float64).reshape(H, W)
        y[ring] = 0
        ys.append(y)
        ws.append(float(meta["weight"]))
    return np.stack(xs), np.stack(ys), np.array(ws)


def test_gradients_match_oracle(pkg):
    W = H = 128
    c = 16
    rng = np.random.default_rng(11)
    params = _params(pkg, rng, 2)
    ht, hn = _fields(rng, 2, W, H, params)
    with pkg.Surrogate(W, H, base_channels=c, batch=2, seed=3) as s:
        p0 = so.init_params(c, seed=4).astype(np.float32)
        s.set_params(p0)
        s.reserve(2)
        s.add_samples(ht, hn, params)
        loss = s.grad([0, 1])
        g = s.grads().astype(np.float64)
    net = so.Net(c, W, H, bf16=True)
    x, y, w = _oracle_inputs(ht, hn, params, W, H)
    ref_loss, ref, _ = net.loss_grad(p0.astype(np.float64), x, y, w)
    assert loss == pytest.approx(ref_loss, rel=1e-2)
    worst = []
    for l, (wo, bo, cin, cout) in enumerate(net.layout):
        for name, lo, hi in (("w", wo, bo), ("b", bo, bo + cout)):
            err = np.linalg.norm(g[lo:hi] - ref[lo:hi]) / (np.linalg.norm(ref[lo:hi]) + 1e-30)
            worst.append((err, l, name))
    hd = net.head
    err = np.linalg.norm(g[hd:] - ref[hd:]) / np.linalg.norm(ref[hd:])
    worst.append((err, 14, "head"))
    worst.sort(reverse=True)
    assert worst[0][0] < 3e-2, worst[:4]


def test_prediction_matches_oracle_forward(pkg):
    W = H = 128
    c = 16
    rng = np.random.default_rng(5)
    params = _params(pkg, rng, 3)
    ht, _ = _fields(rng, 3, W, H, params)
    with pkg.Surrogate(W, H, base_channels=c, batch=2, seed=3) as s:
        p0 = so.init_params(c, seed=8).astype(np.float32)
        s.set_params(p0)
        out = s.predict(ht, params)        # two passes: a full one and one of 1
    net = so.Net(c, W, H, bf16=True)
    ring = so.ring_mask(W, H).reshape(-1)
    for k, p in enumerate(params):
        meta = so.make_meta(p.keq, p.meq, p.ueq, ht[k].max(), ht[k].max())
        x = so.input_planes(ht[k], meta, W, H, counts=_counts(ht[k], W, H, p))[None]
        z = net.forward(p0.astype(np.float64), x)["z"][0].reshape(-1)
        ref = ht[k] + float(meta["u"]) * z
        ref[ring] = ht[k][ring]
        assert np.array_equal(out[k][ring], ht[k][ring])
        scale = float(meta["u"]) * (np.abs(z).max() + 1)
        assert np.max(np.abs(out[k] - ref)) < 2e-2 * scale


def test_training_lowers_heldout_loss_and_beats_uplift_only(pkg):
    W = H = 128
    with pkg.Surrogate(W, H, base_channels=16, batch=8, seed=7) as s:
        s.reserve(96)
        got = s.generate(ntraj=24, per_traj=4, max_spinup=400, seed=21)
        assert got == 96
        s.set_holdout(16)
        before = s.eval()
        train_loss = s.train(200, lr=1e-3)
        after = s.eval()
        assert np.isfinite(train_loss)
        assert after < 0.7 * before, (before, after)
        # what the network gains over the jumps that need none: uplift only
        # (h + u on the interior) and no change
        uplift_only, no_change = s.eval_baselines()
        assert after < uplift_only and after < no_change, (after, uplift_only, no_change)
        ms, flops = s.train_stats()
        assert ms > 0 and flops > 0


def test_judge_measures_match_numpy(pkg):
    W, H = 40, 30
    rng = np.random.default_rng(2)
    p = pkg.workload_params()
    a = rng.uniform(0, 10, (3, H * W))
    b = a + rng.normal(0, 0.3, a.shape)
    b[1] = a[1]
    rel, ag = pkg.compare_fields(W, H, [p] * 3, a, b)
    ring = so.ring_mask(W, H).reshape(-1)
    offs = [-1, -W - 1, -W, -W + 1, 1, W + 1, W, W - 1]
    dr = [p.dr_orth, p.dr_diag] * 4

    def receivers(h):
        out = np.full(H * W, -2)
        for cidx in np.flatnonzero(~ring):
            best, r = 0.0, -1
            for k in range(8):
                sl = (h[cidx] - h[cidx + offs[k]]) / dr[k]
                if sl > best:
                    best, r = sl, k
            out[cidx] = r
        return out

    for k in range(3):
        d = (a[k] - b[k])[~ring]
        ref_rel = np.sqrt(np.mean(d * d)) / (b[k].max() - b[k].min())
        assert rel[k] == pytest.approx(ref_rel, rel=1e-12)
        ra, rb = receivers(a[k]), receivers(b[k])
        assert ag[k] == pytest.approx(np.mean(ra[~ring] == rb[~ring]), rel=1e-12)
    assert rel[1] == 0 and ag[1] == 1


def test_subset_timesteps_are_bit_identical(pkg):
    sides = [64, 96, 80, 128, 72]
    rng = np.random.default_rng(1)
    params = _params(pkg, rng, len(sides))
    seeds = list(range(40, 45))
    b = pkg.FastScapeBatch(sides, sides, params, init=pkg.INIT_PHILOX, seeds=seeds)
    full = pkg.FastScapeBatch(sides, sides, params, init=pkg.INIT_PHILOX, seeds=seeds)
    h0 = [b.getH(r) for r in range(len(sides))]
    b.set_active([3, 1])
    b.step(4)
    full.step(4)
    for r in range(len(sides)):
        if r in (1, 3):
            assert np.array_equal(b.getH(r), full.getH(r))
            assert np.array_equal(b.receivers(r), full.receivers(r))
            assert b.levels(r)[1] == full.levels(r)[1]
        else:
            assert np.array_equal(b.getH(r), h0[r])
    b.set_active([0])                      # a subset of one
    b.step(4)
    assert np.array_equal(b.getH(0), full.getH(0))
    b.set_active(None)
    b.step(3)
    full.step(3)
    for r in (0, 1, 3):
        assert np.array_equal(b.getH(r), full.getH(r))
    b.close()
    full.close()


def test_ensemble_that_falls_back_everywhere_equals_plain_run(pkg):
    W = H = 128
    n = 4
    rng = np.random.default_rng(3)
    params = _params(pkg, rng, n)
    seeds = list(range(7, 7 + n))
    nsteps = 2 * 51 + 3
    with pkg.Surrogate(W, H, base_channels=16, batch=4, seed=1) as s:
        b = pkg.FastScapeBatch([W] * n, [H] * n, params, init=pkg.INIT_PHILOX, seeds=seeds)
        stats, fallen = s.ensemble(b, nsteps, judge_fraction=1.0, max_rel_rms=0.0)
        ref = pkg.FastScapeBatch([W] * n, [H] * n, params, init=pkg.INIT_PHILOX, seeds=seeds)
        ref.step(nsteps)
        for r in range(n):
            assert np.array_equal(b.getH(r), ref.getH(r))
        assert fallen.tolist() == [1] * n
        assert stats["cycles"] == 2 and stats["judged"] == n and stats["fallbacks"] == n
        b.close()
        ref.close()


def test_ensemble_without_judge_jumps_every_cycle(pkg):
    W = H = 128
    n = 3
    rng = np.random.default_rng(4)
    params = _params(pkg, rng, n)
    with pkg.Surrogate(W, H, base_channels=16, batch=2, seed=1) as s:
        b = pkg.FastScapeBatch([W] * n, [H] * n, params, init=pkg.INIT_PHILOX, seeds=[1, 2, 3])
        stats, fallen = s.ensemble(b, 3 * 51, judge_fraction=0.0)
        assert stats["cycles"] == 3 and stats["jumps"] == 3 * n and stats["judged"] == 0
        assert fallen.tolist() == [0] * n
        for r in range(n):
            assert np.all(np.isfinite(b.getH(r)))
        b.close()
