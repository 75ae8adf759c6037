"""Ragged batches (fs_batch_*): every realization of a batch must evolve
exactly like a model of its own -- bit for bit, receivers, level ids,
accumulation and elevation -- whatever its neighbours in the batch, with
direct launches or a replayed CUDA graph, and after the autotuner ran."""
import numpy as np
import pytest

from oracle.pyoracle import Params

pytestmark = pytest.mark.gpu


def ensemble(n, seed, smin=5, smax=160, neq=1.0):
    """Sides log-uniform, K log-U[1e-6,1e-5], m U[0.3,0.6], U log-U[1e-4,5e-3]
    (the ensemble workload's distributions at small sizes)."""
    import importlib
    pkg = importlib.import_module("barnes2019-landscape_gb300")
    rng = np.random.default_rng(seed)
    ws, hs, ps = [], [], []
    for _ in range(n):
        ws.append(int(np.exp(rng.uniform(np.log(smin), np.log(smax)))))
        hs.append(int(np.exp(rng.uniform(np.log(smin), np.log(smax)))))
        p = pkg.workload_params(keq=float(10 ** rng.uniform(-6, -5)),
                                meq=float(rng.uniform(0.3, 0.6)),
                                ueq=float(10 ** rng.uniform(-4, np.log10(5e-3))), neq=neq)
        ps.append(p)
    return ws, hs, ps


def compare_with_singles(pkg, b, ws, hs, ps, singles, tag):
    for r in range(len(ws)):
        m = singles[r]
        assert np.array_equal(b.receivers(r), m.receivers()), f"{tag} rec r={r}"
        lb, nb = b.levels(r)
        lm, nm = m.levels()
        assert nb == nm and np.array_equal(lb, lm), f"{tag} levels r={r}"
        assert np.array_equal(b.accumulation(r), m.accumulation()), f"{tag} acc r={r}"
        assert np.array_equal(b.getH(r), m.getH()), f"{tag} h r={r}"


@pytest.mark.parametrize("graph,int_sub,cta", [(False, False, False), (True, False, False),
                                               (True, True, False), (False, False, True),
                                               (True, True, True)])
def test_batch_equals_independent_models(pkg, graph, int_sub, cta):
    ws, hs, ps = ensemble(9, 11)
    seeds = list(range(100, 109))
    with pkg.FastScapeBatch(ws, hs, ps, init=pkg.INIT_PHILOX, seeds=seeds) as b:
        b.use_graph(graph)
        b.use_int_sub(int_sub)
        b.use_cta_walk(cta)
        assert b.launch_config()["cta_walk"] == cta
        assert b.launch_config()["erode_int_sub"] == int_sub
        singles = [pkg.FastScape_RBP(w, h, params=p, init=pkg.INIT_PHILOX, seed=s)
                   for w, h, p, s in zip(ws, hs, ps, seeds)]
        for r in range(len(ws)):
            assert np.array_equal(b.getH(r), singles[r].getH())
        for k in (1, 4, 7):
            b.step(k)
            for m in singles:
                m.step(k)
            compare_with_singles(pkg, b, ws, hs, ps, singles, f"k={k}")
        for m in singles:
            m.close()


@pytest.mark.parametrize("int_sub", [False, True])
def test_batch_against_oracle(pkg, oracle, int_sub):
    ws, hs, ps = ensemble(5, 3, smin=6, smax=90)
    with pkg.FastScapeBatch(ws, hs, ps, init=pkg.INIT_PHILOX, seeds=[1, 2, 3, 4, 5]) as b:
        b.use_int_sub(int_sub)
        hs0 = [b.getH(r) for r in range(len(ws))]
        b.step(6)
        for r in range(len(ws)):
            h = hs0[r].copy()
            oracle.steps(h, ws[r], hs[r], Params(*ps[r].as_tuple()), 6)
            assert np.array_equal(b.getH(r), h), f"r={r}"


def test_batch_reference_constants(pkg):
    """n = 2 everywhere (the reference's exponent) also batches exactly."""
    ws, hs, ps = ensemble(4, 5, neq=2.0)
    with pkg.FastScapeBatch(ws, hs, ps, init=pkg.INIT_PHILOX, seeds=[7, 8, 9, 10]) as b:
        singles = [pkg.FastScape_RBP(w, h, params=p, init=pkg.INIT_PHILOX, seed=s)
                   for w, h, p, s in zip(ws, hs, ps, [7, 8, 9, 10])]
        b.step(5)
        for m in singles:
            m.step(5)
        compare_with_singles(pkg, b, ws, hs, ps, singles, "n=2")


def test_autotune_keeps_state(pkg):
    ws, hs, ps = ensemble(6, 21, smin=40, smax=300)
    with pkg.FastScapeBatch(ws, hs, ps, init=pkg.INIT_PHILOX, seeds=list(range(6))) as a, \
            pkg.FastScapeBatch(ws, hs, ps, init=pkg.INIT_PHILOX, seeds=list(range(6))) as b:
        a.step(2)
        b.step(2)
        before = [a.getH(r) for r in range(6)]
        choice = a.autotune(probe_steps=2)
        assert choice["erode_blocks_per_sm"] in (1, 2)
        assert choice["erode_int_sub"] in (False, True)
        assert choice["order_blocks_per_sm"] in (2, 3)
        for r in range(6):
            assert np.array_equal(a.getH(r), before[r])
        a.step(5)
        b.step(5)
        for r in range(6):
            assert np.array_equal(a.getH(r), b.getH(r))


def test_single_model_autotune_keeps_state(pkg):
    p = pkg.workload_params()
    with pkg.FastScape_RBP(300, 200, params=p, init=pkg.INIT_PHILOX, seed=4) as a, \
            pkg.FastScape_RBP(300, 200, params=p, init=pkg.INIT_PHILOX, seed=4) as b:
        a.step(3)
        b.step(3)
        h = a.getH()
        cfg = a.autotune(probe_steps=2)
        assert cfg["order_blocks_per_sm"] in (2, 3) and cfg["erode_blocks_per_sm"] in (1, 2)
        assert np.array_equal(a.getH(), h)
        a.step(4)
        b.step(4)
        assert np.array_equal(a.getH(), b.getH())


def test_batch_run_semantics_and_errors(pkg):
    ws, hs, ps = ensemble(3, 8)
    with pkg.FastScapeBatch(ws, hs, ps, seeds=[1, 2, 3]) as b:
        b.run(3)
        assert b.cells() == sum(w * h for w, h in zip(ws, hs))
        with pytest.raises(pkg.FastScapeError):
            b.getH(3)
    p1 = pkg.workload_params()
    p2 = pkg.workload_params(neq=2.0)
    with pytest.raises(pkg.FastScapeError):
        pkg.FastScapeBatch([10, 10], [10, 10], [p1, p2])


def test_large_and_small_mixed(pkg):
    """A 1000x900 realization beside tiny ones; the tiny ones finish their
    levels early and must not disturb the big one."""
    ws = [1000, 5, 7, 64]
    hs = [900, 5, 40, 3]
    ps = [pkg.workload_params()] * 4
    with pkg.FastScapeBatch(ws, hs, ps, init=pkg.INIT_PHILOX, seeds=[4, 5, 6, 7]) as b:
        singles = [pkg.FastScape_RBP(w, h, params=p, init=pkg.INIT_PHILOX, seed=s)
                   for w, h, p, s in zip(ws, hs, ps, [4, 5, 6, 7])]
        b.step(3)
        for m in singles:
            m.step(3)
        compare_with_singles(pkg, b, ws, hs, ps, singles, "mixed")


@pytest.mark.parametrize("cta", [False, True])
def test_batch_table_growth_in_one_realization(pkg, cta):
    """A realization whose drainage counts outgrow its erosion table (a
    valley draining ~W*H cells to one outlet) stops the whole batch's
    timestep before any elevation changes; the host grows that table and
    redoes it. Every realization must still match its single model."""
    W, H = 420, 400
    yy, xx = np.divmod(np.arange(W * H), W)
    hv = 1.0 + 0.5 * np.abs(xx - W // 2) + 0.05 * yy
    hv[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    ws0, hs0, ps0 = ensemble(4, 11, smin=20, smax=200)
    ws, hs = [ws0[0], W, ws0[1], ws0[2]], [hs0[0], H, hs0[1], hs0[2]]
    p = pkg.workload_params()
    ps = [ps0[0], p, ps0[1], ps0[2]]
    with pkg.FastScapeBatch(ws, hs, ps, init=pkg.INIT_PHILOX, seeds=[3, 0, 4, 5]) as b:
        b.use_cta_walk(cta)
        b.setH(1, hv)
        singles = []
        for r in range(4):
            m = pkg.FastScape_RBP(ws[r], hs[r], params=ps[r], init=pkg.INIT_PHILOX,
                                  seed=[3, 0, 4, 5][r])
            if r == 1:
                m.setH(hv)
            singles.append(m)
        b.step(3)
        for m in singles:
            m.step(3)
        compare_with_singles(pkg, b, ws, hs, ps, singles, "valley")
        assert b.accumulation(1).max() / p.cell_area > 65536
        for m in singles:
            m.close()


def test_ragged_ensemble_at_its_own_scale(pkg, oracle):
    """The 256-realization ragged ensemble's own draws (bench.ensemble_spec:
    sides log-uniform in [256, 2048], K, m, U as drawn there), 200 timesteps:
    the largest, the smallest and two more realizations of that draw, run as
    one batch with the launch shape the autotuner picks, each bit-identical to
    a model of its own (receivers, level ids, accumulation, elevation) after
    the deep level structures of 200 timesteps, and the smallest bit-identical
    to the oracle's restatement of the reference as well."""
    import bench
    sides, params = bench.ensemble_spec(pkg, 256, seed=2019)
    order = np.argsort(sides)
    pick = [int(order[-1]), int(order[0]), int(order[len(order) // 3]),
            int(order[2 * len(order) // 3])]
    ws = [sides[i] for i in pick]
    ps = [params[i] for i in pick]
    seeds = [1000 + i for i in pick]
    assert max(ws) > 1800 and min(ws) < 300
    nsteps = 200
    with pkg.FastScapeBatch(ws, ws, ps, init=pkg.INIT_PHILOX, seeds=seeds) as b:
        h_small = b.getH(1)
        b.autotune(probe_steps=2)
        b.step(nsteps)
        singles = [pkg.FastScape_RBP(w, w, params=p, init=pkg.INIT_PHILOX, seed=s)
                   for w, p, s in zip(ws, ps, seeds)]
        for m in singles:
            m.step(nsteps)
        compare_with_singles(pkg, b, ws, ws, ps, singles, f"{nsteps} timesteps")
        assert max(b.levels(r)[1] for r in range(len(ws))) > 20
        p = ps[1]
        ref = oracle.steps(h_small.copy(), ws[1], ws[1], Params(*p.as_tuple()), nsteps)
        assert np.array_equal(b.getH(1), ref)
        for m in singles:
            m.close()


@pytest.mark.parametrize("nmode", [1, 2])
def test_cta_walk_equals_grid_walk_on_deep_levels(pkg, nmode):
    """Long runs under strong uplift grow hundreds of levels (the regime the
    per-realization walk is for): both walks give the same receivers, level
    ids, accumulation and elevation bit for bit after 600 timesteps, with
    and without the integer subtractions, also for a subset of the batch."""
    n = 6
    ws = [96, 128, 64, 128, 80, 112]
    kw = dict(keq=1e-5, meq=0.6, ueq=5e-3, neq=float(nmode))
    ps = [pkg.workload_params(**kw) for _ in range(n)]
    seeds = list(range(30, 30 + n))
    with pkg.FastScapeBatch(ws, ws, ps, init=pkg.INIT_PHILOX, seeds=seeds) as g, \
            pkg.FastScapeBatch(ws, ws, ps, init=pkg.INIT_PHILOX, seeds=seeds) as c:
        c.use_cta_walk(True)
        c.use_int_sub(True)
        g.step(600)
        c.step(600)
        assert max(g.levels(r)[1] for r in range(n)) > 60
        for r in range(n):
            assert np.array_equal(c.receivers(r), g.receivers(r)), r
            lc, nc = c.levels(r)
            lg, ng = g.levels(r)
            assert nc == ng and np.array_equal(lc, lg), r
            assert np.array_equal(c.accumulation(r), g.accumulation(r)), r
            assert np.array_equal(c.getH(r), g.getH(r)), r
        c.set_active([4, 1, 2])
        g.set_active([4, 1, 2])
        c.step(5)
        g.step(5)
        for r in range(n):
            assert np.array_equal(c.getH(r), g.getH(r)), r
