"""GPU parity: the CUDA timestep through the C ABI against the golden fixtures
(produced by the reference's own code) and against the oracle.

Tolerances:
  * receivers, donor masks, level ids, accumulation: bit-exact, always;
  * elevation with n = 1 (the workload): bit-exact (0 ulp) -- the device
    follows the reference's operation order with no multiply-add
    contraction, every division is correctly rounded, and
    pow(k*cell_area, m) comes from a table evaluated with the C library's pow;
  * elevation with n != 1 (the reference's own constants use n = 2): within
    1e-12 relative per timestep, because pow(x, n) of the Newton update is
    evaluated on the device (x*x for n = 2) while the reference calls the C
    library's pow, which is not always correctly rounded. Each timestep is
    then checked from the reference's own input elevation.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle.pyoracle import Params, donor_mask_from_rec, level_ids

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
STEP_CASES = sorted(p.stem for p in GOLDEN.glob("*.npz")
                    if not p.stem.startswith(("run_", "terrain_")))
RUN_CASES = sorted(p.stem for p in GOLDEN.glob("run_*.npz"))


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def gpu_params(pkg, arr):
    return pkg.Params(*[float(x) for x in arr])


RTOL_GENERAL_N = 1e-12


def assert_step_equal(m, W, H, ref, tag="", exact_h=True):
    rec = m.receivers()
    assert np.array_equal(rec, ref["rec"].astype(np.int32)), f"receivers {tag}"
    assert np.array_equal(m.donor_mask(), donor_mask_from_rec(rec, W, H)), f"donor mask {tag}"
    lid, nl = m.levels()
    want_lid = level_ids(ref["stack"], ref["levels"], W * H)
    # the reference's level table has nlevel = levels + 2 entries
    # (fastscape_RB.cpp:246-251 leaves an empty last level plus a duplicate)
    assert nl == len(ref["levels"]) - 2, f"nlevels {tag}"
    assert np.array_equal(lid, want_lid), f"level ids {tag}"
    assert np.array_equal(m.accumulation(), ref["accum"]), f"accumulation {tag}"
    got = m.getH()
    if exact_h:
        assert np.array_equal(got, ref["h"]), f"elevation {tag}"
    else:
        np.testing.assert_allclose(got, ref["h"], rtol=RTOL_GENERAL_N, atol=0,
                                   err_msg=f"elevation {tag}")


@pytest.mark.parametrize("name", STEP_CASES)
def test_golden_per_timestep(pkg, name):
    g = load(name)
    W, H, ns = int(g["W"]), int(g["H"]), int(g["nsteps"])
    exact = float(g["params"][1]) == 1.0
    with pkg.FastScape_RBP(W, H, params=gpu_params(pkg, g["params"]), init=pkg.INIT_ZERO) as m:
        m.setH(g["h0"])
        for s in range(ns):
            if not exact:
                m.setH(g["h0"] if s == 0 else g[f"h_{s - 1}"])
            m.step(1)
            ref = {"rec": g[f"rec_{s}"], "stack": g[f"stack_{s}"], "levels": g[f"levels_{s}"],
                   "accum": g[f"accum_{s}"], "h": g[f"h_{s}"]}
            assert_step_equal(m, W, H, ref, f"{name} step {s}", exact_h=exact)


@pytest.mark.parametrize("name", RUN_CASES)
def test_golden_run(pkg, name):
    g = load(name)
    W = int(g["W"])
    exact = float(g["params"][1]) == 1.0
    with pkg.FastScape_RBP(W, W, params=gpu_params(pkg, g["params"]),
                           init=pkg.INIT_REFERENCE) as m:
        assert np.array_equal(m.getH(), g["h0"])
        m.run(int(g["nstep"]))
        assert m.steps_executed() == int(g["nstep"]) + 1
        if exact:
            assert np.array_equal(m.getH(), g["h_final"])
        else:
            # 121 timesteps with the device's x*x in place of pow(x, 2)
            np.testing.assert_allclose(m.getH(), g["h_final"], rtol=1e-10, atol=0)


@pytest.mark.parametrize("W,H,steps,seed,n", [
    (5, 5, 4, 1, 1), (7, 5, 4, 2, 1), (64, 64, 10, 3, 1), (129, 67, 10, 4, 2),
    (333, 250, 6, 5, 1), (512, 512, 12, 6, 2),
])
def test_oracle_trajectory(pkg, oracle, W, H, steps, seed, n):
    rng = np.random.default_rng(seed)
    p = pkg.workload_params() if n == 1 else pkg.reference_params()
    op = Params(*p.as_tuple())
    h = rng.uniform(0, 3, W * H)
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
        m.setH(h)
        for s in range(steps):
            if n != 1:
                m.setH(h)
            m.step(1)
            ref = oracle.phases(h, W, H, op)
            assert_step_equal(m, W, H, ref, f"step {s}", exact_h=(n == 1))


@pytest.mark.parametrize("W,H,steps,seed", [(64, 64, 10, 3), (333, 250, 6, 5)])
def test_oracle_trajectory_integer_subtractions(pkg, oracle, W, H, steps, seed):
    """The erosion with its elevation subtractions in integer arithmetic,
    bit-identical to the oracle. The terrain mixes the cases each integer
    path declines (negative and zero elevations, receivers below half the
    cell's elevation, erosion close to the elevation itself) with ordinary
    cells, so both the integer paths and their FP64 fallbacks run."""
    rng = np.random.default_rng(seed)
    p = pkg.workload_params()
    op = Params(*p.as_tuple())
    h = rng.uniform(0, 3, W * H)
    kind = rng.integers(0, 6, W * H)
    h[kind == 1] *= 1e-3                          # near zero: large relative drops
    h[kind == 2] = -rng.uniform(0, 5, (kind == 2).sum())   # negative elevations
    h[kind == 3] = 0.0
    h[kind == 4] = rng.uniform(100, 3000, (kind == 4).sum())  # steep cliffs
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
        m.use_int_sub(True)
        assert m.launch_config()["erode_int_sub"]
        m.setH(h)
        for s in range(steps):
            m.step(1)
            ref = oracle.phases(h, W, H, op)
            assert_step_equal(m, W, H, ref, f"step {s}")


@pytest.mark.parametrize("int_sub", [False, True])
def test_second_newton_iterate(pkg, oracle, int_sub):
    """Strong erosion (K 5e-5, U 5e-3, 500 m of relief): most cells erode by
    more than tol per timestep and take the unrolled second Newton iterate
    (its zero-residual shortcut included); bit-identical to the oracle at
    every timestep, with FP64 or integer subtractions."""
    W, H, steps = 200, 150, 8
    rng = np.random.default_rng(17)
    p = pkg.workload_params(keq=5e-5, ueq=5e-3, meq=0.5)
    op = Params(*p.as_tuple())
    h = rng.uniform(0, 500, W * H)
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
        m.use_int_sub(int_sub)
        m.setH(h)
        for s in range(steps):
            m.step(1)
            ref = oracle.phases(h, W, H, op)
            assert_step_equal(m, W, H, ref, f"step {s}")


@pytest.mark.parametrize("n,int_sub", [(1, False), (1, True), (2, False), (2, True)])
def test_erosion_equals_literal_newton_loop(pkg, n, int_sub):
    """The unrolled bit-pattern erosion -- n = 1: the first and second
    iterates; n = 2: every iterate -- with FP64 or integer subtractions gives
    bit for bit the elevations of the reference's Newton loop evaluated
    literally (FP64 division every iterate, pow(x,1) = x, pow(x,2) = x*x),
    on terrain whose cells take several iterates. (n = 2 cannot be compared
    bit for bit with the oracle, whose glibc pow(x, 2) is not always x*x.)"""
    L = pkg.library()
    W, H = 300, 200
    rng = np.random.default_rng(31 + n)
    p = pkg.workload_params(keq=5e-5, ueq=5e-3, meq=0.5) if n == 1 else pkg.reference_params()
    h = rng.uniform(0, 300, W * H)
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as a, \
            pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as b:
        a.use_int_sub(int_sub)
        assert a.launch_config()["erode_int_sub"] == int_sub
        pkg.check(L.fs_test_set_erosion_path(b.handle, 1))
        a.setH(h)
        b.setH(h)
        for s in range(6):
            a.step(1)
            b.step(1)
            assert np.array_equal(a.receivers(), b.receivers()), f"step {s}"
            assert np.array_equal(a.getH(), b.getH()), f"step {s}"


def test_workload_1000_integer_subtractions(pkg, oracle):
    """run(120) of the 1000x1000 workload with the integer subtractions:
    bit-identical to the oracle, like the default erosion."""
    W = 1000
    p = pkg.workload_params()
    with pkg.FastScape_RBP(W, W, params=p, init=pkg.INIT_REFERENCE) as m:
        m.use_int_sub(True)
        m.run(120)
        got = m.getH()
    h = oracle.terrain(W, W, 0)
    oracle.run(h, W, W, Params(*p.as_tuple()), 120, parallel=True)
    assert np.array_equal(got, h)


def test_integer_subtractions_ignored_for_general_n(pkg):
    p = pkg.workload_params(neq=1.5)
    with pkg.FastScape_RBP(64, 64, params=p, init=pkg.INIT_PHILOX) as m:
        m.use_int_sub(True)
        assert not m.launch_config()["erode_int_sub"]


def test_reference_field_generator(pkg, oracle):
    for W, H in [(16, 16), (101, 37)]:
        with pkg.FastScape_RBP(W, H, init=pkg.INIT_REFERENCE, seed=123) as m:
            assert np.array_equal(m.getH(), oracle.terrain(W, H, 0))
        with pkg.FastScape_RBP(W, H, init=pkg.INIT_MT19937, seed=77) as m:
            assert np.array_equal(m.getH(), oracle.terrain(W, H, 77))


def test_philox_field(pkg):
    W, H = 300, 200
    with pkg.FastScape_RBP(W, H, init=pkg.INIT_PHILOX, seed=42) as a, \
            pkg.FastScape_RBP(W, H, init=pkg.INIT_PHILOX, seed=42) as b, \
            pkg.FastScape_RBP(W, H, init=pkg.INIT_PHILOX, seed=43) as c:
        ha, hb, hc = a.getH(), b.getH(), c.getH()
    assert np.array_equal(ha, hb) and not np.array_equal(ha, hc)
    g = ha.reshape(H, W)
    assert np.all(g[:2, :] == 0) and np.all(g[-2:, :] == 0)
    assert np.all(g[:, :2] == 0) and np.all(g[:, -2:] == 0)
    inner = g[2:-2, 2:-2]
    assert inner.min() >= 0 and inner.max() < 1 and abs(inner.mean() - 0.5) < 0.01


def test_workload_1000_full_run(pkg, oracle):
    """The 1000x1000 workload: run(120) = 121 timesteps, final elevation
    bit-identical to the oracle (fastscape_RB+P semantics)."""
    W = 1000
    p = pkg.workload_params()
    with pkg.FastScape_RBP(W, W, params=p, init=pkg.INIT_REFERENCE) as m:
        m.run(120)
        got = m.getH()
        lid, nl = m.levels()
        acc = m.accumulation()
    h = oracle.terrain(W, W, 0)
    oracle.run(h, W, W, Params(*p.as_tuple()), 120, parallel=True)
    assert np.array_equal(got, h)
    assert nl >= 2 and acc.min() == p.cell_area


@pytest.mark.slow
def test_workload_10000_full_run(pkg, oracle):
    """The 10000x10000 workload: run(20) = 21 timesteps, final elevation
    bit-identical to the oracle (OpenMP restatement of fastscape_RB+P, about
    a minute on the host cores), plus size-independent checks of the last
    timestep's receivers, level ids and accumulation."""
    W = H = 10000
    p = pkg.workload_params()
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_REFERENCE) as m:
        m.run(20)
        got = m.getH()
        rec = m.receivers()
        lid, nl = m.levels()
        acc = m.accumulation()
    # every cell drains to exactly one root: the roots' drainage areas add
    # up to the grid; a non-root cell sits one level above its receiver
    roots = rec == -1
    assert np.count_nonzero(lid[roots] == 0) == np.count_nonzero(roots)
    assert np.sum(acc[roots] / p.cell_area, dtype=np.float64) == W * H
    off = np.array([-1, -W - 1, -W, -W + 1, 1, W + 1, W, W - 1], dtype=np.int64)
    for y0 in range(0, H, 1000):
        sl = slice(y0 * W, (y0 + 1000) * W)
        r = rec[sl]
        c = np.nonzero(r >= 0)[0] + y0 * W
        assert np.array_equal(lid[c], lid[c + off[rec[c]]] + 1)
        assert np.all(acc[c] < acc[c + off[rec[c]]])
    assert nl == lid.max() + 1
    del rec, lid, acc
    h = oracle.terrain(W, H, 0)
    oracle.run(h, W, H, Params(*p.as_tuple()), 20, parallel=True)
    assert np.array_equal(got, h)


def test_run_then_run_equals_one_run(pkg):
    """State carried between run() calls is only h (fastscape_RB.cpp:334-340)."""
    W = 200
    p = pkg.workload_params()
    with pkg.FastScape_RBP(W, W, params=p) as a, pkg.FastScape_RBP(W, W, params=p) as b:
        a.run(4); a.run(9)          # 5 + 10 timesteps
        b.step(15)
        assert np.array_equal(a.getH(), b.getH())


def test_deterministic_repeat(pkg):
    W = 700
    p = pkg.workload_params()
    outs = []
    for _ in range(2):
        with pkg.FastScape_RBP(W, W, params=p, init=pkg.INIT_PHILOX, seed=9) as m:
            m.step(6)
            outs.append((m.getH(), m.receivers(), m.levels()[0], m.accumulation()))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_timing_counters(pkg):
    with pkg.FastScape_RBP(256, 256, params=pkg.workload_params()) as m:
        m.set_timing(True)
        m.step(3)
        t = m.phase_times(reset=True)
        assert np.all(t > 0)
        assert t[3] >= t[0] + t[1] + t[2] * 0.99
        assert t[2] == pytest.approx(t[7] + t[8] + t[9], rel=1e-9)  # the walk's kernels
        assert np.all(m.phase_times() == 0)


def test_receiver_filter_equals_fp64_formula(pkg):
    """The FP32 filter + FP64 fix-up path gives the receivers of the FP64
    reference formula on every cell, over an evolving landscape."""
    import ctypes as C
    W, H = 1500, 1100
    p = pkg.workload_params()
    L = pkg.library()
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_PHILOX, seed=5) as a, \
            pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_PHILOX, seed=5) as b:
        L.fs_test_set_receiver_path(b.handle, 1)
        for s in range(8):
            a.step(1)
            b.step(1)
            assert np.array_equal(a.receivers(), b.receivers()), f"step {s}"
            assert np.array_equal(a.getH(), b.getH()), f"step {s}"
        n = C.c_int32(0)
        pkg.check(L.fs_test_receiver_fixups(a.handle, C.byref(n)))
        assert 0 < n.value < W * H // 100


def serpentine(W, H):
    """A channel snaking along every other row between walls 1000 m high,
    descending 1 cm per cell to a single outlet next to the base-level
    ring: one drainage path of thousands of cells, so thousands of levels
    (2489 at 120x50)."""
    h = np.full((H, W), 1000.0)
    rows = list(range(3, H - 3, 2))
    p = 0
    for k, y in enumerate(rows):
        xs = range(3, W - 3) if k % 2 == 0 else range(W - 4, 2, -1)
        for x in xs:
            p += 1
            h[y, x] = p * 0.01
        if k + 1 < len(rows):
            p += 1
            h[y + 1, W - 4 if k % 2 == 0 else 3] = p * 0.01
    h[2, 3] = 0.005
    h = h.reshape(-1).copy()
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    return h


def test_thousands_of_levels(pkg, oracle):
    """More levels than the walk kernels keep in shared memory (2048): every
    level of a 2489-level drainage path, one-pass ordering chunks, the
    level-table fallback of accumulation and erosion -- bit-identical to the
    oracle at every timestep, alone and inside a batch."""
    W, H = 120, 50
    h = serpentine(W, H)
    p = pkg.workload_params()
    op = Params(*p.as_tuple())
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
        m.setH(h)
        ho = h.copy()
        for s in range(3):
            m.step(1)
            ref = oracle.phases(ho, W, H, op)
            assert len(ref["levels"]) - 2 > 2048
            assert_step_equal(m, W, H, ref, f"step {s}")
    ws, hs = [W, 40, 90], [H, 30, 70]
    with pkg.FastScapeBatch(ws, hs, [p] * 3, init=pkg.INIT_PHILOX, seeds=[1, 2, 3]) as b:
        b.setH(0, h)
        singles = []
        for r in range(3):
            mm = pkg.FastScape_RBP(ws[r], hs[r], params=p, init=pkg.INIT_ZERO)
            mm.setH(b.getH(r))
            singles.append(mm)
        b.step(2)
        for r, mm in enumerate(singles):
            mm.step(2)
            assert np.array_equal(b.getH(r), mm.getH()), f"batch r={r}"
            mm.close()


def test_receiver_fixup_on_flat_ground(pkg):
    """Flat-heavy terrain -- integer terraces (exact ties and zero slopes),
    +0 and -0, negative heights, neighbours one ulp apart -- sends most cells
    to the FP64 fix-up; its lower-neighbour shortcut must give the verbatim
    formula's receivers."""
    import ctypes as C
    W, H = 700, 500
    rng = np.random.default_rng(23)
    h = rng.integers(0, 4, W * H).astype(np.float64)
    k = rng.integers(0, 6, W * H)
    h[k == 1] = np.nextafter(h[k == 1], np.inf)        # one ulp above a terrace
    h[k == 2] = -h[k == 2]                             # -0 and negative terraces
    h[k == 3] = 1e-300 * rng.integers(0, 3, (k == 3).sum())
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    p = pkg.workload_params()
    L = pkg.library()
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as a, \
            pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as b:
        L.fs_test_set_receiver_path(b.handle, 1)
        a.setH(h)
        b.setH(h)
        for s in range(3):
            a.step(1)
            b.step(1)
            assert np.array_equal(a.receivers(), b.receivers()), f"step {s}"
            assert np.array_equal(a.getH(), b.getH()), f"step {s}"
        n = C.c_int32(0)
        pkg.check(L.fs_test_receiver_fixups(a.handle, C.byref(n)))
        assert n.value > W * H // 10


def relief(W, H, base, scale):
    """A smooth tilted surface with gentle bumps, `base` metres up, rings at 0."""
    yy, xx = np.divmod(np.arange(W * H), W)
    h = base + scale * (0.05 * xx + 0.03 * yy + 4.0 * np.sin(xx / 53.0) * np.sin(yy / 41.0))
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    return h


def test_receiver_filter_high_ground(pkg):
    """Tiles whose heights reach 128 m are staged relative to their first
    value, so the filter's error bound follows the tile's relief rather than
    its height: the same relief 4000 m up sends no more cells to the FP64
    fix-up than near sea level (staged by truncation), and the receivers
    equal the FP64 formula's -- also on tiles mixing negative ground, zeros
    and subnormals with high ground, values across a binade boundary, exact
    flats, and heights beyond the relative range (1e35; with K = 0 there,
    since no Newton iteration meets a 1e-3 m tolerance at 1e35 m)."""
    import ctypes as C
    W, H = 900, 700
    p = pkg.workload_params()
    L = pkg.library()
    counts = []
    for base in (1.0, 4000.0):
        with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
            m.setH(relief(W, H, base, 1.0))
            m.step(1)
            n = C.c_int32(0)
            pkg.check(L.fs_test_receiver_fixups(m.handle, C.byref(n)))
            counts.append(n.value)
    assert counts[1] <= counts[0] + 100, counts

    rng = np.random.default_rng(31)
    h = relief(W, H, 4000.0, 1.0)
    yy, xx = np.divmod(np.arange(W * H), W)
    interior = (xx > 1) & (yy > 1) & (xx < W - 2) & (yy < H - 2)
    a_neg = interior & (xx < 150) & (yy < 200)
    h[a_neg] = -3000.0 + rng.uniform(0, 50, a_neg.sum())
    a_tiny = interior & (xx >= 200) & (xx < 300) & (yy < 300) & (np.arange(W * H) % 7 == 0)
    h[a_tiny] = rng.choice([0.0, -0.0, 1e-300, 5e-324], a_tiny.sum())
    a_huge = interior & (xx >= 400) & (xx < 440) & (yy >= 100) & (yy < 200)
    h[a_huge] = 1e35 * rng.uniform(1, 2, a_huge.sum())
    a_flat = interior & (xx >= 500) & (xx < 700) & (yy >= 300) & (yy < 400)
    h[a_flat] = 5000.0
    a_binade = interior & (xx >= 100) & (xx < 400) & (yy >= 450)
    h[a_binade] = 4096.0 + rng.uniform(-1e-3, 1e-3, a_binade.sum())
    p0 = pkg.workload_params(keq=0.0)
    with pkg.FastScape_RBP(W, H, params=p0, init=pkg.INIT_ZERO) as a, \
            pkg.FastScape_RBP(W, H, params=p0, init=pkg.INIT_ZERO) as b:
        L.fs_test_set_receiver_path(b.handle, 1)
        a.setH(h)
        b.setH(h)
        for s in range(3):
            a.step(1)
            b.step(1)
            assert np.array_equal(a.receivers(), b.receivers()), f"step {s}"
            assert np.array_equal(a.getH(), b.getH()), f"step {s}"


@pytest.mark.parametrize("W,H", [(1000, 900), (902, 641)])
def test_receiver_filter_tma_staging(pkg, W, H):
    """The receiver filter's tiles staged by one TMA box (even widths)
    give the same receivers, levels and elevations as staged by loads, bit
    for bit, on the reference field and on high ground with negative
    ground, subnormals and flats (the relative restaging reads the same
    shared tile), with the grid's right and bottom edges cutting tiles."""
    p = pkg.workload_params()
    rng = np.random.default_rng(7)
    h = relief(W, H, 4000.0, 1.0)
    yy, xx = np.divmod(np.arange(W * H), W)
    interior = (xx > 1) & (yy > 1) & (xx < W - 2) & (yy < H - 2)
    a_neg = interior & (xx < 150) & (yy < 200)
    h[a_neg] = -3000.0 + rng.uniform(0, 50, a_neg.sum())
    a_tiny = interior & (xx >= 200) & (xx < 300) & (yy < 300) & (np.arange(W * H) % 7 == 0)
    h[a_tiny] = rng.choice([0.0, -0.0, 1e-300, 5e-324], a_tiny.sum())
    a_flat = interior & (xx >= 500) & (xx < 700) & (yy >= 300) & (yy < 400)
    h[a_flat] = 5000.0
    for init in (None, h):
        with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_REFERENCE, seed=3) as a, \
                pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_REFERENCE, seed=3) as b:
            b.use_tma_staging(True)
            assert b.launch_config()["receivers_tma"]
            if init is not None:
                a.setH(init)
                b.setH(init)
            for s in range(4):
                a.step(1)
                b.step(1)
                assert np.array_equal(a.receivers(), b.receivers()), f"step {s}"
                assert np.array_equal(a.levels()[0], b.levels()[0]), f"step {s}"
                assert np.array_equal(a.getH(), b.getH()), f"step {s}"


def test_tma_staging_refused_where_it_does_not_apply(pkg):
    """Odd widths and batches of several realizations keep the loads."""
    p = pkg.workload_params()
    with pkg.FastScape_RBP(301, 200, params=p, init=pkg.INIT_REFERENCE, seed=1) as m:
        with pytest.raises(pkg.FastScapeError):
            m.use_tma_staging(True)
    with pkg.FastScapeBatch([64, 64], [64, 64], [p, p], init=pkg.INIT_PHILOX, seeds=[1, 2]) as b:
        with pytest.raises(pkg.FastScapeError):
            b.use_tma_staging(True)


def valley(W, H):
    """V-shaped valley whose axis runs down to the base-level ring at y = 1:
    nearly every cell drains into the axis, so the axis cell next to base
    level (a level-1 cell) carries a drainage count of ~W*H."""
    yy, xx = np.divmod(np.arange(W * H), W)
    h = 1.0 + 0.5 * np.abs(xx - W // 2) + 0.05 * yy
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    return h


@pytest.mark.parametrize("n", [1, 2])
def test_table_growth_large_basin(pkg, oracle, n):
    """Counts beyond the initial erosion table (65536) make the timestep stop
    before touching h, grow the table and redo it: still bit-exact."""
    import ctypes as C
    W, H = 420, 400
    p = pkg.workload_params() if n == 1 else pkg.reference_params()
    op = Params(*p.as_tuple())
    h = valley(W, H)
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
        m.setH(h)
        cap = C.c_int32(0)
        pkg.check(pkg.library().fs_test_table_capacity(m.handle, C.byref(cap)))
        assert cap.value == 65536
        for s in range(3):
            if n != 1:
                m.setH(h)
            m.step(1)
            ref = oracle.phases(h, W, H, op)
            assert_step_equal(m, W, H, ref, f"step {s}", exact_h=(n == 1))
        pkg.check(pkg.library().fs_test_table_capacity(m.handle, C.byref(cap)))
        assert cap.value > 65536 and ref["accum"].max() / p.cell_area > 65536
        assert m.steps_executed() == 3


@pytest.mark.parametrize("W,H,n", [(64, 64, 1), (301, 157, 1), (90, 90, 2)])
def test_braun_willett_order(pkg, oracle, W, H, n):
    """fs_get_stack_dfs equals the reference Braun-Willett stack order
    (fastscape_BW.cpp:201-221, pinned against the reference by
    tests/test_oracle_pin.py::test_bw_dfs_order) and its stack_start."""
    p = pkg.workload_params() if n == 1 else pkg.reference_params()
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_PHILOX, seed=W) as m:
        for _ in range(3):
            m.step(1)
            stack, starts = m.stack_dfs()
            want, want_starts = oracle.order_bw(m.receivers(), W, H)
            assert np.array_equal(stack, want)
            assert np.array_equal(starts, want_starts)


def test_braun_willett_order_valley(pkg, oracle):
    """Deep trees (hundreds of levels) through one basin."""
    W, H = 200, 180
    with pkg.FastScape_RBP(W, H, params=pkg.workload_params(), init=pkg.INIT_ZERO) as m:
        m.setH(valley(W, H))
        m.step(2)
        stack, starts = m.stack_dfs()
        want, want_starts = oracle.order_bw(m.receivers(), W, H)
        assert np.array_equal(stack, want) and np.array_equal(starts, want_starts)
