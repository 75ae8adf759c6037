"""Pins the oracle restatement against the reference compiled from its own
sources (oracle/_ref, built by oracle/build.py where the reference tree is
available). Skipped where that build does not exist."""
import numpy as np
import pytest

from conftest import ref_harness_available
from oracle.pyoracle import REFERENCE_PARAMS, RefHarness, workload_params

pytestmark = pytest.mark.skipif(not ref_harness_available("pristine"),
                                reason="reference harness not built here")

KEYS = ("rec", "ndon", "donor", "stack", "levels", "accum", "h_uplifted", "h")


def compare_steps(oracle, hr, p, W, H, variant, nsteps, h=None):
    m = hr.model(W, H, p, variant)
    if h is None:
        h = oracle.terrain(W, H, 0)
        assert np.array_equal(h, m.get_h())
    else:
        m.set_h(h)
        h = h.copy()
    for s in range(nsteps):
        r = m.phases()
        q = oracle.phases(h, W, H, p, parallel=bool(variant))
        for k in KEYS:
            assert np.array_equal(r[k], q[k]), f"{k} differs at step {s}"
        assert r["nlevel"] == q["nlevel"]


@pytest.mark.parametrize("W,H", [(5, 5), (6, 7), (33, 17), (96, 96)])
@pytest.mark.parametrize("variant", [0, 1])
def test_pristine_reference_constants(oracle, W, H, variant):
    compare_steps(oracle, RefHarness("pristine", "exact"), REFERENCE_PARAMS, W, H, variant, 6)


@pytest.mark.parametrize("W,H", [(5, 5), (8, 13), (64, 64), (150, 71)])
@pytest.mark.parametrize("variant", [0, 1])
def test_param_workload_constants(oracle, W, H, variant):
    compare_steps(oracle, RefHarness("param", "exact"), workload_params(), W, H, variant, 6)


def test_param_build_equals_pristine():
    # The constant patch changes nothing when given the original constants.
    a = RefHarness("pristine", "exact").model(48, 40, REFERENCE_PARAMS, 0)
    b = RefHarness("param", "exact").model(48, 40, REFERENCE_PARAMS, 0)
    for _ in range(5):
        ra, rb = a.phases(), b.phases()
        for k in KEYS:
            assert np.array_equal(ra[k], rb[k])


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_fields_and_parameters(oracle, seed):
    rng = np.random.default_rng(seed)
    W, H = int(rng.integers(5, 70)), int(rng.integers(5, 70))
    p = workload_params(dx=float(rng.uniform(1, 200)), keq=float(10 ** rng.uniform(-6, -5)),
                        meq=float(rng.uniform(0.3, 0.6)), ueq=float(10 ** rng.uniform(-4, -2.3)))
    h = rng.uniform(0, 50, W * H)
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    compare_steps(oracle, RefHarness("param", "exact"), p, W, H, seed % 2, 8, h=h)


def test_reference_run_semantics(oracle):
    # run(n) executes n+1 timesteps (fastscape_RB.cpp:366).
    m = RefHarness("param", "exact").model(40, 40, workload_params(), 1)
    m.run(7)
    h = oracle.terrain(40, 40, 0)
    oracle.steps(h, 40, 40, workload_params(), 8, parallel=True)
    assert np.array_equal(m.get_h(), h)


@pytest.mark.parametrize("W,H,text", [(30, 30, "pristine"), (57, 41, "param"), (5, 5, "param")])
def test_bw_dfs_order(oracle, W, H, text):
    """fso_order_bw == the reference Braun-Willett FastScape_BW's stack
    (fastscape_BW.cpp:201-221), over several timesteps; its elevations equal
    the level-ordered RB's."""
    from oracle.pyoracle import REFERENCE_PARAMS
    p = REFERENCE_PARAMS if text == "pristine" else workload_params()
    bw = RefHarness(text, "exact").model(W, H, p, 2)
    h = oracle.terrain(W, H, 0)
    for s in range(5):
        r = bw.bw_phases()
        q = oracle.phases(h, W, H, p)
        stack, starts = oracle.order_bw(q["rec"], W, H)
        assert np.array_equal(r["rec"], q["rec"])
        assert np.array_equal(r["stack"], stack), f"step {s}"
        assert np.array_equal(r["h"], q["h"]), f"step {s}"
        assert starts[-1] == W * H and np.all(q["rec"][stack[starts[:-1]]] == -1)
