"""Failure detection on the GPU without faulting it: every error is made on
the host side (bad input, an impossible receiver array, a wait on a count
nothing completes, bounded to tens of milliseconds) and must come back as a
status code with the device still usable afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_nonfinite_input_rejected(pkg):
    with pkg.FastScape_RBP(32, 32, params=pkg.workload_params()) as m:
        h = m.getH()
        h[100] = np.nan
        with pytest.raises(pkg.FastScapeError) as e:
            m.setH(h)
        assert e.value.status == -5
        h[100] = 0.5
        m.setH(h)
        m.step(2)


def test_cycle_in_receivers_is_reported(pkg):
    W = H = 12
    with pkg.FastScape_RBP(W, H, params=pkg.workload_params()) as m:
        rec = np.full(W * H, -1, np.int32)
        # two interior cells pointing at each other: (5,5) -> E, (5,6) -> W
        rec[5 * W + 5] = 4
        rec[5 * W + 6] = 0
        # a third cell draining into the pair never reaches base level either
        rec[6 * W + 5] = 2
        with pytest.raises(pkg.FastScapeError) as e:
            pkg.check(pkg.library().fs_test_order_from_receivers(
                m.handle, rec.ctypes.data_as(pkg.C.POINTER(pkg.C.c_int32))))
        assert e.value.status == -6
        # the model (and GPU) still works afterwards
        m.step(3)
        assert np.all(np.isfinite(m.getH()))


def test_valid_injected_receivers_order(pkg):
    W = H = 9
    with pkg.FastScape_RBP(W, H, params=pkg.workload_params()) as m:
        rec = np.full(W * H, -1, np.int32)
        # a chain along row 4 draining west: x=6 -> 5 -> 4 -> 3 -> 2 -> 1(base)
        for x in range(2, 7):
            rec[4 * W + x] = 0
        pkg.check(pkg.library().fs_test_order_from_receivers(
            m.handle, rec.ctypes.data_as(pkg.C.POINTER(pkg.C.c_int32))))
        lid, nl = m.levels()
        assert nl == 6
        assert [lid[4 * W + x] for x in range(1, 7)] == [0, 1, 2, 3, 4, 5]
        acc = m.accumulation() / m.params.cell_area
        assert [acc[4 * W + x] for x in range(1, 7)] == [6, 5, 4, 3, 2, 1]


def test_invalid_injected_receivers_rejected(pkg):
    W = H = 9
    with pkg.FastScape_RBP(W, H, params=pkg.workload_params()) as m:
        rec = np.full(W * H, -1, np.int32)
        rec[0] = 3  # ring cell with a receiver
        st = pkg.library().fs_test_order_from_receivers(
            m.handle, rec.ctypes.data_as(pkg.C.POINTER(pkg.C.c_int32)))
        assert st == -1


def test_barrier_wait_times_out_and_gpu_stays_usable(pkg):
    with pkg.FastScape_RBP(64, 64, params=pkg.workload_params()) as m:
        st = pkg.library().fs_test_barrier_timeout(m.handle, 30.0)
        assert st == -3
        assert "timed out" in pkg.last_error()
        m.step(2)
        assert np.all(np.isfinite(m.getH()))


def test_bad_arguments(pkg):
    with pkg.FastScape_RBP(16, 16, params=pkg.workload_params()) as m:
        with pytest.raises(pkg.FastScapeError):
            m.step(-1)
        with pytest.raises(pkg.FastScapeError):
            m.run(-2)
        with pytest.raises(pkg.FastScapeError):
            m.set_barrier_timeout(-1)
        m.run(-1)  # zero timesteps, like the reference's loop with nstep=-1
        assert m.steps_executed() == 0
        with pytest.raises(pkg.FastScapeError) as e:
            m.accumulation()
        assert e.value.status == -9
