"""fs_step_noalloc: timesteps on a caller-owned device buffer with all scratch
in one static device array, for callers that may not allocate device memory
while running (an application that owns every device byte through its own
pool, a latency-critical loop where cudaMalloc/cudaFree would synchronize
the device, a plugin with a fixed footprint).

The caller's buffer is a torch CUDA tensor here (torch only provides device
memory). The result must equal the allocating entry point's (fs_create +
fs_set_elevation + fs_step) bit for bit -- the tolerance of the n = 1 parity
tests -- over two calls in a row, since the static scratch keeps the previous
call's contents. This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(pkg):
    lib = pkg.library()
    f = lib.fs_step_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(pkg.Params), C.c_int, C.c_void_p]
    f.restype = C.c_int
    return f


def _field(W, H, seed):
    rng = np.random.default_rng(seed)
    h = rng.uniform(0, 1, W * H)
    yy, xx = np.divmod(np.arange(W * H), W)
    h[(xx <= 1) | (yy <= 1) | (xx >= W - 2) | (yy >= H - 2)] = 0
    return h


@pytest.mark.parametrize("W,H,n", [(300, 200, 1), (512, 512, 1), (300, 200, 2)])
def test_noalloc_matches_allocating_entry_point(pkg, W, H, n):
    torch = pytest.importorskip("torch")
    step_noalloc = _noalloc(pkg)
    p = pkg.workload_params() if n == 1 else pkg.reference_params()
    h0 = _field(W, H, W + H)
    d_h = torch.from_numpy(h0.copy()).cuda()
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
        m.setH(h0)
        for k in (3, 2):                       # two calls in a row
            st = step_noalloc(C.c_void_p(d_h.data_ptr()), W, H, C.byref(p), k, None)
            assert st == 0, pkg.last_error()
            torch.cuda.synchronize()
            m.step(k)
            got = d_h.cpu().numpy()
            assert np.array_equal(got, m.getH())


def test_noalloc_rejects_grids_over_the_limit(pkg):
    torch = pytest.importorskip("torch")
    step_noalloc = _noalloc(pkg)
    p = pkg.workload_params()
    d_h = torch.zeros(8, dtype=torch.float64, device="cuda")
    st = step_noalloc(C.c_void_p(d_h.data_ptr()), 1024, 1024, C.byref(p), 1, None)
    assert st == -1
    assert "FS_NOALLOC_MAX_CELLS" in pkg.last_error()


def test_noalloc_refuses_nonfinite_input(pkg):
    """Like fs_set_elevation, the entry point refuses NaN/Inf in the caller's
    field and leaves the buffer as it was; the next call still works."""
    torch = pytest.importorskip("torch")
    step_noalloc = _noalloc(pkg)
    p = pkg.workload_params()
    W, H = 64, 48
    h0 = _field(W, H, 5)
    bad = h0.copy()
    bad[10 * W + 20] = np.nan
    d_h = torch.from_numpy(bad.copy()).cuda()
    st = step_noalloc(C.c_void_p(d_h.data_ptr()), W, H, C.byref(p), 2, None)
    assert st == -5, pkg.last_error()
    got = d_h.cpu().numpy()
    assert np.array_equal(np.isnan(got), np.isnan(bad))
    assert np.array_equal(got[~np.isnan(got)], bad[~np.isnan(bad)])
    d_h = torch.from_numpy(h0.copy()).cuda()
    assert step_noalloc(C.c_void_p(d_h.data_ptr()), W, H, C.byref(p), 2, None) == 0
    with pkg.FastScape_RBP(W, H, params=p, init=pkg.INIT_ZERO) as m:
        m.setH(h0)
        m.step(2)
        torch.cuda.synchronize()
        assert np.array_equal(d_h.cpu().numpy(), m.getH())
