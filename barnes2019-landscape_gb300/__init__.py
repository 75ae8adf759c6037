"""GB300 FastScape timestep -- Python mirror of the reference's model object.

The reference's public surface is one class per variant
(``FastScape_RBP(width, height)``, ``run(nstep)``, ``getH()``;
fastscape_RB+P.cpp:46-431). ``FastScape_RBP`` below keeps those names and
their meaning on top of the C ABI in ``include/fastscape_gb300.h`` (bound with
ctypes to ``lib/libfastscape_gb300.so``); every timestep runs on the GPU.
There is no CPU fallback: if the CUDA library is missing or no GPU is
present, constructing a model raises.

The package directory name contains a hyphen, so import it with
``importlib.import_module("barnes2019-landscape_gb300")`` (or use
``load()`` from ``__graft_entry__``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libfastscape_gb300.so"

SQRT2 = 1.414213562373095048801688724209698078569671875376948

NO_FLOW = -1
FS_OK = 0
STATUS = {
    -1: "FS_ERR_ARG", -2: "FS_ERR_CUDA", -3: "FS_ERR_TIMEOUT",
    -4: "FS_ERR_LEVEL_OVERFLOW", -5: "FS_ERR_NONFINITE", -6: "FS_ERR_ORDER",
    -7: "FS_ERR_NEWTON", -8: "FS_ERR_NOMEM", -9: "FS_ERR_STATE",
}
INIT_ZERO, INIT_REFERENCE, INIT_MT19937, INIT_PHILOX = 0, 1, 2, 3
# fs_set_timing modes: per-kernel events (direct launches) or whole calls
# (the launch path in use, CUDA-graph replay included)
TIMING_OFF, TIMING_KERNELS, TIMING_CALL = 0, 1, 2

# Exported C symbols, in header order (include/fastscape_gb300.h and
# include/fastscape_gb300_testing.h).
ABI_SYMBOLS = [
    "fs_params_reference", "fs_params_workload", "fs_create", "fs_destroy",
    "fs_run", "fs_step", "fs_get_elevation", "fs_set_elevation",
    "fs_get_accumulation", "fs_get_receivers", "fs_get_receiver_index",
    "fs_get_levels", "fs_get_donor_mask", "fs_get_stack_dfs", "fs_get_shape", "fs_get_params",
    "fs_steps_executed", "fs_set_timing", "fs_get_phase_times",
    "fs_set_barrier_timeout", "fs_synchronize", "fs_last_error", "fs_version",
    "fs_batch_create", "fs_batch_destroy", "fs_batch_step", "fs_batch_run",
    "fs_batch_get_elevation", "fs_batch_set_elevation", "fs_batch_get_accumulation",
    "fs_batch_get_receivers", "fs_batch_get_levels", "fs_batch_get_stack_dfs", "fs_batch_info",
    "fs_batch_set_timing", "fs_batch_get_phase_times", "fs_batch_use_graph",
    "fs_batch_use_int_sub", "fs_use_int_sub",
    "fs_batch_autotune", "fs_batch_launch_config", "fs_batch_synchronize",
    "fs_autotune", "fs_launch_config",
    "fs_step_noalloc",
    "fs_test_order_from_receivers", "fs_test_barrier_timeout",
    "fs_test_set_receiver_path", "fs_test_set_erosion_path", "fs_test_receiver_fixups",
    "fs_test_table_capacity", "fs_test_sg_conv",
]


class FastScapeError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Params(C.Structure):
    """fs_params: the constants the reference hard-codes at
    fastscape_RB.cpp:58-65."""
    _fields_ = [(n, C.c_double) for n in
                ("keq", "neq", "meq", "ueq", "dt", "dr_orth", "dr_diag", "tol",
                 "cell_area")]

    def __repr__(self):
        return "Params(" + ", ".join(f"{n}={getattr(self, n)!r}" for n, _ in self._fields_) + ")"

    def as_tuple(self):
        return tuple(getattr(self, n) for n, _ in self._fields_)


def reference_params() -> Params:
    """K 2e-6, n 2, m 0.8, U 2e-3, dt 1000, dr {1, SQRT2}, tol 1e-3,
    cell_area 40000 (fastscape_RB.cpp:58-65)."""
    return Params(2e-6, 2.0, 0.8, 2e-3, 1000.0, 1.0, SQRT2, 1e-3, 40000.0)


def workload_params(dx: float = 100.0, keq: float = 2e-6, meq: float = 0.4,
                    ueq: float = 2e-3, neq: float = 1.0) -> Params:
    """K 2e-6, n 1, m 0.4, U 2e-3, dt 1000, dr {dx, dx*SQRT2}, tol 1e-3,
    cell_area dx*dx (the 1000^2 and 10000^2 workloads, dx = 100 m)."""
    return Params(keq, neq, meq, ueq, 1000.0, dx, dx * SQRT2, 1e-3, dx * dx)


_lib = None


def library() -> C.CDLL:
    """Loads the CUDA library; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise FastScapeError(-2, f"CUDA library not built: {LIB_PATH} "
                                 "(run __graft_entry__.build())")
    L = C.CDLL(str(LIB_PATH))
    vp, dp, i32p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
    pp = C.POINTER(Params)
    L.fs_params_reference.argtypes = [pp]
    L.fs_params_workload.argtypes = [pp, C.c_double]
    L.fs_create.argtypes = [C.c_int, C.c_int, pp, C.c_int, C.c_uint64, C.POINTER(C.c_int)]
    L.fs_create.restype = vp
    L.fs_destroy.argtypes = [vp]
    L.fs_run.argtypes = [vp, C.c_int]
    L.fs_step.argtypes = [vp, C.c_int]
    L.fs_get_elevation.argtypes = [vp, dp]
    L.fs_set_elevation.argtypes = [vp, dp]
    L.fs_get_accumulation.argtypes = [vp, dp]
    L.fs_get_receivers.argtypes = [vp, i32p]
    L.fs_get_receiver_index.argtypes = [vp, C.POINTER(C.c_int64)]
    L.fs_get_levels.argtypes = [vp, i32p, i32p]
    L.fs_get_donor_mask.argtypes = [vp, C.POINTER(C.c_uint8)]
    L.fs_get_stack_dfs.argtypes = [vp, i32p, i32p, i32p]
    L.fs_batch_get_stack_dfs.argtypes = [vp, C.c_int, i32p, i32p, i32p]
    L.fs_get_shape.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.fs_get_params.argtypes = [vp, pp]
    L.fs_steps_executed.argtypes = [vp]
    L.fs_steps_executed.restype = C.c_int64
    L.fs_set_timing.argtypes = [vp, C.c_int]
    L.fs_get_phase_times.argtypes = [vp, dp, C.c_int]
    L.fs_set_barrier_timeout.argtypes = [vp, C.c_double]
    L.fs_synchronize.argtypes = [vp]
    L.fs_last_error.argtypes = [C.c_char_p, C.c_size_t]
    L.fs_last_error.restype = C.c_size_t
    L.fs_version.restype = C.c_char_p
    ip = C.POINTER(C.c_int)
    L.fs_batch_create.argtypes = [C.c_int, ip, ip, pp, C.c_int, C.POINTER(C.c_uint64), ip]
    L.fs_batch_create.restype = vp
    L.fs_batch_destroy.argtypes = [vp]
    L.fs_batch_step.argtypes = [vp, C.c_int]
    L.fs_batch_run.argtypes = [vp, C.c_int]
    L.fs_batch_get_elevation.argtypes = [vp, C.c_int, dp]
    L.fs_batch_set_elevation.argtypes = [vp, C.c_int, dp]
    L.fs_batch_get_accumulation.argtypes = [vp, C.c_int, dp]
    L.fs_batch_get_receivers.argtypes = [vp, C.c_int, i32p]
    L.fs_batch_get_levels.argtypes = [vp, C.c_int, i32p, i32p]
    L.fs_batch_info.argtypes = [vp, ip, C.POINTER(C.c_int64)]
    L.fs_batch_set_timing.argtypes = [vp, C.c_int]
    L.fs_batch_get_phase_times.argtypes = [vp, dp, C.c_int]
    L.fs_batch_use_graph.argtypes = [vp, C.c_int]
    L.fs_batch_use_int_sub.argtypes = [vp, C.c_int]
    L.fs_use_int_sub.argtypes = [vp, C.c_int]
    L.fs_batch_autotune.argtypes = [vp, C.c_int, ip]
    L.fs_batch_launch_config.argtypes = [vp, ip, ip, ip, ip]
    L.fs_autotune.argtypes = [vp, C.c_int, ip]
    L.fs_launch_config.argtypes = [vp, ip, ip, ip, ip]
    L.fs_batch_synchronize.argtypes = [vp]
    L.fs_step_noalloc.argtypes = [vp, C.c_int, C.c_int, pp, C.c_int, vp]
    L.fs_test_order_from_receivers.argtypes = [vp, i32p]
    L.fs_test_barrier_timeout.argtypes = [vp, C.c_double]
    L.fs_test_set_receiver_path.argtypes = [vp, C.c_int]
    L.fs_test_set_erosion_path.argtypes = [vp, C.c_int]
    L.fs_test_receiver_fixups.argtypes = [vp, i32p]
    L.fs_test_table_capacity.argtypes = [vp, i32p]
    u16p = C.POINTER(C.c_uint16)
    L.fs_test_sg_conv.argtypes = [C.c_int] * 7 + [u16p, u16p, C.POINTER(C.c_float), C.c_int,
                                                  u16p, vp]
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    library().fs_last_error(buf, len(buf))
    return buf.value.decode()


def check(status: int) -> None:
    if status != FS_OK:
        raise FastScapeError(status, last_error())


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


class FastScape_RBP:
    """Drop-in for the reference's ``FastScape_RBP`` (fastscape_RB+P.cpp:46).

    ``FastScape_RBP(width, height)`` draws the reference's initial field
    (fastscape_RB.cpp:111-130) and uses the reference's constants unless
    ``params`` is given; ``run(nstep)`` executes nstep+1 timesteps like the
    reference (fastscape_RB.cpp:366); ``getH()`` returns the elevation (a
    host copy -- the reference returns a reference to its own vector).
    """

    def __init__(self, width: int, height: int, params: Params | None = None,
                 init: int = INIT_REFERENCE, seed: int = 123):
        L = library()
        self.width, self.height = int(width), int(height)
        self.size = self.width * self.height
        self.params = reference_params() if params is None else params
        st = C.c_int(0)
        self._m = L.fs_create(self.width, self.height, C.byref(self.params), int(init),
                              int(seed) & 0xFFFFFFFFFFFFFFFF, C.byref(st))
        if not self._m:
            raise FastScapeError(st.value, last_error())

    def close(self):
        if getattr(self, "_m", None):
            library().fs_destroy(self._m)
            self._m = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- the reference's interface ---------------------------------------
    def run(self, nstep: int) -> None:
        """nstep+1 timesteps (fastscape_RB.cpp:341-398)."""
        check(library().fs_run(self._m, int(nstep)))

    def getH(self) -> np.ndarray:
        out = np.empty(self.size, np.float64)
        check(library().fs_get_elevation(self._m, _p(out, C.c_double)))
        return out

    # -- additions ----------------------------------------------------------
    def step(self, k: int = 1) -> None:
        """Exactly k timesteps."""
        check(library().fs_step(self._m, int(k)))

    def setH(self, h) -> None:
        h = np.ascontiguousarray(h, np.float64).reshape(-1)
        if h.size != self.size:
            raise ValueError(f"expected {self.size} elevations, got {h.size}")
        check(library().fs_set_elevation(self._m, _p(h, C.c_double)))

    def accumulation(self) -> np.ndarray:
        out = np.empty(self.size, np.float64)
        check(library().fs_get_accumulation(self._m, _p(out, C.c_double)))
        return out

    def receivers(self) -> np.ndarray:
        out = np.empty(self.size, np.int32)
        check(library().fs_get_receivers(self._m, _p(out, C.c_int32)))
        return out

    def receiver_index(self) -> np.ndarray:
        out = np.empty(self.size, np.int64)
        check(library().fs_get_receiver_index(self._m, _p(out, C.c_int64)))
        return out

    def levels(self):
        """(level id per cell, number of levels)."""
        out = np.empty(self.size, np.int32)
        n = C.c_int32(0)
        check(library().fs_get_levels(self._m, _p(out, C.c_int32), C.byref(n)))
        return out, n.value

    def stack_dfs(self):
        """(stack, stack_start) of the Braun-Willett order
        (fastscape_BW.cpp:201-221, fastscape_BW+P.cpp:223-240)."""
        stack = np.empty(self.size, np.int32)
        starts = np.empty(self.size + 1, np.int32)
        n = C.c_int32(0)
        check(library().fs_get_stack_dfs(self._m, _p(stack, C.c_int32), _p(starts, C.c_int32),
                                         C.byref(n)))
        return stack, starts[:n.value + 1].copy()

    def donor_mask(self) -> np.ndarray:
        out = np.empty(self.size, np.uint8)
        check(library().fs_get_donor_mask(self._m, _p(out, C.c_uint8)))
        return out

    def steps_executed(self) -> int:
        return int(library().fs_steps_executed(self._m))

    def set_timing(self, on=True) -> None:
        """True / TIMING_KERNELS: per-kernel events (direct launches);
        TIMING_CALL: events around whole calls only (graph replay kept);
        False: off."""
        check(library().fs_set_timing(self._m, int(on)))

    TIMERS = ("receivers", "donors_level0", "walk", "total",
              "walk_order", "walk_accumulation", "walk_erosion",
              "order_kernel", "erode_kernel", "accum_kernel")

    def phase_times(self, reset: bool = False):
        """Device milliseconds per timer in TIMERS (fs_get_phase_times)."""
        out = np.zeros(len(self.TIMERS), np.float64)
        check(library().fs_get_phase_times(self._m, _p(out, C.c_double), int(reset)))
        return out

    def autotune(self, probe_steps: int = 2):
        """Picks the fastest launch configuration (kernel blocks per SM,
        graph replay) on the model's own state, which it restores."""
        out = (C.c_int * 2)()
        check(library().fs_autotune(self._m, int(probe_steps), out))
        return self.launch_config()

    def use_int_sub(self, on: bool = True) -> None:
        """n = 1 or 2: the erosion's elevation subtractions in integer
        arithmetic (same results; fs_autotune chooses by speed)."""
        check(library().fs_use_int_sub(self._m, int(bool(on))))

    def launch_config(self):
        o, e, g, i = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(library().fs_launch_config(self._m, C.byref(o), C.byref(e), C.byref(g),
                                         C.byref(i)))
        return {"order_blocks_per_sm": o.value, "erode_blocks_per_sm": e.value,
                "graph": bool(g.value), "erode_int_sub": bool(i.value)}

    def set_barrier_timeout(self, ms: float) -> None:
        check(library().fs_set_barrier_timeout(self._m, float(ms)))

    def synchronize(self) -> None:
        check(library().fs_synchronize(self._m))

    @property
    def handle(self):
        return self._m


# The serial reference class has the same interface.
FastScape_RB = FastScape_RBP


class FastScapeBatch:
    """A ragged batch of independent realizations stepped together
    (fs_batch_* in the C ABI). Each realization r has its own grid
    ``widths[r] x heights[r]`` and constants ``params[r]`` (one n for all)
    and evolves exactly as a FastScape_RBP of its own would."""

    def __init__(self, widths, heights, params, init: int = INIT_PHILOX, seeds=None):
        L = library()
        n = len(widths)
        if not (len(heights) == n and len(params) == n):
            raise ValueError("widths, heights and params must have the same length")
        self.n = n
        self.widths = [int(w) for w in widths]
        self.heights = [int(h) for h in heights]
        self.params = list(params)
        w = (C.c_int * n)(*self.widths)
        h = (C.c_int * n)(*self.heights)
        pa = (Params * n)(*self.params)
        sd = None
        if seeds is not None:
            sd = (C.c_uint64 * n)(*[int(s) & 0xFFFFFFFFFFFFFFFF for s in seeds])
        st = C.c_int(0)
        self._b = L.fs_batch_create(n, w, h, pa, int(init), sd, C.byref(st))
        if not self._b:
            raise FastScapeError(st.value, last_error())

    def close(self):
        if getattr(self, "_b", None):
            library().fs_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def size(self, r: int) -> int:
        if not 0 <= int(r) < self.n:
            raise FastScapeError(-1, f"realization {r} out of range [0, {self.n})")
        return self.widths[r] * self.heights[r]

    def cells(self) -> int:
        n, c = C.c_int(0), C.c_int64(0)
        check(library().fs_batch_info(self._b, C.byref(n), C.byref(c)))
        return c.value

    def step(self, k: int = 1) -> None:
        check(library().fs_batch_step(self._b, int(k)))

    def run(self, nstep: int) -> None:
        check(library().fs_batch_run(self._b, int(nstep)))

    def getH(self, r: int) -> np.ndarray:
        out = np.empty(self.size(r), np.float64)
        check(library().fs_batch_get_elevation(self._b, int(r), _p(out, C.c_double)))
        return out

    def setH(self, r: int, h) -> None:
        h = np.ascontiguousarray(h, np.float64).reshape(-1)
        if h.size != self.size(r):
            raise ValueError(f"expected {self.size(r)} elevations, got {h.size}")
        check(library().fs_batch_set_elevation(self._b, int(r), _p(h, C.c_double)))

    def accumulation(self, r: int) -> np.ndarray:
        out = np.empty(self.size(r), np.float64)
        check(library().fs_batch_get_accumulation(self._b, int(r), _p(out, C.c_double)))
        return out

    def receivers(self, r: int) -> np.ndarray:
        out = np.empty(self.size(r), np.int32)
        check(library().fs_batch_get_receivers(self._b, int(r), _p(out, C.c_int32)))
        return out

    def levels(self, r: int):
        out = np.empty(self.size(r), np.int32)
        n = C.c_int32(0)
        check(library().fs_batch_get_levels(self._b, int(r), _p(out, C.c_int32), C.byref(n)))
        return out, n.value

    def set_timing(self, on=True) -> None:
        """As FastScape_RBP.set_timing."""
        check(library().fs_batch_set_timing(self._b, int(on)))

    def phase_times(self, reset: bool = False):
        out = np.zeros(len(FastScape_RBP.TIMERS), np.float64)
        check(library().fs_batch_get_phase_times(self._b, _p(out, C.c_double), int(reset)))
        return out

    def use_graph(self, on: bool = True) -> None:
        check(library().fs_batch_use_graph(self._b, int(bool(on))))

    def use_int_sub(self, on: bool = True) -> None:
        check(library().fs_batch_use_int_sub(self._b, int(bool(on))))

    def autotune(self, probe_steps: int = 2):
        """Picks the fastest launch configuration; returns it."""
        out = (C.c_int * 2)()
        check(library().fs_batch_autotune(self._b, int(probe_steps), out))
        return self.launch_config()

    def launch_config(self):
        o, e, g, i = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(library().fs_batch_launch_config(self._b, C.byref(o), C.byref(e), C.byref(g),
                                               C.byref(i)))
        return {"order_blocks_per_sm": o.value, "erode_blocks_per_sm": e.value,
                "graph": bool(g.value), "erode_int_sub": bool(i.value)}

    def synchronize(self) -> None:
        check(library().fs_batch_synchronize(self._b))

    @property
    def handle(self):
        return self._b


def version() -> str:
    return library().fs_version().decode()


def sg_conv(mode: int, x_bits: np.ndarray, w_bits: np.ndarray, taps: int = 9, bias=None,
            relu: bool = False, mask_bits=None) -> np.ndarray:
    """One convolution of the surrogate's tensor-core kernels on host arrays
    (fs_test_sg_conv). mode 0: forward, x [B,H,W,cin], w [cout,taps,cin] ->
    BF16 bits [B,H,W,cout]; mode 1: data gradient, x = dy [B,H,W,cout], w as
    above, mask [B,H,W,cin] or None -> BF16 bits [B,H,W,cin]; mode 2: weight
    gradient, x [B,H,W,cin], w = dy [B,H,W,cout] -> FP32 [cout,taps,cin]."""
    x_bits = np.ascontiguousarray(x_bits, np.uint16)
    w_bits = np.ascontiguousarray(w_bits, np.uint16)
    B, H, W = x_bits.shape[:3]
    if mode == 2:
        cin, cout = x_bits.shape[3], w_bits.shape[3]
        out = np.empty((cout, taps, cin), np.float32)
    else:
        cout, t, cin = w_bits.shape
        if t != taps:
            raise ValueError("weights do not match taps")
        out = np.empty((B, H, W, cout if mode == 0 else cin), np.uint16)
    u16 = C.POINTER(C.c_uint16)
    bp = None
    if bias is not None:
        bias = np.ascontiguousarray(bias, np.float32)
        bp = bias.ctypes.data_as(C.POINTER(C.c_float))
    mp = None
    if mask_bits is not None:
        mask_bits = np.ascontiguousarray(mask_bits, np.uint16)
        mp = mask_bits.ctypes.data_as(u16)
    check(library().fs_test_sg_conv(int(mode), B, H, W, cin, cout, int(taps),
                                    x_bits.ctypes.data_as(u16), w_bits.ctypes.data_as(u16), bp,
                                    int(bool(relu)), mp, out.ctypes.data_as(C.c_void_p)))
    return out
