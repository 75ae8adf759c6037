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
    "fs_batch_use_cta_walk", "fs_batch_walk_mode",
    "fs_batch_use_tma_staging", "fs_batch_tma_staging", "fs_use_tma_staging", "fs_tma_staging",
    "fs_batch_set_active", "fs_batch_analyze", "fs_batch_drainage_counts",
    "fs_batch_device_elevation", "fs_batch_stream",
    "fs_batch_get_params", "fs_batch_get_shape",
    "fs_step_noalloc",
    "fs_test_order_from_receivers", "fs_test_barrier_timeout",
    "fs_test_set_receiver_path", "fs_test_set_erosion_path", "fs_test_receiver_fixups",
    "fs_test_table_capacity", "fs_test_sg_conv",
    "fs_sg_config_default", "fs_sg_create", "fs_sg_destroy", "fs_sg_get_config",
    "fs_sg_param_count", "fs_sg_get_params", "fs_sg_set_params", "fs_sg_get_grads",
    "fs_sg_save", "fs_sg_load", "fs_sg_reserve", "fs_sg_add_samples", "fs_sg_generate",
    "fs_sg_set_holdout", "fs_sg_dataset_info", "fs_sg_get_sample", "fs_sg_train", "fs_sg_eval",
    "fs_sg_eval_baselines", "fs_sg_grad", "fs_sg_train_stats", "fs_sg_predict_host", "fs_sg_predict_batch",
    "fs_sg_time_forward", "fs_sg_infer_flops", "fs_sg_ensemble_defaults", "fs_sg_compare_host", "fs_sg_ensemble_run",
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


class SgConfig(C.Structure):
    """fs_sg_config (include/fastscape_surrogate.h)."""
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("base_channels", C.c_int),
                ("batch", C.c_int), ("jump", C.c_int), ("dt", C.c_double),
                ("seed", C.c_uint64)]


class EnsembleOpts(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("plain_steps", C.c_int), ("judge_fraction", C.c_double),
                ("max_rel_rms", C.c_double), ("min_agreement", C.c_double),
                ("seed", C.c_uint64)]


class EnsembleStats(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("cycles", "jumps", "judged", "fallbacks")] + \
               [(n, C.c_double) for n in ("rel_rms_mean", "rel_rms_max", "agreement_mean",
                                          "agreement_min", "ms_total", "ms_infer", "ms_exact",
                                          "ms_plain", "ms_judge", "rel_rms_unchanged_mean",
                                          "agreement_unchanged_mean")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


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
    L.fs_batch_use_cta_walk.argtypes = [vp, C.c_int]
    L.fs_batch_walk_mode.argtypes = [vp, ip]
    L.fs_batch_use_tma_staging.argtypes = [vp, C.c_int]
    L.fs_batch_tma_staging.argtypes = [vp, ip]
    L.fs_use_tma_staging.argtypes = [vp, C.c_int]
    L.fs_tma_staging.argtypes = [vp, ip]
    L.fs_batch_set_active.argtypes = [vp, C.c_int, ip]
    L.fs_batch_analyze.argtypes = [vp]
    L.fs_batch_drainage_counts.argtypes = [vp, C.c_int, vp]
    L.fs_batch_device_elevation.argtypes = [vp, C.c_int, C.POINTER(C.c_void_p)]
    L.fs_batch_stream.argtypes = [vp, C.POINTER(C.c_void_p)]
    L.fs_batch_get_params.argtypes = [vp, C.c_int, pp]
    L.fs_batch_get_shape.argtypes = [vp, C.c_int, ip, ip]
    L.fs_step_noalloc.argtypes = [vp, C.c_int, C.c_int, pp, C.c_int, vp]
    L.fs_test_order_from_receivers.argtypes = [vp, i32p]
    L.fs_test_barrier_timeout.argtypes = [vp, C.c_double]
    L.fs_test_set_receiver_path.argtypes = [vp, C.c_int]
    L.fs_test_set_erosion_path.argtypes = [vp, C.c_int]
    L.fs_test_receiver_fixups.argtypes = [vp, i32p]
    L.fs_test_table_capacity.argtypes = [vp, i32p]
    sgc = C.POINTER(SgConfig)
    L.fs_sg_config_default.argtypes = [sgc]
    L.fs_sg_config_default.restype = None
    L.fs_sg_create.argtypes = [sgc, ip]
    L.fs_sg_create.restype = vp
    L.fs_sg_destroy.argtypes = [vp]
    L.fs_sg_destroy.restype = None
    L.fs_sg_get_config.argtypes = [vp, sgc]
    L.fs_sg_param_count.argtypes = [vp, C.POINTER(C.c_int64)]
    fp = C.POINTER(C.c_float)
    L.fs_sg_get_params.argtypes = [vp, fp]
    L.fs_sg_set_params.argtypes = [vp, fp]
    L.fs_sg_get_grads.argtypes = [vp, fp]
    L.fs_sg_save.argtypes = [vp, C.c_char_p]
    L.fs_sg_load.argtypes = [vp, C.c_char_p]
    L.fs_sg_reserve.argtypes = [vp, C.c_int]
    L.fs_sg_add_samples.argtypes = [vp, C.c_int, dp, dp, pp]
    L.fs_sg_generate.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_uint64, ip]
    L.fs_sg_set_holdout.argtypes = [vp, C.c_int]
    L.fs_sg_dataset_info.argtypes = [vp, ip, ip]
    L.fs_sg_get_sample.argtypes = [vp, C.c_int, fp, fp]
    L.fs_sg_train.argtypes = [vp, C.c_int, C.c_float, dp]
    L.fs_sg_eval.argtypes = [vp, dp]
    L.fs_sg_eval_baselines.argtypes = [vp, dp, dp]
    L.fs_sg_grad.argtypes = [vp, C.c_int, ip, dp]
    L.fs_sg_train_stats.argtypes = [vp, dp, dp]
    L.fs_sg_predict_host.argtypes = [vp, C.c_int, dp, pp, dp]
    L.fs_sg_predict_batch.argtypes = [vp, vp, C.c_int, ip, C.POINTER(C.c_void_p)]
    L.fs_sg_time_forward.argtypes = [vp, C.c_int, dp, dp]
    L.fs_sg_infer_flops.argtypes = [vp, dp]
    L.fs_sg_ensemble_defaults.argtypes = [C.POINTER(EnsembleOpts)]
    L.fs_sg_ensemble_defaults.restype = None
    L.fs_sg_compare_host.argtypes = [C.c_int, C.c_int, pp, C.c_int, dp, dp, dp, dp]
    L.fs_sg_ensemble_run.argtypes = [vp, vp, C.POINTER(EnsembleOpts), C.POINTER(EnsembleStats),
                                     ip]
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
        o, e, g, i, t = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(library().fs_launch_config(self._m, C.byref(o), C.byref(e), C.byref(g),
                                         C.byref(i)))
        check(library().fs_tma_staging(self._m, C.byref(t)))
        return {"order_blocks_per_sm": o.value, "erode_blocks_per_sm": e.value,
                "graph": bool(g.value), "erode_int_sub": bool(i.value),
                "receivers_tma": bool(t.value)}

    def use_tma_staging(self, on: bool = True) -> None:
        """The receiver filter stages its tiles by TMA instead of loads
        (even widths); identical results."""
        check(library().fs_use_tma_staging(self._m, int(bool(on))))

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
        o, e, g, i, w = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(library().fs_batch_launch_config(self._b, C.byref(o), C.byref(e), C.byref(g),
                                               C.byref(i)))
        check(library().fs_batch_walk_mode(self._b, C.byref(w)))
        t = C.c_int()
        check(library().fs_batch_tma_staging(self._b, C.byref(t)))
        return {"order_blocks_per_sm": o.value, "erode_blocks_per_sm": e.value,
                "graph": bool(g.value), "erode_int_sub": bool(i.value),
                "cta_walk": bool(w.value), "receivers_tma": bool(t.value)}

    def use_tma_staging(self, on: bool = True) -> None:
        """A single grid's receiver filter stages its tiles by TMA instead of
        loads (even widths); identical results."""
        check(library().fs_batch_use_tma_staging(self._b, int(bool(on))))

    def use_cta_walk(self, on: bool = True) -> None:
        """One CTA per realization walks its levels (block barriers only)
        instead of the grid-wide lock step; identical results."""
        check(library().fs_batch_use_cta_walk(self._b, int(bool(on))))

    def synchronize(self) -> None:
        check(library().fs_batch_synchronize(self._b))

    def set_active(self, idx=None) -> None:
        """Advance only the realizations in idx from now on (None: all)."""
        if idx is None or len(idx) == 0:
            check(library().fs_batch_set_active(self._b, 0, None))
            return
        a = (C.c_int * len(idx))(*[int(i) for i in idx])
        check(library().fs_batch_set_active(self._b, len(idx), a))

    def analyze(self) -> None:
        """Receivers, levels and accumulation of the current fields, without
        uplift or erosion (fs_batch_analyze)."""
        check(library().fs_batch_analyze(self._b))

    def device_elevation(self, r: int) -> int:
        """Device address of realization r's elevation field."""
        p = C.c_void_p()
        check(library().fs_batch_device_elevation(self._b, int(r), C.byref(p)))
        return int(p.value)

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
    gradient, x [B,H,W,cin], w = dy [B,H,W,cout] -> FP32 [cout,taps,cin];
    mode 3: mode 0 written into the middle planes of a wider tensor (the
    library checks the others stay untouched); mode 4: mode 3 stored
    upsampled 2x (nearest) -> [B,2H,2W,cout]."""
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
        f = 2 if mode == 4 else 1
        out = np.empty((B, f * H, f * W, cin if mode == 1 else cout), np.uint16)
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


class Surrogate:
    """The learned surrogate (include/fastscape_surrogate.h): a BF16
    encoder-decoder trained on the GPU on data the plain method generates,
    jumping realizations `jump` timesteps ahead."""

    def __init__(self, width=512, height=512, base_channels=32, batch=32, jump=50, dt=1000.0,
                 seed=1):
        L = library()
        self.cfg = SgConfig(int(width), int(height), int(base_channels), int(batch), int(jump),
                            float(dt), int(seed))
        st = C.c_int(0)
        self._s = L.fs_sg_create(C.byref(self.cfg), C.byref(st))
        if not self._s:
            raise FastScapeError(st.value, last_error())
        self.size = self.cfg.width * self.cfg.height

    def close(self):
        if getattr(self, "_s", None):
            library().fs_sg_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def param_count(self) -> int:
        n = C.c_int64(0)
        check(library().fs_sg_param_count(self._s, C.byref(n)))
        return n.value

    def params(self) -> np.ndarray:
        out = np.empty(self.param_count(), np.float32)
        check(library().fs_sg_get_params(self._s, _p(out, C.c_float)))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.param_count():
            raise ValueError("wrong parameter count")
        check(library().fs_sg_set_params(self._s, _p(p, C.c_float)))

    def grads(self) -> np.ndarray:
        out = np.empty(self.param_count(), np.float32)
        check(library().fs_sg_get_grads(self._s, _p(out, C.c_float)))
        return out

    def save(self, path) -> None:
        check(library().fs_sg_save(self._s, str(path).encode()))

    def load(self, path) -> None:
        check(library().fs_sg_load(self._s, str(path).encode()))

    def reserve(self, n: int) -> None:
        check(library().fs_sg_reserve(self._s, int(n)))

    def add_samples(self, h_t, h_next, params) -> None:
        h_t = np.ascontiguousarray(h_t, np.float64).reshape(-1, self.size)
        h_next = np.ascontiguousarray(h_next, np.float64).reshape(-1, self.size)
        n = h_t.shape[0]
        pa = (Params * n)(*params)
        check(library().fs_sg_add_samples(self._s, n, _p(h_t, C.c_double),
                                          _p(h_next, C.c_double), pa))

    def generate(self, ntraj: int, per_traj: int, max_spinup: int, seed: int = 0) -> int:
        got = C.c_int(0)
        check(library().fs_sg_generate(self._s, int(ntraj), int(per_traj), int(max_spinup),
                                       int(seed) & 0xFFFFFFFFFFFFFFFF, C.byref(got)))
        return got.value

    def set_holdout(self, n: int) -> None:
        check(library().fs_sg_set_holdout(self._s, int(n)))

    def dataset_info(self):
        n, h = C.c_int(0), C.c_int(0)
        check(library().fs_sg_dataset_info(self._s, C.byref(n), C.byref(h)))
        return n.value, h.value

    def sample(self, k: int):
        h = np.empty(self.size, np.float32)
        y = np.empty(self.size, np.float32)
        check(library().fs_sg_get_sample(self._s, int(k), _p(h, C.c_float), _p(y, C.c_float)))
        return h, y

    def train(self, steps: int, lr: float = 1e-3) -> float:
        loss = C.c_double(0)
        check(library().fs_sg_train(self._s, int(steps), float(lr), C.byref(loss)))
        return loss.value

    def eval(self) -> float:
        loss = C.c_double(0)
        check(library().fs_sg_eval(self._s, C.byref(loss)))
        return loss.value

    def eval_baselines(self):
        """(uplift-only loss, no-change loss) over the held-out split."""
        a, b = C.c_double(0), C.c_double(0)
        check(library().fs_sg_eval_baselines(self._s, C.byref(a), C.byref(b)))
        return a.value, b.value

    def grad(self, idx) -> float:
        a = (C.c_int * len(idx))(*[int(i) for i in idx])
        loss = C.c_double(0)
        check(library().fs_sg_grad(self._s, len(idx), a, C.byref(loss)))
        return loss.value

    def train_stats(self):
        ms, fl = C.c_double(0), C.c_double(0)
        check(library().fs_sg_train_stats(self._s, C.byref(ms), C.byref(fl)))
        return ms.value, fl.value

    def time_forward(self, reps: int = 5):
        """(ms per forward pass over a full batch, conv FLOPs of that pass)."""
        ms, fl = C.c_double(0), C.c_double(0)
        check(library().fs_sg_time_forward(self._s, int(reps), C.byref(ms), C.byref(fl)))
        return ms.value, fl.value

    def infer_flops(self) -> float:
        f = C.c_double(0)
        check(library().fs_sg_infer_flops(self._s, C.byref(f)))
        return f.value

    def predict(self, h, params) -> np.ndarray:
        h = np.ascontiguousarray(h, np.float64).reshape(-1, self.size)
        n = h.shape[0]
        out = np.empty_like(h)
        pa = (Params * n)(*params)
        check(library().fs_sg_predict_host(self._s, n, _p(h, C.c_double), pa,
                                           _p(out, C.c_double)))
        return out

    def predict_batch(self, batch: "FastScapeBatch", idx) -> None:
        a = (C.c_int * len(idx))(*[int(i) for i in idx])
        check(library().fs_sg_predict_batch(self._s, batch.handle, len(idx), a, None))

    def ensemble(self, batch: "FastScapeBatch", nsteps: int, judge_fraction: float = 0.05,
                 max_rel_rms: float = 0.01, min_agreement: float = 0.99, plain_steps: int = 1,
                 seed: int = 2019):
        """Judged surrogate-accelerated run of every realization of `batch`
        (fs_sg_ensemble_run); returns (stats dict, fallen flags)."""
        o = EnsembleOpts()
        library().fs_sg_ensemble_defaults(C.byref(o))
        o.nsteps, o.plain_steps = int(nsteps), int(plain_steps)
        o.judge_fraction, o.max_rel_rms = float(judge_fraction), float(max_rel_rms)
        o.min_agreement, o.seed = float(min_agreement), int(seed)
        st = EnsembleStats()
        fallen = (C.c_int * batch.n)()
        check(library().fs_sg_ensemble_run(batch.handle, self._s, C.byref(o), C.byref(st),
                                           fallen))
        return st.as_dict(), np.array(fallen[:], dtype=np.int32)


def compare_fields(width: int, height: int, params, a, b):
    """The ensemble judge's measures for host field pairs: (relief-normalised
    RMS error, receiver agreement) per pair (fs_sg_compare_host)."""
    a = np.ascontiguousarray(a, np.float64).reshape(-1, width * height)
    b = np.ascontiguousarray(b, np.float64).reshape(-1, width * height)
    n = a.shape[0]
    rel = np.empty(n, np.float64)
    ag = np.empty(n, np.float64)
    pa = (Params * n)(*params)
    check(library().fs_sg_compare_host(width, height, pa, n, _p(a, C.c_double),
                                       _p(b, C.c_double), _p(rel, C.c_double),
                                       _p(ag, C.c_double)))
    return rel, ag
