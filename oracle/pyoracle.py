"""ctypes bindings for the oracle (test infrastructure only).

``Oracle`` wraps ``oracle/_build/libfsoracle.so`` (the C restatement).
``RefHarness`` wraps ``oracle/_ref/libfsref_*.so`` (the reference's own
classes, built here from its sources by ``oracle/build.py``); it exists only
where the reference tree was available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

SQRT2 = 1.414213562373095048801688724209698078569671875376948


class FsoParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("keq", "neq", "meq", "ueq", "dt", "dr_orth", "dr_diag", "tol", "cell_area")]


@dataclass(frozen=True)
class Params:
    """Physical constants of one realization (fastscape_RB.cpp:58-65)."""
    keq: float = 2e-6
    neq: float = 2.0
    meq: float = 0.8
    ueq: float = 2e-3
    dt: float = 1000.0
    dr_orth: float = 1.0
    dr_diag: float = SQRT2
    tol: float = 1e-3
    cell_area: float = 40000.0

    def as_tuple(self):
        return (self.keq, self.neq, self.meq, self.ueq, self.dt,
                self.dr_orth, self.dr_diag, self.tol, self.cell_area)

    def c(self) -> FsoParams:
        return FsoParams(*self.as_tuple())


# The constants hard-coded in the reference (fastscape_RB.cpp:58-65).
REFERENCE_PARAMS = Params()


def workload_params(dx: float = 100.0, keq: float = 2e-6, meq: float = 0.4,
                    ueq: float = 2e-3, neq: float = 1.0) -> Params:
    """The 1000^2 / 10000^2 workload: K 2e-6, m 0.4, n 1, U 2e-3, dt 1000,
    dx = dy = 100 m (diagonal dx*SQRT2), cell area dx*dx."""
    return Params(keq=keq, neq=neq, meq=meq, ueq=ueq, dt=1000.0, dr_orth=dx,
                  dr_diag=dx * SQRT2, tol=1e-3, cell_area=dx * dx)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    def __init__(self, path: Path | None = None):
        if path is None:
            from oracle.build import build_oracle  # noqa: WPS433
            path = build_oracle()
        self.lib = L = C.CDLL(str(path))
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        pp = C.POINTER(FsoParams)
        L.fso_terrain_mt19937.argtypes = [dp, C.c_int, C.c_int, C.c_uint32]
        L.fso_mt19937_stream.argtypes = [C.c_uint32, C.POINTER(C.c_uint32), C.c_int]
        L.fso_receivers.argtypes = [dp, C.c_int, C.c_int, pp, ip]
        L.fso_donors.argtypes = [ip, C.c_int, C.c_int, ip, ip]
        L.fso_order.argtypes = [ip, ip, ip, C.c_int, C.c_int, ip, ip]
        L.fso_order.restype = C.c_int
        L.fso_flowacc.argtypes = [ip, ip, C.c_int, C.c_int, pp, dp]
        L.fso_uplift.argtypes = [dp, C.c_int, C.c_int, pp]
        L.fso_erode.argtypes = [dp, ip, ip, dp, C.c_int, C.c_int, pp]
        L.fso_erode_levels.argtypes = [dp, ip, ip, ip, C.c_int, dp, C.c_int, C.c_int, pp]
        L.fso_run.argtypes = [dp, C.c_int, C.c_int, pp, C.c_int, C.c_int]
        L.fso_level_ids.argtypes = [ip, ip, C.c_int, C.c_int, C.c_int, ip]
        L.fso_order_bw.argtypes = [ip, ip, ip, C.c_int, C.c_int, ip, ip]
        L.fso_order_bw.restype = C.c_int
        L.fso_omp_threads.restype = C.c_int

    # -- primitives -------------------------------------------------------
    def terrain(self, W: int, H: int, engine_seed: int = 0) -> np.ndarray:
        h = np.empty(W * H, np.float64)
        self.lib.fso_terrain_mt19937(_ptr(h, C.c_double), W, H, engine_seed)
        return h

    def mt_stream(self, seed: int, n: int) -> np.ndarray:
        out = np.empty(n, np.uint32)
        self.lib.fso_mt19937_stream(seed, _ptr(out, C.c_uint32), n)
        return out

    def phases(self, h: np.ndarray, W: int, H: int, p: Params, parallel=False):
        """One timestep; returns dict of every intermediate (h updated)."""
        size = W * H
        pc = p.c()
        rec = np.empty(size, np.int32)
        ndon = np.empty(size, np.int32)
        donor = np.zeros(8 * size, np.int32)
        stack = np.empty(size, np.int32)
        levels = np.empty(size + 2, np.int32)
        accum = np.empty(size, np.float64)
        L = self.lib
        ip = C.c_int32
        L.fso_receivers(_ptr(h, C.c_double), W, H, C.byref(pc), _ptr(rec, ip))
        L.fso_donors(_ptr(rec, ip), W, H, _ptr(ndon, ip), _ptr(donor, ip))
        nlevel = L.fso_order(_ptr(rec, ip), _ptr(ndon, ip), _ptr(donor, ip), W, H,
                             _ptr(stack, ip), _ptr(levels, ip))
        L.fso_flowacc(_ptr(rec, ip), _ptr(stack, ip), W, H, C.byref(pc),
                      _ptr(accum, C.c_double))
        h_upl = h.copy()
        L.fso_uplift(_ptr(h, C.c_double), W, H, C.byref(pc))
        h_upl = h.copy()
        if parallel:
            L.fso_erode_levels(_ptr(h, C.c_double), _ptr(rec, ip), _ptr(stack, ip),
                               _ptr(levels, ip), nlevel, _ptr(accum, C.c_double),
                               W, H, C.byref(pc))
        else:
            L.fso_erode(_ptr(h, C.c_double), _ptr(rec, ip), _ptr(stack, ip),
                        _ptr(accum, C.c_double), W, H, C.byref(pc))
        level_id = np.empty(size, np.int32)
        L.fso_level_ids(_ptr(stack, ip), _ptr(levels, ip), nlevel, W, H,
                        _ptr(level_id, ip))
        return dict(rec=rec, ndon=ndon, donor=donor.reshape(size, 8), stack=stack,
                    levels=levels[:nlevel].copy(), nlevel=nlevel, accum=accum,
                    h_uplifted=h_upl, h=h, level_id=level_id)

    def order_bw(self, rec: np.ndarray, W: int, H: int):
        """Braun-Willett DFS stack and root starts from receiver codes
        (fastscape_BW.cpp:201-221)."""
        size = W * H
        ip = C.c_int32
        rec = np.ascontiguousarray(rec, np.int32)
        ndon = np.empty(size, np.int32)
        donor = np.zeros(8 * size, np.int32)
        self.lib.fso_donors(_ptr(rec, ip), W, H, _ptr(ndon, ip), _ptr(donor, ip))
        stack = np.empty(size, np.int32)
        starts = np.empty(size + 1, np.int32)
        n = self.lib.fso_order_bw(_ptr(rec, ip), _ptr(ndon, ip), _ptr(donor, ip), W, H,
                                  _ptr(stack, ip), _ptr(starts, ip))
        return stack, starts[:n + 1].copy()

    def run(self, h: np.ndarray, W: int, H: int, p: Params, nstep: int,
            parallel=False) -> np.ndarray:
        """fastscape_RB::run semantics: nstep+1 timesteps, in place."""
        pc = p.c()
        self.lib.fso_run(_ptr(h, C.c_double), W, H, C.byref(pc), nstep, int(parallel))
        return h

    def steps(self, h: np.ndarray, W: int, H: int, p: Params, k: int,
              parallel=False) -> np.ndarray:
        """Exactly k timesteps, in place."""
        if k <= 0:
            return h
        return self.run(h, W, H, p, k - 1, parallel)

    def threads(self) -> int:
        return self.lib.fso_omp_threads()


def donor_mask_from_rec(rec: np.ndarray, W: int, H: int) -> np.ndarray:
    """8-bit donor mask: bit k of cell c is set when neighbour c+nshift[k]
    drains into c (its receiver code is (k+4)%8). Pure numpy, for tests."""
    r = rec.reshape(H, W)
    mask = np.zeros((H, W), np.uint8)
    offs = [(0, -1), (-1, -1), (-1, 0), (-1, 1), (0, 1), (1, 1), (1, 0), (1, -1)]
    for k, (dy, dx) in enumerate(offs):
        src = np.full((H, W), -2, np.int32)
        ys0, ys1 = max(0, -dy), H - max(0, dy)
        xs0, xs1 = max(0, -dx), W - max(0, dx)
        src[ys0:ys1, xs0:xs1] = r[ys0 + dy:ys1 + dy, xs0 + dx:xs1 + dx]
        mask |= ((src == (k + 4) % 8).astype(np.uint8) << k)
    return mask.reshape(-1)


class RefHarness:
    """The reference's own FastScape_RB (variant 0) / FastScape_RBP (1)."""

    def __init__(self, text: str = "param", flags: str = "exact"):
        path = HERE / "_ref" / f"libfsref_{text}_{flags}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        self.text = text
        self.lib = L = C.CDLL(str(path))
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.fsref_create.argtypes = [C.c_int, C.c_int, C.c_int]
        L.fsref_create.restype = vp
        L.fsref_destroy.argtypes = [C.c_int, vp]
        L.fsref_seed.argtypes = [C.c_ulong]
        L.fsref_set_params.argtypes = [dp]
        L.fsref_constants.argtypes = [C.c_int, vp, dp]
        for n in ("fsref_get_h", "fsref_set_h", "fsref_get_accum"):
            getattr(L, n).argtypes = [C.c_int, vp, dp]
        for n in ("fsref_get_rec", "fsref_get_ndon", "fsref_get_donor", "fsref_get_stack"):
            getattr(L, n).argtypes = [C.c_int, vp, ip]
        L.fsref_get_levels.argtypes = [C.c_int, vp, ip, C.c_int]
        L.fsref_prepare.argtypes = [C.c_int, vp]
        L.fsref_phase.argtypes = [C.c_int, vp, C.c_int]
        L.fsref_step.argtypes = [C.c_int, vp]
        L.fsref_nlevel.argtypes = [C.c_int, vp]
        L.fsref_nlevel.restype = C.c_int
        L.fsref_run.argtypes = [C.c_int, vp, C.c_int]
        L.fsref_print_dem.argtypes = [C.c_int, vp, C.c_char_p]

    def set_params(self, p: Params):
        if self.text != "param":
            if p != REFERENCE_PARAMS:
                raise ValueError("pristine reference build only has its own constants")
            return
        arr = np.array(p.as_tuple(), np.float64)
        self.lib.fsref_set_params(_ptr(arr, C.c_double))

    def model(self, W: int, H: int, p: Params, variant: int = 0, seed: int = 123):
        return RefModel(self, W, H, p, variant, seed)


class RefModel:
    def __init__(self, hr: RefHarness, W, H, p, variant, seed):
        self.hr, self.W, self.H, self.v = hr, W, H, variant
        hr.set_params(p)
        hr.lib.fsref_seed(seed)
        self.obj = hr.lib.fsref_create(variant, W, H)
        self.size = W * H

    def __del__(self):
        try:
            self.hr.lib.fsref_destroy(self.v, self.obj)
        except Exception:
            pass

    def constants(self):
        out = np.empty(9, np.float64)
        self.hr.lib.fsref_constants(self.v, self.obj, _ptr(out, C.c_double))
        return out

    def get_h(self):
        out = np.empty(self.size, np.float64)
        self.hr.lib.fsref_get_h(self.v, self.obj, _ptr(out, C.c_double))
        return out

    def set_h(self, h):
        h = np.ascontiguousarray(h, np.float64)
        self.hr.lib.fsref_set_h(self.v, self.obj, _ptr(h, C.c_double))

    def prepare(self):
        self.hr.lib.fsref_prepare(self.v, self.obj)

    def phase(self, i):
        self.hr.lib.fsref_phase(self.v, self.obj, i)

    def step(self):
        self.hr.lib.fsref_step(self.v, self.obj)

    def run(self, nstep):
        self.hr.lib.fsref_run(self.v, self.obj, nstep)

    def print_dem(self, path):
        """The reference's PrintDEM of the current elevation."""
        self.hr.lib.fsref_print_dem(self.v, self.obj, str(path).encode())

    def get(self, name):
        L, ip = self.hr.lib, C.c_int32
        if name == "accum":
            out = np.empty(self.size, np.float64)
            L.fsref_get_accum(self.v, self.obj, _ptr(out, C.c_double))
            return out
        if name == "donor":
            out = np.empty(8 * self.size, np.int32)
            L.fsref_get_donor(self.v, self.obj, _ptr(out, ip))
            return out.reshape(self.size, 8)
        if name == "levels":
            n = L.fsref_nlevel(self.v, self.obj)
            out = np.empty(n, np.int32)
            L.fsref_get_levels(self.v, self.obj, _ptr(out, ip), n)
            return out
        if name == "nlevel":
            return L.fsref_nlevel(self.v, self.obj)
        out = np.empty(self.size, np.int32)
        getattr(L, f"fsref_get_{name}")(self.v, self.obj, _ptr(out, ip))
        return out

    def bw_phases(self):
        """One timestep of the Braun-Willett variant (variant 2); returns
        receivers, its DFS stack and the eroded h."""
        self.prepare()
        for i in range(6):
            self.phase(i)
        return dict(rec=self.get("rec"), stack=self.get("stack"), h=self.get_h())

    def phases(self):
        """One timestep; returns the intermediates like Oracle.phases."""
        self.prepare()
        self.phase(0); self.phase(1); self.phase(2); self.phase(3)
        self.phase(4)
        h_upl = self.get_h()
        self.phase(5)
        return dict(rec=self.get("rec"), ndon=self.get("ndon"), donor=self.get("donor"),
                    stack=self.get("stack"), levels=self.get("levels"),
                    nlevel=self.get("nlevel"), accum=self.get("accum"),
                    h_uplifted=h_upl, h=self.get_h())


def level_ids(stack, levels, size):
    lid = np.full(size, -1, np.int32)
    for li in range(len(levels) - 1):
        lid[stack[levels[li]:levels[li + 1]]] = li
    return lid


def is_close_rel(a, b, rtol):
    a = np.asarray(a); b = np.asarray(b)
    denom = np.maximum(np.abs(b), np.finfo(np.float64).tiny)
    return np.abs(a - b) <= rtol * denom


__all__ = ["Oracle", "RefHarness", "Params", "REFERENCE_PARAMS", "workload_params",
           "donor_mask_from_rec", "level_ids", "SQRT2", "math"]
