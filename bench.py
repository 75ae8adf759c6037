"""Benchmark: FastScape timestep on a 10000x10000 FP64 grid, one GB300.

Workload (the reference's 10000^2 configuration): the reference's initial
field (uniform [0,1) m, rings 0 and 1 at 0 m), K 2e-6, m 0.4, n 1,
U 2e-3 m/yr, dt 1000 yr, dx = dy = 100 m. A bench "step" is one FastScape
timestep over the whole grid (1e8 cell-steps): receivers, donors, level
ordering, accumulation, uplift, erosion.

  value      cell-steps/s with the field resident in HBM, timed with CUDA
             events on the model's stream (K timesteps after W warm-up
             timesteps). h (800 MB) is larger than L2, so no flush is needed.
  e2e        the same metric through the reference-facing call sequence with
             host buffers: fs_set_elevation (pinned host -> device), fs_run(20)
             (21 timesteps, the reference's run semantics) and
             fs_get_elevation (device -> pinned host), all inside the timed
             region (host clock; the median of --e2e-calls calls after one
             warm-up call).
  roofline   the dominant kernel's algorithmic bytes per launch / its mean
             launch time (CUDA events), against the measured HBM copy peak.
  cpu_baseline  the oracle's fastscape_RB+P restatement (OpenMP on every host
             core) on a bounded sample of the same workload, rank 0 only.

--impl reference times the reference's CPU implementation of the timestep:
the reference's own FastScape_RBP compiled from its sources (oracle/_ref)
where that build exists, else the oracle's restatement of it.

The default run's line also carries `ensemble_ragged` (the 256-member
ragged ensemble, 200 timesteps) and `surrogate` (the learned surrogate's
training throughput at 512^2, batch 32, and the judged surrogate ensemble
against the plain batched method, 1024 x 512^2, 2000 timesteps, with the
committed parameters), each with its own clocks; --no-extras drops them.
Other workloads (--workload): ensemble, sweep, deep, refconst, surrogate
(generation, training and the judged ensemble), conv (the surrogate's
convolutions alone).

Multi-GPU (torchrun): one independent replica per rank ("replicas only": a
single grid does not shard); value = all ranks' cell-steps / max time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-steps/s at 10000^2 FP64"
UNIT = "cell-steps/s"
SIDE = 10000
RUN_NSTEP = 20            # run(20) executes 21 timesteps
# Algorithmic bytes per cell for each kernel in this layout (h f64, rec i8,
# mask u8, stack i32, cnt u32): each array the kernel must touch, once.
ALG_BYTES = {
    "receivers": 8 + 1,                     # h read, rec write
    "donors_level0": 1 + 1,                 # rec read, mask write (+ pit list)
    "order": 4 + 1 + 4 + 1 + 4 + 4,
    # k_order: entry read, mask read, entry + direction + receiver-position
    # write, unit count write
    "accum": 4 + 4 + 4,
    # k_accum: own count and receiver position read, reduction into the
    # receiver's count
    "erode": 4 + 1 + 4 + 8 + 8,
    # k_erode: entry, direction, count, h read, h write
}
# k_erode leans on the FP64 pipe: per eroded cell fact*dh and the
# division's one multiplication (its residual and rounding run in integer
# arithmetic), plus h0 - hn and h0 - q unless those run in integer
# arithmetic too (the autotuner's erode_int_sub); the uplift always runs in
# integer arithmetic. Peak measured here with a probe kernel: 1.59 FP64
# lanes/clock/SM x 152 SMs x 2.07 GHz.
def erode_fp64_per_cell(int_sub: bool) -> int:
    return 2 if int_sub else 4


FP64_PEAK_TFLOPS = 1.59 * 152 * 2.07e9 / 1e12
STEP_ALG_BYTES = 79        # compulsory streaming bytes per cell-step with int32 receivers


def grid_config(side: int) -> dict:
    """The workload description both arms print (identical dictionaries)."""
    return {"workload": f"FastScape timestep, {side}x{side} FP64, reference initial field, "
                        "K 2e-6 m 0.4 n 1 U 2e-3 dt 1000 dx 100",
            "grid": [side, side], "step": "one timestep over the whole grid",
            "l2": "inputs larger than L2 (h is 800 MB at 10000^2)"}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"fs_bench_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            self.proc.wait()
            self.f.close()
            self._text = self.path.read_text() if self.path.exists() else ""
            try:
                self.path.unlink()
            except OSError:
                pass

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "_text", "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        loaded = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return dist, rank, ws, local


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def pinned_buffer(n: int):
    """n float64 in page-locked host memory (torch is used only to pin)."""
    import torch
    t = torch.empty(n, dtype=torch.float64, pin_memory=True)
    return t, t.numpy()


def cpu_sample(side: int, nsteps: int, prefer_reference: bool):
    """Times the CPU implementation of the timestep on a side^2 grid.
    Returns (cell-steps/s, kind, threads, description)."""
    import ctypes

    from oracle.pyoracle import Oracle, workload_params
    p = workload_params()
    if prefer_reference:
        path = ROOT / "oracle" / "_ref" / "libfsref_param_shipped.so"
        if path.exists():
            try:
                from oracle.pyoracle import RefHarness
                hr = RefHarness("param", "shipped")
                m = hr.model(side, side, p, 1)
                m.prepare()
                m.step()                       # warm-up timestep
                t0 = time.perf_counter()
                for _ in range(nsteps):
                    m.step()
                dt = time.perf_counter() - t0
                thr = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
                return (side * side * nsteps / dt, "reference", thr,
                        f"reference FastScape_RBP (oracle/_ref, -O3 -march=native), "
                        f"{side}^2, {nsteps} timesteps after 1 warm-up")
            except OSError:
                pass
    o = Oracle()
    h = o.terrain(side, side, 0)
    lib = o.lib
    from oracle.pyoracle import FsoParams

    class Work(ctypes.Structure):
        _fields_ = [("W", ctypes.c_int), ("H", ctypes.c_int)] + \
                   [(n, ctypes.c_void_p) for n in ("rec", "ndon", "donor", "stack", "levels", "accum")] + \
                   [("nlevel", ctypes.c_int)]
    lib.fso_work_init.argtypes = [ctypes.POINTER(Work), ctypes.c_int, ctypes.c_int]
    lib.fso_work_free.argtypes = [ctypes.POINTER(Work)]
    lib.fso_step.argtypes = [ctypes.POINTER(Work), ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(FsoParams), ctypes.c_int,
                             ctypes.POINTER(ctypes.c_double)]
    w = Work()
    if lib.fso_work_init(ctypes.byref(w), side, side) != 0:
        raise MemoryError("oracle work arrays")
    pc = p.c()
    hp = h.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    lib.fso_step(ctypes.byref(w), hp, ctypes.byref(pc), 1, None)   # warm-up
    t0 = time.perf_counter()
    for _ in range(nsteps):
        lib.fso_step(ctypes.byref(w), hp, ctypes.byref(pc), 1, None)
    dt = time.perf_counter() - t0
    lib.fso_work_free(ctypes.byref(w))
    return (side * side * nsteps / dt, "port", o.threads(),
            f"oracle restatement of fastscape_RB+P (level-parallel erosion, OpenMP), "
            f"{side}^2, {nsteps} timesteps after 1 warm-up")


def cpu_steps_from(h: np.ndarray, side: int, params, nsteps: int):
    """Times the oracle's restatement of fastscape_RB+P for nsteps timesteps
    from the elevation h (copied) with the given oracle Params. Returns
    (cell-steps/s, threads)."""
    import ctypes

    from oracle.pyoracle import FsoParams, Oracle
    o = Oracle()
    lib = o.lib

    class Work(ctypes.Structure):
        _fields_ = [("W", ctypes.c_int), ("H", ctypes.c_int)] + \
                   [(n, ctypes.c_void_p) for n in ("rec", "ndon", "donor", "stack", "levels", "accum")] + \
                   [("nlevel", ctypes.c_int)]
    lib.fso_work_init.argtypes = [ctypes.POINTER(Work), ctypes.c_int, ctypes.c_int]
    lib.fso_work_free.argtypes = [ctypes.POINTER(Work)]
    lib.fso_step.argtypes = [ctypes.POINTER(Work), ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(FsoParams), ctypes.c_int,
                             ctypes.POINTER(ctypes.c_double)]
    w = Work()
    if lib.fso_work_init(ctypes.byref(w), side, side) != 0:
        raise MemoryError("oracle work arrays")
    hh = np.array(h, dtype=np.float64, copy=True)
    pc = params.c()
    hp = hh.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    lib.fso_step(ctypes.byref(w), hp, ctypes.byref(pc), 1, None)   # warm-up
    t0 = time.perf_counter()
    for _ in range(nsteps):
        lib.fso_step(ctypes.byref(w), hp, ctypes.byref(pc), 1, None)
    dt = time.perf_counter() - t0
    lib.fso_work_free(ctypes.byref(w))
    return side * side * nsteps / dt, o.threads()


def run_reference_arm(args, dist, rank, ws):
    if rank != 0:
        return
    side = args.side
    t_all = []
    # one bounded CPU timestep per bench step
    import ctypes
    from oracle.pyoracle import workload_params
    p = workload_params()
    kind, desc, thr = None, None, None
    path = ROOT / "oracle" / "_ref" / "libfsref_param_shipped.so"
    stepper = None
    if path.exists():
        try:
            from oracle.pyoracle import RefHarness
            hr = RefHarness("param", "shipped")
            m = hr.model(side, side, p, 1)
            m.prepare()
            stepper = m.step
            kind = "reference"
            thr = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
            desc = f"reference FastScape_RBP compiled from its sources (-O3 -march=native), {side}^2"
        except OSError:
            stepper = None
    if stepper is None:
        from oracle.pyoracle import FsoParams, Oracle
        o = Oracle()
        h = o.terrain(side, side, 0)

        class Work(ctypes.Structure):
            _fields_ = [("W", ctypes.c_int), ("H", ctypes.c_int)] + \
                       [(n, ctypes.c_void_p) for n in ("rec", "ndon", "donor", "stack", "levels", "accum")] + \
                       [("nlevel", ctypes.c_int)]
        lib = o.lib
        lib.fso_work_init.argtypes = [ctypes.POINTER(Work), ctypes.c_int, ctypes.c_int]
        lib.fso_step.argtypes = [ctypes.POINTER(Work), ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(FsoParams), ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double)]
        w = Work()
        lib.fso_work_init(ctypes.byref(w), side, side)
        pc = p.c()
        hp = h.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        stepper = lambda: lib.fso_step(ctypes.byref(w), hp, ctypes.byref(pc), 1, None)  # noqa: E731
        kind = "port"
        thr = o.threads()
        desc = f"oracle restatement of fastscape_RB+P (OpenMP), {side}^2"
    for _ in range(args.warmup):
        stepper()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        stepper()
        t_all.append(time.perf_counter() - t0)
    tot = sum(t_all)
    value = side * side * args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": grid_config(side), "parallelism": "host cores",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": thr, "kind": kind,
                         "sample": f"{desc}, {args.steps} timesteps after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


ENSEMBLE_STEPS = 200      # timesteps of one ensemble run


def ensemble_spec(pkg, n: int, seed: int = 2019, side: int = 0):
    """The ragged ensemble: square sides log-uniform in [256, 2048], K
    log-uniform in [1e-6, 1e-5], m uniform in [0.3, 0.6], U log-uniform in
    [1e-4, 5e-3] m/yr, n 1, dt 1000 yr, dx 100 m, seeded. With `side` > 0
    every realization is side x side (the parameters are drawn the same
    way)."""
    rng = np.random.default_rng(seed)
    sides = np.exp(rng.uniform(np.log(256), np.log(2048), n)).astype(int)
    if side > 0:
        sides = np.full(n, side)
    params = [pkg.workload_params(keq=float(10 ** rng.uniform(-6, -5)),
                                  meq=float(rng.uniform(0.3, 0.6)),
                                  ueq=float(10 ** rng.uniform(-4, np.log10(5e-3))))
              for _ in range(n)]
    return [int(s) for s in sides], params


def ensemble_result(pkg, n, side, nsteps, seed, rank, ws, dist, local, walk="auto",
                    int_sub="auto"):
    """Batched ensemble: realizations/s of nsteps-timestep runs from the
    initial fields (the launch shape the autotuner picks, CUDA events around
    the whole run on the batch's stream), then the same run once more from
    the same initial fields with an event between kernels for the split."""
    sides, params = ensemble_spec(pkg, n, seed=seed, side=side)
    seeds = list(range(1000 * rank, 1000 * rank + len(sides)))
    b = pkg.FastScapeBatch(sides, sides, params, init=pkg.INIT_PHILOX, seeds=seeds)
    cells = b.cells()
    # warm-up: the autotuner's probe timesteps (9 launch configurations x 3),
    # after which it restores the initial fields
    tune = b.autotune(probe_steps=2)
    if walk != "auto":
        b.use_cta_walk(walk == "cta")
    if int_sub != "auto":
        b.use_int_sub(int_sub == "1")
    tune = b.launch_config()
    b.set_timing(pkg.TIMING_CALL)
    b.phase_times(reset=True)
    b.synchronize()
    barrier(dist)
    with Clocks(local) as clk:
        b.step(nsteps)                       # the whole run from the initial fields
    barrier(dist)
    dt = max_over_ranks(dist, float(b.phase_times(reset=True)[3]) * 1e-3)
    levels = max(b.levels(r)[1] for r in range(len(sides)))
    b.close()
    b = pkg.FastScapeBatch(sides, sides, params, init=pkg.INIT_PHILOX, seeds=seeds)
    b.use_cta_walk(tune.get("cta_walk", False))
    b.use_int_sub(tune.get("erode_int_sub", False))
    b.set_timing(pkg.TIMING_KERNELS)
    b.phase_times(reset=True)
    b.step(nsteps)
    t = b.phase_times(reset=True) / nsteps
    b.close()
    per_step = dt / nsteps
    shape = "equal-size" if side > 0 else "ragged"
    side_desc = f"{side}" if side > 0 else "log-U[256,2048]"
    peak, peak_kind = load_peaks()
    kern = {"receivers": t[0], "donors_level0": t[1], "order": t[7], "accum": t[9],
            "erode": t[8]}
    dom = max(("order", "accum", "erode"), key=kern.get)
    achieved = ALG_BYTES[dom] * cells / (kern[dom] * 1e-3) / 1e9
    return {
        "metric": f"ensemble realizations/s ({nsteps}-timestep runs)",
        "value": ws * len(sides) / (nsteps * per_step),
        "unit": "realizations/s", "n_gpus": ws, "steps": nsteps, "warmup": 9 * 3,
        "ms_per_step": 1e3 * per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{shape} ensemble of {len(sides)} realizations, sides "
                               f"{side_desc}, K log-U[1e-6,1e-5], m U[0.3,0.6], "
                               "U log-U[1e-4,5e-3], n 1, dt 1000, dx 100",
                   "cells_per_step": cells, "cell_steps_per_s": cells / per_step,
                   "launch": tune, "l2": "inputs larger than L2",
                   "timed": f"the whole {nsteps}-timestep run from the initial fields "
                            "(launch path of the autotuner's choice)",
                   "kernel_split": "a second run from the same fields, direct launches "
                                   "with events between kernels",
                   "levels_at_end": levels},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "alg_bytes_per_cell": ALG_BYTES[dom],
                     "peak_source": f"{peak_kind} hbm_gbs", "kernel_ms": kern},
        "gpu_launches": 6 * nsteps,
        "clocks": clk.summary(),
    }


def run_ensemble(args, dist, rank, ws, local):
    """Batched ragged ensemble: realizations/s of 200-timestep runs, one
    batched launch sequence per timestep (autotuned). The timed region is the
    whole run from the initial fields, so deepening level structures count."""
    import __graft_entry__ as ge
    import torch  # noqa: F401
    pkg = ge.load()
    if ws > 1:
        torch.cuda.set_device(local)
    res = ensemble_result(pkg, args.realizations, args.ensemble_side, args.ensemble_steps,
                          2019 + rank, rank, ws, dist, local, walk=args.walk,
                          int_sub=args.int_sub)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


SG_WEIGHTS = ROOT / "barnes2019-landscape_gb300" / "weights" / "surrogate_512_c32_j50.bin"


def load_bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["bf16_tflops"]), float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), \
            "measured"
    return 1900.0, 1700.0, "fallback"


def surrogate_ensemble(pkg, net, n, side, nsteps, judge, seed, clk_index):
    """The judged surrogate ensemble and the plain batched method on the
    same n realizations (parameters and initial fields as the ragged
    ensemble's, all side x side); returns a dict of both."""
    import torch  # noqa: F401
    sides, params = ensemble_spec(pkg, n, seed=seed, side=side)
    seeds = list(range(5000, 5000 + n))
    out = {}
    # plain batched method (the yardstick), its launch shape autotuned
    plain = pkg.FastScapeBatch(sides, sides, params, init=pkg.INIT_PHILOX, seeds=seeds)
    tune = plain.autotune(probe_steps=2)
    plain.synchronize()
    with Clocks(clk_index) as clk:
        t0 = time.perf_counter()
        plain.step(nsteps)
        plain.synchronize()
        t_plain = time.perf_counter() - t0
    out["plain"] = {"seconds": t_plain, "realizations_per_s": n / t_plain, "launch": tune,
                    "levels_at_end": max(plain.levels(r)[1] for r in range(n)),
                    "clocks": clk.summary()}
    h_plain = [plain.getH(r) for r in range(min(n, 16))]
    plain.close()
    b = pkg.FastScapeBatch(sides, sides, params, init=pkg.INIT_PHILOX, seeds=seeds)
    b.autotune(probe_steps=2)
    b.use_graph(False)
    b.synchronize()
    with Clocks(clk_index) as clk:
        t0 = time.perf_counter()
        stats, fallen = net.ensemble(b, nsteps, judge_fraction=judge, seed=seed)
        b.synchronize()
        t_sg = time.perf_counter() - t0
    # end state against the plain run (realizations that never fell back
    # carry the surrogate's errors; the others are exact from their fallback)
    rel = []
    for r in range(len(h_plain)):
        h = b.getH(r)
        relief = h_plain[r].max() - h_plain[r].min()
        rel.append(float(np.sqrt(np.mean((h - h_plain[r]) ** 2)) / relief))
    b.close()
    out["surrogate"] = {"seconds": t_sg, "realizations_per_s": n / t_sg, "stats": stats,
                        "fallen": int(np.sum(fallen)),
                        "end_rel_rms_vs_plain_first16": {"mean": float(np.mean(rel)),
                                                         "max": float(np.max(rel))},
                        "clocks": clk.summary()}
    out["ratio"] = out["surrogate"]["realizations_per_s"] / out["plain"]["realizations_per_s"]
    return out


def run_surrogate(args, dist, rank, ws, local):
    """Configs 3 and 4: the surrogate trained on data the plain method
    generates on the device (config 3: --sg-traj x --sg-per samples of
    512^2 spun up 0..--sg-spinup timesteps, --sg-train-steps Adam steps at
    batch 32), then the judged surrogate ensemble (config 4: --realizations
    x 512^2, --ensemble-steps timesteps, --sg-judge of the jumps re-run
    exactly) against the plain batched method on the same realizations.
    --sg-load skips generation and training and uses saved parameters."""
    import __graft_entry__ as ge
    import torch  # noqa: F401
    pkg = ge.load()
    if ws > 1:
        torch.cuda.set_device(local)
    side = 512
    peak_b, peak_s, peak_kind = load_bf16_peak()
    line = {"metric": "ensemble realizations/s, surrogate vs plain (512^2, judged)",
            "unit": "realizations/s", "n_gpus": ws, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 network, f64 timestep", "data": "synthetic"}
    net = pkg.Surrogate(side, side, base_channels=32, batch=32, jump=50, seed=1 + rank)
    train = None
    nsamp = args.sg_traj * args.sg_per
    if args.sg_load:
        net.load(args.sg_load)
        net.reserve(64)
        net.generate(16, 4, 400, seed=99 + rank)        # samples for the timing pass
    else:
        net.reserve(nsamp)
        t0 = time.perf_counter()
        got = net.generate(args.sg_traj, args.sg_per, args.sg_spinup, seed=2019 + rank)
        t_gen = time.perf_counter() - t0
        held = max(32, nsamp // 20)
        net.set_holdout(held)
        before = net.eval()
        curve = []
        t0 = time.perf_counter()
        done = 0
        steps_total = 0.0
        ms_total = 0.0
        chunk = max(1, args.sg_train_steps // 10)
        while done < args.sg_train_steps:
            k = min(chunk, args.sg_train_steps - done)
            frac = done / max(1, args.sg_train_steps)
            lr = args.sg_lr * (0.5 * (1 + np.cos(np.pi * frac)))  # cosine decay
            lr = max(lr, args.sg_lr * 0.02)
            loss = net.train(k, lr=float(lr))
            ms, flops = net.train_stats()
            ms_total += ms
            steps_total += k
            done += k
            curve.append({"step": done, "train_loss": loss, "heldout_loss": net.eval()})
        t_train = time.perf_counter() - t0
        uplift_only, no_change = net.eval_baselines()
        after = curve[-1]["heldout_loss"] if curve else before
        _, flops_step = net.train_stats()
        achieved = flops_step * steps_total / (ms_total * 1e-3) / 1e12
        train = {"samples": got, "heldout": held, "generate_s": t_gen, "train_s": t_train,
                 "steps": args.sg_train_steps, "batch": 32,
                 "samples_per_s": 32 * steps_total / (ms_total * 1e-3),
                 "ms_per_step": ms_total / steps_total,
                 "conv_tflops": achieved, "conv_frac_of_bf16_sustained": achieved / peak_s,
                 "heldout_loss_before": before, "heldout_loss_after": after,
                 "heldout_loss_uplift_only": uplift_only, "heldout_loss_no_change": no_change,
                 "curve": curve}
        if args.sg_save:
            net.save(args.sg_save)
    fwd_ms, fwd_flops = net.time_forward(reps=5)
    fwd_tf = fwd_flops / (fwd_ms * 1e-3) / 1e12
    ens = surrogate_ensemble(pkg, net, args.realizations, side, args.ensemble_steps, args.sg_judge,
                             2019 + rank, local)
    net.close()
    if rank == 0:
        line["value"] = ens["surrogate"]["realizations_per_s"]
        line["steps"] = args.ensemble_steps
        line["warmup"] = args.warmup
        line["ms_per_step"] = 1e3 * ens["surrogate"]["seconds"] / args.ensemble_steps
        line["config"] = {"workload": f"{args.realizations} realizations of {side}x{side}, "
                                      "K log-U[1e-6,1e-5], m U[0.3,0.6], U log-U[1e-4,5e-3], n 1, "
                                      f"{args.ensemble_steps} timesteps, 50-step jumps + 1 plain "
                                      f"timestep per cycle, {args.sg_judge:g} of jumps judged",
                          "network": "4-level conv encoder-decoder, 32-256 channels, BF16, "
                                     f"{net_param_count(pkg)} parameters"}
        line["plain_realizations_per_s"] = ens["plain"]["realizations_per_s"]
        line["surrogate_vs_plain"] = ens["ratio"]
        line["ensemble"] = ens
        line["training"] = train
        line["roofline"] = {"bound": "tensor", "kernel": "forward pass (14 tcgen05 convolutions "
                                                         "+ pooling/concat), batch 32",
                            "achieved": fwd_tf, "peak": peak_b, "unit": "TFLOP/s",
                            "frac": fwd_tf / peak_b, "ms_per_pass": fwd_ms,
                            "flops_per_pass": fwd_flops,
                            "peak_source": f"{peak_kind} bf16_tflops (burst)"}
        line["clocks"] = ens["surrogate"]["clocks"]
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def training_speed(pkg, batch, steps, local, peak_b, peak_s, peak_kind, seed=1):
    """The surrogate's training throughput at 512^2 and `batch` (Adam, on
    2*batch samples the plain method generates on the device over 0..200
    timesteps; three warm-up steps, then `steps` timed with CUDA events on the
    network's stream) and one forward pass over a batch (five passes after a
    warm-up). Returns (the network, the result dict)."""
    net = pkg.Surrogate(512, 512, base_channels=32, batch=batch, jump=50, seed=seed)
    net.reserve(2 * batch)
    net.generate(batch, 2, 200, seed=7)
    net.train(3, lr=1e-4)                      # warm-up steps
    with Clocks(local) as clk:
        net.train(steps, lr=1e-4)
    ms, flops = net.train_stats()
    tf = flops * steps / (ms * 1e-3) / 1e12
    fwd_ms, fwd_flops = net.time_forward(reps=5)
    fwd_tf = fwd_flops / (fwd_ms * 1e-3) / 1e12
    res = {
        "metric": f"surrogate training samples/s (512^2, batch {batch}, BF16 tcgen05, Adam)",
        "value": batch * steps / (ms * 1e-3), "unit": "samples/s", "steps": steps, "warmup": 3,
        "ms_per_step": ms / steps, "conv_tflops_per_step": flops / 1e12,
        "roofline": {"bound": "tensor", "kernel": "training step (14 convolutions forward, "
                                                   "data and weight gradients, and the rest)",
                     "achieved": tf, "peak": peak_s, "unit": "TFLOP/s", "frac": tf / peak_s,
                     "peak_source": f"{peak_kind} bf16_tflops_sustained"},
        "forward_pass": {"ms": fwd_ms, "flops": fwd_flops, "achieved_tflops": fwd_tf,
                         "peak": peak_b, "frac": fwd_tf / peak_b,
                         "peak_source": f"{peak_kind} bf16_tflops (burst)"},
        "data": f"{2 * batch} samples of 512^2 the plain method generated on the device "
                "(0..200 timesteps); the full 20000-sample run is --workload surrogate",
        "clocks": clk.summary()}
    return net, res


def run_conv(args, dist, rank, ws, local):
    """The surrogate's tensor-core convolutions alone: training throughput and
    one forward pass at 512^2, --sg-batch samples (no ensemble, no long
    training; a case small enough for a profiler capture at --sg-batch 8)."""
    import __graft_entry__ as ge
    import torch  # noqa: F401
    pkg = ge.load()
    if ws > 1:
        torch.cuda.set_device(local)
    peak_b, peak_s, peak_kind = load_bf16_peak()
    net, res = training_speed(pkg, args.sg_batch, args.sg_bench_steps, local, peak_b, peak_s,
                              peak_kind, seed=1 + rank)
    net.close()
    line = dict(res)
    line.update({"n_gpus": ws, "higher_is_better": True, "scaling": "weak",
                 "vs_baseline": None, "dtype": "bf16",
                 "config": {"workload": f"surrogate convolutions, 512^2, batch {args.sg_batch}, "
                                        "c 32 (1.95M parameters)",
                            "l2": "inputs larger than L2 (activations of one pass)"}})
    line["ms_per_step"] = max_over_ranks(dist, line["ms_per_step"])
    line["value"] = ws * args.sg_batch / (line["ms_per_step"] * 1e-3)
    if rank == 0:
        print(json.dumps(line), flush=True)


def surrogate_extras(pkg, args, local):
    """Configs 3 and 4 for the default run: the surrogate's training
    throughput (512^2, batch 32, Adam, on samples the plain method generates
    on the device; short, timed with CUDA events on the network's stream)
    and the judged surrogate ensemble against the plain batched method with
    the committed trained parameters (SG_WEIGHTS)."""
    peak_b, peak_s, peak_kind = load_bf16_peak()
    out = {}
    net, out["training"] = training_speed(pkg, 32, args.sg_bench_steps, local, peak_b, peak_s,
                                          peak_kind)
    if SG_WEIGHTS.exists():
        net.load(SG_WEIGHTS)
        ens = surrogate_ensemble(pkg, net, args.sg_realizations, 512, args.sg_ensemble_steps,
                                 0.05, 2019, local)
        out["ensemble"] = {
            "metric": "ensemble realizations/s, surrogate vs plain (512^2, judged)",
            "value": ens["surrogate"]["realizations_per_s"], "unit": "realizations/s",
            "plain_realizations_per_s": ens["plain"]["realizations_per_s"],
            "surrogate_vs_plain": ens["ratio"], "steps": args.sg_ensemble_steps,
            "realizations": args.sg_realizations, "parameters": SG_WEIGHTS.name,
            "detail": ens}
    else:
        out["ensemble"] = {"unavailable": f"no trained parameters at {SG_WEIGHTS.name}"}
    net.close()
    return out


def net_param_count(pkg):
    with pkg.Surrogate(512, 512, base_channels=32, batch=1) as s:
        return s.param_count()


SWEEP_SIDES = (100, 200, 400, 700, 1000, 1500, 2000, 3000, 4000, 5000, 7000, 10000,
               14000, 20000)
SWEEP_NSTEP = 120          # run(120): 121 timesteps, the reference's sweep length


def run_sweep(args, dist, rank, ws, local):
    """Size sweep mirroring the reference's scaling runs (edge 100 ... 20000,
    run(120) = 121 timesteps, reference initial field, workload constants).
    Per size: device-resident cell-steps/s (CUDA events over run(120)), the
    reference-style wall time of run(120) from the host, and the CPU
    restatement of fastscape_RB+P on a bounded sample (sizes <= 10000)."""
    import __graft_entry__ as ge
    import torch  # noqa: F401
    pkg = ge.load()
    if ws > 1:
        torch.cuda.set_device(local)
    sides = [int(s) for s in args.sizes.split(",")] if args.sizes else list(SWEEP_SIDES)
    p = pkg.workload_params()
    rows = []
    for side in sides:
        m = pkg.FastScape_RBP(side, side, params=p, init=pkg.INIT_REFERENCE, seed=123)
        m.step(args.warmup)
        m.set_timing(True)
        m.phase_times(reset=True)
        m.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        m.run(SWEEP_NSTEP)
        m.synchronize()
        wall = max_over_ranks(dist, time.perf_counter() - t0)
        t = m.phase_times(reset=True)
        dev_s = max_over_ranks(dist, float(t[3]) * 1e-3)
        nstep = SWEEP_NSTEP + 1
        nl = m.levels()[1]
        m.close()
        row = {"side": side, "cells": side * side, "timesteps": nstep, "levels": int(nl),
               "ms_per_step": 1e3 * dev_s / nstep,
               "cell_steps_per_s": ws * side * side * nstep / dev_s,
               "run_wall_s": wall,
               "run_cell_steps_per_s": ws * side * side * nstep / wall,
               "kernel_ms": {"receivers": t[0] / nstep, "donors_level0": t[1] / nstep,
                             "order": t[7] / nstep, "accum": t[9] / nstep,
                             "erode": t[8] / nstep}}
        if rank == 0 and ws == 1 and not args.no_cpu_baseline and side <= 10000:
            nst = int(max(1, min(nstep, 4e7 / (side * side))))
            v, kind, thr, _ = cpu_sample(side, nst, prefer_reference=False)
            row["cpu"] = {"cell_steps_per_s": v, "kind": kind, "cores": thr, "timesteps": nst}
        rows.append(row)
        if rank == 0:
            print(json.dumps({"sweep_row": row}), flush=True)
    if rank == 0:
        best = max(rows, key=lambda r: r["cell_steps_per_s"])
        print(json.dumps({
            "metric": "cell-steps/s by grid size (run(120), FP64)",
            "value": best["cell_steps_per_s"], "unit": UNIT, "n_gpus": ws,
            "steps": SWEEP_NSTEP + 1, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "size sweep, edge " + ",".join(map(str, sides)) +
                                   ", reference initial field, K 2e-6 m 0.4 n 1 U 2e-3 "
                                   "dt 1000 dx 100", "best_side": best["side"]},
            "sweep": rows}), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_refconst(args, dist, rank, ws, local):
    """The reference's own constants (fastscape_RB.cpp:58-65: K 2e-6, n 2,
    m 0.8, U 2e-3, dt 1000, dr {1, sqrt 2}, cell area 40000) on the 10000^2
    reference field: n = 2 runs the multi-iterate Newton erosion. Device
    cell-steps/s over --steps timesteps (CUDA events, after --warmup and the
    autotuner), with the CPU restatement of fastscape_RB+P on a bounded
    sample (2000^2, 2 timesteps) with the same constants."""
    import __graft_entry__ as ge
    import torch  # noqa: F401
    from oracle.pyoracle import Oracle, Params as OParams
    pkg = ge.load()
    if ws > 1:
        torch.cuda.set_device(local)
    side = args.side
    p = pkg.reference_params()
    m = pkg.FastScape_RBP(side, side, params=p, init=pkg.INIT_REFERENCE, seed=123)
    m.step(args.warmup)
    tune = m.autotune(probe_steps=2)
    m.set_timing(True)
    m.phase_times(reset=True)
    m.synchronize()
    barrier(dist)
    with Clocks(local) as clk:
        m.step(args.steps)
    t = m.phase_times(reset=True)
    dev_s = max_over_ranks(dist, float(t[3]) * 1e-3)
    levels = int(m.levels()[1])
    m.close()
    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            cs, nst = 2000, 2
            h = Oracle().terrain(cs, cs, 0)
            v, thr = cpu_steps_from(h, cs, OParams(*p.as_tuple()), nst)
            cpu = {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                   "sample": f"oracle restatement of fastscape_RB+P (OpenMP) with the same "
                             f"constants, {cs}^2 reference field, {nst} timesteps after 1 warm-up"}
        print(json.dumps({
            "metric": f"cell-steps/s at {side}^2 FP64, reference constants (n 2)",
            "value": ws * side * side * args.steps / dev_s, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"FastScape timestep, {side}x{side} FP64, reference initial "
                                   "field, K 2e-6 n 2 m 0.8 U 2e-3 dt 1000 dr {1, sqrt 2}",
                       "levels": levels, "launch": tune},
            "kernel_ms": {"receivers": t[0] / args.steps, "donors_level0": t[1] / args.steps,
                          "order": t[7] / args.steps, "accum": t[9] / args.steps,
                          "erode": t[8] / args.steps},
            "gpu_launches": 6 * args.steps,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }), flush=True)
    if dist is not None:
        dist.destroy_process_group()


DEEP_SIDE = 512
DEEP_SPINUP = 2000
DEEP_PARAMS = {"keq": 1e-5, "meq": 0.6, "ueq": 5e-3}


def run_deep(args, dist, rank, ws, local):
    """Long-run regime: a 512^2 grid after 2000 timesteps of strong uplift and
    erosion (K 1e-5, m 0.6, U 5e-3: ~290 levels of at most a few thousand
    cells each), where a timestep is dominated by the per-level latency of
    the three level walks rather than by bandwidth or FP64 throughput.
    Device cell-steps/s over 10 x --steps timesteps of that state (CUDA
    events; the spin-up is untimed), with the CPU restatement of
    fastscape_RB+P timed from the same elevations."""
    import __graft_entry__ as ge
    import torch  # noqa: F401
    from oracle.pyoracle import workload_params as oracle_params
    pkg = ge.load()
    if ws > 1:
        torch.cuda.set_device(local)
    side = DEEP_SIDE
    p = pkg.workload_params(**DEEP_PARAMS)
    m = pkg.FastScape_RBP(side, side, params=p, init=pkg.INIT_PHILOX, seed=7 + rank)
    m.step(DEEP_SPINUP)
    tune = m.autotune(probe_steps=2)
    m.step(args.warmup)
    nsteps = 10 * args.steps
    m.set_timing(True)
    m.phase_times(reset=True)
    m.synchronize()
    barrier(dist)
    with Clocks(local) as clk:
        m.step(nsteps)
    t = m.phase_times(reset=True)
    dev_s = max_over_ranks(dist, float(t[3]) * 1e-3)
    levels = int(m.levels()[1])
    h = m.getH()
    m.close()
    if rank == 0:
        value = ws * side * side * nsteps / dev_s
        cpu = None
        if ws == 1 and not args.no_cpu_baseline:
            nst = 20
            v, thr = cpu_steps_from(h, side, oracle_params(**DEEP_PARAMS), nst)
            cpu = {"value": v, "unit": UNIT, "cores": thr, "kind": "port",
                   "sample": f"oracle restatement of fastscape_RB+P (OpenMP) from the same "
                             f"{side}^2 state, {nst} timesteps after 1 warm-up"}
        print(json.dumps({
            "metric": f"cell-steps/s, {side}^2 after {DEEP_SPINUP} timesteps "
                      "(K 1e-5 m 0.6 U 5e-3)",
            "value": value, "unit": UNIT, "n_gpus": ws, "steps": nsteps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / nsteps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{side}x{side} FP64, Philox initial field, K 1e-5 m 0.6 "
                                   f"n 1 U 5e-3 dt 1000 dx 100, after {DEEP_SPINUP} "
                                   "untimed timesteps", "levels": levels, "launch": tune},
            "kernel_ms": {"receivers": t[0] / nsteps, "donors_level0": t[1] / nsteps,
                          "order": t[7] / nsteps, "accum": t[9] / nsteps,
                          "erode": t[8] / nsteps},
            "per_level_us": {"order": 1e3 * t[7] / nsteps / levels,
                             "accum": 1e3 * t[9] / nsteps / levels,
                             "erode": 1e3 * t[8] / nsteps / levels},
            "gpu_launches": 6 * nsteps,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--side", type=int, default=SIDE)
    ap.add_argument("--e2e-calls", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="grid",
                    choices=["grid", "ensemble", "sweep", "deep", "refconst", "surrogate",
                             "conv"],
                    help="grid: the 10000^2 timestep (default); ensemble: the ragged "
                         "256-realization batch; sweep: grid sizes 100..20000; deep: a "
                         "512^2 grid after 2000 timesteps of strong erosion (~290 levels); "
                         "refconst: the 10000^2 timestep with the reference's own "
                         "constants (n 2); surrogate: generation, training and the judged "
                         "ensemble; conv: the surrogate's convolutions alone")
    ap.add_argument("--realizations", type=int, default=256)
    ap.add_argument("--ensemble-steps", type=int, default=ENSEMBLE_STEPS,
                    help="ensemble: timesteps of the timed run (the metric's run length)")
    ap.add_argument("--ensemble-side", type=int, default=0,
                    help="ensemble: give every realization this edge instead of the ragged "
                         "draw (1024 x 512 with 2000 timesteps is the plain batched method "
                         "at the surrogate ensemble's shape)")
    ap.add_argument("--sizes", default="", help="sweep: comma-separated grid edges")
    ap.add_argument("--walk", default="auto", choices=["auto", "grid", "cta"],
                    help="ensemble: level walk (auto: the library's choice)")
    ap.add_argument("--int-sub", default="auto", choices=["auto", "0", "1"],
                    help="ensemble: erosion subtractions in integer arithmetic")
    ap.add_argument("--sg-traj", type=int, default=2000,
                    help="surrogate: realizations generating training data")
    ap.add_argument("--sg-per", type=int, default=10, help="surrogate: samples per realization")
    ap.add_argument("--sg-spinup", type=int, default=2000,
                    help="surrogate: samples spread over timesteps [0, spinup)")
    ap.add_argument("--sg-train-steps", type=int, default=2000)
    ap.add_argument("--sg-lr", type=float, default=1e-3)
    ap.add_argument("--sg-judge", type=float, default=0.05)
    ap.add_argument("--sg-save", default="", help="surrogate: write the trained parameters here")
    ap.add_argument("--sg-bench-steps", type=int, default=20,
                    help="default run and conv: timed surrogate training steps")
    ap.add_argument("--sg-batch", type=int, default=32, help="conv: samples per batch")
    ap.add_argument("--sg-realizations", type=int, default=1024,
                    help="default run: realizations of the surrogate ensemble")
    ap.add_argument("--sg-ensemble-steps", type=int, default=2000,
                    help="default run: timesteps of the surrogate ensemble")
    ap.add_argument("--no-extras", action="store_true",
                    help="default run: only the 10000^2 timestep (no ensemble or surrogate "
                         "keys)")
    ap.add_argument("--sg-load", default="",
                    help="surrogate: use these parameters (no generation or training)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")

    dist, rank, ws, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, dist, rank, ws)
        return
    if args.workload == "ensemble":
        run_ensemble(args, dist, rank, ws, local)
        return
    if args.workload == "sweep":
        run_sweep(args, dist, rank, ws, local)
        return
    if args.workload == "deep":
        run_deep(args, dist, rank, ws, local)
        return
    if args.workload == "refconst":
        run_refconst(args, dist, rank, ws, local)
        return
    if args.workload == "surrogate":
        run_surrogate(args, dist, rank, ws, local)
        return
    if args.workload == "conv":
        run_conv(args, dist, rank, ws, local)
        return

    import __graft_entry__ as ge
    pkg = ge.load()
    lib = pkg.library()
    import torch  # noqa: F401  (pinned host buffers)
    if ws > 1:
        torch.cuda.set_device(local)
    side = args.side
    p = pkg.workload_params()
    m = pkg.FastScape_RBP(side, side, params=p, init=pkg.INIT_REFERENCE, seed=123)
    h0 = m.getH()

    # ---- device-resident throughput -------------------------------------
    m.step(args.warmup)
    tune = m.autotune(probe_steps=2)      # launch shape; restores the state
    m.step(1)
    # the timed region: the launch path the autotuner chose (graph replay or
    # direct launches), CUDA events around the whole call on the model's
    # stream and none between its kernels
    m.set_timing(pkg.TIMING_CALL)
    m.phase_times(reset=True)
    barrier(dist)
    m.synchronize()
    with Clocks(local) as clk:
        m.step(args.steps)
    barrier(dist)
    total_ms = max_over_ranks(dist, float(m.phase_times(reset=True)[3]))
    # the same number of timesteps again, launched directly with an event
    # between kernels, for the per-kernel split and the roofline
    m.set_timing(pkg.TIMING_KERNELS)
    m.phase_times(reset=True)
    m.step(args.steps)
    t = m.phase_times(reset=True)
    m.set_timing(pkg.TIMING_OFF)
    split_total_ms = float(t[3])
    cells = side * side
    value = ws * cells * args.steps / (total_ms * 1e-3)
    # receivers filter + fix-up, donors/level 0, ordering, accumulation,
    # erosion: six launches a timestep
    launches = 6 * args.steps

    # ---- roofline of the dominant kernel ----------------------------------
    peak, peak_kind = load_peaks()
    kern = {"receivers": t[0], "donors_level0": t[1], "order": t[7], "accum": t[9],
            "erode": t[8]}
    dom = max(kern, key=kern.get)
    per_launch_ms = kern[dom] / args.steps
    achieved = ALG_BYTES[dom] * cells / (per_launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                "alg_bytes_per_cell": ALG_BYTES[dom], "peak_source": f"{peak_kind} hbm_gbs",
                "kernel_ms": {k: v / args.steps for k, v in kern.items()},
                "walk_split_ms": {"ordering": t[4] / args.steps,
                                  "accumulation": t[5] / args.steps,
                                  "erosion": t[6] / args.steps}}
    # the erosion kernel against the FP64 pipe (eroded cells: all but level 0)
    lid, _ = m.levels()
    eroded = int(np.count_nonzero(lid >= 1))
    del lid
    fp64_ops = erode_fp64_per_cell(bool(tune.get("erode_int_sub")))
    erode_tf = fp64_ops * eroded / (t[8] / args.steps * 1e-3) / 1e12
    roofline["erode_fp64"] = {"bound": "fp64", "achieved": erode_tf, "peak": FP64_PEAK_TFLOPS,
                              "unit": "TFLOP/s", "frac": erode_tf / FP64_PEAK_TFLOPS,
                              "ops_per_eroded_cell": fp64_ops,
                              "eroded_cells": eroded,
                              "peak_source": "probe-kernel FP64 rate (no FP64 figure in "
                                             "MEASURED_PEAKS.json)"}
    step_rf = cells * args.steps / (total_ms * 1e-3) * STEP_ALG_BYTES / 1e9
    prof = ROOT / "profiles" / "traffic.json"
    if prof.exists():
        try:
            tr = json.loads(prof.read_text())
            if dom in tr:   # ncu DRAM bytes per cell of the 4000^2 capture x cells
                roofline["traffic"] = tr[dom]["bytes_per_cell"] * cells
        except (ValueError, KeyError):
            pass

    # ---- end to end through the reference-facing calls ------------------
    hbuf_t, hbuf = pinned_buffer(cells)
    obuf_t, obuf = pinned_buffer(cells)
    hbuf[:] = h0
    dp = C.POINTER(C.c_double)
    hptr = hbuf.ctypes.data_as(dp)
    optr = obuf.ctypes.data_as(dp)
    pkg.check(lib.fs_set_elevation(m.handle, hptr))   # warm-up of the e2e path
    pkg.check(lib.fs_run(m.handle, RUN_NSTEP))
    pkg.check(lib.fs_get_elevation(m.handle, optr))
    call_s = []
    for _ in range(args.e2e_calls):
        barrier(dist)
        t0 = time.perf_counter()
        pkg.check(lib.fs_set_elevation(m.handle, hptr))
        pkg.check(lib.fs_run(m.handle, RUN_NSTEP))
        pkg.check(lib.fs_get_elevation(m.handle, optr))
        call_s.append(max_over_ranks(dist, time.perf_counter() - t0))
    e2e_s = statistics.median(call_s)   # one call; host-side jitter is not the library's
    e2e_value = ws * cells * (RUN_NSTEP + 1) / e2e_s
    checksum = float(np.sum(obuf))
    m.close()

    # ---- CPU baseline (rank 0, N = 1 only) --------------------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        v, kind, thr, desc = cpu_sample(side, args.cpu_steps, prefer_reference=False)
        cpu = {"value": v, "unit": UNIT, "cores": thr, "kind": kind, "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": grid_config(side),
            "parallelism": "replicas" if ws > 1 else "single GPU",
            "launch": dict(tune, timed_region="graph replay" if tune.get("graph")
                           else "direct launches",
                           kernel_split="direct launches with events between kernels, "
                                        f"{args.steps} more timesteps",
                           kernel_split_ms_per_step=split_total_ms / args.steps),
            "roofline": roofline,
            "step_roofline": {"alg_bytes_per_cell_step": STEP_ALG_BYTES,
                              "achieved_gbs": step_rf, "frac": step_rf / peak},
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": 8 * cells / (RUN_NSTEP + 1),
                    "d2h_bytes_per_step": 8 * cells / (RUN_NSTEP + 1),
                    "step": "one timestep; a call is fs_set_elevation + "
                            f"fs_run({RUN_NSTEP}) ({RUN_NSTEP + 1} timesteps) + "
                            "fs_get_elevation",
                    "h2d_bytes_per_call": 8 * cells, "d2h_bytes_per_call": 8 * cells,
                    "calls": args.e2e_calls, "call_ms": [1e3 * x for x in call_s],
                    "statistic": "median call", "checksum": checksum},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        if ws == 1 and not args.no_extras:
            # the ensemble half of the metric: the 256-realization ragged
            # ensemble (200 timesteps) and the surrogate against the plain
            # batched method, each with its own clock record
            line["ensemble_ragged"] = ensemble_result(pkg, 256, 0, ENSEMBLE_STEPS, 2019, 0, 1,
                                                      None, local)
            line["surrogate"] = surrogate_extras(pkg, args, local)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
