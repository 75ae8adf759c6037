"""Generates the golden fixtures in tests/golden/ from the reference itself.

The reference has no golden vectors or known-answer tests of its own (its
only check is compare.sh, which diffs whole DEMs at 6 significant digits).
This script runs the reference's own FastScape_RB / FastScape_RBP classes,
compiled from its sources by oracle/build.py into oracle/_ref/, and records
every intermediate of a few timesteps for small grids:

  h0        initial field (the reference's own generator, random.cpp)
  rec_s, ndon_s, donor_s, stack_s, levels_s, accum_s, hup_s, h_s
            receivers, donor counts and lists, stack, level offsets,
            accumulation, uplifted and eroded elevation after timestep s

plus end-of-run elevations of the reference's own run() (nstep+1 timesteps)
and hand-built known-answer grids (tilted plane, single pit, tie cases).
Run it where the reference tree is available:

    python oracle/build.py --ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle.pyoracle import REFERENCE_PARAMS, Params, RefHarness, workload_params  # noqa: E402


def record(model, nsteps):
    out = {"h0": model.get_h()}
    for s in range(nsteps):
        r = model.phases()
        out[f"rec_{s}"] = r["rec"].astype(np.int8)
        out[f"ndon_{s}"] = r["ndon"].astype(np.int8)
        out[f"donor_{s}"] = r["donor"].astype(np.int32)
        out[f"stack_{s}"] = r["stack"].astype(np.int32)
        out[f"levels_{s}"] = r["levels"].astype(np.int32)
        out[f"accum_{s}"] = r["accum"]
        out[f"hup_{s}"] = r["h_uplifted"]
        out[f"h_{s}"] = r["h"]
    return out


def params_array(p: Params):
    return np.array(p.as_tuple(), np.float64)


def known_answer_fields():
    """Hand-built inputs: name -> (W, H, h)."""
    cases = {}
    W, H = 9, 8
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    # tilted plane rising to the east: every interior cell drains west
    h = 0.5 * xx + 0.01 * yy
    h[:2, :] = 0; h[-2:, :] = 0; h[:, :2] = 0; h[:, -2:] = 0
    cases["plane"] = (W, H, h.reshape(-1).copy())
    # single pit in a dome: the centre is NO_FLOW, neighbours drain into it
    W, H = 9, 9
    h = np.full((H, W), 5.0)
    h[4, 4] = 1.0
    h[:2, :] = 0; h[-2:, :] = 0; h[:, :2] = 0; h[:, -2:] = 0
    cases["pit"] = (W, H, h.reshape(-1).copy())
    # exact ties between neighbours: first in neighbour order must win
    W, H = 7, 7
    h = np.full((H, W), 3.0)
    h[3, 3] = 4.0          # centre: equal drop to all orthogonal neighbours
    h[2, 2] = 2.0; h[2, 4] = 2.0   # tie between NW and NE diagonals
    h[:2, :] = 0; h[-2:, :] = 0; h[:, :2] = 0; h[:, -2:] = 0
    cases["ties"] = (W, H, h.reshape(-1).copy())
    # flat interior: every interior cell equals its neighbours except rings
    W, H = 8, 6
    h = np.full((H, W), 1.0)
    h[:2, :] = 0; h[-2:, :] = 0; h[:, :2] = 0; h[:, -2:] = 0
    cases["flat"] = (W, H, h.reshape(-1).copy())
    return cases


def main():
    pristine = RefHarness("pristine", "exact")
    param = RefHarness("param", "exact")
    wl = workload_params()
    written = []

    def save(name, **arrays):
        path = HERE / f"{name}.npz"
        np.savez_compressed(path, **arrays)
        written.append(path)

    # per-timestep intermediates
    for name, hr, p, W, H, ns, variant in [
        ("refconst_32x32", pristine, REFERENCE_PARAMS, 32, 32, 4, 0),
        ("refconst_rbp_23x31", pristine, REFERENCE_PARAMS, 23, 31, 3, 1),
        ("workload_40x48", param, wl, 40, 48, 4, 0),
        ("workload_rbp_57x19", param, wl, 57, 19, 3, 1),
        ("workload_5x5", param, wl, 5, 5, 3, 0),
        ("workload_6x9", param, wl, 6, 9, 3, 0),
    ]:
        m = hr.model(W, H, p, variant)
        rec = record(m, ns)
        save(name, W=W, H=H, nsteps=ns, variant=variant, params=params_array(p), **rec)

    # whole runs through the reference's own run(): nstep+1 timesteps
    for name, hr, p, W, nstep, variant in [
        ("run_refconst_64", pristine, REFERENCE_PARAMS, 64, 120, 0),
        ("run_workload_64", param, wl, 64, 120, 1),
        ("run_workload_101", param, wl, 101, 40, 0),
    ]:
        m = hr.model(W, W, p, variant)
        h0 = m.get_h()
        m.run(nstep)
        save(name, W=W, H=W, nstep=nstep, variant=variant, params=params_array(p),
             h0=h0, h_final=m.get_h())

    # known-answer grids, one timestep, both constant sets
    for kname, (W, H, h) in known_answer_fields().items():
        for pname, hr, p in (("refconst", pristine, REFERENCE_PARAMS), ("workload", param, wl)):
            m = hr.model(W, H, p, 0)
            m.set_h(h)
            rec = record(m, 2)
            save(f"known_{kname}_{pname}", W=W, H=H, nsteps=2, variant=0,
                 params=params_array(p), **rec)

    # the reference's own DEM output (PrintDEM after run(nstep)), as its CLI
    # writes it: compare.sh's artefact
    for name, hr, p, W, nstep in [("dem_refconst_40_30", pristine, REFERENCE_PARAMS, 40, 30),
                                  ("dem_workload_33_25", param, wl, 33, 25)]:
        m = hr.model(W, W, p, 0)
        m.run(nstep)
        path = HERE / f"{name}.dem"
        m.print_dem(path)
        written.append(path)

    # the reference's own generator stream: first draws of the field for
    # seeds that seed_rand turns into engine seed 0
    m = pristine.model(16, 16, REFERENCE_PARAMS, 0, seed=999)
    save("terrain_seed999_16x16", W=16, H=16, h=m.get_h())

    total = sum(p.stat().st_size for p in written)
    print(f"wrote {len(written)} fixtures, {total / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
