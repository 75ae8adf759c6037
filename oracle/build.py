"""Build recipe for the oracle (test infrastructure only).

Two products:

* ``oracle/_build/libfsoracle.so`` -- the C restatement
  (``oracle/fastscape_oracle.c``), compiled with ``-O3 -ffp-contract=off
  -fopenmp``. Built on every machine, including the GPU host, because the
  parity tests and the CPU baseline use it.

* ``oracle/_ref/libfsref_<text>_<flags>.so`` -- the reference's own
  ``FastScape_RB`` / ``FastScape_RBP`` classes, compiled from the reference
  sources where they lie (``$FS_REFERENCE_DIR``, default ``/root/reference``)
  together with ``oracle/ref_harness.cpp``. Only built where the reference
  tree exists. ``text`` is ``pristine`` (reference text unchanged) or
  ``param`` (the eight constants of fastscape_RB.cpp:58-65 read from a
  settable array); ``flags`` is ``exact`` (-O3 -ffp-contract=off, the
  parity build) or ``shipped`` (Makefile:4's -O3 -march=native -g, for
  timing only). The translation unit is assembled in memory and piped to
  g++; no copy of the reference sources is written anywhere.

Usage: ``python oracle/build.py [--ref]``.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_SO = BUILD_DIR / "libfsoracle.so"


def reference_dir() -> Path:
    return Path(os.environ.get("FS_REFERENCE_DIR", "/root/reference"))


def _newer(target: Path, *sources: Path) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in sources if s.exists())


def build_oracle(force: bool = False) -> Path:
    """Compile the C restatement into oracle/_build/libfsoracle.so."""
    src = HERE / "fastscape_oracle.c"
    hdr = HERE / "fastscape_oracle.h"
    if not force and _newer(ORACLE_SO, src, hdr, Path(__file__)):
        return ORACLE_SO
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = ORACLE_SO.with_suffix(".so.tmp")
    cmd = ["gcc", "-std=c11", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC",
           "-shared", "-Wall", "-Wextra", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


# --- reference harness ------------------------------------------------------

_CONST_PATCHES = [
    (r"(const double keq\s*=\s*)[^;]+;", r"\1fsref_p[0];"),
    (r"(const double neq\s*=\s*)[^;]+;", r"\1fsref_p[1];"),
    (r"(const double meq\s*=\s*)[^;]+;", r"\1fsref_p[2];"),
    (r"(const double ueq\s*=\s*)[^;]+;", r"\1fsref_p[3];"),
    (r"(const double dt\s*=\s*)[^;]+;", r"\1fsref_p[4];"),
    (r"(const double dr\[8\]\s*=\s*)\{[^}]*\};",
     r"\1{fsref_p[5],fsref_p[6],fsref_p[5],fsref_p[6],"
     r"fsref_p[5],fsref_p[6],fsref_p[5],fsref_p[6]};"),
    (r"(const double tol\s*=\s*)[^;]+;", r"\1fsref_p[7];"),
    (r"(const double cell_area\s*=\s*)[^;]+;", r"\1fsref_p[8];"),
]


def _patch_constants(text: str, name: str) -> str:
    for pat, rep in _CONST_PATCHES:
        text, n = re.subn(pat, rep, text)
        if n != 1:
            raise RuntimeError(f"constant patch {pat!r} matched {n}x in {name}")
    return text


def _translation_unit(ref: Path, param: bool) -> str:
    harness = (HERE / "ref_harness.cpp").read_text()
    pre_start = harness.index("//@@PRELUDE")
    drv_start = harness.index("//@@DRIVER")
    prelude = harness[pre_start:drv_start]
    driver = harness[drv_start:]
    drv_line = harness[:drv_start].count("\n") + 1
    parts = []
    if param:
        parts.append("#define FSREF_PARAM_BUILD 1\n")
    parts.append(f'#line {harness[:pre_start].count(chr(10)) + 1} "{HERE / "ref_harness.cpp"}"\n')
    parts.append(prelude)
    for ns, fname in (("fsref_rb", "fastscape_RB.cpp"), ("fsref_rbp", "fastscape_RB+P.cpp"),
                      ("fsref_bw", "fastscape_BW.cpp")):
        text = (ref / fname).read_text()
        if param:
            text = _patch_constants(text, fname)
        parts.append(f"namespace {ns} {{\n#line 1 \"{ref / fname}\"\n")
        parts.append(text)
        parts.append("\n}\n")
    parts.append(f'#line {drv_line} "{HERE / "ref_harness.cpp"}"\n')
    parts.append(driver)
    return "".join(parts)


def build_ref(force: bool = False) -> list[Path]:
    """Compile the reference harness variants into oracle/_ref/."""
    ref = reference_dir()
    if not (ref / "fastscape_RB.cpp").exists():
        return []
    REF_OUT.mkdir(exist_ok=True)
    sources = [ref / "fastscape_RB.cpp", ref / "fastscape_RB+P.cpp", ref / "fastscape_BW.cpp",
               ref / "random.cpp", ref / "CumulativeTimer.cpp",
               HERE / "ref_harness.cpp", Path(__file__)]
    flagsets = {
        "exact": ["-O3", "-ffp-contract=off"],
        "shipped": ["-O3", "-march=native", "-g"],
    }
    outs = []
    procs = []
    for text in ("pristine", "param"):
        tu = _translation_unit(ref, text == "param")
        for fl_name, fl in flagsets.items():
            out = REF_OUT / f"libfsref_{text}_{fl_name}.so"
            outs.append(out)
            if not force and _newer(out, *sources):
                continue
            tmp = out.with_suffix(".so.tmp")
            cmd = (["g++", "-std=c++14"] + fl +
                   ["-fopenmp", "-fPIC", "-shared", "-w",
                    f"-I{ref}", '-DGIT_HASH="reference"',
                    '-DCOMPILE_TIME="reference"',
                    "-o", str(tmp), "-x", "c++", "-",
                    str(ref / "random.cpp"), str(ref / "CumulativeTimer.cpp")])
            p = subprocess.Popen(cmd, stdin=subprocess.PIPE)
            procs.append((p, tu, tmp, out))
    for p, tu, tmp, out in procs:
        p.communicate(tu.encode())
        if p.returncode != 0:
            raise RuntimeError(f"reference harness build failed for {out.name}")
        os.replace(tmp, out)
    return outs


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    if "--ref" in sys.argv:
        for o in build_ref(force="--force" in sys.argv):
            print(o)
