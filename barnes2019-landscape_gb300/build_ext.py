"""Builds the CUDA library of the package in-tree.

Compiles every ``csrc/*.cu`` for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``) with ``-fmad=false`` (the timestep must
not contract multiply-adds, to keep the reference's rounding) and links
``lib/libfastscape_gb300.so`` with the CUDA runtime linked statically.
Objects go to ``_build/`` next to this file. Translation units compile in
parallel. Also builds ``bin/fastscape_gb300``, the command-line program with
the reference's interface. Usage: ``python build_ext.py [--force] [--verbose]``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libfastscape_gb300.so"
BINDIR = PKG / "bin"
CLI = BINDIR / "fastscape_gb300"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def cflags(verbose: bool = False) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17",
                "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    hdrs = _headers() + [Path(__file__)]
    jobs = []
    objs = []
    for src in sources:
        obj = OBJ / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc()] + cflags(verbose) + ["-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for msg in ex.map(compile_one, jobs):
            if verbose and msg:
                sys.stderr.write(msg)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + \
              ["-Xcompiler", "-fPIC", "-lpthread"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    build_cli(force)
    return LIB


def build_cli(force: bool = False) -> Path:
    """The reference-style command-line program, linked to the library."""
    BINDIR.mkdir(exist_ok=True)
    src = CSRC / "fs_cli.cpp"
    deps = [src, LIB, ROOT / "include" / "fastscape_gb300.hpp", ROOT / "include" / "fastscape_gb300.h"]
    if not force and not _stale(CLI, deps):
        return CLI
    tmp = CLI.with_suffix(".tmp")
    cmd = ["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(src), "-o", str(tmp),
           f"-L{LIBDIR}", "-lfastscape_gb300", "-Wl,-rpath,$ORIGIN/../lib"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
