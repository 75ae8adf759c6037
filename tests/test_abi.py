"""CPU-side checks of the C-ABI library: it loads, exports every function
the public headers declare, and validates arguments before touching the GPU.
No timestep runs here."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
DECL = re.compile(r"^[A-Za-z_][\w\s\*]*?\b(fs_\w+)\s*\(", re.M)


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += DECL.findall(text)
    return names


def test_headers_declare_functions():
    names = declared_functions()
    assert "fs_create" in names and "fs_run" in names and "fs_get_elevation" in names


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"symbols declared but not exported: {missing}"
    assert sorted(set(declared_functions())) == sorted(set(pkg.ABI_SYMBOLS))


def test_version(pkg):
    assert "sm_103a" in pkg.version()


def test_parameter_presets(pkg):
    lib = pkg.library()
    p = pkg.Params()
    lib.fs_params_reference(C.byref(p))
    assert p.as_tuple() == pkg.reference_params().as_tuple()
    assert p.as_tuple() == (2e-6, 2.0, 0.8, 2e-3, 1000.0, 1.0, pkg.SQRT2, 1e-3, 40000.0)
    lib.fs_params_workload(C.byref(p), 100.0)
    assert p.as_tuple() == pkg.workload_params().as_tuple()
    assert p.dr_diag == 100.0 * pkg.SQRT2 and p.cell_area == 1e4


@pytest.mark.parametrize("w,h", [(2, 10), (10, 2), (0, 0), (-5, 7), (50000, 50000)])
def test_create_rejects_bad_shapes_before_any_cuda_call(pkg, w, h):
    lib = pkg.library()
    st = C.c_int(0)
    m = lib.fs_create(w, h, None, 1, 0, C.byref(st))
    assert not m and st.value == -1
    assert "width" in pkg.last_error() or "exceeds" in pkg.last_error()


def test_null_model_is_an_argument_error(pkg):
    lib = pkg.library()
    assert lib.fs_run(None, 3) == -1
    assert lib.fs_step(None, 1) == -1
    assert lib.fs_get_elevation(None, None) == -1
    assert lib.fs_steps_executed(None) == -1
    lib.fs_destroy(None)


def test_bad_params_rejected(pkg):
    lib = pkg.library()
    p = pkg.workload_params()
    p.dr_orth = 0.0
    st = C.c_int(0)
    assert not lib.fs_create(10, 10, C.byref(p), 1, 0, C.byref(st))
    assert st.value == -1
    p = pkg.workload_params()
    p.keq = float("nan")
    assert not lib.fs_create(10, 10, C.byref(p), 1, 0, C.byref(st))
    assert st.value == -1
    assert not lib.fs_create(10, 10, None, 7, 0, C.byref(st))
    assert st.value == -1


def test_python_mirror_matches_reference_interface(pkg):
    cls = pkg.FastScape_RBP
    for name in ("run", "getH"):
        assert callable(getattr(cls, name))
