"""The kernels' integer-arithmetic operations (csrc/fs_bits.h, the same
source the kernels compile) checked on the host: the erosion's additions and
subtractions of elevations against the hardware's RN operations, the second
Newton iterate's FP32 step decision against the exact iterate, the
receiver filter's fixed-point staging of high ground against its error
bound, and the filter's decisions (restated in FP32 on the host) against the
FP64 reference formula. The GPU parity tests check the device results bit
for bit against the oracle."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_uplift_add_matches_hardware(tmp_path):
    exe = tmp_path / "uplift_add_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "barnes2019-landscape_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "uplift_add_check.cpp"), "-o", str(exe)],
                   check=True)
    for seed in (1, 2, 3):
        out = subprocess.run([str(exe), "5000000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "all equal to the hardware operation" in out.stdout


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_second_iterate_step_decision(tmp_path):
    """fs::newton_step_in_spacing: the second Newton iterate decided from an
    FP32 quotient (perturbed by +-2^-20) equals the exact double iterate."""
    exe = tmp_path / "newton_step_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "barnes2019-landscape_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "newton_step_check.cpp"), "-o", str(exe)],
                   check=True)
    for seed in (1, 2):
        out = subprocess.run([str(exe), "3000000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "all decisions equal to the exact iterate" in out.stdout


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_high_ground_staging_bound(tmp_path):
    """fs::fixed_in_binade: a tile of high ground staged relative to its
    first value, f = RN32(X - X_ref) * u, is within 2^-24 |h - X_ref u| + 1.01 u
    of the exact relative height (checked in 128-bit integers)."""
    exe = tmp_path / "tile_fixed_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "barnes2019-landscape_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "tile_fixed_check.cpp"), "-o", str(exe)],
                   check=True)
    for seed in (1, 2, 3):
        out = subprocess.run([str(exe), "2000000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "all within the staging bound" in out.stdout


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_receiver_filter_decisions(tmp_path):
    """The receiver filter's FP32 decisions, restated operation for operation
    on the host with both stagings (truncated; relative to the tile's first
    cell with a per-cell bound), never differ from the FP64 reference formula
    on cells they settle -- over random terrain with planted near-ties,
    ties, jumps to base level and special values."""
    exe = tmp_path / "filter_bound_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "barnes2019-landscape_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "filter_bound_check.cpp"), "-o", str(exe)],
                   check=True)
    for seed in (1, 2):
        out = subprocess.run([str(exe), "30000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "all decisions exact" in out.stdout
