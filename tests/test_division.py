"""The erosion kernel's three-operation quotient (neg_div_rn_bits) replayed
on the host: every quotient its fast path accepts must equal the IEEE
division, on random operands and on operands next to rounding midpoints.
The GPU parity tests check the device code itself bit for bit against the
oracle."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fast_quotient_matches_ieee(tmp_path):
    exe = tmp_path / "division_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    str(ROOT / "tests" / "native" / "division_check.cpp"), "-o", str(exe)],
                   check=True)
    for seed in (1, 2, 3):
        out = subprocess.run([str(exe), "3000000", str(seed)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "all equal to the IEEE quotient" in out.stdout
