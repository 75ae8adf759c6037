"""The erosion kernels' quotients replayed on the host: the n = 1 form with a
tabled reciprocal (neg_div_rn_bits: one FP64 multiplication, rounding from
the exact integer residual), its earlier fused multiply-add form, and the
n = 2 form for any denominator (fdiv_rn_bits: FP32 seed, one Newton step,
round_quotient_bits from fs_bits.h, the function the kernels compile). Every
quotient a form accepts must equal the IEEE division, on random operands and
on operands next to rounding midpoints. The GPU parity tests check the
device code itself bit for bit against the oracle."""
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
