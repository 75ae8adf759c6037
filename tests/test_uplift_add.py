"""The erosion kernel's integer uplift addition (fs::add_pos_rn_bits in
csrc/fs_bits.h, the same source the kernel compiles) checked on the host
against the hardware's RN addition: random operands at every exponent
difference, sums next to rounding ties, carries through the rounding,
overflow to +Inf, and the operand filter. The GPU parity tests check the
device results bit for bit against the oracle."""
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
