"""The reference-style command-line program: same arguments, same tagged
stdout lines, and a DEM file byte-identical to the one the reference's own
PrintDEM writes for the same run (tests/golden/dem_*.dem, produced by the
reference; compare.sh's comparison, done byte for byte instead of to
printed precision)."""
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
CLI = ROOT / "barnes2019-landscape_gb300" / "bin" / "fastscape_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("golden,args", [
    ("dem_refconst_40_30.dem", ["40", "30"]),
    ("dem_workload_33_25.dem", ["33", "25", "--workload"]),
])
def test_cli_dem_matches_reference(tmp_path, golden, args):
    assert CLI.exists(), "CLI not built"
    out = tmp_path / "out.dem"
    cmd = [str(CLI), args[0], args[1], str(out), "123"] + args[2:]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert out.read_bytes() == (GOLDEN / golden).read_bytes()
    lines = r.stdout.splitlines()
    tags = {ln[0] for ln in lines if ln}
    assert {"A", "C", "h", "m", "p", "t"} <= tags
    steps = [int(ln.split("=")[1]) for ln in lines if ln.startswith("p Step")]
    nstep = int(args[1])
    assert steps == list(range(0, nstep + 1, 20))
    # the reference's timer columns, as its tests/d.make_tabular names them
    # (tag, then the name with ':' dropped and spaces as '_')
    cols = {}
    for ln in lines:
        if ln.startswith("t ") and "=" in ln:
            name, val = ln[2:].split("=", 1)
            cols[name.strip().replace(":", "").replace(" ", "_")] = val.split()[0]
    want = ["Step1_Initialize", "Step2_DetermineReceivers", "Step3_DetermineDonors",
            "Step4_GenerateOrder", "Step5_FlowAcc", "Step6_Uplift", "Step7_Erosion",
            "Overall"]
    assert all(c in cols for c in want), sorted(cols)
    assert all(int(cols[c]) >= 0 for c in want)
    assert int(cols["Step7_Erosion"]) > 0 and int(cols["Step6_Uplift"]) == 0


def test_cli_usage_error():
    r = subprocess.run([str(CLI), "10"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "Syntax" in r.stderr
