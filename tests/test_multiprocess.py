"""The N > 1 launch path of bench.py on CPU: world_size-2 gloo ranks.

A single grid does not shard ("replicas only"); what N ranks share is the
rendezvous, the barriers around the timed region and the max over ranks of
the timings. These run here on CPU with the gloo backend; the GPU arms only
add the per-rank device.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _max_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    dist, r, ws, _ = bench.dist_setup()
    assert (r, ws) == (rank, world)
    bench.barrier(dist)
    q.put((rank, bench.max_over_ranks(dist, 1.5 + rank)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 2.5, 1: 2.5}


def test_reference_arm_under_torchrun():
    """Rank 0 alone runs the CPU reference timestep and prints one line; the
    other rank exits 0 without work."""
    pytest.importorskip("torch")
    lib = ROOT / "oracle" / "_build" / "libfsoracle.so"
    if not lib.exists():
        pytest.skip("oracle not built")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
           "--side", "48", "--steps", "1", "--warmup", "3"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(line) for line in out.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
