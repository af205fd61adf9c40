"""The N > 1 path of bench.py on the CPU (gloo, world size 2).

A transpose does not shard, so N GPUs run N independent replicas; what
crosses ranks is only the barrier around the timed region and the maximum
of the per-rank times.  These tests run those helpers in two gloo processes,
and run the reference arm under torchrun with two ranks (rank 0 alone works
and prints the single JSON line; the other rank exits 0).
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench

    r, _, w = bench.dist_setup(world)
    assert (r, w) == (rank, world)
    bench.barrier(w)
    m = bench.max_over_ranks(1.5 + r, w)
    Path(out_dir, f"rank{r}.txt").write_text(repr(m))
    bench.barrier(w)


def test_barrier_and_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("exercises the CPU (gloo) path")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_replica, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert [float((tmp_path / f"rank{r}.txt").read_text()) for r in (0, 1)] == [2.5, 2.5]


def test_reference_arm_two_ranks():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("exercises the CPU (gloo) path")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "c1", "--steps", "2", "--warmup", "1"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(x) for x in res.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
