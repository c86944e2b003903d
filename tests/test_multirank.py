"""The multi-rank path of bench.py on CPU: world size 2 over gloo.

The time-stepping path runs as independent replicas, one per GPU (no collective on the
data path); the ranks only meet at the timing barriers and in the max-over-ranks of the
measured times, and rank 0 alone prints.  These tests run that host logic as two CPU
processes.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    w, r, local = bench.dist_setup(None)
    bench.barrier(w)
    m = bench.allmax(w, 10.0 * r + 1.0)  # max over ranks of each rank's time
    bench.barrier(w)
    Path(out_dir, f"rank{r}.json").write_text(json.dumps({"world": w, "rank": r, "local": local, "max": m}))
    dist.destroy_process_group()


def test_timing_helpers_two_ranks(tmp_path):
    """dist_setup joins a gloo group from the torchrun variables, barrier returns on both
    ranks, allmax gives every rank the maximum."""
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    assert [g["rank"] for g in got] == [0, 1] and all(g["world"] == 2 for g in got)
    assert all(g["max"] == 11.0 for g in got)


def test_reference_arm_two_ranks_prints_once():
    """Under torchrun with two ranks the reference arm runs on rank 0 alone and prints one
    JSON line; the other rank exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--cpu-sample", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(l) for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
