"""The benchmark's multi-rank path on CPU (gloo, world size 2): the max over
ranks of the timed region and the barrier, and the reference arm launched by
torchrun, where rank 0 alone runs and prints."""
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


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        got = bench.reduce_max(float(10 * (rank + 1)), world)
        Path(out_dir, f"rank{rank}.txt").write_text(repr(got))
    finally:
        dist.destroy_process_group()


def test_reduce_max_and_barrier_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    assert [float((tmp_path / f"rank{r}.txt").read_text()) for r in range(2)] == [20.0, 20.0]


def test_reference_arm_under_torchrun_prints_once(tmp_path):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--workload", "c1", "--steps", "1", "--warmup", "0",
           "--cpu-threads", "2", "--gpus", "2"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
