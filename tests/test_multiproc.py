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


def test_partition_systems_is_contiguous_complete_and_balanced():
    """The batching form's shards: contiguous system ranges covering every
    system once, the largest rank cost (sum of N log2 N) within total /
    world + the largest system's cost."""
    from astro_gb300 import shard

    import numpy as np

    rng = np.random.default_rng(1004)
    # 256 systems, log-uniform in [1024, 65536] (the batching workload's law).
    sizes = np.exp(rng.uniform(np.log(1024), np.log(65536), 256)).astype(int)
    costs = [shard.system_cost(s) for s in sizes]
    for world in (1, 2, 3, 4, 8):
        ranges = shard.partition_systems(sizes, world)
        assert len(ranges) == world
        assert ranges[0][0] == 0 and ranges[-1][1] == len(sizes)
        assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
        worst = max(shard.rank_cost(sizes, r) for r in ranges)
        assert worst <= sum(costs) / world + max(costs)
    # Fewer systems than ranks: the extra ranks get empty ranges.
    assert shard.partition_systems([10, 20], 4) == [(0, 1), (1, 2), (2, 2), (2, 2)]
    assert shard.particle_range([10, 20, 30], (1, 3)) == (10, 60)


def _shard_worker(rank, world, port, out_dir):
    import numpy as np
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), OMP_NUM_THREADS="2")
    sys.path.insert(0, str(ROOT))
    from astro_gb300 import ic, layouts as L, shard
    from oracle import oracle as orc

    ic.use_generator_library(orc.lib())
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes, scales = ic.system_sizes(9, 77, 300, 3000)
        pm, vr, _ = ic.plummer_batch(9, 77, 300, 3000)
        p = L.host_default_params(L.PRESET_PHYSICAL, lbits=8, softening=0.01, far_ratio=0.2)
        rng = shard.partition_systems(sizes, world)[rank]
        a, b = shard.particle_range(sizes, rng)
        mine = [int(s) for s in sizes[rng[0]:rng[1]]]
        pm_r, vr_r = pm[a:b].copy(), vr[a:b].copy()
        out = orc.phys_run(p, pm_r, vr_r, sizes=mine, dt=1e-3, steps=2) if mine else None
        acc = out["acc4"] if out is not None else np.zeros((0, 4), np.float32)
        gathered = [None] * world
        dist.all_gather_object(gathered, (rank, acc, pm_r, vr_r))
        if rank == 0:
            gathered.sort(key=lambda t: t[0])
            np.savez(Path(out_dir, "sharded.npz"),
                     acc=np.concatenate([g[1] for g in gathered]),
                     pm=np.concatenate([g[2] for g in gathered]),
                     vr=np.concatenate([g[3] for g in gathered]))
    finally:
        dist.destroy_process_group()


def test_sharded_batch_concatenates_to_the_single_rank_result(tmp_path):
    """Two gloo ranks each step their own contiguous range of systems with
    the CPU restatement (no exchange); their results, concatenated, are the
    single-rank batched step's bit for bit."""
    import numpy as np
    import torch.multiprocessing as mp

    sys.path.insert(0, str(ROOT))
    from astro_gb300 import ic, layouts as L
    from oracle import oracle as orc

    mp.spawn(_shard_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    got = np.load(tmp_path / "sharded.npz")
    ic.use_generator_library(orc.lib())
    try:
        sizes, _ = ic.system_sizes(9, 77, 300, 3000)
        pm, vr, _ = ic.plummer_batch(9, 77, 300, 3000)
    finally:
        ic.use_generator_library(None)
    p = L.host_default_params(L.PRESET_PHYSICAL, lbits=8, softening=0.01, far_ratio=0.2)
    orc.set_threads(2)
    ref = orc.phys_run(p, pm, vr, sizes=[int(s) for s in sizes], dt=1e-3, steps=2)
    assert np.array_equal(got["acc"], ref["acc4"])
    assert np.array_equal(got["pm"], pm) and np.array_equal(got["vr"], vr)
